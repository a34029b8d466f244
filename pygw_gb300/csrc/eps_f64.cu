// Dielectric build and inverse per frequency, FP64 (the comparator path).
//
// Restates the ε block of MatrixElements2Band.calc_eps (pygw.py:3229-3271):
//     eps = (eps + epsᴴ)/2 ; eps += I ; eps = inv(eps)
//     if q = 0: bw1 = eps·epsw1 ; w2b = conj(eps·epsw2) ; ww = epsw2·bw1
//               head = 1/(1 + head − ww) ; epsw1 = −head·bw1 ; epsw2 = −head·w2b
//               eps += head·outer(bw1, w2b) ; head −= 1
//     eps −= I
// The inverse is an in-place Gauss–Jordan elimination with partial pivoting
// (pivot = largest |Re|+|Im| in the column, first on ties — LAPACK's getrf
// rule), one frequency per grid slice, three launches per pivot step.
// Layout: eps[I + N*J + N*N*ω] (the reference's Fortran-ordered array).
#include <cuda_runtime.h>
#include <stdint.h>
#include "pygw_status.h"
#include "launches.h"
#include "eps_internal.h"

namespace pge {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 crecip(double2 a) {
  // Smith's algorithm for 1/a.
  if (fabs(a.x) >= fabs(a.y)) {
    const double r = a.y / a.x, d = a.x + a.y * r;
    return make_double2(1.0 / d, -r / d);
  } else {
    const double r = a.x / a.y, d = a.x * r + a.y;
    return make_double2(r / d, -1.0 / d);
  }
}

// eps ← (eps + epsᴴ)/2 + I
__global__ void k_sym_add_identity(double2* eps, int N) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y;
  const int w = blockIdx.z;
  if (I >= N || I > J) return;
  double2* E = eps + (size_t)N * N * w;
  const double2 a = E[(size_t)I + (size_t)N * J];
  const double2 b = E[(size_t)J + (size_t)N * I];
  double2 v = make_double2((a.x + b.x) / 2.0, (a.y - b.y) / 2.0);
  if (I == J) {
    v.y = 0.0 * v.y;  // (x + conj x)/2 has a zero imaginary part
    v.x += 1.0;
    E[(size_t)I + (size_t)N * I] = v;
  } else {
    E[(size_t)I + (size_t)N * J] = v;
    E[(size_t)J + (size_t)N * I] = make_double2(v.x, -v.y);
  }
}

// Pivot search, row swap and pivot-row scaling for step k (one block per ω).
__global__ void k_gj_pivot(double2* eps, int N, int k, int* perm) {
  const int w = blockIdx.x;
  double2* E = eps + (size_t)N * N * w;
  __shared__ double sv[256];
  __shared__ int si[256];
  double best = -1.0;
  int bi = N;
  for (int i = k + threadIdx.x; i < N; i += blockDim.x) {
    const double2 a = E[(size_t)i + (size_t)N * k];
    const double v = fabs(a.x) + fabs(a.y);
    if (v > best) { best = v; bi = i; }
  }
  sv[threadIdx.x] = best;
  si[threadIdx.x] = bi;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      const double v2 = sv[threadIdx.x + s];
      const int i2 = si[threadIdx.x + s];
      if (v2 > sv[threadIdx.x] || (v2 == sv[threadIdx.x] && i2 < si[threadIdx.x])) {
        sv[threadIdx.x] = v2;
        si[threadIdx.x] = i2;
      }
    }
    __syncthreads();
  }
  const int p = (si[0] < N) ? si[0] : k;   // a column without a finite pivot keeps its row
  if (threadIdx.x == 0) perm[(size_t)N * w + k] = p;
  if (p != k) {
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
      const double2 t = E[(size_t)k + (size_t)N * j];
      E[(size_t)k + (size_t)N * j] = E[(size_t)p + (size_t)N * j];
      E[(size_t)p + (size_t)N * j] = t;
    }
  }
  __syncthreads();
  const double2 r = crecip(E[(size_t)k + (size_t)N * k]);
  __syncthreads();
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    if (j == k) E[(size_t)k + (size_t)N * k] = r;
    else E[(size_t)k + (size_t)N * j] = cmul(E[(size_t)k + (size_t)N * j], r);
  }
}

// A[i,j] −= A[i,k]·A[k,j] for i ≠ k, j ≠ k.
__global__ void k_gj_eliminate(double2* eps, int N, int k) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  const int w = blockIdx.z;
  if (i >= N || i == k || j == k) return;
  double2* E = eps + (size_t)N * N * w;
  const double2 f = E[(size_t)i + (size_t)N * k];
  const double2 a = E[(size_t)k + (size_t)N * j];
  double2& d = E[(size_t)i + (size_t)N * j];
  d.x -= f.x * a.x - f.y * a.y;
  d.y -= f.x * a.y + f.y * a.x;
}

// A[i,k] ← −A[i,k]·A[k,k] for i ≠ k (A[k,k] already holds 1/pivot).
__global__ void k_gj_column(double2* eps, int N, int k) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int w = blockIdx.y;
  if (i >= N || i == k) return;
  double2* E = eps + (size_t)N * N * w;
  const double2 r = E[(size_t)k + (size_t)N * k];
  const double2 f = E[(size_t)i + (size_t)N * k];
  const double2 v = cmul(f, r);
  E[(size_t)i + (size_t)N * k] = make_double2(-v.x, -v.y);
}

// Undo the row interchanges on the columns of the inverse (reverse order).
__global__ void k_gj_unpermute(double2* eps, int N, const int* perm) {
  const int w = blockIdx.x;
  double2* E = eps + (size_t)N * N * w;
  for (int k = N - 1; k >= 0; k--) {
    const int p = perm[(size_t)N * w + k];
    if (p != k && p >= 0 && p < N) {
      for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const double2 t = E[(size_t)i + (size_t)N * k];
        E[(size_t)i + (size_t)N * k] = E[(size_t)i + (size_t)N * p];
        E[(size_t)i + (size_t)N * p] = t;
      }
    }
    __syncthreads();
  }
}

// y[I, ω] = Σ_J A[I,J]·x[J, ω]   (conj_out: y = conj(A·x))
__global__ void k_matvec(const double2* eps, int N, const double2* x, double2* y, int conj_out) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int w = blockIdx.y;
  if (I >= N) return;
  const double2* E = eps + (size_t)N * N * w;
  double re = 0.0, im = 0.0;
  for (int J = 0; J < N; J++) {
    const double2 a = E[(size_t)I + (size_t)N * J];
    const double2 b = x[(size_t)N * w + J];
    re += a.x * b.x - a.y * b.y;
    im += a.x * b.y + a.y * b.x;
  }
  y[(size_t)N * w + I] = conj_out ? make_double2(re, -im) : make_double2(re, im);
}

// Per ω: ww = epsw2·bw1, new head, new wings (one block per ω).
__global__ void k_head_update(int N, const double2* bw1, const double2* w2b, double2* epsw1, double2* epsw2,
                              double2* head) {
  const int w = blockIdx.x;
  __shared__ double sr[256], si[256];
  double re = 0.0, im = 0.0;
  for (int J = threadIdx.x; J < N; J += blockDim.x) {
    const double2 a = epsw2[(size_t)N * w + J];
    const double2 b = bw1[(size_t)N * w + J];
    re += a.x * b.x - a.y * b.y;
    im += a.x * b.y + a.y * b.x;
  }
  sr[threadIdx.x] = re; si[threadIdx.x] = im;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) { sr[threadIdx.x] += sr[threadIdx.x + s]; si[threadIdx.x] += si[threadIdx.x + s]; }
    __syncthreads();
  }
  __shared__ double2 hnew;
  if (threadIdx.x == 0) {
    const double2 h = head[w];
    const double2 den = make_double2(1.0 + h.x - sr[0], h.y - si[0]);
    hnew = crecip(den);
  }
  __syncthreads();
  const double2 hn = hnew;
  for (int J = threadIdx.x; J < N; J += blockDim.x) {
    const double2 v1 = cmul(hn, bw1[(size_t)N * w + J]);
    const double2 v2 = cmul(hn, w2b[(size_t)N * w + J]);
    epsw1[(size_t)N * w + J] = make_double2(-v1.x, -v1.y);
    epsw2[(size_t)N * w + J] = make_double2(-v2.x, -v2.y);
  }
  if (threadIdx.x == 0) head[w] = make_double2(hn.x, hn.y);  // "−1" applied after the rank-1 update
}

// eps += head·outer(bw1, w2b), then head −= 1.
__global__ void k_head_rank1(double2* eps, int N, const double2* bw1, const double2* w2b, const double2* head) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y;
  const int w = blockIdx.z;
  if (I >= N) return;
  const double2 h = head[w];
  const double2 t = cmul(h, cmul(bw1[(size_t)N * w + I], w2b[(size_t)N * w + J]));
  double2& d = eps[(size_t)N * N * w + (size_t)I + (size_t)N * J];
  d.x += t.x;
  d.y += t.y;
}

__global__ void k_head_minus_one(double2* head, int nom) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w < nom) head[w].x -= 1.0;
}

__global__ void k_sub_identity(double2* eps, int N) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int w = blockIdx.y;
  if (I < N) eps[(size_t)N * N * w + (size_t)I + (size_t)N * I].x -= 1.0;
}

void launch_sym_add_identity(double2* eps, int N, int nom, cudaStream_t s) {
  const int TB = 128;
  k_sym_add_identity<<<dim3((N + TB - 1) / TB, N, nom), TB, 0, s>>>(eps, N);
  pg_count_launches(1);
}

void launch_finish(double2* eps, int N, int nom, double2* epsw1, double2* epsw2, double2* head, double2* bw1,
                   double2* w2b, cudaStream_t s) {
  const int TB = 128;
  if (epsw1) {
    dim3 gv((N + TB - 1) / TB, nom);
    k_matvec<<<gv, TB, 0, s>>>(eps, N, epsw1, bw1, 0);
    k_matvec<<<gv, TB, 0, s>>>(eps, N, epsw2, w2b, 1);
    k_head_update<<<nom, 256, 0, s>>>(N, bw1, w2b, epsw1, epsw2, head);
    k_head_rank1<<<dim3((N + TB - 1) / TB, N, nom), TB, 0, s>>>(eps, N, bw1, w2b, head);
    k_head_minus_one<<<(nom + 127) / 128, 128, 0, s>>>(head, nom);
    pg_count_launches(5);
  }
  k_sub_identity<<<dim3((N + TB - 1) / TB, nom), TB, 0, s>>>(eps, N);
  pg_count_launches(1);
}

// out[j][e] = Σ_i in[i][e]·U[i + nin·j]: complex arrays whose leading index is
// a frequency or SVD-basis index, transformed by a real (nin, nout) matrix
// (the basis changes dot(eps, Ul) and dot(eps, dUl) of pygw.py:3226, 3276-3280).
__global__ void k_basis_change(const double2* __restrict__ in, int nin, double2* __restrict__ out, int nout,
                               const double* __restrict__ U, long long nelem) {
  extern __shared__ double us[];
  for (int i = threadIdx.x; i < nin * nout; i += blockDim.x) us[i] = U[i];
  __syncthreads();
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nelem) return;
  for (int j = 0; j < nout; j++) {
    double re = 0.0, im = 0.0;
    for (int i = 0; i < nin; i++) {
      const double2 v = in[(size_t)i * nelem + e];
      re += v.x * us[i + nin * j];
      im += v.y * us[i + nin * j];
    }
    out[(size_t)j * nelem + e] = make_double2(re, im);
  }
}

}  // namespace pge

using namespace pge;

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

extern "C" size_t pg_eps_inverse_f64_workspace(int npb, int nom) {
  if (npb <= 0 || nom <= 0) return 0;
  return align256(sizeof(int) * (size_t)npb * nom) + 2 * align256(sizeof(double2) * (size_t)npb * nom);
}

// eps: χ0 part accumulated by pg_chi0_accumulate_f64 (+ mirror); on return it
// holds ε⁻¹ − 1.  epsw1/epsw2/head (device, complex128, [nom][N] / [nom]) are
// updated in place when non-null (q = 0).
extern "C" int pg_eps_inverse_f64(void* eps_, int npb, int nom, void* epsw1_, void* epsw2_, void* head_, void* work,
                                  size_t work_bytes, void* stream) {
  if (!eps_ || npb <= 0 || nom <= 0 || !work) return PG_EARG;
  const bool q0 = epsw1_ != nullptr;
  if (q0 && (!epsw2_ || !head_)) return PG_EARG;
  if (work_bytes < pg_eps_inverse_f64_workspace(npb, nom)) return PG_EWORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  double2* eps = (double2*)eps_;
  const int N = npb;
  char* wp = (char*)work;
  int* perm = (int*)wp; wp += align256(sizeof(int) * (size_t)N * nom);
  double2* bw1 = (double2*)wp; wp += align256(sizeof(double2) * (size_t)N * nom);
  double2* w2b = (double2*)wp;
  const int TB = 128;
  dim3 gsq((N + TB - 1) / TB, N, nom);
  launch_sym_add_identity(eps, N, nom, s);
  for (int k = 0; k < N; k++) {
    k_gj_pivot<<<nom, 256, 0, s>>>(eps, N, k, perm);
    k_gj_eliminate<<<gsq, TB, 0, s>>>(eps, N, k);
    k_gj_column<<<dim3((N + TB - 1) / TB, nom), TB, 0, s>>>(eps, N, k);
  }
  k_gj_unpermute<<<nom, 256, 0, s>>>(eps, N, perm);
  pg_count_launches(1 + 3ull * N);
  launch_finish(eps, N, nom, q0 ? (double2*)epsw1_ : nullptr, (double2*)epsw2_, (double2*)head_, bw1, w2b, s);
  return cudaGetLastError() == cudaSuccess ? PG_OK : PG_ECUDA;
}

// Basis change along the leading (frequency / SVD) index: out[nout][nelem] =
// in[nin][nelem] · U, U real (nin, nout) Fortran order (device); in ≠ out.
extern "C" int pg_basis_change(const void* in, int nin, void* out, int nout, const double* U, long long nelem,
                               void* stream) {
  if (!in || !out || !U || nin <= 0 || nout <= 0 || nelem <= 0 || in == out) return PG_EARG;
  if ((size_t)nin * nout * sizeof(double) > 48 * 1024) return PG_ETOOBIG;
  k_basis_change<<<(unsigned)((nelem + 127) / 128), 128, (size_t)nin * nout * sizeof(double), (cudaStream_t)stream>>>(
      (const double2*)in, nin, (double2*)out, nout, U, nelem);
  pg_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? PG_OK : PG_ECUDA;
}
