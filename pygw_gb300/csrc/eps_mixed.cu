// ε⁻¹ in mixed precision: FP32 Gauss–Jordan inverse, refined in FP64 with
// the residual on the tensor cores.
//
// The ε block of calc_eps (pygw.py:3229-3271) inverts the Hermitian
// A = (ε + εᴴ)/2 + I per frequency with scipy.linalg.inv in FP64.  Here:
//   1. X0 = A⁻¹ in FP32 (complex Gauss–Jordan, partial pivoting by |Re|+|Im|,
//      the FP64 path's algorithm, blocked: panels of b columns factored in
//      shared memory, then a rank-b update of the other columns);
//   2. `iters` refinement steps  R = I − A·X (split-precision digit GEMM on
//      tcgen05: A and X split into six 8-bit digits per value, digit pairs
//      s + t ≤ 5 summed exactly, ≈ 2^-48 relative to the row scales),
//      X ← X + X·R (FP32 product, FP64 sum: R is small, so FP32 suffices);
//   3. the q → 0 head/wings update and −I in FP64 (shared with the FP64 path).
// Each refinement step squares the relative error of X (‖I − X·A‖ < 1), so
// one or two steps take the FP32 inverse (≈ κ·1e-7) to the FP64 level.
//
// Real form of the complex product C = A·X used by the digit GEMM:
//   A_real (2N × 2N) = [[Re A, −Im A], [Im A, Re A]],  B (N × 2N): B[j] = [Re X(:,j); Im X(:,j)],
//   G = A_real · Bᵀ,  C(i,j) = G[i][j] + i·G[N+i][j].
// A is Hermitian, so row r of A is the conjugate of its column r and every
// digit row is read from contiguous memory.
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include "pygw_status.h"
#include "launches.h"
#include "ozaki.h"
#include "eps_internal.h"

namespace pgx {

using pgm::digit_index;
using pgm::row_exponent;
constexpr int S = 6;            // digits per value in the residual (≈ 2^-48 of the row scales)

// ------------------------------------------------------------ FP32 inverse
__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 crecipf(float2 a) {
  // Smith's algorithm for 1/a.
  if (fabsf(a.x) >= fabsf(a.y)) {
    const float r = a.y / a.x, d = a.x + a.y * r;
    return make_float2(1.0f / d, -r / d);
  } else {
    const float r = a.x / a.y, d = a.x * r + a.y;
    return make_float2(r / d, -1.0f / d);
  }
}

__global__ void k_to_f32(const double2* __restrict__ a, float2* __restrict__ x, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = make_float2((float)a[i].x, (float)a[i].y);
}

// ---- blocked Gauss–Jordan: the same elimination (partial pivoting by
// |Re|+|Im|, first on ties; row swaps over the whole matrix; the inverse
// built in place) organised in panels of b columns.  Within a panel the b
// elementary steps are applied to the panel columns only; their product M
// differs from I only in the panel's (pivot) rows, so the other columns follow
// as A_o ← A_o + W·S − I_p·S with W the factored panel columns and S the
// panel rows of A_o (a rank-b update).

// Panel factorisation, one CTA per ω; the panel (N × b) lives in shared memory
// as P[j][i].  Row swaps of the non-panel columns are made here in global
// memory (they precede the rank-b update of those columns).
__global__ void __launch_bounds__(512) k_gj32_panel(float2* X, int N, int c0, int b, int* perm) {
  extern __shared__ float2 Pn[];                 // [b][N]
  __shared__ float sv[512];
  __shared__ int si[512];
  const int w = blockIdx.x;
  float2* E = X + (size_t)N * N * w;
  for (int e = threadIdx.x; e < b * N; e += blockDim.x) {
    const int j = e / N, i = e - j * N;
    Pn[e] = E[(size_t)i + (size_t)N * (c0 + j)];
  }
  __syncthreads();
  for (int jj = 0; jj < b; jj++) {
    const int k = c0 + jj;
    float2* col = Pn + (size_t)jj * N;
    float best = -1.0f;
    int bi = N;
    for (int i = k + threadIdx.x; i < N; i += blockDim.x) {
      const float v = fabsf(col[i].x) + fabsf(col[i].y);
      if (v > best) { best = v; bi = i; }
    }
    sv[threadIdx.x] = best;
    si[threadIdx.x] = bi;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) {
        const float v2 = sv[threadIdx.x + s];
        const int i2 = si[threadIdx.x + s];
        if (v2 > sv[threadIdx.x] || (v2 == sv[threadIdx.x] && i2 < si[threadIdx.x])) {
          sv[threadIdx.x] = v2;
          si[threadIdx.x] = i2;
        }
      }
      __syncthreads();
    }
    const int p = (si[0] < N) ? si[0] : k;       // a column without a finite pivot keeps its row
    if (threadIdx.x == 0) perm[(size_t)N * w + k] = p;
    if (p != k) {
      for (int c = threadIdx.x; c < N; c += blockDim.x) {
        if (c >= c0 && c < c0 + b) {
          float2* pc = Pn + (size_t)(c - c0) * N;
          const float2 t = pc[k]; pc[k] = pc[p]; pc[p] = t;
        } else {
          const float2 t = E[(size_t)k + (size_t)N * c];
          E[(size_t)k + (size_t)N * c] = E[(size_t)p + (size_t)N * c];
          E[(size_t)p + (size_t)N * c] = t;
        }
      }
    }
    __syncthreads();
    const float2 r = crecipf(col[k]);
    __syncthreads();
    // pivot row of the panel: scaled; the pivot itself becomes 1/pivot
    for (int j = threadIdx.x; j < b; j += blockDim.x) {
      if (j == jj) Pn[(size_t)j * N + k] = r;
      else Pn[(size_t)j * N + k] = cmulf(Pn[(size_t)j * N + k], r);
    }
    __syncthreads();
    // other rows: P[j][i] −= P[jj][i]·P[j][k] (j ≠ jj), then P[jj][i] = −P[jj][i]·r
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
      if (i == k) continue;
      const float2 f = col[i];
      for (int j = 0; j < b; j++) {
        if (j == jj) continue;
        float2& d = Pn[(size_t)j * N + i];
        const float2 a = Pn[(size_t)j * N + k];
        d.x -= f.x * a.x - f.y * a.y;
        d.y -= f.x * a.y + f.y * a.x;
      }
      const float2 v = cmulf(f, r);
      col[i] = make_float2(-v.x, -v.y);
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < b * N; e += blockDim.x) {
    const int j = e / N, i = e - j * N;
    E[(size_t)i + (size_t)N * (c0 + j)] = Pn[e];
  }
}

// Rank-b update of the non-panel columns: A[i,c] ← (i in panel ? 0 : A[i,c]) + Σ_j W[i,j]·S[j,c],
// S[j,c] = A[c0+j, c] read before any write of column c.  Block: 32 columns
// (panel columns skipped) × all rows of one ω; grid (ceil(N/32), nw).  Each
// thread loads eight columns of its row before it updates them, so eight
// loads per warp are in flight (one at a time left the kernel bound by
// DRAM latency, at about a fifth of the copy bandwidth).
constexpr int GJ_BMAX = 16;
__global__ void __launch_bounds__(256) k_gj32_update(float2* X, int N, int c0, int b) {
  __shared__ float2 Ss[GJ_BMAX][32];
  const int w = blockIdx.y;
  const int cbase = blockIdx.x * 32;
  float2* E = X + (size_t)N * N * w;
  for (int e = threadIdx.x; e < b * 32; e += blockDim.x) {
    const int j = e / 32, cc = e % 32, c = cbase + cc;
    Ss[j][cc] = (c < N && (c < c0 || c >= c0 + b)) ? E[(size_t)(c0 + j) + (size_t)N * c] : make_float2(0.0f, 0.0f);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    float2 wr[GJ_BMAX];
#pragma unroll
    for (int j = 0; j < GJ_BMAX; j++) wr[j] = (j < b) ? E[(size_t)i + (size_t)N * (c0 + j)] : make_float2(0.0f, 0.0f);
    const bool prow = i >= c0 && i < c0 + b;
    for (int c8 = 0; c8 < 32; c8 += 8) {
      float2 acc[8];
      bool upd[8];
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const int c = cbase + c8 + q;
        upd[q] = c < N && (c < c0 || c >= c0 + b);
        acc[q] = (upd[q] && !prow) ? E[(size_t)i + (size_t)N * c] : make_float2(0.0f, 0.0f);
      }
#pragma unroll
      for (int q = 0; q < 8; q++) {
#pragma unroll
        for (int j = 0; j < GJ_BMAX; j++) {
          if (j < b) {
            const float2 sj = Ss[j][c8 + q];
            acc[q].x += wr[j].x * sj.x - wr[j].y * sj.y;
            acc[q].y += wr[j].x * sj.y + wr[j].y * sj.x;
          }
        }
      }
#pragma unroll
      for (int q = 0; q < 8; q++)
        if (upd[q]) E[(size_t)i + (size_t)N * (cbase + c8 + q)] = acc[q];
    }
  }
}

// Undo the row interchanges on the columns of the inverse (reverse order).
__global__ void k_gj32_unpermute(float2* X, int N, const int* perm) {
  const int w = blockIdx.x;
  float2* E = X + (size_t)N * N * w;
  for (int k = N - 1; k >= 0; k--) {
    const int p = perm[(size_t)N * w + k];
    if (p != k && p >= 0 && p < N) {
      for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const float2 t = E[(size_t)i + (size_t)N * k];
        E[(size_t)i + (size_t)N * k] = E[(size_t)i + (size_t)N * p];
        E[(size_t)i + (size_t)N * p] = t;
      }
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------ digits
__device__ __forceinline__ double2 ld2(const double2* p) { return *p; }
__device__ __forceinline__ double2 ld2(const float2* p) { const float2 v = *p; return make_double2(v.x, v.y); }

// Exponent of column j of M (max over k of |Re|, |Im|) for row j of the real
// form (and row N + j when two_rows).  Grid (N, nw), 256 threads.
template <typename T>
__global__ void k_col_exp(const T* M, int N, int R_pad, int two_rows, int* e) {
  const int j = blockIdx.x, w = blockIdx.y;
  const T* col = M + (size_t)N * N * w + (size_t)N * j;
  double m = 0.0;
  for (int k = threadIdx.x; k < N; k += blockDim.x) {
    const double2 v = ld2(col + k);
    m = fmax(m, fmax(fabs(v.x), fabs(v.y)));
  }
  __shared__ double sm[256];
  sm[threadIdx.x] = m;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const int ex = row_exponent(__double2float_ru(sm[0]));
    e[(size_t)R_pad * w + j] = ex;
    if (two_rows) e[(size_t)R_pad * w + N + j] = ex;
  }
}

// ND signed 8-bit digits of x relative to 2^e (exact FP64 arithmetic).
template <int ND>
__device__ __forceinline__ void digitsS(double x, int e, __nv_bfloat16 (&d)[ND]) {
  double y = ldexp(x, -e);
#pragma unroll
  for (int s = 0; s < ND; s++) {
    const double t = y * 256.0;
    const double dg = rint(t);
    y = t - dg;
    d[s] = __float2bfloat16_rn((float)dg);
  }
}

// A digits: rows r and N + r of A_real from column r of the Hermitian A.
// Grid (ceil(N/256), N, nw).
__global__ void k_digits_herm(const double2* __restrict__ A, int N, int R_pad, int nkb, const int* eA,
                              __nv_bfloat16* adig) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y, w = blockIdx.z;
  if (k >= N) return;
  const double2 x = A[(size_t)N * N * w + (size_t)N * r + k];   // A(k, r) = conj A(r, k)
  const int e = eA[(size_t)R_pad * w + r];
  __nv_bfloat16 dre[S], dim[S];
  digitsS<S>(x.x, e, dre);
  digitsS<S>(x.y, e, dim);
#pragma unroll
  for (int s = 0; s < S; s++) {
    const int pl = w * S + s;
    adig[digit_index(pl, r, k, R_pad, nkb)] = dre[s];                 //  Re A(r,k)
    adig[digit_index(pl, r, N + k, R_pad, nkb)] = dim[s];             // −Im A(r,k)
    adig[digit_index(pl, N + r, k, R_pad, nkb)] = __hneg(dim[s]);     //  Im A(r,k)
    adig[digit_index(pl, N + r, N + k, R_pad, nkb)] = dre[s];         //  Re A(r,k)
  }
}

// B digits: row j = [Re X(:, j); Im X(:, j)].  Grid (ceil(N/256), N, nw).
template <typename T, int ND>
__global__ void k_digits_cols(const T* __restrict__ X, int N, int R_pad, int nkb, const int* fB, __nv_bfloat16* bdig) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y, w = blockIdx.z;
  if (k >= N) return;
  const double2 x = ld2(X + (size_t)N * N * w + (size_t)N * j + k);
  const int e = fB[(size_t)R_pad * w + j];
  __nv_bfloat16 dre[ND], dim[ND];
  digitsS<ND>(x.x, e, dre);
  digitsS<ND>(x.y, e, dim);
#pragma unroll
  for (int s = 0; s < ND; s++) {
    const int pl = w * ND + s;
    bdig[digit_index(pl, j, k, R_pad, nkb)] = dre[s];
    bdig[digit_index(pl, j, N + k, R_pad, nkb)] = dim[s];
  }
}

// R = I − A·X from the digit-GEMM tiles.  Grid (ceil(N/128), N, nw).
__global__ void k_residual(const double* __restrict__ out, const int* eA, const int* fB, int N, int R_padA, int R_padB,
                           int nTb, int ntile, double2* R) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y, w = blockIdx.z;
  if (i >= N) return;
  const float2* out2 = reinterpret_cast<const float2*>(out);      // float-pair tiles
  auto G = [&](int r, int c) -> double {
    const int tile = (r >> 7) * nTb + (c >> 7);
    const float2 t = out2[((size_t)w * ntile + tile) * 16384 + (size_t)(c & 127) * 128 + (r & 127)];
    return ldexp((double)t.x + (double)t.y, eA[(size_t)R_padA * w + r] + fB[(size_t)R_padB * w + c] - 16);
  };
  const double re = G(i, j), im = G(N + i, j);
  R[(size_t)N * N * w + (size_t)N * j + i] = make_double2((i == j ? 1.0 : 0.0) - re, -im);
}

// Xnew = X + X·R (complex, FP32 products and accumulation, FP64 sum with X).
// 64×64 output tile per block, 16×16 threads with 4×4 outputs each; the next
// 16-wide K slice is loaded into registers while the current one is used.
template <typename T>
__global__ void __launch_bounds__(256) k_correct(const T* __restrict__ X, const double2* __restrict__ R, int N,
                                                 double2* __restrict__ Xnew) {
  __shared__ float2 sx[16][64];
  __shared__ float2 sr[16][64];
  const int w = blockIdx.z;
  const int i0 = blockIdx.x * 64, j0 = blockIdx.y * 64;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const T* Xw = X + (size_t)N * N * w;
  const double2* Rw = R + (size_t)N * N * w;
  float2 acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) acc[a][b] = make_float2(0.0f, 0.0f);
  double2 vx[4], vr[4];                                   // this thread's loads of one K slice
  auto load = [&](int k0) {
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int e = threadIdx.x + 256 * q;
      const int ii = e & 63, kk = e >> 6;                 // X(i0+ii, k0+kk): 64 consecutive rows
      const int i = i0 + ii, k = k0 + kk;
      vx[q] = (i < N && k < N) ? ld2(Xw + (size_t)N * k + i) : make_double2(0.0, 0.0);
      const int kr = e & 15, jj = e >> 4;                 // R(k0+kr, j0+jj): 16 consecutive rows
      const int k2 = k0 + kr, j = j0 + jj;
      vr[q] = (k2 < N && j < N) ? Rw[(size_t)N * j + k2] : make_double2(0.0, 0.0);
    }
  };
  load(0);
  for (int k0 = 0; k0 < N; k0 += 16) {
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int e = threadIdx.x + 256 * q;
      sx[e >> 6][e & 63] = make_float2((float)vx[q].x, (float)vx[q].y);
      sr[e & 15][e >> 4] = make_float2((float)vr[q].x, (float)vr[q].y);
    }
    __syncthreads();
    if (k0 + 16 < N) load(k0 + 16);
#pragma unroll
    for (int kk = 0; kk < 16; kk++) {
      float2 xa[4], rb[4];
#pragma unroll
      for (int a = 0; a < 4; a++) xa[a] = sx[kk][ty * 4 + a];
#pragma unroll
      for (int b = 0; b < 4; b++) rb[b] = sr[kk][tx * 4 + b];
#pragma unroll
      for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) {
          acc[a][b].x = fmaf(xa[a].x, rb[b].x, fmaf(-xa[a].y, rb[b].y, acc[a][b].x));
          acc[a][b].y = fmaf(xa[a].x, rb[b].y, fmaf(xa[a].y, rb[b].x, acc[a][b].y));
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) {
      const int i = i0 + ty * 4 + a, j = j0 + tx * 4 + b;
      if (i < N && j < N) {
        const double2 x = ld2(Xw + (size_t)N * j + i);
        Xnew[(size_t)N * N * w + (size_t)N * j + i] = make_double2(x.x + (double)acc[a][b].x, x.y + (double)acc[a][b].y);
      }
    }
}

__global__ void k_to_f64(const float2* __restrict__ x, double2* __restrict__ a, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = make_double2((double)x[i].x, (double)x[i].y);
}

// ------------------------------------------------------------ workspace
static size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

struct Layout {
  int N, nb, R_padA, R_padB, nkb, nTb, ntile;
  long long K_pad;
  size_t perm, x32, x64, res, adig, bdig, eA, fB, out, bw1, w2b, total;
};

static Layout layout(int N, int nom, int nb) {
  Layout L;
  L.N = N;
  L.nb = nb;
  L.R_padA = (2 * N + pgm::OZ_BLOCK - 1) / pgm::OZ_BLOCK * pgm::OZ_BLOCK;
  L.R_padB = (N + pgm::OZ_BLOCK - 1) / pgm::OZ_BLOCK * pgm::OZ_BLOCK;
  L.K_pad = (2LL * N + pgm::OZ_KB - 1) / pgm::OZ_KB * pgm::OZ_KB;
  L.nkb = (int)(L.K_pad / pgm::OZ_KB);
  L.nTb = L.R_padB / pgm::OZ_TILE;
  L.ntile = (L.R_padA / pgm::OZ_TILE) * L.nTb;
  const size_t NN = (size_t)N * N;
  size_t o = 0;
  L.perm = o; o += al256(sizeof(int) * (size_t)N * nb);
  L.x32 = o; o += al256(sizeof(float2) * NN * nb);
  L.x64 = o; o += al256(sizeof(double2) * NN * nb);
  L.res = o; o += al256(sizeof(double2) * NN * nb);
  L.adig = o; o += al256((size_t)2 * S * L.R_padA * L.K_pad * nb);
  L.bdig = o; o += al256((size_t)2 * S * L.R_padB * L.K_pad * nb);
  L.eA = o; o += al256(sizeof(int) * (size_t)L.R_padA * nb);
  L.fB = o; o += al256(sizeof(int) * (size_t)L.R_padB * nb);
  L.out = o; o += al256(sizeof(double) * (size_t)L.ntile * 16384 * nb);
  L.bw1 = o; o += al256(sizeof(double2) * (size_t)N * nom);
  L.w2b = o; o += al256(sizeof(double2) * (size_t)N * nom);
  L.total = o;
  return L;
}

// One refinement step: dst = X + X·(I − A·X) for the nw frequencies of a batch
// (A's digits and exponents are already in the workspace; dst ≠ X).
template <typename T>
static int refine_step(const T* X, double2* dst, const Layout& L, char* w, int nw, unsigned* status, cudaStream_t s) {
  const int N = L.N;
  int* fB = (int*)(w + L.fB);
  __nv_bfloat16* bdig = (__nv_bfloat16*)(w + L.bdig);
  if (cudaMemsetAsync(fB, 0, sizeof(int) * (size_t)L.R_padB * nw, s) != cudaSuccess) return PG_ECUDA;
  if (cudaMemsetAsync(bdig, 0, (size_t)2 * S * L.R_padB * L.K_pad * nw, s) != cudaSuccess) return PG_ECUDA;
  k_col_exp<T><<<dim3(N, nw), 256, 0, s>>>(X, N, L.R_padB, 0, fB);
  k_digits_cols<T, S><<<dim3((N + 255) / 256, N, nw), 256, 0, s>>>(X, N, L.R_padB, L.nkb, fB, bdig);
  pg_count_launches(2);
  double* out = (double*)(w + L.out);
  const int rc = pgm::launch_gemm_general((const __nv_bfloat16*)(w + L.adig), bdig, S, 1, L.R_padA, L.R_padB,
                                          (N + pgm::OZ_TILE - 1) / pgm::OZ_TILE, L.nkb, nw, out, status, s);
  if (rc != PG_OK) return rc;
  double2* R = (double2*)(w + L.res);
  k_residual<<<dim3((N + 127) / 128, N, nw), 128, 0, s>>>(out, (const int*)(w + L.eA), fB, N, L.R_padA, L.R_padB,
                                                         L.nTb, L.ntile, R);
  k_correct<T><<<dim3((N + 63) / 64, (N + 63) / 64, nw), 256, 0, s>>>(X, R, N, dst);
  pg_count_launches(2);
  return PG_OK;
}

// Exponents and nd (5 or 6) digits of the columns of X[nw][N][N] complex128
// as B rows [Re X(:,j); Im X(:,j)] (bdig and fB zeroed first).
int launch_cols_digits(const double2* X, int N, int nw, int R_pad, int nkb, int nd, int* fB, __nv_bfloat16* bdig,
                       cudaStream_t s) {
  if (nd != 5 && nd != 6) return PG_EARG;
  if (cudaMemsetAsync(fB, 0, sizeof(int) * (size_t)R_pad * nw, s) != cudaSuccess) return PG_ECUDA;
  if (cudaMemsetAsync(bdig, 0, (size_t)2 * nd * R_pad * nkb * 64 * nw, s) != cudaSuccess) return PG_ECUDA;
  k_col_exp<double2><<<dim3(N, nw), 256, 0, s>>>(X, N, R_pad, 0, fB);
  if (nd == 5)
    k_digits_cols<double2, 5><<<dim3((N + 255) / 256, N, nw), 256, 0, s>>>(X, N, R_pad, nkb, fB, bdig);
  else
    k_digits_cols<double2, 6><<<dim3((N + 255) / 256, N, nw), 256, 0, s>>>(X, N, R_pad, nkb, fB, bdig);
  pg_count_launches(2);
  return cudaGetLastError() == cudaSuccess ? PG_OK : PG_ECUDA;
}

}  // namespace pgx

using namespace pgx;

extern "C" size_t pg_eps_inverse_mixed_workspace(int npb, int nom, int omega_batch) {
  if (npb <= 0 || nom <= 0) return 0;
  const int nb = (omega_batch > 0 && omega_batch < nom) ? omega_batch : nom;
  return layout(npb, nom, nb).total;
}

// eps: the χ0 part (as for pg_eps_inverse_f64); on return ε⁻¹ − 1.
// omega_batch frequencies are inverted together (0 = all); iters (0, 1 or 2)
// refinement steps follow the FP32 inverse (0 = the FP32 inverse alone).
extern "C" int pg_eps_inverse_mixed(void* eps_, int npb, int nom, void* epsw1_, void* epsw2_, void* head_, void* work,
                                    size_t work_bytes, int omega_batch, int iters, unsigned* d_status, void* stream) {
  if (!eps_ || npb <= 0 || nom <= 0 || !work || iters < 0 || iters > 2) return PG_EARG;
  const bool q0 = epsw1_ != nullptr;
  if (q0 && (!epsw2_ || !head_)) return PG_EARG;
  const int nb = (omega_batch > 0 && omega_batch < nom) ? omega_batch : nom;
  const Layout L = layout(npb, nom, nb);
  if (work_bytes < L.total) return PG_EWORKSPACE;
  if ((long long)S * L.nkb * 64 * 16641 >= (1ll << 35)) return PG_ETOOBIG;
  cudaStream_t s = (cudaStream_t)stream;
  double2* eps = (double2*)eps_;
  const int N = npb;
  const size_t NN = (size_t)N * N;
  char* w = (char*)work;
  int* perm = (int*)(w + L.perm);
  float2* x32 = (float2*)(w + L.x32);
  double2* x64 = (double2*)(w + L.x64);
  int* eA = (int*)(w + L.eA);
  __nv_bfloat16* adig = (__nv_bfloat16*)(w + L.adig);
  pge::launch_sym_add_identity(eps, N, nom, s);
  for (int w0 = 0; w0 < nom; w0 += nb) {
    const int nw = (w0 + nb <= nom) ? nb : nom - w0;
    double2* A = eps + NN * w0;
    const size_t n = NN * nw;
    k_to_f32<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(A, x32, n);
    // panel width: the panel (b × N complex floats) must fit in shared memory
    int bw = GJ_BMAX;
    while (bw > 1 && (size_t)bw * N * sizeof(float2) > (size_t)200 * 1024) bw /= 2;
    const size_t psm = (size_t)bw * N * sizeof(float2);
    if (psm > (size_t)200 * 1024) return PG_ETOOBIG;
    if (cudaFuncSetAttribute(k_gj32_panel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psm) != cudaSuccess)
      return PG_ECUDA;
    unsigned long long nl = 2;
    for (int c0 = 0; c0 < N; c0 += bw) {
      const int b = (c0 + bw <= N) ? bw : N - c0;
      k_gj32_panel<<<nw, 512, psm, s>>>(x32, N, c0, b, perm);
      k_gj32_update<<<dim3((N + 31) / 32, nw), 256, 0, s>>>(x32, N, c0, b);
      nl += 2;
    }
    k_gj32_unpermute<<<nw, 256, 0, s>>>(x32, N, perm);
    pg_count_launches(nl);
    if (iters == 0) {
      k_to_f64<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(x32, A, n);
      pg_count_launches(1);
      continue;
    }
    // digits of A (shared by the refinement steps of this batch)
    if (cudaMemsetAsync(eA, 0, sizeof(int) * (size_t)L.R_padA * nw, s) != cudaSuccess) return PG_ECUDA;
    if (cudaMemsetAsync(adig, 0, (size_t)2 * S * L.R_padA * L.K_pad * nw, s) != cudaSuccess) return PG_ECUDA;
    k_col_exp<double2><<<dim3(N, nw), 256, 0, s>>>(A, N, L.R_padA, 1, eA);
    k_digits_herm<<<dim3((N + 255) / 256, N, nw), 256, 0, s>>>(A, N, L.R_padA, L.nkb, eA, adig);
    pg_count_launches(2);
    for (int it = 0; it < iters; it++) {
      // the last step writes the result over A (no longer needed once its residual is formed)
      double2* dst = (it == iters - 1) ? A : x64;
      const int rc = (it == 0) ? refine_step<float2>(x32, dst, L, w, nw, d_status, s)
                               : refine_step<double2>(x64, dst, L, w, nw, d_status, s);
      if (rc != PG_OK) return rc;
    }
  }
  pge::launch_finish(eps, N, nom, q0 ? (double2*)epsw1_ : nullptr, (double2*)epsw2_, (double2*)head_,
                     (double2*)(w + L.bw1), (double2*)(w + L.w2b), s);
  return cudaGetLastError() == cudaSuccess ? PG_OK : PG_ECUDA;
}
