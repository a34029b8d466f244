// Plain FP64 χ0 contraction on sm_103a (the comparator path).
//
// Restates the per-k, per-ω update of MatrixElements2Band.calc_eps
// (pygw.py:3170-3185):
//     tmat = minm2ᵀ·coef ⊙ kcw[:, :, k, ω].ravel()       (coef = −fspin = −2)
//     eps[:, :, ω] += tmat @ conj(minm2)
// i.e.  eps[I,J,ω] += Σ_p (M[p,I]·coef·w_p(k,ω)) · conj(M[p,J]),
// with p = ie1·nb2 + ie2 (C order of kcw[:nb1,:nb2]) and
// M = minm[nb1, nb2, matsiz] reshaped to [P, matsiz].
//
// The sum is Hermitian in (I, J); only tiles on or above the diagonal are
// accumulated and pg_chi0_mirror_f64 copies their conjugates below it, so the
// result equals the reference's full matrix up to rounding.  Layouts:
//   minm  : [nk_chunk][P][N] complex128 (the per-k minm2 blocks stacked)
//   kcw   : [nb1, nb2, nkp, nom] Fortran order (as returned by the weights)
//   eps   : [nom][N][N] with I fastest — eps[I + N*J + N*N*ω], i.e. the
//           reference's (matsiz, matsiz, nom) Fortran-ordered array.
//   pm    : [nk_chunk][P] complex128 (q→0 wings, optional)
//   epsw1 : [nom][N] complex128 (optional)
#include <cuda_runtime.h>
#include <stdint.h>
#include "pygw_status.h"
#include "launches.h"

namespace pgc {

constexpr int TILE = 64;
constexpr int KC = 16;

__device__ __forceinline__ void tile_pair(int lin, int ntile, int& ti, int& tj) {
  // lin enumerates (ti, tj) with ti ≤ tj, row by row.
  int t = 0, rem = lin;
  while (rem >= ntile - t) { rem -= ntile - t; t++; }
  ti = t; tj = t + rem;
}

__global__ void __launch_bounds__(256) k_chi0_f64(const double2* __restrict__ minm, int nkc, int k0,
                                                  const double* __restrict__ kcw, int nb1, int nb2, int nkp,
                                                  int N, double coef, double2* __restrict__ eps) {
  __shared__ double2 As[KC][TILE];
  __shared__ double2 Bs[KC][TILE];
  const int ntile = (N + TILE - 1) / TILE;
  int ti, tj;
  tile_pair(blockIdx.x, ntile, ti, tj);
  const int w = blockIdx.y;
  const int P = nb1 * nb2;
  const long long K = (long long)nkc * P;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int i0 = ti * TILE, j0 = tj * TILE;
  double2 acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) acc[a][b] = make_double2(0.0, 0.0);
  for (long long kb = 0; kb < K; kb += KC) {
    // 256 threads load KC×TILE complex for each operand: 4 each.
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const int idx = threadIdx.x + 256 * r;    // 0..1023
      const int kk = idx / TILE, ii = idx % TILE;
      const long long K1 = kb + kk;
      double2 a = make_double2(0.0, 0.0), b = make_double2(0.0, 0.0);
      if (K1 < K) {
        const int kl = (int)(K1 / P), p = (int)(K1 - (long long)kl * P);
        const int ib = p / nb2, jb = p - ib * nb2;
        const double wv = kcw[(size_t)ib + (size_t)nb1 * ((size_t)jb + (size_t)nb2 * ((size_t)(k0 + kl) + (size_t)nkp * w))];
        const double2* row = minm + ((size_t)kl * P + p) * N;
        if (i0 + ii < N) {
          const double2 m = row[i0 + ii];
          a = make_double2((m.x * coef) * wv, (m.y * coef) * wv);
        }
        if (j0 + ii < N) b = row[j0 + ii];
      }
      As[kk][ii] = a;
      Bs[kk][ii] = b;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < KC; kk++) {
      double2 av[4], bv[4];
#pragma unroll
      for (int a = 0; a < 4; a++) av[a] = As[kk][tx + 16 * a];
#pragma unroll
      for (int b = 0; b < 4; b++) bv[b] = Bs[kk][ty + 16 * b];
#pragma unroll
      for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) {
          // acc += a · conj(b)
          acc[a][b].x = fma(av[a].x, bv[b].x, fma(av[a].y, bv[b].y, acc[a][b].x));
          acc[a][b].y = fma(av[a].y, bv[b].x, fma(-av[a].x, bv[b].y, acc[a][b].y));
        }
    }
    __syncthreads();
  }
  double2* E = eps + (size_t)N * N * w;
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) {
      const int I = i0 + tx + 16 * a, J = j0 + ty + 16 * b;
      if (I < N && J < N) {
        double2& d = E[(size_t)I + (size_t)N * J];
        d.x += acc[a][b].x;
        d.y += acc[a][b].y;
      }
    }
}

// Lower tiles ← conjugate of the upper tiles (tile-granular, as accumulated).
__global__ void k_mirror(double2* eps, int N) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y;
  const int w = blockIdx.z;
  if (I >= N) return;
  if (J / TILE < I / TILE) {
    double2* E = eps + (size_t)N * N * w;
    const double2 v = E[(size_t)J + (size_t)N * I];
    E[(size_t)I + (size_t)N * J] = make_double2(v.x, -v.y);
  }
}

// epsw1[I, ω] += Σ_p (M[p,I]·coef·w_p) · pm_p   (pygw.py:3192-3195; no conjugate)
__global__ void k_wings_f64(const double2* __restrict__ minm, int nkc, int k0, const double* __restrict__ kcw,
                            int nb1, int nb2, int nkp, int N, double coef, const double2* __restrict__ pm,
                            double2* __restrict__ epsw1) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int w = blockIdx.y;
  if (I >= N) return;
  const int P = nb1 * nb2;
  double re = 0.0, im = 0.0;
  for (int kl = 0; kl < nkc; kl++) {
    for (int p = 0; p < P; p++) {
      const int ib = p / nb2, jb = p - ib * nb2;
      const double wv = kcw[(size_t)ib + (size_t)nb1 * ((size_t)jb + (size_t)nb2 * ((size_t)(k0 + kl) + (size_t)nkp * w))];
      const double2 m = minm[((size_t)kl * P + p) * N + I];
      const double tr = (m.x * coef) * wv, ti = (m.y * coef) * wv;
      const double2 q = pm[(size_t)kl * P + p];
      re = fma(tr, q.x, fma(-ti, q.y, re));
      im = fma(tr, q.y, fma(ti, q.x, im));
    }
  }
  epsw1[(size_t)N * w + I].x += re;
  epsw1[(size_t)N * w + I].y += im;
}

}  // namespace pgc

using namespace pgc;

extern "C" int pg_chi0_accumulate_f64(const void* minm, int nk_chunk, int k0, const double* kcw, int nb1, int nb2,
                                      int nkp, int nom, int npb, double coef, void* eps, const void* pm, void* epsw1,
                                      void* stream) {
  if (!minm || !kcw || !eps || nk_chunk <= 0 || k0 < 0 || k0 + nk_chunk > nkp || nb1 <= 0 || nb2 <= 0 || nom <= 0 ||
      npb <= 0)
    return PG_EARG;
  if ((pm == nullptr) != (epsw1 == nullptr)) return PG_EARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int ntile = (npb + TILE - 1) / TILE;
  dim3 grid(ntile * (ntile + 1) / 2, nom);
  k_chi0_f64<<<grid, 256, 0, s>>>((const double2*)minm, nk_chunk, k0, kcw, nb1, nb2, nkp, npb, coef, (double2*)eps);
  pg_count_launches(1);
  if (pm) {
    dim3 g2((npb + 127) / 128, nom);
    k_wings_f64<<<g2, 128, 0, s>>>((const double2*)minm, nk_chunk, k0, kcw, nb1, nb2, nkp, npb, coef,
                                   (const double2*)pm, (double2*)epsw1);
    pg_count_launches(1);
  }
  return cudaGetLastError() == cudaSuccess ? PG_OK : PG_ECUDA;
}

extern "C" int pg_chi0_mirror_f64(void* eps, int npb, int nom, void* stream) {
  if (!eps || npb <= 0 || nom <= 0) return PG_EARG;
  dim3 g((npb + 127) / 128, npb, nom);
  k_mirror<<<g, 128, 0, (cudaStream_t)stream>>>((double2*)eps, npb);
  pg_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? PG_OK : PG_ECUDA;
}

// q→0 wings only (the mixed-precision path computes χ0 itself).
extern "C" int pg_wings_f64(const void* minm, int nk_chunk, int k0, const double* kcw, int nb1, int nb2, int nkp,
                            int nom, int npb, double coef, const void* pm, void* epsw1, void* stream) {
  if (!minm || !kcw || !pm || !epsw1 || nk_chunk <= 0 || k0 < 0 || k0 + nk_chunk > nkp || nb1 <= 0 || nb2 <= 0 ||
      nom <= 0 || npb <= 0)
    return PG_EARG;
  dim3 g2((npb + 127) / 128, nom);
  k_wings_f64<<<g2, 128, 0, (cudaStream_t)stream>>>((const double2*)minm, nk_chunk, k0, kcw, nb1, nb2, nkp, npb, coef,
                                                    (const double2*)pm, (double2*)epsw1);
  pg_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? PG_OK : PG_ECUDA;
}
