// Synthetic matrix elements generated on the device, per k-chunk, from a seed.
//
// The measured workloads have no LAPW inputs: their matrix elements are
//     M_{p,I}(k) = z · √(1/2) / (1 + |E_n(k) − E_m(k−q)|) · √v_I,   z ~ CN(0, 1),
// p = ie1·nb2k + ie2 (occupied n = ncg + ie1, unoccupied m = ncg + numin + ie2).
// Host generation with numpy costs seconds per GB; the large workloads need
// tens to hundreds of GB per q, so they draw M here instead, one k-chunk at a
// time (never fully resident), keyed by (seed, q, k, n, m, I) so any chunk can be
// regenerated independently.  Normal deviates: SplitMix64 (Steele, Lea &
// Flood, OOPSLA 2014) on the counter, two 32-bit uniforms, Box–Muller.  The
// values differ from the numpy generator's (a different random stream with the
// same distribution); parity tests use the numpy generator and the oracle.
#include <cuda_runtime.h>
#include <stdint.h>
#include "pygw_status.h"
#include "launches.h"

namespace pgs {

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// One thread per (row, I); row = (k, p) of the chunk.
__global__ void k_synth_minm(int nk, int k0, int iq, const double* __restrict__ enk, int nbnd,
                             const int* __restrict__ kqid, int ncg, int numin, int nb1, int nb2,
                             const int* __restrict__ kstart, const int* __restrict__ knb2,
                             const double* __restrict__ sqv, int N, long long rows, uint64_t seed,
                             double2* __restrict__ out) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= rows * N) return;
  const long long row = idx / N;
  const int I = (int)(idx - row * N);
  int kc, pp, n2;
  if (kstart) {
    int lo = 0, hi = nk;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if ((long long)kstart[mid] <= row) lo = mid; else hi = mid;
    }
    kc = lo;
    pp = (int)(row - kstart[kc]);
    n2 = knb2[kc];
  } else {
    kc = (int)(row / ((long long)nb1 * nb2));
    pp = (int)(row - (long long)kc * nb1 * nb2);
    n2 = nb2;
  }
  const int k = k0 + kc;
  const int ie1 = pp / n2, ie2 = pp - ie1 * n2;
  const double en = enk[(size_t)ie1 + (size_t)nbnd * k];
  const double em = enk[(size_t)(ncg + numin + ie2) + (size_t)nbnd * kqid[k]];
  const double scale = 0.7071067811865476 / (1.0 + fabs(en - em)) * sqv[I];
  // key (q, k, n, m, I): the same value whatever the chunking or window layout
  const uint64_t kq = splitmix64((uint64_t)iq * 1000003ull + (uint64_t)k);
  const uint64_t r = splitmix64(seed ^ splitmix64(kq ^ (((uint64_t)ie1 << 48) | ((uint64_t)ie2 << 32) | (uint64_t)I)));
  // two uniforms in (0, 1]: 32 bits each
  const double u1 = ((double)(uint32_t)(r >> 32) + 1.0) * (1.0 / 4294967296.0);
  const double u2 = ((double)(uint32_t)r + 0.5) * (1.0 / 4294967296.0);
  const double rad = sqrt(-2.0 * log(u1));
  double sn, cs;
  sincospi(2.0 * u2, &sn, &cs);
  out[(size_t)row * N + I] = make_double2(rad * cs * scale, rad * sn * scale);
}

}  // namespace pgs

// Matrix elements of the k-points k0 .. k0+nk-1 for one q: out [rows][N]
// complex128 with rows = nk·nb1·nb2 (kstart = NULL) or kstart[nk] (ragged
// windows: point i has nb1·knb2[i] rows starting at kstart[i]).  enk
// [nbnd][nkp] column-major (the weights' layout), kqid the k−q indices of
// this q (nkp, 0-based), sqv √v_I (N).  All pointers are device pointers.
extern "C" int pg_synth_minm(int nk, int k0, int iq, const double* enk, int nbnd, const int* kqid, int ncg,
                             int numin, int nb1, int nb2, const int* kstart, const int* knb2, long long nrows,
                             const double* sqv, int npb, unsigned long long seed, void* out, void* stream) {
  if (nk <= 0 || k0 < 0 || !enk || !kqid || !sqv || !out || nb1 <= 0 || nb2 <= 0 || npb <= 0 || nbnd <= 0)
    return PG_EARG;
  if (kstart && !knb2) return PG_EARG;
  const long long rows = kstart ? nrows : (long long)nk * nb1 * nb2;
  if (rows <= 0 || rows * npb / 256 >= 2147483647ll) return PG_EARG;
  const long long nthr = rows * npb;
  pgs::k_synth_minm<<<(unsigned)((nthr + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      nk, k0, iq, enk, nbnd, kqid, ncg, numin, nb1, nb2, kstart, knb2, sqv, npb, rows, (uint64_t)seed,
      (double2*)out);
  pg_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? PG_OK : PG_ECUDA;
}
