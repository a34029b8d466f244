// Split-precision χ0 on sm_103a tensor cores (tcgen05 + TMA).
//
// χ0(ω) = Σ_K M[K,I]·c·w_K(ω)·conj(M[K,J])   (K = (k, band pair), c = −2,
// pygw.py:3170-3185) is rewritten as the real symmetric product
//     G(ω) = V · diag(c·w(ω)) · Vᵀ,   V = [Re M ; Im M]  (2N × K),
//     χ0_IJ = G[I,J] + G[N+I,N+J] + i (G[N+I,J] − G[I,N+J]).
// Both factors are split into S = 5 signed 8-bit digits with one exponent per
// row (an Ozaki-type error-free slicing):
//     V[r,K]      = 2^eA[r] Σ_s a_s[r,K] 2^(−8(s+1)),   |a_s| ≤ 129
//     c·w·V[r,K]  = 2^fB[r] Σ_t b_t[r,K] 2^(−8(t+1))
// Every digit is an integer that bf16 holds exactly, so every bf16×bf16
// product is an exact integer below 2^15.  The digit pairs are grouped by
// d = s+t (pairs with d ≥ 5 are dropped: their weight is below 2^-40):
//     G[r,c] = 2^(eA[r]+fB[c]−16) Σ_d 2^(−8d) I_d[r,c],
//     I_d    = Σ_{s+t=d} Σ_K a_s[r,K] b_t[c,K]   (an integer).
// I_d is accumulated EXACTLY: the tensor core adds integer-valued products
// into an FP32 TMEM accumulator; every ≤ 14 K-blocks (896 K-values, sum
// < 2^24) the epilogue warps move the multiples of 2^12 into a second TMEM
// accumulator (exact while below 2^36 — the host splits K so it stays
// below 2^35) and leave the remainder in place.  Each group's integer is
// then combined in FP64.  The only rounding is the dropped 5th-digit
// residual and the dropped d ≥ 5 pairs (≈ 1e-11 relative per row scale).
//
// Kernel layout: one CTA per 128×128 tile of the upper triangle of G, per
// frequency, per K-split; warp 0 issues TMA loads (one A-digit and one
// B-digit 128×64 bf16 tile per stage, 128-byte swizzle, 6 stages), warp 1
// allocates TMEM and issues tcgen05.mma (M=128, N=128, K=16), warps 2–5
// renormalise the accumulators.  Two accumulators alternate so the tensor
// core keeps working while the previous chunk is renormalised.  Every wait
// is bounded (≈ 5 s of %globaltimer); on expiry the kernel records
// PG_ERR_TIMEOUT, drains its own in-flight work, frees TMEM and returns.
#include <cuda_runtime.h>
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include <string.h>
#include "pygw_status.h"
#include "launches.h"

namespace pgm {

constexpr int S = 5;            // digits per value
constexpr int TM = 128;         // tile rows (A) = tile cols (B)
constexpr int KB = 64;          // K per stage (one 128-byte swizzle row of bf16)
constexpr int NST = 6;          // pipeline stages
constexpr int LBLK = 14;        // K-blocks per exact chunk: 14·64·129² + 2^12 < 2^24
constexpr int TILE_BYTES = TM * KB * 2;           // 16 KB
constexpr int STAGE_BYTES = 2 * TILE_BYTES;       // A + B
constexpr int NTHREADS = 192;                     // 6 warps
constexpr uint32_t TMEM_COLS = 512;
constexpr unsigned long long WAIT_NS = 5000000000ull;   // 5 s per wait

struct OzParams {
  double* out;          // [nsplit][wb][npair][128 (col)][128 (row)]
  unsigned* status;
  int R_pad, nT, npair, nkb, kb_per_split, nsplit, wb;
};

// ------------------------------------------------------------ PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ unsigned long long gtime() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: false (and the abort flag set) if the phase did not complete in WAIT_NS.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag, unsigned* status) {
  if (mbar_test(bar, parity)) return true;
  const unsigned long long t0 = gtime();
  while (true) {
    if (*abort_flag) return false;
    if (mbar_test(bar, parity)) return true;
    if (gtime() - t0 > WAIT_NS) {
      *abort_flag = 1;
      if (status) atomicOr(status, PG_ERR_TIMEOUT);
      return false;
    }
  }
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
          smem_u32(dst)),
      "l"((uint64_t)map), "r"(smem_u32(bar)), "r"(x), "r"(y)
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
      : "memory");
}
// 32 lanes × 32 consecutive 32-bit columns per warp.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
      "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const float (&v)[32]) {
  uint32_t r[32];
#pragma unroll
  for (int i = 0; i < 32; i++) r[i] = __float_as_uint(v[i]);
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
      "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]),
      "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]), "r"(r[16]), "r"(r[17]), "r"(r[18]),
      "r"(r[19]), "r"(r[20]), "r"(r[21]), "r"(r[22]), "r"(r[23]), "r"(r[24]), "r"(r[25]), "r"(r[26]), "r"(r[27]),
      "r"(r[28]), "r"(r[29]), "r"(r[30]), "r"(r[31])
      : "memory");
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle,
// 8-row core groups 1024 bytes apart (tcgen05 descriptor format, version 1).
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);          // start address
  d |= (uint64_t)1 << 16;                             // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;                   // stride byte offset
  d |= (uint64_t)1 << 46;                             // descriptor version
  d |= (uint64_t)2 << 61;                             // 128-byte swizzle
  return d;
}
// Instruction descriptor, kind::f16: D=F32, A=B=BF16, both K-major, M=128, N=128.
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TM >> 3) << 17) | ((uint32_t)(TM >> 4) << 24);

__device__ __forceinline__ void tile_pair(int lin, int nT, int& ti, int& tj) {
  int t = 0, rem = lin;
  while (rem >= nT - t) { rem -= nT - t; t++; }
  ti = t; tj = t + rem;
}

// ------------------------------------------------------ the digit GEMM
__global__ void __launch_bounds__(NTHREADS, 1)
    k_ozaki_gemm(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, OzParams p) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + NST * STAGE_BYTES);
  uint64_t* empty = full + NST;
  uint64_t* acc_full = empty + NST;      // [2]
  uint64_t* acc_empty = acc_full + 2;    // [2]
  uint64_t* group_done = acc_empty + 2;  // [1]
  uint64_t* drain = group_done + 1;      // [1]
  uint32_t* tmem_base_slot = (uint32_t*)(drain + 1);
  volatile int* abort_flag = (volatile int*)(tmem_base_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int ti, tj;
  tile_pair(blockIdx.x, p.nT, ti, tj);
  const int wl = blockIdx.y;        // frequency within the batch
  const int split = blockIdx.z;
  const int kb0 = split * p.kb_per_split;
  const int kb1 = min(p.nkb, kb0 + p.kb_per_split);

  if (threadIdx.x == 0) {
    for (int i = 0; i < NST; i++) { mbar_init(full + i, 1); mbar_init(empty + i, 1); }
    // acc_empty / group_done: every epilogue thread arrives (no unbounded named barrier)
    for (int i = 0; i < 2; i++) { mbar_init(acc_full + i, 1); mbar_init(acc_empty + i, 128); }
    mbar_init(group_done, 128);
    mbar_init(drain, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_base_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_base_slot;
  // column layout: [0,128) low0, [128,256) low1, [256,384) high
  const int nchunk_per_pass = (kb1 - kb0 + LBLK - 1) / LBLK;

  if (warp == 0) {
    // ---------------------------------------------------------- TMA producer
    if (lane == 0 && kb1 > kb0) {
      int it = 0;
      bool ok = true;
      for (int d = 0; d < S && ok; d++)
        for (int s = 0; s <= d && ok; s++) {
          const int t = d - s;
          const int ya = s * p.R_pad + ti * TM;
          const int yb = (wl * S + t) * p.R_pad + tj * TM;
          for (int kb = kb0; kb < kb1 && ok; kb++, it++) {
            const int st = it % NST;
            if (it >= NST) ok = mbar_wait(empty + st, ((it / NST) - 1) & 1, abort_flag, p.status);
            if (!ok) break;
            unsigned char* sa = smem + st * STAGE_BYTES;
            mbar_expect_tx(full + st, STAGE_BYTES);
            tma_load_2d(sa, &tmA, full + st, kb * KB, ya);
            tma_load_2d(sa + TILE_BYTES, &tmB, full + st, kb * KB, yb);
          }
        }
      // drain: every stage issued must have landed before the CTA exits
      const int issued = it;
      for (int j = max(0, issued - NST); j < issued; j++) {
        const int st = j % NST;
        const unsigned long long t0 = gtime();
        while (!mbar_test(full + st, (j / NST) & 1) && gtime() - t0 < WAIT_NS) {}
      }
    }
  } else if (warp == 1) {
    // ---------------------------------------------------------- MMA issuer
    if (lane == 0 && kb1 > kb0) {
      int it = 0, c = 0;
      bool ok = true;
      for (int d = 0; d < S && ok; d++) {
        if (d > 0) ok = mbar_wait(group_done, (d - 1) & 1, abort_flag, p.status);
        if (!ok) break;
        bool used[2] = {false, false};
        for (int s = 0; s <= d && ok; s++) {
          for (int ch = 0; ch < nchunk_per_pass && ok; ch++, c++) {
            const int b = c & 1;
            if (c >= 2) ok = mbar_wait(acc_empty + b, ((c >> 1) - 1) & 1, abort_flag, p.status);
            if (!ok) break;
            tc_fence_after();
            const uint32_t dcol = tmem + (uint32_t)(b * TM);
            const int cb0 = kb0 + ch * LBLK, cb1 = min(kb1, cb0 + LBLK);
            for (int kb = cb0; kb < cb1; kb++, it++) {
              const int st = it % NST;
              ok = mbar_wait(full + st, (it / NST) & 1, abort_flag, p.status);
              if (!ok) break;
              tc_fence_after();
              const uint32_t sa = smem_u32(smem + st * STAGE_BYTES);
              const uint64_t ad = sdesc_sw128(sa), bd = sdesc_sw128(sa + TILE_BYTES);
#pragma unroll
              for (int k = 0; k < KB / 16; k++) {
                const uint32_t accumulate = (used[b] || kb > cb0 || k > 0) ? 1u : 0u;
                tc_mma(dcol, ad + (uint64_t)(2 * k), bd + (uint64_t)(2 * k), IDESC, accumulate);
              }
              tc_commit(empty + st);     // stage free once these MMAs have read it
            }
            if (!ok) break;
            used[b] = true;
            tc_commit(acc_full + b);     // chunk complete
          }
        }
      }
      // drain: wait for every MMA this thread issued
      tc_commit(drain);
      const unsigned long long t0 = gtime();
      while (!mbar_test(drain, 0) && gtime() - t0 < WAIT_NS) {}
    }
  } else {
    // ---------------------------------------------------------- epilogue (warps 2–5)
    const int q = warp & 3;                        // TMEM lane quarter this warp may access
    const int row = q * 32 + lane;                 // accumulator row (A tile row)
    const uint32_t lane_off = (uint32_t)(q * 32) << 16;
    const uint32_t t_low0 = tmem + lane_off, t_low1 = tmem + lane_off + TM, t_high = tmem + lane_off + 2 * TM;
    double* out = p.out + ((((size_t)split * p.wb + wl) * p.npair + blockIdx.x) * TM) * TM;
    int c = 0;
    bool ok = kb1 > kb0;
    for (int d = 0; d < S && ok; d++) {
      bool used[2] = {false, false};
      bool high_init = false;
      const int nchunks_group = (d + 1) * nchunk_per_pass;
      for (int gc = 0; gc < nchunks_group && ok; gc++, c++) {
        const int b = c & 1;
        ok = mbar_wait(acc_full + b, (c >> 1) & 1, abort_flag, p.status);
        if (!ok) break;
        tc_fence_after();
        const uint32_t tl = b ? t_low1 : t_low0;
        for (int cb = 0; cb < TM; cb += 32) {
          float lo[32], hi[32];
          tmem_ld32(tl + cb, lo);
          if (high_init) tmem_ld32(t_high + cb, hi);
#pragma unroll
          for (int i = 0; i < 32; i++) {
            const float h = rintf(lo[i] * (1.0f / 4096.0f)) * 4096.0f;   // multiple of 2^12
            lo[i] = lo[i] - h;                                            // |residual| ≤ 2^11
            hi[i] = high_init ? hi[i] + h : h;                            // exact below 2^36
          }
          tmem_st32(tl + cb, lo);
          tmem_st32(t_high + cb, hi);
        }
        high_init = true;
        used[b] = true;
        if (gc == nchunks_group - 1) {
          // group complete: I_d = high + low0 + low1 (exact in FP64), scaled by 2^(−8d)
          const double scale = ldexp(1.0, -8 * d);
          for (int cb = 0; cb < TM; cb += 32) {
            float h[32], l0[32], l1[32];
            tmem_ld32(t_high + cb, h);
            if (used[0]) tmem_ld32(t_low0 + cb, l0);
            if (used[1]) tmem_ld32(t_low1 + cb, l1);
#pragma unroll
            for (int i = 0; i < 32; i++) {
              double v = (double)h[i];
              if (used[0]) v += (double)l0[i];
              if (used[1]) v += (double)l1[i];
              double& o = out[(size_t)(cb + i) * TM + row];
              o = (d == 0) ? v * scale : o + v * scale;
            }
          }
        }
        tc_fence_before();
        mbar_arrive(acc_empty + b);
        if (gc == nchunks_group - 1) mbar_arrive(group_done);
      }
    }
    if (kb1 <= kb0) {
      for (int i = 0; i < TM; i++) out[(size_t)i * TM + row] = 0.0;        // empty K-split
    } else if (!ok) {
      for (int i = 0; i < TM; i++) out[(size_t)i * TM + row] = __longlong_as_double(0x7ff8dead00000000LL);
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

// ------------------------------------------------------------ digit prep
// Per 64-value K-block maxima of |Re M| and |Im M| for every product-basis
// index: tmax[r][kb] (r < N real parts, N ≤ r < 2N imaginary parts).
__global__ void k_block_max(const double2* __restrict__ minm, long long K, int N, int R_pad, int nkb, float* tmax) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int kb = blockIdx.y;
  if (I >= N) return;
  double mr = 0.0, mi = 0.0;
  for (int j = 0; j < KB; j++) {
    const long long k = (long long)kb * KB + j;
    if (k >= K) break;
    const double2 m = minm[(size_t)k * N + I];
    mr = fmax(mr, fabs(m.x));
    mi = fmax(mi, fabs(m.y));
  }
  // round up so the float bound is never below the double value
  tmax[(size_t)I * nkb + kb] = __double2float_ru(mr);
  tmax[(size_t)(N + I) * nkb + kb] = __double2float_ru(mi);
}

// Row exponent e with max|x|·(1+2^-20) < 2^(e−1): every value of the row is then
// |x / 2^e| < 1/2 and its leading digit |rint(256·x/2^e)| ≤ 128.
__device__ __forceinline__ int row_exponent(float bound) {
  if (!(bound > 0.0f)) return 0;
  int e;
  frexpf(bound * 1.000001f, &e);   // bound·(1+eps) in [2^(e−1), 2^e)
  return e + 1;
}

__global__ void k_row_exp_A(const float* tmax, int R, int R_pad, int nkb, int* eA) {
  const int r = blockIdx.x;
  float m = 0.0f;
  if (r < R)
    for (int kb = threadIdx.x; kb < nkb; kb += blockDim.x) m = fmaxf(m, tmax[(size_t)r * nkb + kb]);
  __shared__ float sm[256];
  sm[threadIdx.x] = m;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sm[threadIdx.x] = fmaxf(sm[threadIdx.x], sm[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) eA[r] = row_exponent(sm[0]);
}

// A digits: adig[s][r][k] (bf16), K contiguous; computed exactly in FP64.
__global__ void k_digits_A(const double2* __restrict__ minm, long long K, int N, int R_pad, long long K_pad,
                           const int* eA, __nv_bfloat16* adig) {
  __shared__ double2 tile[32][33];
  const int k0 = blockIdx.x * 32, I0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 32 × 8
  for (int j = ty; j < 32; j += 8) {
    const long long k = k0 + j;
    const int I = I0 + tx;
    tile[j][tx] = (k < K && I < N) ? minm[(size_t)k * N + I] : make_double2(0.0, 0.0);
  }
  __syncthreads();
  for (int j = ty; j < 32; j += 8) {
    const int I = I0 + j;
    const long long k = k0 + tx;
    if (I >= N || k >= K_pad) continue;
    const double2 m = tile[tx][j];
    for (int part = 0; part < 2; part++) {
      const int r = part ? N + I : I;
      double y = ldexp(part ? m.y : m.x, -eA[r]);
      for (int s = 0; s < S; s++) {
        const double t = y * 256.0;
        const double dg = rint(t);
        y = t - dg;
        adig[((size_t)s * R_pad + r) * K_pad + k] = __float2bfloat16_rn((float)dg);
      }
    }
  }
}

// Weights for a batch of frequencies: c·w as an FP32 pair (hi + lo ≈ 48 bits).
__global__ void k_weights_prep(const double* __restrict__ kcw, int nb1, int nb2, int nkp, int om0, int wb, double coef,
                               long long K, long long K_pad, float2* wpair) {
  const int kb = blockIdx.x, wl = blockIdx.y;
  const int P = nb1 * nb2;
  for (int j = threadIdx.x; j < KB; j += blockDim.x) {
    const long long k = (long long)kb * KB + j;
    float2 pr = make_float2(0.0f, 0.0f);
    if (k < K) {
      const int kpt = (int)(k / P), pp = (int)(k - (long long)kpt * P);
      const int ib = pp / nb2, jb = pp - ib * nb2;
      const double w = coef * kcw[(size_t)ib + (size_t)nb1 * ((size_t)jb + (size_t)nb2 * ((size_t)kpt + (size_t)nkp * (om0 + wl)))];
      const float hi = __double2float_rn(w);
      const float lo = __double2float_rn(w - (double)hi);
      pr = make_float2(hi, lo);
    }
    wpair[(size_t)wl * K_pad + k] = pr;
  }
}

// Exact row maxima of |V_trunc·c·w| per frequency (V relative to 2^eA), as
// float bits: nonnegative floats order like unsigned integers.
__global__ void k_rowmax_B(const __nv_bfloat16* __restrict__ adig, const float2* __restrict__ wpair, int R, int R_pad,
                           long long K_pad, unsigned* rmax) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y, wl = blockIdx.z;
  float m = 0.0f;
  if (k < K_pad && r < R) {
    const float a0 = __bfloat162float(adig[((size_t)0 * R_pad + r) * K_pad + k]);
    const float a1 = __bfloat162float(adig[((size_t)1 * R_pad + r) * K_pad + k]);
    const float a2 = __bfloat162float(adig[((size_t)2 * R_pad + r) * K_pad + k]);
    const float vhi = (a0 * 0x1p-8f + a1 * 0x1p-16f) + a2 * 0x1p-24f;
    m = __fmul_ru(fabsf(vhi), fabsf(wpair[(size_t)wl * K_pad + k].x));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  __shared__ float sm[8];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    float mm = sm[0];
    for (int i = 1; i < (int)(blockDim.x >> 5); i++) mm = fmaxf(mm, sm[i]);
    if (mm > 0.0f) atomicMax(rmax + (size_t)wl * R_pad + r, __float_as_uint(mm));
  }
}

// fB = eA + exponent of the row maximum (with margin for the low-order terms
// of the product, which row_exponent's 1+1e-6 factor covers).
__global__ void k_row_exp_B(const unsigned* rmax, const int* eA, int R, int R_pad, int nw, int* fB) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nw * R_pad) return;
  const int r = i % R_pad;
  fB[i] = (r < R) ? eA[r] + row_exponent(__uint_as_float(rmax[i])) : 0;
}

// B digits of c·w_K·V[r,K] from the A digits, in FP32 pair arithmetic:
// V = 2^eA (hi + lo) exactly (hi: digits 0-2, lo: digits 3-4), c·w = wh + wl,
// product to ~46 bits with one exact FMA error term, then 5 signed digits
// relative to 2^fB carried as an unevaluated float pair.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
__global__ void k_digits_B(const __nv_bfloat16* __restrict__ adig, const int* eA, const float2* __restrict__ wpair,
                           const int* fB, int R, int R_pad, long long K_pad, int wb, __nv_bfloat16* bdig) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y, wl = blockIdx.z;
  if (k >= K_pad) return;
  float a[S];
#pragma unroll
  for (int s = 0; s < S; s++) a[s] = __bfloat162float(adig[((size_t)s * R_pad + r) * K_pad + k]);
  const float vhi = ((a[0] * 0x1p-8f + a[1] * 0x1p-16f) + a[2] * 0x1p-24f);   // exact
  const float vlo = (a[3] * 0x1p-32f + a[4] * 0x1p-40f);                       // exact
  const float2 w = wpair[(size_t)wl * K_pad + k];
  const float ph = vhi * w.x;
  const float pe = fmaf(vhi, w.x, -ph);
  const float pl = pe + (vhi * w.y + vlo * w.x);
  const int sh = (r < R) ? (eA[r] - fB[(size_t)wl * R_pad + r]) : 0;
  float yh = ldexpf(ph, sh), yl = ldexpf(pl, sh);
  two_sum(yh, yl, yh, yl);
#pragma unroll
  for (int s = 0; s < S; s++) {
    const float t = yh * 256.0f;
    const float dg = rintf(t);
    const float rh = t - dg;              // exact
    two_sum(rh, yl * 256.0f, yh, yl);
    bdig[(((size_t)wl * S + s) * R_pad + r) * K_pad + k] = __float2bfloat16_rn(dg);
  }
}

// χ0[ω][J][I] (complex, full matrix) from the digit-group sums.
__global__ void k_assemble(const double* __restrict__ out, const int* eA, const int* fB, int N, int R_pad, int nT,
                           int npair, int nsplit, int wb, int om0, double2* __restrict__ eps) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y;
  const int wl = blockIdx.z;
  if (I >= N) return;
  auto G = [&](int r, int c) -> double {
    int a = r, b = c;
    if (a / TM > b / TM) { a = c; b = r; }    // stored tiles are ti ≤ tj
    const int ti = a / TM, tj = b / TM;
    const int pair = ti * nT - ti * (ti - 1) / 2 + (tj - ti);
    double s = 0.0;
    for (int sp = 0; sp < nsplit; sp++)
      s += out[((((size_t)sp * wb + wl) * npair + pair) * TM + (b % TM)) * TM + (a % TM)];
    return ldexp(s, eA[a] + fB[(size_t)wl * R_pad + b] - 16);
  };
  const double re = G(I, J) + G(N + I, N + J);
  const double im = G(N + I, J) - G(I, N + J);
  eps[((size_t)(om0 + wl) * N + J) * N + I] = make_double2(re, im);
}

}  // namespace pgm

// ---------------------------------------------------------------- host side
using namespace pgm;

static size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

struct MixedLayout {
  long long K, K_pad;
  int N, R, R_pad, nT, npair, nkb, nsplit, kb_per_split, wb;
  size_t off_adig, off_bdig, off_tmax, off_wpair, off_rmax, off_eA, off_fB, off_out, total;
};

static MixedLayout mixed_layout(int nb1, int nb2, int nkp, int npb, int wb, int kb_split) {
  MixedLayout L;
  L.K = (long long)nkp * nb1 * nb2;
  L.K_pad = (L.K + KB - 1) / KB * KB;
  L.nkb = (int)(L.K_pad / KB);
  L.N = npb;
  L.R = 2 * npb;
  L.R_pad = (L.R + TM - 1) / TM * TM;
  L.nT = L.R_pad / TM;
  L.npair = L.nT * (L.nT + 1) / 2;
  // Exact-range split: a group sum over one split stays below 2^35
  // (5 pairs · kb·64 · 129² < 2^35  →  kb ≤ 6452).
  const int kb_max = (kb_split > 0 && kb_split < 6400) ? kb_split : 6400;
  L.nsplit = (L.nkb + kb_max - 1) / kb_max;
  L.kb_per_split = (L.nkb + L.nsplit - 1) / L.nsplit;
  L.wb = wb;
  size_t o = 0;
  L.off_adig = o; o += al256((size_t)S * L.R_pad * L.K_pad * 2);
  L.off_bdig = o; o += al256((size_t)wb * S * L.R_pad * L.K_pad * 2);
  L.off_tmax = o; o += al256((size_t)L.R_pad * L.nkb * 4);
  L.off_wpair = o; o += al256((size_t)wb * L.K_pad * 8);
  L.off_rmax = o; o += al256((size_t)wb * L.R_pad * 4);     // row maxima of |V·c·w| (float bits)
  L.off_eA = o; o += al256((size_t)L.R_pad * 4);
  L.off_fB = o; o += al256((size_t)wb * L.R_pad * 4);
  L.off_out = o; o += al256((size_t)L.nsplit * wb * L.npair * TM * TM * 8);
  L.total = o;
  return L;
}

static PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return nullptr;
    fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  }
  return fn;
}

static bool make_map(CUtensorMap* m, void* base, long long cols, long long rows) {
  auto enc = get_encode();
  if (!enc) return false;
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
  cuuint32_t box[2] = {(cuuint32_t)KB, (cuuint32_t)TM};
  cuuint32_t es[2] = {1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

extern "C" size_t pg_chi0_mixed_workspace(int nb1, int nb2, int nkp, int npb, int omega_batch, int kb_split) {
  if (nb1 <= 0 || nb2 <= 0 || nkp <= 0 || npb <= 0 || omega_batch <= 0) return 0;
  return mixed_layout(nb1, nb2, nkp, npb, omega_batch, kb_split).total;
}

// χ0 for frequencies [0, nom) from the matrix elements of all k (device,
// [nkp][P][N] complex128) and kcw (device, Fortran (nb1, nb2, nkp, nom)).
// Writes the full Hermitian χ0 (before symmetrisation, +1 and inversion) to
// eps[ω][J][I].  Frequencies are processed omega_batch at a time; kb_split
// (> 0) caps the 64-value K-blocks one CTA sums (0 = the largest exact range).
extern "C" int pg_chi0_mixed(const void* minm, int nkp, const double* kcw, int nb1, int nb2, int nom, int npb,
                             double coef, void* eps, void* work, size_t work_bytes, int omega_batch, int kb_split,
                             unsigned* d_status, void* stream) {
  if (!minm || !kcw || !eps || !work || nkp <= 0 || nb1 <= 0 || nb2 <= 0 || nom <= 0 || npb <= 0 || omega_batch <= 0)
    return PG_EARG;
  const int wb = omega_batch < nom ? omega_batch : nom;
  MixedLayout L = mixed_layout(nb1, nb2, nkp, npb, wb, kb_split);
  if (work_bytes < L.total) return PG_EWORKSPACE;
  if (L.R_pad > (1 << 20) || L.K_pad > (1ll << 31)) return PG_ETOOBIG;
  cudaStream_t s = (cudaStream_t)stream;
  char* w = (char*)work;
  __nv_bfloat16* adig = (__nv_bfloat16*)(w + L.off_adig);
  __nv_bfloat16* bdig = (__nv_bfloat16*)(w + L.off_bdig);
  float* tmax = (float*)(w + L.off_tmax);
  float2* wpair = (float2*)(w + L.off_wpair);
  unsigned* rmax = (unsigned*)(w + L.off_rmax);
  int* eA = (int*)(w + L.off_eA);
  int* fB = (int*)(w + L.off_fB);
  double* out = (double*)(w + L.off_out);
  const double2* M = (const double2*)minm;

  // padding rows of the digit arrays must be zero
  if (cudaMemsetAsync(adig, 0, (size_t)S * L.R_pad * L.K_pad * 2, s) != cudaSuccess) return PG_ECUDA;
  if (cudaMemsetAsync(tmax, 0, (size_t)L.R_pad * L.nkb * 4, s) != cudaSuccess) return PG_ECUDA;
  k_block_max<<<dim3((npb + 127) / 128, L.nkb), 128, 0, s>>>(M, L.K, npb, L.R_pad, L.nkb, tmax);
  k_row_exp_A<<<L.R_pad, 256, 0, s>>>(tmax, L.R, L.R_pad, L.nkb, eA);
  k_digits_A<<<dim3((unsigned)((L.K_pad + 31) / 32), (npb + 31) / 32), 256, 0, s>>>(M, L.K, npb, L.R_pad, L.K_pad, eA,
                                                                                    adig);
  pg_count_launches(3);

  CUtensorMap mapA, mapB;
  if (!make_map(&mapA, adig, L.K_pad, (long long)S * L.R_pad)) return PG_ECUDA;
  if (!make_map(&mapB, bdig, L.K_pad, (long long)wb * S * L.R_pad)) return PG_ECUDA;
  const size_t smem = (size_t)NST * STAGE_BYTES + 1024 + 256;
  if (cudaFuncSetAttribute(k_ozaki_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return PG_ECUDA;
  OzParams op;
  op.out = out; op.status = d_status; op.R_pad = L.R_pad; op.nT = L.nT; op.npair = L.npair; op.nkb = L.nkb;
  op.kb_per_split = L.kb_per_split; op.nsplit = L.nsplit;
  for (int om0 = 0; om0 < nom; om0 += wb) {
    const int nw = (om0 + wb <= nom) ? wb : nom - om0;
    op.wb = wb;
    k_weights_prep<<<dim3(L.nkb, nw), 64, 0, s>>>(kcw, nb1, nb2, nkp, om0, nw, coef, L.K, L.K_pad, wpair);
    if (cudaMemsetAsync(rmax, 0, (size_t)L.wb * L.R_pad * 4, s) != cudaSuccess) return PG_ECUDA;
    k_rowmax_B<<<dim3((unsigned)((L.K_pad + 255) / 256), L.R_pad, nw), 256, 0, s>>>(adig, wpair, L.R, L.R_pad,
                                                                                   L.K_pad, rmax);
    k_row_exp_B<<<(nw * L.R_pad + 255) / 256, 256, 0, s>>>(rmax, eA, L.R, L.R_pad, nw, fB);
    k_digits_B<<<dim3((unsigned)((L.K_pad + 255) / 256), L.R_pad, nw), 256, 0, s>>>(adig, eA, wpair, fB, L.R, L.R_pad,
                                                                                   L.K_pad, nw, bdig);
    k_ozaki_gemm<<<dim3(L.npair, nw, L.nsplit), NTHREADS, smem, s>>>(mapA, mapB, op);
    k_assemble<<<dim3((npb + 127) / 128, npb, nw), 128, 0, s>>>(out, eA, fB, npb, L.R_pad, L.nT, L.npair, L.nsplit,
                                                               wb, om0, (double2*)eps);
    pg_count_launches(6);
  }
  return cudaGetLastError() == cudaSuccess ? PG_OK : PG_ECUDA;
}

// Workspace layout of pg_chi0_mixed, for inspection by tests:
// offs = {adig, bdig, tmax, wpair, rmax, eA, fB, out, total} (bytes),
// dims = {K, K_pad, R, R_pad, nT, npair, nkb, nsplit, kb_per_split}.
extern "C" int pg_chi0_mixed_layout(int nb1, int nb2, int nkp, int npb, int omega_batch, int kb_split, size_t* offs,
                                    long long* dims) {
  if (nb1 <= 0 || nb2 <= 0 || nkp <= 0 || npb <= 0 || omega_batch <= 0 || !offs || !dims) return PG_EARG;
  MixedLayout L = mixed_layout(nb1, nb2, nkp, npb, omega_batch, kb_split);
  const size_t o[9] = {L.off_adig, L.off_bdig, L.off_tmax, L.off_wpair, L.off_rmax, L.off_eA, L.off_fB, L.off_out,
                       L.total};
  const long long d[9] = {L.K, L.K_pad, L.R, L.R_pad, L.nT, L.npair, L.nkb, L.nsplit, L.kb_per_split};
  for (int i = 0; i < 9; i++) { offs[i] = o[i]; dims[i] = d[i]; }
  return PG_OK;
}
