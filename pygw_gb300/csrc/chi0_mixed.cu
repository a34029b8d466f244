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
// < 2^24) the epilogue warps move the multiples of 2^12 into an FP32 register
// accumulator (exact while below 2^36 — the host splits K so it stays
// below 2^35) and leave the remainder in place.  Each group's integer is
// then combined into the output tile: in FP64 for the symmetric χ0 product,
// as a float pair (≈ 2^-47 relative) for the general product.  The only other
// rounding is the dropped 5th-digit residual and the dropped d ≥ 5 pairs
// (≈ 1e-11 relative per row scale).
//
// Kernel layout: a cluster of two CTAs (a CTA pair) owns a 256×256 block of
// the upper block triangle of G, per frequency, per K-split, computed by
// 2-SM MMAs (tcgen05.mma.cta_group::2, M = 256, N = 256, K = 16) that the
// pair's first CTA issues: CTA r holds the 128 A rows of tile ti = 2·rp + r
// and the 128 B rows cb·256 + r·128 … of the block in its own shared memory
// (plain TMA loads into its own shared memory, completing on the first CTA's
// barrier), and its 128 rows × 256 columns of the accumulator in its own
// tensor memory.  Each SM thus reads 32 KB from L2 per 64-wide K-block, and a
// stage is 32 KB, so six stages fit.
// Warp 0 issues the TMA loads (A tile + the CTA's B half per stage, 128-byte
// swizzle, 6 stages), warp 1 allocates TMEM and (first CTA) issues the MMAs, warps 2 …
// renormalise: the low accumulators (two 256-column TMEM buffers used in
// turn, so the tensor core keeps working while the previous chunk is
// renormalised) and a high accumulator per group held in registers (each
// epilogue thread owns one row × 128 or × 64 columns, see epi_warps).  A stage is refilled only when
// the pair's MMAs have read it (each MMA commit arrives on both CTAs' "empty"
// barriers); the MMA issuer reuses an accumulator when the epilogue threads
// of both CTAs have arrived on its barrier.
// Every wait is bounded by OzParams::wait_ns of %globaltimer (5 s unless the
// host sets another limit with pg_set_wait_limit_ns); on expiry the kernel
// records PG_ERR_TIMEOUT, stops issuing, waits (bounded by a fixed 5 s, never
// by the shortened limit) until its issued TMA loads have landed and its
// issued MMAs have completed, frees TMEM and returns.
#include <cuda_runtime.h>
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include <string.h>
#include "pygw_status.h"
#include "launches.h"
#include "ozaki.h"
#include "tc_ptx.h"

namespace pgm {

constexpr int S = OZ_S;         // digits per value
constexpr int TM = 128;         // tile rows (A) = B rows loaded by one CTA
constexpr int TN = 256;         // columns of a cluster's block
constexpr int KB = 64;          // K per stage (one 128-byte swizzle row of bf16)
constexpr int NST = 6;          // pipeline stages
constexpr int LBLK = 14;        // K-blocks per exact chunk: 14·64·129² + 2^11 < 2^24
constexpr int CL = 2;           // CTAs per cluster: the pair of a 2-SM MMA
constexpr int TILE_BYTES = TM * KB * 2;           // 16 KB: one 128-row digit tile
constexpr int STAGE_BYTES = 2 * TILE_BYTES;       // A tile + this CTA's B half
// Epilogue warps: 8 (each thread one row × 128 columns) for the symmetric χ0
// product, whose long K hides the epilogue behind the MMAs; 16 (one row × 64
// columns) for the general product, whose short K leaves the digit-group ends
// on the critical path — half the registers per thread, more tile loads in
// flight (C3 self-energy step 8.12 → 6.66 s; χ0 at C3 76.3 → 79.9 ms with 16).
__host__ __device__ constexpr int epi_warps(bool general) { return general ? 16 : 8; }
__host__ __device__ constexpr int gemm_threads(bool general) { return 32 * (2 + epi_warps(general)); }
constexpr uint32_t TMEM_COLS = 512;               // two 256-column low accumulators
constexpr unsigned long long WAIT_NS = 5000000000ull;   // default limit of one wait (5 s)
constexpr unsigned long long DRAIN_NS = 5000000000ull;  // limit of the drain waits before exit (fixed)

struct OzParams {
  double* out;          // [nsplit][wb][npair][128 (col)][128 (row)]: FP64, or in the general
                        // product float pairs (hi, lo) whose sum is the value (see df_add2)
  unsigned* status;
  int R_pad, nT, nTv, nC, npair, nkb, kb_per_split, nsplit, wb;
  // general (full, non-symmetric) product: A digits per frequency, B with its own rows
  int gen;              // 0: upper block triangle of V·diag(w)·Vᵀ; 1: full A·Bᵀ
  int a_per_w;          // A planes per frequency (1) or shared by the batch (0)
  int nTb, nTbv, nCb;   // B: 128-row tiles, tiles with real rows, 256-row blocks
  int nw;               // frequencies of this launch (≤ wb, the output's frequency stride)
  int wl0;              // B planes of this launch start at frequency wl0 of the digit array
  unsigned long long wait_ns;   // limit of one pipeline wait (%globaltimer ns)
};

// ------------------------------------------------ 2-SM (CTA pair) helpers
// Shared::cluster address of this CTA's shared variable at `a` in CTA `rank`.
__device__ __forceinline__ uint32_t mapa_rank(uint32_t a, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
// Arrive on an mbarrier given by its shared::cluster address (either CTA of the pair).
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t bar_cluster) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(bar_cluster) : "memory");
}
// TMA tile load into this CTA's shared memory, completing on the barrier at
// shared::cluster address bar_cluster (which may be the pair's other CTA's).
__device__ __forceinline__ void tma_load_3d_pair(void* dst, const CUtensorMap* map, uint32_t bar_cluster, int x,
                                                 int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, "
      "%5}], [%2];" ::"r"(smem_u32(dst)),
      "l"((uint64_t)map), "r"(bar_cluster), "r"(x), "r"(y), "r"(z)
      : "memory");
}
// 2-SM MMA: D (both CTAs' tensor memory, 128 lanes each) += A (128 rows from
// each CTA) · B (N/2 rows from each CTA), operands at the same shared-memory
// offsets in both CTAs.
__device__ __forceinline__ void tc_mma_pair(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                            uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
      : "memory");
}
// Arrive on the barrier at this shared-memory offset in both CTAs of the pair
// once the pair's MMAs issued so far by this thread have completed.
__device__ __forceinline__ void tc_commit_pair(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::
                   "r"(smem_u32(bar)),
               "h"((uint16_t)3)
               : "memory");
}
// The same, on this CTA's barrier only.
__device__ __forceinline__ void tc_commit_pair_local(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
// Instruction descriptor, kind::f16: D=F32, A=B=BF16, both K-major, M=256 (pair), N=n.
__host__ __device__ constexpr uint32_t idesc_m256(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(256 >> 4) << 24);
}

// (v.x + v.y) + a + b as a normalised float pair (hi, lo) by Knuth's two-sum:
// with a, b exact (group integers times 2^-8d) the pair holds the running
// tile value to ≈ 2^-47 relative, with FP32 operations only (FP64 runs at a
// small fraction of the FP32 rate on this GPU, and the general product's short
// K leaves the epilogue's group ends on the critical path).  The _rn
// intrinsics keep the compiler from fusing products into the sums.
__device__ __forceinline__ void two_sum_rn(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ float2 df_add2(float2 v, float a, float b) {
  float s1, e1, s2, e2, x, y;
  two_sum_rn(v.x, a, s1, e1);
  two_sum_rn(s1, b, s2, e2);
  two_sum_rn(s2, __fadd_rn(__fadd_rn(e1, e2), v.y), x, y);
  return make_float2(x, y);
}

// Linear index → (i, j), i ≤ j < n, row-major over the upper triangle.
__host__ __device__ __forceinline__ void tri_pair(int lin, int n, int& i, int& j) {
  int t = 0, rem = lin;
  while (rem >= n - t) { rem -= n - t; t++; }
  i = t; j = t + rem;
}

// Coordinates of load i of a CTA: digit pair (s, t) in the order d = 0..SD−1,
// s = 0..d, then the K-block; ya / yb = first rows of the A tile and of this
// CTA's 128-row half of the block's B tile, za / zb = their (plane, K-block) slices.
template <int SD>
__device__ __forceinline__ void load_coords(const OzParams& p, int i, int nkbs, int kb0, int ti, int wl, int cb,
                                            int crank, int& ya, int& za, int& yb, int& zb) {
  const int pi = i / nkbs;
  int d = 0;
  while ((d + 1) * (d + 2) / 2 <= pi) d++;
  const int s_ = pi - d * (d + 1) / 2, t_ = d - s_;
  const int kb = kb0 + (i - pi * nkbs);
  ya = ti * TM;
  za = ((p.a_per_w ? wl * SD : 0) + s_) * p.nkb + kb;
  yb = cb * TN + crank * TM;
  zb = ((p.wl0 + wl) * SD + t_) * p.nkb + kb;
}

// ------------------------------------------------------ the digit GEMM
// SD digits per value; digit pairs s + t ≤ SD − 1 (SD = 5 for χ0, 6 for the
// residual of the ε⁻¹ refinement).
template <int SD, bool DF>
__global__ void __launch_bounds__(gemm_threads(DF), 1)
    k_ozaki_gemm(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, OzParams p) {
  constexpr int NEPI = epi_warps(DF);             // epilogue warps: NEPI/4 per TMEM lane quarter
  constexpr int CW = TN / (NEPI / 4);             // columns per epilogue thread
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
  const int crank = (int)cluster_rank();
  // Work units (output block, frequency, K split), numbered with the output
  // block fastest; cluster cid takes units cid, cid + ncl, …  (the host launches
  // one cluster per unit; a smaller grid makes the kernel persistent).
  const int ncl = gridDim.x / CL, cid = blockIdx.x / CL;
  const int nitems = p.gen ? p.nC * p.nCb : p.nC * (p.nC + 1) / 2;
  const int nunits = nitems * p.nw * p.nsplit;

  if (threadIdx.x == 0) {
    for (int i = 0; i < NST; i++) { mbar_init(full + i, 1); mbar_init(empty + i, 1); }
    // acc_empty / group_done: one arrival per epilogue warp (no unbounded named
    // barrier); the first CTA's barriers take the epilogue warps of both CTAs
    for (int i = 0; i < 2; i++) { mbar_init(acc_full + i, 1); mbar_init(acc_empty + i, CL * NEPI); }
    mbar_init(group_done, CL * NEPI);
    mbar_init(drain, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    // one warp of each CTA of the pair allocates, together
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_base_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  cluster_sync_all();            // the pair's barriers exist before either CTA signals the other's
  tc_fence_after();
  const uint32_t tmem = *tmem_base_slot;

  // One unit: output block (rp, cb), this CTA's row tile ti, frequency wl and
  // K range [kb0, kb1); the pair's MMA computes both 128-column tiles of the
  // block (the one below the diagonal of a diagonal block is not stored).
  struct Unit { int rp, cb, ti, wl, split, kb0, kb1; };
  auto unit = [&](int u) {
    Unit U;
    const int item = u % nitems, rest = u / nitems;
    U.wl = rest % p.nw;
    U.split = rest / p.nw;
    if (p.gen) { U.rp = item / p.nCb; U.cb = item % p.nCb; }
    else tri_pair(item, p.nC, U.rp, U.cb);
    U.ti = 2 * U.rp + crank;
    U.kb0 = U.split * p.kb_per_split;
    U.kb1 = min(p.nkb, U.kb0 + p.kb_per_split);
    return U;
  };

  if (warp == 0) {
    // ---------------------------------------------------------- TMA producer
    // Per unit, load order: for d = 0..SD−1, s = 0..d (t = d − s), K-blocks kb0..kb1−1.
    if (lane == 0) {
      int it = 0;
      bool ok = true;
      for (int u = cid; u < nunits && ok; u += ncl) {
        const Unit U = unit(u);
        const int nkbs = U.kb1 - U.kb0;
        const int total = (SD * (SD + 1) / 2) * nkbs;
        for (int i = 0; i < total && ok; i++, it++) {
          const int st = it % NST;
          if (it >= NST) ok = mbar_wait(empty + st, ((it / NST) - 1) & 1, abort_flag, p.status, p.wait_ns);
          if (!ok) break;
          int ya, za, yb, zb;
          load_coords<SD>(p, i, nkbs, U.kb0, U.ti, U.wl, U.cb, crank, ya, za, yb, zb);
          unsigned char* sa = smem + st * STAGE_BYTES;
          // both CTAs' loads of this stage complete on the first CTA's barrier,
          // which expects the bytes of both
          if (crank == 0) mbar_expect_tx(full + st, CL * STAGE_BYTES);
          const uint32_t bar = mapa_rank(smem_u32(full + st), 0);
          tma_load_3d_pair(sa, &tmA, bar, 0, ya, za);
          tma_load_3d_pair(sa + TILE_BYTES, &tmB, bar, 0, yb, zb);
        }
      }
      // drain: the last phase of every stage has been read by the pair's MMAs
      // (so every load into this CTA has landed) before the CTA may exit
      const int issued = it;
      const unsigned long long t0 = gtime();
      for (int j = max(0, issued - NST); j < issued; j++) {
        const int st = j % NST;
        while (!mbar_test(empty + st, (j / NST) & 1) && gtime() - t0 < DRAIN_NS) {}
      }
    }
  } else if (warp == 1) {
    // ---------------------------------------------------------- MMA issuer (first CTA of the pair)
    if (lane == 0 && crank == 0) {
      int it = 0, c = 0, G = 0;          // loads, chunks and digit groups consumed so far
      bool ok = true;
      const uint32_t idesc = idesc_m256(TN);
      for (int u = cid; u < nunits && ok; u += ncl) {
        const Unit U = unit(u);
        const int nchunk_per_pass = (U.kb1 - U.kb0 + LBLK - 1) / LBLK;
        for (int d = 0; d < SD && ok; d++, G++) {
          // the epilogue has combined the previous group (its remainders are read)
          if (G > 0) ok = mbar_wait(group_done, (G - 1) & 1, abort_flag, p.status, p.wait_ns);
          if (!ok) break;
          bool used[2] = {false, false};
          for (int s = 0; s <= d && ok; s++) {
            for (int ch = 0; ch < nchunk_per_pass && ok; ch++, c++) {
              const int b = c & 1;
              if (c >= 2) ok = mbar_wait(acc_empty + b, ((c >> 1) - 1) & 1, abort_flag, p.status, p.wait_ns);
              if (!ok) break;
              tc_fence_after();
              const uint32_t dcol = tmem + (uint32_t)(b * TN);
              const int cb0 = U.kb0 + ch * LBLK, cb1 = min(U.kb1, cb0 + LBLK);
              for (int kb = cb0; kb < cb1; kb++, it++) {
                const int st = it % NST;
                ok = mbar_wait(full + st, (it / NST) & 1, abort_flag, p.status, p.wait_ns);
                if (!ok) break;
                tc_fence_after();
                const uint32_t sa = smem_u32(smem + st * STAGE_BYTES);
                const uint64_t ad = sdesc_sw128(sa), bd = sdesc_sw128(sa + TILE_BYTES);
#pragma unroll
                for (int k = 0; k < KB / 16; k++) {
                  const uint32_t accumulate = (used[b] || kb > cb0 || k > 0) ? 1u : 0u;
                  tc_mma_pair(dcol, ad + (uint64_t)(2 * k), bd + (uint64_t)(2 * k), idesc, accumulate);
                }
                tc_commit_pair(empty + st);   // stage free in both CTAs once these MMAs have read it
              }
              if (!ok) break;
              used[b] = true;
              tc_commit_pair(acc_full + b);     // chunk complete in both CTAs' tensor memory
            }
          }
        }
      }
      // drain: wait for every MMA this thread issued
      tc_commit_pair_local(drain);
      const unsigned long long t0 = gtime();
      while (!mbar_test(drain, 0) && gtime() - t0 < DRAIN_NS) {}
    }
  } else {
    // ---------------------------------------------------------- epilogue (warps 2 … 2+NEPI−1)
    const int q = warp & 3;                        // TMEM lane quarter this warp may access
    const int sl = (warp - 2) >> 2;                // column slice of the block (CW columns)
    const int h = (sl * CW) / TM;                  // its 128-column tile of the block
    const int co = (sl * CW) % TM;                 // its first column within that tile
    const int row = q * 32 + lane;                 // accumulator row (A tile row)
    const uint32_t t_b0 = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(sl * CW);
    const uint32_t t_b1 = t_b0 + TN;
    float hi[CW];                                  // high accumulator: multiples of 2^12, exact below 2^36
    int c = 0;
    bool ok = true;
    for (int u = cid; u < nunits && ok; u += ncl) {
      const Unit U = unit(u);
      const int tj = 2 * U.cb + h;
      const bool stored = p.gen || tj >= U.ti;     // tile (ti, tj) is kept
      // a tile below the diagonal is computed by the pair's MMA but neither
      // read nor stored (its accumulator columns are left to grow)
      const bool active = stored;
      const int pair = p.gen ? U.ti * p.nTb + tj : stored ? U.ti * p.nT - U.ti * (U.ti - 1) / 2 + (tj - U.ti) : 0;
      double* out = p.out + ((((size_t)U.split * p.wb + U.wl) * p.npair + pair) * TM) * TM;
      const int nchunk_per_pass = (U.kb1 - U.kb0 + LBLK - 1) / LBLK;
      for (int d = 0; d < SD && ok; d++) {
#pragma unroll
        for (int i = 0; i < CW; i++) hi[i] = 0.0f;
        const int nchunks_group = (d + 1) * nchunk_per_pass;
        const int c_first = c;
        for (int gc = 0; gc < nchunks_group && ok; gc++, c++) {
          const int b = c & 1;
          // warp-uniform outcome: the tcgen05.ld/st below are warp-collective
          ok = __all_sync(0xffffffffu, mbar_wait(acc_full + b, (c >> 1) & 1, abort_flag, p.status, p.wait_ns));
          if (!ok) break;
          tc_fence_after();
          if (active) {
            const uint32_t tl = b ? t_b1 : t_b0;
#pragma unroll
            for (int cc = 0; cc < CW / 16; cc++) {
              float lo[16];
              tmem_ld16(tl + cc * 16, lo);
#pragma unroll
              for (int i = 0; i < 16; i++) {
                // nearest multiple of 2^12 (ties to even): lo + 1.5·2^35 lies in
                // [2^35, 2^36), where the float spacing is 2^12 (|lo| < 2^24), so
                // the addition rounds lo there and the subtraction is exact — two
                // additions instead of a multiply, a rounding and a multiply
                const float hh = __fsub_rn(__fadd_rn(lo[i], 0x1.8p35f), 0x1.8p35f);
                lo[i] = __fsub_rn(lo[i], hh);                                  // |residual| ≤ 2^11
                hi[cc * 16 + i] += hh;
              }
              tmem_st16(tl + cc * 16, lo);
            }
          }
          if (gc == nchunks_group - 1 && active) {
            // group complete: I_d = high + both low remainders (|r| ≤ 2^11, so r0 + r1 is
            // exact in FP32 and high + r0 + r1 exact in FP64), scaled by 2^(−8d);
            // 8 columns at a time keep the live registers to hi[] + 16
            const bool used0 = nchunks_group >= 2 || (c_first & 1) == 0;
            const bool used1 = nchunks_group >= 2 || (c_first & 1) == 1;
            if constexpr (!DF) {
              const double scale = ldexp(1.0, -8 * d);
#pragma unroll
              for (int cc = 0; cc < CW / 8; cc++) {
                float l0[8], l1[8];
                if (used0) tmem_ld8(t_b0 + cc * 8, l0);
                if (used1) tmem_ld8(t_b1 + cc * 8, l1);
#pragma unroll
                for (int i = 0; i < 8; i++) {
                  const float r = (used0 ? l0[i] : 0.0f) + (used1 ? l1[i] : 0.0f);
                  const double v = (double)hi[cc * 8 + i] + (double)r;
                  double& o = out[(size_t)(co + cc * 8 + i) * TM + row];
                  o = (d == 0) ? v * scale : o + v * scale;
                }
              }
            } else {
              // float-pair tile: hi·2^-8d and r·2^-8d are exact floats
              float2* out2 = reinterpret_cast<float2*>(out);
              const float fscale = __int_as_float((127 - 8 * d) << 23);
#pragma unroll
              for (int cc = 0; cc < CW / 8; cc++) {
                float l0[8], l1[8];
                if (used0) tmem_ld8(t_b0 + cc * 8, l0);
                if (used1) tmem_ld8(t_b1 + cc * 8, l1);
#pragma unroll
                for (int i = 0; i < 8; i++) {
                  const float r = __fadd_rn(used0 ? l0[i] : 0.0f, used1 ? l1[i] : 0.0f);
                  float2& o = out2[(size_t)(co + cc * 8 + i) * TM + row];
                  const float2 prev = (d == 0) ? make_float2(0.0f, 0.0f) : o;
                  o = df_add2(prev, __fmul_rn(hi[cc * 8 + i], fscale), __fmul_rn(r, fscale));
                }
              }
            }
          }
          // the MMA issuer (first CTA) waits for the epilogue warps of both CTAs:
          // each thread's tensor-memory accesses are complete (waited above) and
          // fenced, the warp converges, and one lane arrives for all 32
          tc_fence_before();
          __syncwarp();
          if (lane == 0) {
            mbar_arrive_cluster(mapa_rank(smem_u32(acc_empty + b), 0));
            if (gc == nchunks_group - 1) mbar_arrive_cluster(mapa_rank(smem_u32(group_done), 0));
          }
        }
      }
      if (stored && !ok) {
        for (int i = 0; i < CW; i++) out[(size_t)(co + i) * TM + row] = __longlong_as_double(0x7ff8dead00000000LL);
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  cluster_sync_all();            // neither CTA leaves while the other may still write to it
  tc_fence_after();
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
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

// Knuth's two-sum: s = fl(a + b), e = the exact rounding error (s + e = a + b).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// One digit step of a float pair carried scaled by 256, (Yh, Yl) = 256·(yh, yl)
// with |Yl| ≤ ulp(Yh)/2: d = the nearest integer to Yh, and (Yh, Yl) ← 256 ×
// the pair of (Yh − d) + Yl.  r = Yh − d is exact and a multiple of u = ulp(Yh)
// (u ≤ 1 whenever Yh is not an integer; r = 0 otherwise), while |Yl| ≤ u/2, so
// r = 0 or |r| ≥ |Yl|: Dekker's fast two-sum is then exact.  Its sum and error
// are formed already scaled by 256 (256·r is exact, so fma(r, 256, ·) rounds
// once, as the unscaled sum does), six operations per digit; |Yl| ≤ ulp(Yh)/2
// holds again.  The digits are those of the unscaled two-sum step: scaling by
// 256 commutes with rounding wherever a digit can be nonzero.
__device__ __forceinline__ float digit_step(float& Yh, float& Yl) {
  const float d = rintf(Yh);
  const float r = Yh - d;               // exact
  const float B = Yl * 256.0f;          // exact
  const float S = fmaf(r, 256.0f, B);   // 256·fl(r + Yl)
  Yl = B + fmaf(r, 256.0f, -S);         // 256 × the exact rounding error of fl(r + Yl)
  Yh = S;
  return d;
}

// A digits (bf16, K-block major, see digit_index).  The value scaled by 2^-eA
// is split once into a float pair (hi = nearest float, lo = nearest float to
// the rest, ≈ 48 bits), and the digits are taken from the pair in FP32 with
// exact two-sums, as k_digits_B does: |value − digits| stays below 2^(eA−40),
// and FP64 work drops from ≈ 17 operations per value to 4 (GB300 runs FP64
// at a small fraction of the FP32 rate).
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
      // ·2^(8−e) (the row scaling and the first digit's 256) as a multiply by
      // a normal double: the same correctly rounded product as ldexp (which
      // costs several FP64 operations)
      const int e = eA[r];
      const double x = part ? m.y : m.x;
      const double y = (e >= -1014 && e <= 1030) ? x * __longlong_as_double((long long)(1031 - e) << 52)
                                                 : ldexp(x, 8 - e);
      const float h = __double2float_rn(y);
      float yh = h, yl = __double2float_rn(y - (double)h);
      for (int s = 0; s < S; s++) {
        const float d = digit_step(yh, yl);
        adig[digit_index(s, r, k, R_pad, (int)(K_pad >> 6))] = __float2bfloat16_rn(d);
      }
    }
  }
}

// Weights for a batch of frequencies: c·w as an FP32 pair (hi + lo ≈ 48 bits).
// K-value k of the chunk → (point kpt, pair pp): uniform windows (kstart null)
// have P = nb1·nb2 pairs per point; ragged ones have nb1·knb2[kpt] pairs
// starting at kstart[kpt], pp = ib·knb2[kpt] + jb.
__global__ void k_weights_prep(const double* __restrict__ kcw, int nb1, int nb2, int nkp, int k0, int nkc,
                               const int* __restrict__ kstart, const int* __restrict__ knb2, int om0, int wb,
                               double coef, long long K, long long K_pad, float2* wpair) {
  const int kb = blockIdx.x, wl = blockIdx.y;
  const int P = nb1 * nb2;
  for (int j = threadIdx.x; j < KB; j += blockDim.x) {
    const long long k = (long long)kb * KB + j;
    float2 pr = make_float2(0.0f, 0.0f);
    if (k < K) {
      int kpt, ib, jb;
      if (kstart) {
        int lo = 0, hi = nkc;                    // kstart[lo] ≤ k < kstart[hi]
        while (hi - lo > 1) {
          const int mid = (lo + hi) >> 1;
          if ((long long)kstart[mid] <= k) lo = mid; else hi = mid;
        }
        kpt = lo;
        const int pp = (int)(k - kstart[kpt]), n2 = knb2[kpt];
        ib = pp / n2;
        jb = pp - ib * n2;
      } else {
        kpt = (int)(k / P);
        const int pp = (int)(k - (long long)kpt * P);
        ib = pp / nb2;
        jb = pp - ib * nb2;
      }
      const double w =
          coef * kcw[(size_t)ib + (size_t)nb1 * ((size_t)jb + (size_t)nb2 * ((size_t)(k0 + kpt) + (size_t)nkp * (om0 + wl)))];
      const float hi = __double2float_rn(w);
      const float lo = __double2float_rn(w - (double)hi);
      pr = make_float2(hi, lo);
    }
    wpair[(size_t)wl * K_pad + k] = pr;
  }
}

// Four consecutive bf16 digits (8 bytes) as floats.
__device__ __forceinline__ void ld_bf16x4(const __nv_bfloat16* p, float (&v)[4]) {
  const uint2 u = *reinterpret_cast<const uint2*>(p);
  v[0] = __uint_as_float(u.x << 16);
  v[1] = __uint_as_float(u.x & 0xffff0000u);
  v[2] = __uint_as_float(u.y << 16);
  v[3] = __uint_as_float(u.y & 0xffff0000u);
}
// Four floats holding integers |d| ≤ 256 (exact in bf16) stored as 8 bytes.
__device__ __forceinline__ void st_bf16x4(__nv_bfloat16* p, const float (&v)[4]) {
  uint2 u;
  u.x = (__float_as_uint(v[0]) >> 16) | (__float_as_uint(v[1]) & 0xffff0000u);
  u.y = (__float_as_uint(v[2]) >> 16) | (__float_as_uint(v[3]) & 0xffff0000u);
  *reinterpret_cast<uint2*>(p) = u;
}

// Exact row maxima of |V_trunc·c·w| for every frequency of the batch (V relative
// to 2^eA), as float bits: nonnegative floats order like unsigned integers.
// One pass over the A digits serves all nw frequencies; 4 K-values per thread.
__global__ void k_rowmax_B(const __nv_bfloat16* __restrict__ adig, const float2* __restrict__ wpair, int R, int R_pad,
                           long long K_pad, int nw, unsigned* rmax) {
  const long long k0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * 4;
  const int r = blockIdx.y;
  const bool in = k0 < K_pad && r < R;
  float v[4] = {0.0f, 0.0f, 0.0f, 0.0f};
  if (in) {
    float a0[4], a1[4], a2[4];
    const int nkb = (int)(K_pad >> 6);
    ld_bf16x4(adig + digit_index(0, r, k0, R_pad, nkb), a0);
    ld_bf16x4(adig + digit_index(1, r, k0, R_pad, nkb), a1);
    ld_bf16x4(adig + digit_index(2, r, k0, R_pad, nkb), a2);
#pragma unroll
    for (int j = 0; j < 4; j++) v[j] = fabsf((a0[j] * 0x1p-8f + a1[j] * 0x1p-16f) + a2[j] * 0x1p-24f);
  }
  __shared__ float sm[32];
  for (int wl = 0; wl < nw; wl++) {
    float m = 0.0f;
    if (in) {
      const float4* wp = reinterpret_cast<const float4*>(wpair + (size_t)wl * K_pad + k0);
      const float4 w01 = wp[0], w23 = wp[1];
      m = fmaxf(fmaxf(__fmul_ru(v[0], fabsf(w01.x)), __fmul_ru(v[1], fabsf(w01.z))),
                fmaxf(__fmul_ru(v[2], fabsf(w23.x)), __fmul_ru(v[3], fabsf(w23.z))));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
      float mm = sm[0];
      for (int i = 1; i < (int)(blockDim.x >> 5); i++) mm = fmaxf(mm, sm[i]);
      if (mm > 0.0f) atomicMax(rmax + (size_t)wl * R_pad + r, __float_as_uint(mm));
    }
    __syncthreads();
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
// With wnext (the next batch's weights, nwn frequencies) the same pass also
// forms that batch's row maxima into rmax_next, exactly as k_rowmax_B does
// (the three-digit |V| it needs is vhi here), so only the first batch of a
// contraction needs its own k_rowmax_B pass over the A digits.
// Block: DB_ROWS rows × 16 threads (4 values each: one 64-value K-block row,
// 128 bytes), over DB_KB consecutive K-blocks; in the K-block-major digit
// layout the block's rows of one K-block are DB_ROWS·128 contiguous bytes of
// every plane (one row per block scattered its accesses in 128-byte pieces
// R_pad·128 bytes apart).  Dynamic shared memory: nwn·DB_ROWS floats.
constexpr int DB_ROWS = 16, DB_KB = 8;
__global__ void __launch_bounds__(256, 6) k_digits_B(const __nv_bfloat16* __restrict__ adig, const int* eA,
                                                     const float2* __restrict__ wpair, const int* fB, int R, int R_pad,
                                                     long long K_pad, int nw, __nv_bfloat16* bdig,
                                                     const float2* __restrict__ wnext, int nwn, unsigned* rmax_next) {
  extern __shared__ float smax[];                // [nwn][DB_ROWS] row maxima of the next batch
  const int nkb = (int)(K_pad >> 6);
  const int lr = threadIdx.x >> 4, lk = threadIdx.x & 15;
  const int r = blockIdx.y * DB_ROWS + lr;       // < R_pad (a multiple of 256)
  const int eAr = (r < R) ? eA[r] : 0;
  for (int i = threadIdx.x; i < nwn * DB_ROWS; i += blockDim.x) smax[i] = 0.0f;
  __syncthreads();
  for (int kbi = 0; kbi < DB_KB; kbi++) {
    const int kb = blockIdx.x * DB_KB + kbi;
    if (kb >= nkb) break;                        // uniform across the block
    const long long k0 = (long long)kb * KB + lk * 4;
    float vhi[4], vlo[4];
    {
      float a[S][4];
#pragma unroll
      for (int s = 0; s < S; s++) ld_bf16x4(adig + digit_index(s, r, k0, R_pad, nkb), a[s]);
#pragma unroll
      for (int j = 0; j < 4; j++) {
        vhi[j] = ((a[0][j] * 0x1p-8f + a[1][j] * 0x1p-16f) + a[2][j] * 0x1p-24f);   // exact
        vlo[j] = (a[3][j] * 0x1p-32f + a[4][j] * 0x1p-40f);                         // exact
      }
    }
    for (int wl = 0; wl < nw; wl++) {
      const float4* wp = reinterpret_cast<const float4*>(wpair + (size_t)wl * K_pad + k0);
      const float4 w01 = wp[0], w23 = wp[1];
      const float wh[4] = {w01.x, w01.z, w23.x, w23.z}, wo[4] = {w01.y, w01.w, w23.y, w23.w};
      const int sh = (r < R) ? (eAr - fB[(size_t)wl * R_pad + r]) : 0;
      // 2^(sh+8) (the scaling to 2^fB and the first digit's 256) as a float
      // when it is a normal number (a multiply then scales exactly as ldexpf does)
      const bool fast = sh >= -134 && sh <= 119;
      const float p2 = fast ? __int_as_float((sh + 135) << 23) : 1.0f;
      float dg[S][4];
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const float ph = vhi[j] * wh[j];
        const float pe = fmaf(vhi[j], wh[j], -ph);
        const float pl = pe + (vhi[j] * wo[j] + vlo[j] * wh[j]);
        float yh = fast ? ph * p2 : ldexpf(ph, sh + 8), yl = fast ? pl * p2 : ldexpf(pl, sh + 8);
        two_sum(yh, yl, yh, yl);
#pragma unroll
        for (int s = 0; s < S; s++) dg[s][j] = digit_step(yh, yl);
      }
#pragma unroll
      for (int s = 0; s < S; s++) st_bf16x4(bdig + digit_index(wl * S + s, r, k0, R_pad, nkb), dg[s]);
    }
    for (int wl = 0; wl < nwn; wl++) {
      float m = 0.0f;
      if (r < R) {
        const float4* wp = reinterpret_cast<const float4*>(wnext + (size_t)wl * K_pad + k0);
        const float4 w01 = wp[0], w23 = wp[1];
        m = fmaxf(fmaxf(__fmul_ru(fabsf(vhi[0]), fabsf(w01.x)), __fmul_ru(fabsf(vhi[1]), fabsf(w01.z))),
                  fmaxf(__fmul_ru(fabsf(vhi[2]), fabsf(w23.x)), __fmul_ru(fabsf(vhi[3]), fabsf(w23.z))));
      }
      // maximum over the 16 threads of this row (one half of the warp)
      for (int o = 8; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
      if (lk == 0) smax[wl * DB_ROWS + lr] = fmaxf(smax[wl * DB_ROWS + lr], m);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nwn * DB_ROWS; i += blockDim.x) {
    const int rr = blockIdx.y * DB_ROWS + (i % DB_ROWS);
    if (rr < R && smax[i] > 0.0f) atomicMax(rmax_next + (size_t)(i / DB_ROWS) * R_pad + rr, __float_as_uint(smax[i]));
  }
}

// χ0[ω][J][I] (complex, full matrix) from the digit-group sums.
__global__ void k_assemble(const double* __restrict__ out, const int* eA, const int* fB, int N, int R_pad, int nT,
                           int npair, int nsplit, int wb, int om0, int accumulate, double2* __restrict__ eps) {
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
  double2& e = eps[((size_t)(om0 + wl) * N + J) * N + I];
  if (accumulate) e = make_double2(e.x + re, e.y + im);
  else e = make_double2(re, im);
}

}  // namespace pgm

// ---------------------------------------------------------------- host side
using namespace pgm;

static size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

// Limit of one pipeline wait inside k_ozaki_gemm, for every launch after it
// is set (process-wide; 0 restores the default of 5 s).  A short limit makes
// a wait expire on purpose: the launch then records PG_ERR_TIMEOUT in its
// status word, marks its unfinished output tiles with NaN and returns, which
// is how the expiry path is tested.
#include <atomic>
static std::atomic<unsigned long long> g_wait_ns{WAIT_NS};
constexpr int PREP_BATCH = 4;
extern "C" void pg_set_wait_limit_ns(unsigned long long ns) { g_wait_ns.store(ns ? ns : WAIT_NS); }
extern "C" unsigned long long pg_wait_limit_ns(void) { return g_wait_ns.load(); }

struct MixedLayout {
  long long K, K_pad;
  int N, R, R_pad, nT, nTv, nC, nitems, npair, nkb, nsplit, kb_per_split, wb, wbp;
  size_t off_adig, off_bdig, off_tmax, off_wpair, off_rmax, off_eA, off_fB, off_out, total;
};

static size_t gemm_smem_bytes() { return (size_t)NST * STAGE_BYTES + 1024 + 256; }

// CTAs of k_ozaki_gemm that run at once on the current device (cached per device).
#include <algorithm>
#include <mutex>
static std::mutex g_cap_mutex;
static int g_cap[64] = {0};
static int gemm_cta_capacity() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 2 * 74;
  std::lock_guard<std::mutex> lk(g_cap_mutex);
  if (g_cap[dev]) return g_cap[dev];
  int ncl = 0;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(CL, 1, 1);
  cfg.blockDim = dim3(gemm_threads(false));
  cfg.dynamicSmemBytes = gemm_smem_bytes();
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (cudaFuncSetAttribute(k_ozaki_gemm<S, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gemm_smem_bytes()) !=
          cudaSuccess ||
      cudaOccupancyMaxActiveClusters(&ncl, k_ozaki_gemm<S, false>, &cfg) != cudaSuccess || ncl <= 0) {
    cudaGetLastError();
    int sms = 148;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    ncl = sms / CL;
  }
  g_cap[dev] = ncl * CL;
  return g_cap[dev];
}

// Frequencies per B-digit preparation pass (process-wide, read by every
// layout computation after it is set, workspace queries included).  A pass
// reads the five A digit planes once and writes the five B planes of each of
// its frequencies, so a longer pass cuts the A reads per frequency (at C3 a
// frequency's B planes are 24.4 GB and the A planes 24.4 GB: 36.6 GB of
// traffic per frequency with two per pass, 30.5 GB with four) at the cost of
// one set of B planes of workspace per frequency.  0 restores the default, 4.
static std::atomic<int> g_prep_batch{PREP_BATCH};
extern "C" int pg_set_chi0_prep_batch(int n) {
  if (n < 0 || n > 64) return PG_EARG;
  g_prep_batch.store(n ? n : PREP_BATCH);
  return PG_OK;
}
extern "C" int pg_chi0_prep_batch(void) { return g_prep_batch.load(); }

static MixedLayout mixed_layout(int nb1, int nb2, int nkp, int npb, int wb, int kb_split, long long K = -1) {
  MixedLayout L;
  L.K = K >= 0 ? K : (long long)nkp * nb1 * nb2;
  L.K_pad = (L.K + KB - 1) / KB * KB;
  L.nkb = (int)(L.K_pad / KB);
  L.N = npb;
  L.R = 2 * npb;
  L.R_pad = (L.R + TN - 1) / TN * TN;       // whole 256-column blocks
  L.nT = L.R_pad / TM;                      // 128-row tiles (even)
  L.nTv = (L.R + TM - 1) / TM;              // tiles holding real rows
  L.nC = L.R_pad / TN;                      // 256-column blocks
  L.nitems = L.nC * (L.nC + 1) / 2;         // upper-triangle blocks, one cluster each
  L.npair = L.nT * (L.nT + 1) / 2;          // stored 128×128 tiles
  // Exact-range split: a group sum over one split stays below 2^35
  // (5 pairs · kb·64 · 129² < 2^35  →  kb ≤ 6452).
  if (kb_split > 0) {
    const int kb_max = kb_split < 6400 ? kb_split : 6400;
    L.nsplit = (L.nkb + kb_max - 1) / kb_max;
  } else {
    // Automatic: the fewest splits (≥ the exact-range minimum, ≥ 256 K-blocks
    // each) whose CTA count fills the last wave of the device to ≥ 95 %.
    const int cap = gemm_cta_capacity();
    const int ns0 = (L.nkb + 6399) / 6400;
    int best = ns0;
    double best_eff = 0.0;
    for (int ns = ns0; ns <= 4 * ns0 + 8 && (ns == ns0 || L.nkb / ns >= 256); ns++) {
      const double waves = (double)CL * L.nitems * wb * ns / cap;
      const double eff = waves / ceil(waves);
      if (eff > best_eff + 0.01) { best = ns; best_eff = eff; }
      if (eff >= 0.95) break;
    }
    L.nsplit = best;
  }
  L.kb_per_split = (L.nkb + L.nsplit - 1) / L.nsplit;
  L.nsplit = (L.nkb + L.kb_per_split - 1) / L.kb_per_split;   // no empty split
  L.wb = wb;
  // B digits are prepared for several frequencies per pass over the A digits
  // (each pass reads all five A planes; see pg_set_chi0_prep_batch), a whole
  // number of GEMM batches, while the GEMM may take one frequency per launch
  const int pb = g_prep_batch.load();
  L.wbp = wb >= pb ? wb : (pb + wb - 1) / wb * wb;
  size_t o = 0;
  L.off_adig = o; o += al256((size_t)S * L.R_pad * L.K_pad * 2);
  L.off_bdig = o; o += al256((size_t)L.wbp * S * L.R_pad * L.K_pad * 2);
  L.off_tmax = o; o += al256((size_t)L.R_pad * L.nkb * 4);
  // two preparation batches' weights and row maxima (the next batch's maxima
  // are formed while the current batch's digits are written)
  L.off_wpair = o; o += al256((size_t)2 * L.wbp * L.K_pad * 8);
  L.off_rmax = o; o += al256((size_t)2 * L.wbp * L.R_pad * 4);  // row maxima of |V·c·w| (float bits)
  L.off_eA = o; o += al256((size_t)L.R_pad * 4);
  L.off_fB = o; o += al256((size_t)L.wbp * L.R_pad * 4);
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

// 3-D map over a K-block-major digit array: {64 values, R_pad rows, planes·nkb
// K-blocks}; box 64 × 128 × 1 with the 128-byte swizzle the MMA descriptors use.
static bool make_map(CUtensorMap* m, void* base, int R_pad, long long nslices) {
  auto enc = get_encode();
  if (!enc) return false;
  cuuint64_t dims[3] = {(cuuint64_t)KB, (cuuint64_t)R_pad, (cuuint64_t)nslices};
  cuuint64_t strides[2] = {(cuuint64_t)KB * 2, (cuuint64_t)KB * 2 * R_pad};
  cuuint32_t box[3] = {(cuuint32_t)KB, (cuuint32_t)TM, 1};
  cuuint32_t es[3] = {1, 1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
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
// gemm_events (optional): 2 per batch, recorded around each digit-GEMM launch.
static int chi0_mixed_impl(const void* minm, int nkp, int k0, const int* kstart, const int* knb2, long long nK,
                           int nkp_total, const double* kcw, int nb1, int nb2, int nom, int npb, double coef, void* eps,
                           int accumulate, void* work, size_t work_bytes, int omega_batch, int kb_split,
                           unsigned* d_status, void* stream, void* const* gemm_events) {
  if (!minm || !kcw || !eps || !work || nkp <= 0 || nb1 <= 0 || nb2 <= 0 || nom <= 0 || npb <= 0 || omega_batch <= 0 ||
      k0 < 0 || k0 + nkp > nkp_total)
    return PG_EARG;
  if (kstart && (!knb2 || nK <= 0 || nK > (long long)nkp * nb1 * nb2)) return PG_EARG;
  const int wb = omega_batch < nom ? omega_batch : nom;
  MixedLayout L = mixed_layout(nb1, nb2, nkp, npb, wb, kb_split, kstart ? nK : -1);
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

  // padding rows of the digit arrays must be zero: no pass writes them, so
  // they are cleared once per contraction (rows R … R_pad−1 of every
  // (plane, K-block) slice, R_pad·128 bytes apart)
  if (L.R_pad > L.R) {
    const size_t pitch = (size_t)L.R_pad * KB * 2, off = (size_t)L.R * KB * 2, width = pitch - off;
    if (cudaMemset2DAsync((char*)adig + off, pitch, 0, width, (size_t)S * L.nkb, s) != cudaSuccess ||
        cudaMemset2DAsync((char*)bdig + off, pitch, 0, width, (size_t)L.wbp * S * L.nkb, s) != cudaSuccess)
      return PG_ECUDA;
  }
  if (cudaMemsetAsync(tmax, 0, (size_t)L.R_pad * L.nkb * 4, s) != cudaSuccess) return PG_ECUDA;
  k_block_max<<<dim3((npb + 127) / 128, L.nkb), 128, 0, s>>>(M, L.K, npb, L.R_pad, L.nkb, tmax);
  k_row_exp_A<<<L.R_pad, 256, 0, s>>>(tmax, L.R, L.R_pad, L.nkb, eA);
  k_digits_A<<<dim3((unsigned)((L.K_pad + 31) / 32), (npb + 31) / 32), 256, 0, s>>>(M, L.K, npb, L.R_pad, L.K_pad, eA,
                                                                                    adig);
  pg_count_launches(3);

  CUtensorMap mapA, mapB;
  if (!make_map(&mapA, adig, L.R_pad, (long long)S * L.nkb)) return PG_ECUDA;
  if (!make_map(&mapB, bdig, L.R_pad, (long long)L.wbp * S * L.nkb)) return PG_ECUDA;
  const size_t smem = gemm_smem_bytes();
  if (cudaFuncSetAttribute(k_ozaki_gemm<S, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return PG_ECUDA;
  OzParams op;
  op.out = out; op.status = d_status; op.R_pad = L.R_pad; op.nT = L.nT; op.nTv = L.nTv; op.nC = L.nC;
  op.gen = 0; op.a_per_w = 0; op.nTb = L.nT; op.nTbv = L.nTv; op.nCb = L.nC;
  op.npair = L.npair; op.nkb = L.nkb; op.kb_per_split = L.kb_per_split; op.nsplit = L.nsplit; op.wb = wb;
  op.wait_ns = g_wait_ns.load();
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  op.wl0 = 0;
  const int wbp = L.wbp;
  const size_t wstride = (size_t)wbp * L.K_pad, rstride = (size_t)wbp * L.R_pad;
  // first batch: weights and row maxima by their own pass
  {
    const int npw0 = wbp < nom ? wbp : nom;
    k_weights_prep<<<dim3(L.nkb, npw0), 64, 0, s>>>(kcw, nb1, nb2, nkp_total, k0, nkp, kstart, knb2, 0, npw0, coef,
                                                    L.K, L.K_pad, wpair);
    if (cudaMemsetAsync(rmax, 0, rstride * 4, s) != cudaSuccess) return PG_ECUDA;
    k_rowmax_B<<<dim3((unsigned)((L.K_pad + 1023) / 1024), L.R), 256, 0, s>>>(adig, wpair, L.R, L.R_pad, L.K_pad,
                                                                              npw0, rmax);
    pg_count_launches(2);
  }
  for (int op0 = 0, bi = 0; op0 < nom; op0 += wbp, bi++) {
    // B digits of the frequencies op0 … op0+npw−1 (one pass over the A digits),
    // which also forms the next batch's row maxima
    const int npw = (op0 + wbp <= nom) ? wbp : nom - op0;
    const int cur = bi & 1, nxt = cur ^ 1;
    const int on = op0 + wbp, npn = on < nom ? ((on + wbp <= nom) ? wbp : nom - on) : 0;
    float2* wcur = wpair + cur * wstride;
    float2* wnxt = wpair + nxt * wstride;
    unsigned* rcur = rmax + cur * rstride;
    unsigned* rnxt = rmax + nxt * rstride;
    k_row_exp_B<<<(npw * L.R_pad + 255) / 256, 256, 0, s>>>(rcur, eA, L.R, L.R_pad, npw, fB);
    if (npn > 0) {
      k_weights_prep<<<dim3(L.nkb, npn), 64, 0, s>>>(kcw, nb1, nb2, nkp_total, k0, nkp, kstart, knb2, on, npn, coef,
                                                     L.K, L.K_pad, wnxt);
      if (cudaMemsetAsync(rnxt, 0, rstride * 4, s) != cudaSuccess) return PG_ECUDA;
      pg_count_launches(1);
    }
    // real rows only (rounded up to whole row blocks; the rest stay zero)
    k_digits_B<<<dim3((unsigned)((L.nkb + DB_KB - 1) / DB_KB), (L.R + DB_ROWS - 1) / DB_ROWS), 256,
                 (size_t)(npn > 0 ? npn : 1) * DB_ROWS * sizeof(float), s>>>(
        adig, eA, wcur, fB, L.R, L.R_pad, L.K_pad, npw, bdig, npn > 0 ? wnxt : nullptr, npn, rnxt);
    pg_count_launches(2);
    for (int g0 = 0; g0 < npw; g0 += wb) {
      const int nw = (g0 + wb <= npw) ? wb : npw - g0;
      const int om0 = op0 + g0;
      cudaLaunchConfig_t cfg = {};
      op.nw = nw;
      op.wl0 = g0;
      // one cluster per unit: the hardware schedules the units in waves, whose
      // staggered starts spread the digit traffic over time (a grid of
      // co-resident clusters looping over the units measured 12 % slower at C3)
      const int nunits = L.nitems * nw * L.nsplit;
      cfg.gridDim = dim3((unsigned)(CL * nunits), 1, 1);
      cfg.blockDim = dim3(gemm_threads(false));
      cfg.dynamicSmemBytes = smem;
      cfg.stream = s;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      const int batch = om0 / wb;
      if (gemm_events && cudaEventRecord((cudaEvent_t)gemm_events[2 * batch], s) != cudaSuccess) return PG_ECUDA;
      if (cudaLaunchKernelEx(&cfg, k_ozaki_gemm<S, false>, mapA, mapB, op) != cudaSuccess) return PG_ECUDA;
      if (gemm_events && cudaEventRecord((cudaEvent_t)gemm_events[2 * batch + 1], s) != cudaSuccess) return PG_ECUDA;
      k_assemble<<<dim3((npb + 127) / 128, npb, nw), 128, 0, s>>>(out, eA, fB + (size_t)g0 * L.R_pad, npb, L.R_pad,
                                                                 L.nT, L.npair, L.nsplit, wb, om0, accumulate,
                                                                 (double2*)eps);
      pg_count_launches(2);
    }
  }
  return cudaGetLastError() == cudaSuccess ? PG_OK : PG_ECUDA;
}

extern "C" int pg_chi0_mixed(const void* minm, int nkp, const double* kcw, int nb1, int nb2, int nom, int npb,
                             double coef, void* eps, void* work, size_t work_bytes, int omega_batch, int kb_split,
                             unsigned* d_status, void* stream, void* const* gemm_events) {
  return chi0_mixed_impl(minm, nkp, 0, nullptr, nullptr, 0, nkp, kcw, nb1, nb2, nom, npb, coef, eps, 0, work,
                         work_bytes, omega_batch, kb_split, d_status, stream, gemm_events);
}

// The same for the k-points k0 .. k0+nk_chunk−1 (minm holds their blocks;
// kcw covers all nkp points): eps = (accumulate ? eps : 0) + their χ0.  Each
// chunk has its own row exponents; the chunks' sums add in FP64.  With
// kstart (device, nk_chunk+1 offsets) and knb2 (device, nk_chunk counts) the
// points have ragged windows: point i contributes nb1·knb2[i] pairs (the
// first knb2[i] of the nb2 unoccupied bands), its rows of minm starting at
// kstart[i], nK = kstart[nk_chunk] in all.  Workspace:
// pg_chi0_mixed_workspace(nb1, nb2, nk_chunk, npb, omega_batch, kb_split).
extern "C" int pg_chi0_mixed_accumulate(const void* minm, int nk_chunk, int k0, const int* kstart, const int* knb2,
                                        long long nK, const double* kcw, int nb1, int nb2, int nkp, int nom, int npb,
                                        double coef, void* eps, int accumulate, void* work, size_t work_bytes,
                                        int omega_batch, int kb_split, unsigned* d_status, void* stream,
                                        void* const* gemm_events) {
  return chi0_mixed_impl(minm, nk_chunk, k0, kstart, knb2, nK, nkp, kcw, nb1, nb2, nom, npb, coef, eps, accumulate,
                         work, work_bytes, omega_batch, kb_split, d_status, stream, gemm_events);
}

// Full product for the refinement of ε⁻¹ (see ozaki.h).
int pgm::launch_gemm_general(const __nv_bfloat16* adig, const __nv_bfloat16* bdig, int sd, int a_per_w, int R_padA,
                             int R_padB, int nTbv, int nkb, int nw, double* out, unsigned* status, cudaStream_t s) {
  // group sums stay below 2^35: sd pairs · nkb·64 · 129² < 2^35
  if (R_padA <= 0 || R_padB <= 0 || R_padA % TN || R_padB % TN || nkb <= 0 || nw <= 0 || (sd != 5 && sd != 6) ||
      (long long)sd * nkb * 64 * 16641 >= (1ll << 35))
    return PG_EARG;
  CUtensorMap mapA, mapB;
  if (!make_map(&mapA, (void*)adig, R_padA, (long long)(a_per_w ? nw : 1) * sd * nkb)) return PG_ECUDA;
  if (!make_map(&mapB, (void*)bdig, R_padB, (long long)nw * sd * nkb)) return PG_ECUDA;
  const size_t smem = gemm_smem_bytes();
  auto kern = (sd == 6) ? k_ozaki_gemm<6, true> : k_ozaki_gemm<5, true>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return PG_ECUDA;
  OzParams op;
  memset(&op, 0, sizeof(op));
  op.out = out; op.status = status;
  op.R_pad = R_padA; op.nT = R_padA / TM; op.nTv = R_padA / TM; op.nC = R_padA / TN;
  op.gen = 1; op.a_per_w = a_per_w ? 1 : 0; op.nTb = R_padB / TM; op.nTbv = nTbv; op.nCb = R_padB / TN;
  op.npair = op.nT * op.nTb; op.nkb = nkb; op.kb_per_split = nkb; op.nsplit = 1; op.wb = nw;
  op.wait_ns = g_wait_ns.load();
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cudaLaunchConfig_t cfg = {};
  op.nw = nw;
  cfg.gridDim = dim3((unsigned)(CL * op.nC * op.nCb * nw), 1, 1);
  cfg.blockDim = dim3(gemm_threads(true));
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (cudaLaunchKernelEx(&cfg, kern, mapA, mapB, op) != cudaSuccess) return PG_ECUDA;
  pg_count_launches(1);
  return PG_OK;
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
