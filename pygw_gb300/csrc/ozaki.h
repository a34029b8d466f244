// Split-precision (Ozaki-type) digit GEMM shared by the χ0 contraction and
// the refinement of ε⁻¹: internal interface, not part of the C-ABI.
//
// A value x of a row with exponent e is held as five signed 8-bit digits,
//     x ≈ 2^e Σ_s a_s 2^(−8(s+1)),  |a_s| ≤ 129,  |x − that| ≤ 2^(e−40),
// stored as bf16 in K-block-major planes (see digit_index).  The GEMM sums
// the digit products of pairs s + t ≤ 4 exactly and returns, per 128×128
// output tile, Σ_d 2^(−8d) I_d in FP64; the caller scales by 2^(eA + fB − 16).
#pragma once
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stddef.h>

namespace pgm {

constexpr int OZ_S = 5;         // digits per value
constexpr int OZ_TILE = 128;    // output tile edge
constexpr int OZ_BLOCK = 256;   // rows of A and of B are padded to multiples of this
constexpr int OZ_KB = 64;       // K-block width

// Digit arrays are K-block major: plane (digit, or frequency·5 + digit), then
// 64-wide K-block, then row, then 64 values — one 128-row TMA tile is 16 KB of
// contiguous memory.
__host__ __device__ __forceinline__ size_t digit_index(int plane, int r, long long k, int R_pad, int nkb) {
  return (((size_t)plane * nkb + (size_t)(k >> 6)) * R_pad + r) * 64 + (size_t)(k & 63);
}

// Row exponent e with max|x|·(1+2^-20) < 2^(e−1): every value of the row is then
// |x / 2^e| < 1/2 and its leading digit |rint(256·x/2^e)| ≤ 128.
__device__ __forceinline__ int row_exponent(float bound) {
  if (!(bound > 0.0f)) return 0;
  int e;
  frexpf(bound * 1.000001f, &e);   // bound·(1+eps) in [2^(e−1), 2^e)
  return e + 1;
}

// Full product G_w = A_w · B_wᵀ for nw frequencies with sd (5 or 6) digits
// per value and digit pairs s + t ≤ sd − 1 (A digits per frequency, R_padA × K,
// B digits R_padB × K, K = 64·nkb, one K split; sd = 6 takes the result from
// ≈ 2^-40 to ≈ 2^-48 of the row scales).
// out: [nw][R_padA/128 · R_padB/128 tiles][128 (col)][128 (row)] float pairs
// (hi, lo), 8 bytes per element; an element's value is (double)hi + (double)lo.
// nTbv: B tiles holding real rows.  Returns a PG_* code.
// a_per_w: A digits per frequency (1) or one set shared by the frequencies (0).
int launch_gemm_general(const __nv_bfloat16* adig, const __nv_bfloat16* bdig, int sd, int a_per_w, int R_padA,
                        int R_padB, int nTbv, int nkb, int nw, double* out, unsigned* status, cudaStream_t s);

}  // namespace pgm

namespace pgx {
// Exponents and nd (5 or 6) digits of the columns of X[nw][N][N] (complex128,
// column-major per frequency) as B rows [Re X(:,j); Im X(:,j)] of the general
// product; bdig/fB are laid out for R_pad rows and nkb K-blocks.
int launch_cols_digits(const double2* X, int N, int nw, int R_pad, int nkb, int nd, int* fB, __nv_bfloat16* bdig,
                       cudaStream_t s);

}  // namespace pgm
