// Correlation self-energy: the mwm contraction and the Matsubara convolution on sm_103a.
//
// MatrixElements2Band.calc_selfc (pygw.py:3352-3364) forms, per k and frequency,
//     mwm[ω, ib1, ib2] = wkq · Σ_{I,J} conj(M[p,I]) · W_ω[I,J] · M[p,J],   p = ib1·nb2 + ib2,
// with W = ε⁻¹ − 1 from calc_eps, plus for q = 0 head and wing terms on the
// pairs (ie1, ie1 + ncg_c).  Compute_selfc_inside (mcommon.py:80-165) then
// convolves mwm over the Matsubara axis: all_fr_convolutions / fr_convolution2
// (fnc.f90:90-177); on a denser mesh after cubic-spline interpolation
// (iopfreq 4, few_fr_convolutions); or, in the SVD basis, through
// many_fr_convolutions of the basis functions and a contraction with mwm.
//
// The contraction is a complex GEMM C = conj(M)·W (rows r = (k, p) of a
// k-chunk, N columns) followed by the row dots Σ_J C[r,J]·M[r,J]:
//   * FP64: k_mwm_f64, shared-memory tiles of conj(M) and W with the row dot
//     fused into the tile epilogue;
//   * split precision: the general digit GEMM with one digit set for
//     A = [[Re M, Im M], [−Im M, Re M]] shared by the frequencies and B = the
//     columns [Re W; Im W] per frequency (float-pair output tiles), then
//     k_mwm_reduce in float-pair arithmetic against a float-pair copy of M.
// Layouts: minm [nk][P][N], W [nom][N][N] (column-major per frequency),
// mwm [nk][nom][P], enk [nk][nb2], sc [nk][nb1][nom]; all complex128 but enk.
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include "pygw_status.h"
#include "launches.h"
#include "ozaki.h"

namespace pgc {

using pgm::digit_index;
using pgm::row_exponent;

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// ------------------------------------------------------------------ FP64
// Block: 32 rows × one frequency, 256 threads (row ty = tid/8; columns
// tx + 8c, c < 8, of a 64-column tile of W), I in chunks of 16.
__global__ void __launch_bounds__(256) k_mwm_f64(const double2* __restrict__ M, long long R, int N,
                                                 const double2* __restrict__ W, int P, int nom, int om0, double wkq,
                                                 double2* __restrict__ mwm) {
  __shared__ double2 Ms[32][17];
  __shared__ double2 Ws[16][65];
  const int tid = threadIdx.x, ty = tid >> 3, tx = tid & 7;
  const long long r0 = (long long)blockIdx.x * 32;
  const int wl = blockIdx.y;
  const double2* Ww = W + (size_t)N * N * wl;
  const long long r = r0 + ty;
  double2 part = make_double2(0.0, 0.0);
  for (int J0 = 0; J0 < N; J0 += 64) {
    double2 acc[8];
#pragma unroll
    for (int c = 0; c < 8; c++) acc[c] = make_double2(0.0, 0.0);
    for (int I0 = 0; I0 < N; I0 += 16) {
      for (int e = tid; e < 32 * 16; e += 256) {
        const int rr = e >> 4, i = e & 15;
        const long long row = r0 + rr;
        const int I = I0 + i;
        const double2 v = (row < R && I < N) ? M[(size_t)row * N + I] : make_double2(0.0, 0.0);
        Ms[rr][i] = make_double2(v.x, -v.y);                 // conj(M)
      }
      for (int e = tid; e < 16 * 64; e += 256) {
        const int i = e & 15, j = e >> 4;
        const int I = I0 + i, J = J0 + j;
        Ws[i][j] = (I < N && J < N) ? Ww[(size_t)N * J + I] : make_double2(0.0, 0.0);
      }
      __syncthreads();
#pragma unroll
      for (int i = 0; i < 16; i++) {
        const double2 a = Ms[ty][i];
#pragma unroll
        for (int c = 0; c < 8; c++) {
          const double2 b = Ws[i][tx + 8 * c];
          acc[c].x += a.x * b.x - a.y * b.y;
          acc[c].y += a.x * b.y + a.y * b.x;
        }
      }
      __syncthreads();
    }
    if (r < R) {
#pragma unroll
      for (int c = 0; c < 8; c++) {
        const int J = J0 + tx + 8 * c;
        if (J < N) {
          const double2 m = M[(size_t)r * N + J];
          part.x += acc[c].x * m.x - acc[c].y * m.y;
          part.y += acc[c].x * m.y + acc[c].y * m.x;
        }
      }
    }
  }
  // the 8 threads of a row are 8 consecutive lanes
  for (int o = 4; o > 0; o >>= 1) {
    part.x += __shfl_xor_sync(0xffffffffu, part.x, o);
    part.y += __shfl_xor_sync(0xffffffffu, part.y, o);
  }
  if (tx == 0 && r < R) {
    const long long k = r / P, p = r - k * P;
    mwm[((size_t)k * nom + om0 + wl) * P + p] = make_double2(wkq * part.x, wkq * part.y);
  }
}

// ------------------------------------------------------- split precision
// Rows r and R + r of A = [[Re M, Im M], [−Im M, Re M]] (the real form of
// conj(M), K = 2N): a shared exponent from max_I(|Re M|, |Im M|) and five
// digits per value; and X = M·2^-e as float pairs for the reduction.  One
// block per row r.
__global__ void __launch_bounds__(256) k_rows_digits(const double2* __restrict__ M, long long R, int N, int R_pad,
                                                     int nkb, int* eA, __nv_bfloat16* adig, float4* X) {
  const long long r = blockIdx.x;
  const double2* row = M + (size_t)r * N;
  double m = 0.0;
  for (int I = threadIdx.x; I < N; I += blockDim.x) {
    const double2 v = row[I];
    m = fmax(m, fmax(fabs(v.x), fabs(v.y)));
  }
  __shared__ double sm[256];
  __shared__ int se;
  sm[threadIdx.x] = m;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    se = row_exponent(__double2float_ru(sm[0]));
    eA[r] = se;
    eA[R + r] = se;
  }
  __syncthreads();
  const int e = se;
  const int ri = (int)r, rj = (int)(R + r);
  for (int I = threadIdx.x; I < N; I += blockDim.x) {
    const double2 x = row[I];
    double yr = ldexp(x.x, -e), yi = ldexp(x.y, -e);
    // M[r][I]·2^-e as float pairs (hi = nearest float, lo = nearest float to the rest),
    // column-major for the reduction's coalesced reads
    const float xh = __double2float_rn(yr), yh = __double2float_rn(yi);
    X[(size_t)I * R + r] = make_float4(xh, __double2float_rn(yr - (double)xh), yh, __double2float_rn(yi - (double)yh));
#pragma unroll
    for (int s = 0; s < pgm::OZ_S; s++) {
      const double tr = yr * 256.0, ti = yi * 256.0;
      const double dr = rint(tr), di = rint(ti);
      yr = tr - dr;
      yi = ti - di;
      const __nv_bfloat16 br = __float2bfloat16_rn((float)dr), bi = __float2bfloat16_rn((float)di);
      adig[digit_index(s, ri, I, R_pad, nkb)] = br;                 //  Re M
      adig[digit_index(s, ri, N + I, R_pad, nkb)] = bi;             //  Im M
      adig[digit_index(s, rj, I, R_pad, nkb)] = __hneg(bi);         // −Im M
      adig[digit_index(s, rj, N + I, R_pad, nkb)] = br;             //  Re M
    }
  }
}

// (S, C) += (gh + gl)·(xh + xl)·s with s a power of two, in float-pair
// arithmetic: the leading product exactly by FMA, the cross terms (≈ 2^-24 of
// it) into the low part, the sum by Knuth's two-sum.  The _rn intrinsics keep
// the compiler from fusing products into the sums.
__device__ __forceinline__ void df_mac(float gh, float gl, float xh, float xl, float s, float& S, float& C) {
  const float ah = __fmul_rn(gh, s), al = __fmul_rn(gl, s);          // exact
  const float p = __fmul_rn(ah, xh);
  float e = __fmaf_rn(ah, xh, -p);
  e = __fmaf_rn(ah, xl, e);
  e = __fmaf_rn(al, xh, e);
  e = __fmaf_rn(al, xl, e);
  const float t = __fadd_rn(S, p), b = __fsub_rn(t, S);
  C = __fadd_rn(C, __fadd_rn(__fadd_rn(__fsub_rn(S, __fsub_rn(t, b)), __fsub_rn(p, b)), e));
  S = t;
}

// mwm from the digit-GEMM tiles (float pairs): C[r,J] = (G[r][J] + i·G[R+r][J])·2^(eA[r] + fB[J] − 16),
// mwm = wkq·Σ_J C[r,J]·M[r,J] = wkq·2^(2·eA[r] − 16)·Σ_J G·2^fB[J]·X[J][r] with X = M·2^-eA
// (float pairs), summed in float-pair arithmetic: GB300's FP64 rate is a small
// fraction of its FP32 rate, and FP64 is used once per row.  Thread per (row, frequency).
__global__ void k_mwm_reduce(const double* __restrict__ out, const int* eA, const int* fB,
                             const float4* __restrict__ X, long long R, int N, int R_padB, int nTb, int ntile, int P,
                             int nom, int om0, double wkq, double2* __restrict__ mwm) {
  const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int wl = blockIdx.y;
  if (r >= R) return;
  const long long ri = R + r;
  const float2* out2 = reinterpret_cast<const float2*>(out);
  const float2* tr = out2 + ((size_t)wl * ntile + (size_t)(r >> 7) * nTb) * 16384 + (r & 127);
  const float2* ti = out2 + ((size_t)wl * ntile + (size_t)(ri >> 7) * nTb) * 16384 + (ri & 127);
  const int* f = fB + (size_t)R_padB * wl;
  float S1 = 0.0f, C1 = 0.0f, S2 = 0.0f, C2 = 0.0f;
  for (int J = 0; J < N; J++) {
    const size_t o = (size_t)(J >> 7) * 16384 + (size_t)(J & 127) * 128;
    const float2 gr = tr[o], gi = ti[o];
    const float4 x = X[(size_t)J * R + r];
    const float sJ = __int_as_float((f[J] + 127) << 23);
    // Re += G_re·Re X − G_im·Im X,  Im += G_re·Im X + G_im·Re X
    df_mac(gr.x, gr.y, x.x, x.y, sJ, S1, C1);
    df_mac(-gi.x, -gi.y, x.z, x.w, sJ, S1, C1);
    df_mac(gr.x, gr.y, x.z, x.w, sJ, S2, C2);
    df_mac(gi.x, gi.y, x.x, x.y, sJ, S2, C2);
  }
  const double sc = wkq * ldexp(1.0, 2 * eA[r] - 16);
  const long long k = r / P, p = r - k * P;
  mwm[((size_t)k * nom + om0 + wl) * P + p] =
      make_double2(sc * ((double)S1 + (double)C1), sc * ((double)S2 + (double)C2));
}

// q = 0 (pygw.py:3358-3363): for each GW band row ie1 the pair (ie1, ie1 + off)
// gets coefs2·head[ω] + coefs1·Σ_I M·epsw2[ω] + coefs1·Σ_I conj(M)·epsw1[ω]
// (off = ibgw + ncg_c).  Thread per (k, ie1, ω).
__global__ void k_mwm_q0(const double2* __restrict__ M, int nk, int nb1, int nb2, int N, int off, int nom,
                         const double2* __restrict__ head, const double2* __restrict__ epsw1,
                         const double2* __restrict__ epsw2, double coefs1, double coefs2, double2* __restrict__ mwm) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)nk * nb1 * nom) return;
  const int w = (int)(t % nom), ie1 = (int)((t / nom) % nb1), k = (int)(t / ((long long)nom * nb1));
  const int ie2 = ie1 + off;
  if (ie2 >= nb2) return;
  const int P = nb1 * nb2, p = ie1 * nb2 + ie2;
  const double2* m = M + ((size_t)k * P + p) * N;
  double2 a = make_double2(0.0, 0.0), c = make_double2(0.0, 0.0);
  for (int I = 0; I < N; I++) {
    const double2 v = m[I], e2 = epsw2[(size_t)w * N + I], e1 = epsw1[(size_t)w * N + I];
    a.x += v.x * e2.x - v.y * e2.y;            // M·epsw2
    a.y += v.x * e2.y + v.y * e2.x;
    c.x += v.x * e1.x + v.y * e1.y;            // conj(M)·epsw1
    c.y += v.x * e1.y - v.y * e1.x;
  }
  double2& d = mwm[((size_t)k * nom + w) * P + p];
  const double2 h = head[w];
  d.x += coefs2 * h.x + coefs1 * a.x + coefs1 * c.x;
  d.y += coefs2 * h.y + coefs1 * a.y + coefs1 * c.y;
}

// ------------------------------------------------------------ convolution
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
  // Smith's algorithm (R. L. Smith, CACM 5 (1962) 435)
  if (fabs(b.x) >= fabs(b.y)) {
    const double r = b.y / b.x, d = b.x + b.y * r;
    return make_double2((a.x + a.y * r) / d, (a.y - a.x * r) / d);
  } else {
    const double r = b.x / b.y, d = b.x * r + b.y;
    return make_double2((a.x * r + a.y) / d, (a.y * r - a.x) / d);
  }
}
// Principal complex arctangent from atan z = (i/2)·(log(1 − i z) − log(1 + i z)),
// with log|1 + u| = ½·log1p(2 Re u + |u|²) for accuracy near |z| → 0.
__device__ __forceinline__ double2 catan_(double2 z) {
  // 1 − i z = (1 + y) − i x,  1 + i z = (1 − y) + i x
  const double x = z.x, y = z.y, q = x * x + y * y;
  const double lr1 = 0.5 * log1p(2.0 * y + q), li1 = atan2(-x, 1.0 + y);
  const double lr2 = 0.5 * log1p(-2.0 * y + q), li2 = atan2(x, 1.0 - y);
  return make_double2(-0.5 * (li1 - li2), 0.5 * (lr1 - lr2));
}

// One fr_convolution2 term (fnc.f90:90-120): f on the mesh (om, wom, n),
// fi = the value at the output frequency omi, e the band energy.
__device__ __forceinline__ double2 conv_term(double e, const double2* f, size_t stride, double2 fi, double omi,
                                             const double* __restrict__ om, const double* __restrict__ wom, int n) {
  const double PI_F = 3.14159265358979;         // the truncated π of fnc.f90:71
  const double2 eo = make_double2(e, -omi);
  const double2 eo2 = cmul(eo, eo);
  double2 s0 = make_double2(0.0, 0.0);
  for (int i = 0; i < n; i++) {
    const double2 v = f[(size_t)i * stride];
    const double2 num = make_double2((v.x - fi.x) * wom[i], (v.y - fi.y) * wom[i]);
    const double2 q = cdiv(num, make_double2(om[i] * om[i] + eo2.x, eo2.y));
    s0.x += q.x;
    s0.y += q.y;
  }
  const double2 t0 = cmul(eo, s0);
  double2 res = make_double2(t0.x / PI_F, t0.y / PI_F);
  if (hypot(fi.x, fi.y) > 1e-16) {
    const double2 at = catan_(cdiv(make_double2(om[n - 1], 0.0), eo));
    const double2 v = cmul(make_double2(fi.x / PI_F, fi.y / PI_F), at);
    res.x += v.x;
    res.y += v.y;
  }
  return res;
}

// sc[k][ie1][iom] = Σ_ie2 of the fr_convolution2 term of f[k][·][ie1,ie2] at
// enk[k][ie2] and ω_iom, with mwm[k][iom][ie1,ie2] as the value subtracted and
// in the arctangent term: all_fr_convolutions with f = mwm on the same mesh,
// few_fr_convolutions with f = the interpolated mwm on the dense mesh
// (omd, womd, nd).  One block per (k, iom): the weighted inverse denominators
// womd_i/(ωd_i² + (e − iω)²) and the arctangents depend on (k, ie2, iom) only,
// so a block computes them once per chunk of 16 ie2 in shared memory and
// every ie1 row uses them (the per-term complex division was the cost).
// 256 threads = 16 ie1 × 16 ie2 of the chunk; ie1 beyond 16 in further passes.
constexpr int CONV_E2 = 16;
constexpr int CONV_MAXD = 128;      // mesh points held per chunk (larger meshes in slices)
__global__ void __launch_bounds__(256) k_fr_conv(const double2* __restrict__ mwm, const double2* __restrict__ f,
                                                 const double* __restrict__ enk, const double* __restrict__ om,
                                                 const double* __restrict__ omd, const double* __restrict__ womd,
                                                 int nk, int nb1, int nb2, int nom, int nd,
                                                 double2* __restrict__ sc) {
  const double PI_F = 3.14159265358979;         // the truncated π of fnc.f90:71
  __shared__ double2 D[CONV_E2][CONV_MAXD];     // 32 KB
  __shared__ double2 AT[CONV_E2];               // atan(ωd_last/(e − iω))/π
  __shared__ double2 EO[CONV_E2];               // e − iω
  const int iom = blockIdx.x, k = blockIdx.y;
  const int tj = threadIdx.x & 15, ti = threadIdx.x >> 4;
  const size_t P = (size_t)nb1 * nb2;
  const double omi = om[iom];
  for (int e10 = 0; e10 < nb1; e10 += 16) {
    const int ie1 = e10 + ti;
    double2 sum = make_double2(0.0, 0.0);
    for (int c0 = 0; c0 < nb2; c0 += CONV_E2) {
      const int ie2 = c0 + tj;
      const bool live = ie1 < nb1 && ie2 < nb2;
      const size_t p = (size_t)ie1 * nb2 + ie2;
      const double2 fi = live ? mwm[((size_t)k * nom + iom) * P + p] : make_double2(0.0, 0.0);
      double2 s0 = make_double2(0.0, 0.0);
      for (int i0 = 0; i0 < nd; i0 += CONV_MAXD) {
        const int ni = min(CONV_MAXD, nd - i0);
        __syncthreads();
        for (int e = threadIdx.x; e < CONV_E2 * ni; e += blockDim.x) {
          const int jj = e / ni, ii = e - jj * ni;
          const int j2 = c0 + jj, i = i0 + ii;
          if (j2 < nb2) {
            const double2 eo = make_double2(enk[(size_t)k * nb2 + j2], -omi);
            const double2 eo2 = cmul(eo, eo);
            const double2 one = make_double2(womd[i], 0.0);
            D[jj][ii] = cdiv(one, make_double2(omd[i] * omd[i] + eo2.x, eo2.y));
          }
        }
        if (i0 == 0 && threadIdx.x < CONV_E2 && c0 + (int)threadIdx.x < nb2) {
          const double2 eo = make_double2(enk[(size_t)k * nb2 + c0 + threadIdx.x], -omi);
          EO[threadIdx.x] = eo;
          const double2 at = catan_(cdiv(make_double2(omd[nd - 1], 0.0), eo));
          AT[threadIdx.x] = make_double2(at.x / PI_F, at.y / PI_F);
        }
        __syncthreads();
        if (live) {
          const double2* fr = f + (size_t)k * nd * P + p;
          for (int ii = 0; ii < ni; ii++) {
            const double2 v = fr[(size_t)(i0 + ii) * P];
            const double2 dv = make_double2(v.x - fi.x, v.y - fi.y);
            const double2 q = cmul(dv, D[tj][ii]);
            s0.x += q.x;
            s0.y += q.y;
          }
        }
      }
      if (live) {
        const double2 t0 = cmul(EO[tj], s0);
        double2 res = make_double2(t0.x / PI_F, t0.y / PI_F);
        if (hypot(fi.x, fi.y) > 1e-16) {
          const double2 v = cmul(fi, AT[tj]);
          res.x += v.x;
          res.y += v.y;
        }
        sum.x += res.x;
        sum.y += res.y;
      }
    }
    // the 16 ie2 lanes of a row are 16 consecutive threads
    for (int o = 8; o > 0; o >>= 1) {
      sum.x += __shfl_xor_sync(0xffffffffu, sum.x, o);
      sum.y += __shfl_xor_sync(0xffffffffu, sum.y, o);
    }
    if (tj == 0 && ie1 < nb1) sc[((size_t)k * nb1 + ie1) * nom + iom] = sum;
  }
}

// iopfreq 4 (mcommon.py:126-140): f[k][j][p] = Σ_i S[j][i]·(ω_i² + 1)·mwm[k][i][p] / (ωd_j² + 1)
// with S the cubic-spline interpolation matrix from the coarse to the dense
// mesh; the imaginary part is dropped where Σ_i |Im mwm[k][i][p]| / nom ≤ 1e-10.
// Thread per (k, p, j).
__global__ void k_interp(const double2* __restrict__ mwm, const double* __restrict__ S, const double* __restrict__ om,
                         const double* __restrict__ omd, int nk, int P, int nom, int nd, double2* __restrict__ f) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)nk * P * nd) return;
  const int p = (int)(t % P), j = (int)((t / P) % nd), k = (int)(t / ((long long)P * nd));
  const double2* m = mwm + (size_t)k * nom * P + p;
  double sr = 0.0, si = 0.0, aim = 0.0;
  for (int i = 0; i < nom; i++) {
    const double2 v = m[(size_t)i * P];
    const double a = om[i] * om[i] + 1.0;
    const double s = S[(size_t)j * nom + i];
    sr += s * (a * v.x);
    si += s * (a * v.y);
    aim += fabs(v.y);
  }
  const double b = omd[j] * omd[j] + 1.0;
  f[((size_t)k * nd + j) * P + p] = make_double2(sr / b, aim / nom > 1e-10 ? si / b : 0.0);
}

// SVD basis (mcommon.py:115-121): Cnl[k][l][ie2][iom] = conv_term of the basis
// function Ul[l][·] at enk[k][ie2] (many_fr_convolutions, fnc.f90:139-154).
__global__ void k_many_conv(const double2* __restrict__ Ul, const double* __restrict__ enk,
                            const double* __restrict__ om, const double* __restrict__ wom, int nk, int nl, int nb2,
                            int nom, double2* __restrict__ cnl) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)nk * nl * nb2 * nom) return;
  const int iom = (int)(t % nom), ie2 = (int)((t / nom) % nb2), l = (int)((t / ((long long)nom * nb2)) % nl);
  const int k = (int)(t / ((long long)nom * nb2 * nl));
  const double2* f = Ul + (size_t)l * nom;
  cnl[t] = conv_term(enk[(size_t)k * nb2 + ie2], f, 1, f[iom], om[iom], om, wom, nom);
}

// sc[k][ie1][iom] = Σ_l Σ_ie2 mwm[k][l][ie1,ie2]·Cnl[k][l][ie2][iom].  Thread per (k, ie1, iom).
__global__ void k_svd_sc(const double2* __restrict__ mwm, const double2* __restrict__ cnl, int nk, int nb1, int nb2,
                         int nl, int nom, double2* __restrict__ sc) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)nk * nb1 * nom) return;
  const int iom = (int)(t % nom), ie1 = (int)((t / nom) % nb1), k = (int)(t / ((long long)nom * nb1));
  const size_t P = (size_t)nb1 * nb2;
  double2 s = make_double2(0.0, 0.0);
  for (int l = 0; l < nl; l++) {
    const double2* m = mwm + ((size_t)k * nl + l) * P + (size_t)ie1 * nb2;
    const double2* c = cnl + (((size_t)k * nl + l) * nb2) * nom + iom;
    for (int ie2 = 0; ie2 < nb2; ie2++) {
      const double2 v = cmul(m[ie2], c[(size_t)ie2 * nom]);
      s.x += v.x;
      s.y += v.y;
    }
  }
  sc[((size_t)k * nb1 + ie1) * nom + iom] = s;
}

static size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

struct MLayout {
  long long R;
  int N, nw, R_padA, R_padB, nkb, nTb, ntile;
  size_t adig, bdig, eA, fB, X, out, total;
};
static MLayout mlayout(long long R, int N, int nw) {
  MLayout L;
  L.R = R; L.N = N; L.nw = nw;
  L.R_padA = (int)((2 * R + pgm::OZ_BLOCK - 1) / pgm::OZ_BLOCK * pgm::OZ_BLOCK);
  L.R_padB = (N + pgm::OZ_BLOCK - 1) / pgm::OZ_BLOCK * pgm::OZ_BLOCK;
  const long long K_pad = (2LL * N + 63) / 64 * 64;
  L.nkb = (int)(K_pad / 64);
  L.nTb = L.R_padB / pgm::OZ_TILE;
  L.ntile = (L.R_padA / pgm::OZ_TILE) * L.nTb;
  size_t o = 0;
  L.adig = o; o += al256((size_t)2 * pgm::OZ_S * L.R_padA * K_pad);
  L.bdig = o; o += al256((size_t)2 * pgm::OZ_S * L.R_padB * K_pad * nw);
  L.eA = o; o += al256(sizeof(int) * (size_t)L.R_padA);
  L.fB = o; o += al256(sizeof(int) * (size_t)L.R_padB * nw);
  L.X = o; o += al256(sizeof(float4) * (size_t)R * N);
  L.out = o; o += al256(sizeof(double) * (size_t)L.ntile * 16384 * nw);
  L.total = o;
  return L;
}

}  // namespace pgc

using namespace pgc;

extern "C" size_t pg_selfc_mwm_workspace(int nk, int P, int npb, int omega_batch, int mixed) {
  if (nk <= 0 || P <= 0 || npb <= 0 || omega_batch <= 0) return 0;
  if (!mixed) return 256;
  return mlayout((long long)nk * P, npb, omega_batch).total;
}

extern "C" int pg_selfc_mwm(const void* minm, int nk, int P, int npb, const void* eps, int nom, double wkq, void* mwm,
                            int mixed, int omega_batch, void* work, size_t work_bytes, unsigned* d_status,
                            void* stream) {
  if (!minm || !eps || !mwm || nk <= 0 || P <= 0 || npb <= 0 || nom <= 0) return PG_EARG;
  cudaStream_t s = (cudaStream_t)stream;
  const long long R = (long long)nk * P;
  const double2* M = (const double2*)minm;
  const double2* W = (const double2*)eps;
  double2* out = (double2*)mwm;
  const int N = npb;
  if (!mixed) {
    if (nom > 65535 || (R + 31) / 32 > 2147483647ll) return PG_ETOOBIG;
    k_mwm_f64<<<dim3((unsigned)((R + 31) / 32), nom), 256, 0, s>>>(M, R, N, W, P, nom, 0, wkq, out);
    pg_count_launches(1);
    return cudaGetLastError() == cudaSuccess ? PG_OK : PG_ECUDA;
  }
  if (!work || omega_batch <= 0) return PG_EARG;
  const int nb = omega_batch < nom ? omega_batch : nom;
  const MLayout L = mlayout(R, N, nb);
  if (work_bytes < L.total) return PG_EWORKSPACE;
  if (2 * R + pgm::OZ_BLOCK > 2147483647ll || nb > 65535 ||
      (long long)pgm::OZ_S * L.nkb * 64 * 16641 >= (1ll << 35))
    return PG_ETOOBIG;
  char* w = (char*)work;
  __nv_bfloat16* adig = (__nv_bfloat16*)(w + L.adig);
  __nv_bfloat16* bdig = (__nv_bfloat16*)(w + L.bdig);
  int* eA = (int*)(w + L.eA);
  int* fB = (int*)(w + L.fB);
  double* gout = (double*)(w + L.out);
  if (cudaMemsetAsync(adig, 0, (size_t)2 * pgm::OZ_S * L.R_padA * L.nkb * 64, s) != cudaSuccess) return PG_ECUDA;
  if (cudaMemsetAsync(eA, 0, sizeof(int) * (size_t)L.R_padA, s) != cudaSuccess) return PG_ECUDA;
  float4* X = (float4*)(w + L.X);
  k_rows_digits<<<(unsigned)R, 256, 0, s>>>(M, R, N, L.R_padA, L.nkb, eA, adig, X);
  pg_count_launches(1);
  for (int om0 = 0; om0 < nom; om0 += nb) {
    const int nw = (om0 + nb <= nom) ? nb : nom - om0;
    int rc = pgx::launch_cols_digits(W + (size_t)N * N * om0, N, nw, L.R_padB, L.nkb, pgm::OZ_S, fB, bdig, s);
    if (rc != PG_OK) return rc;
    rc = pgm::launch_gemm_general(adig, bdig, pgm::OZ_S, 0, L.R_padA, L.R_padB, (N + 127) / 128, L.nkb, nw, gout,
                                  d_status, s);
    if (rc != PG_OK) return rc;
    k_mwm_reduce<<<dim3((unsigned)((R + 127) / 128), nw), 128, 0, s>>>(gout, eA, fB, X, R, N, L.R_padB, L.nTb,
                                                                      L.ntile, P, nom, om0, wkq, out);
    pg_count_launches(1);
  }
  return cudaGetLastError() == cudaSuccess ? PG_OK : PG_ECUDA;
}

extern "C" int pg_selfc_mwm_q0(const void* minm, int nk, int nb1, int nb2, int npb, int off, int nom, const void* head,
                               const void* epsw1, const void* epsw2, double coefs1, double coefs2, void* mwm,
                               void* stream) {
  if (!minm || !head || !epsw1 || !epsw2 || !mwm || nk <= 0 || nb1 <= 0 || nb2 <= 0 || npb <= 0 || nom <= 0 ||
      off < 0)
    return PG_EARG;
  const long long n = (long long)nk * nb1 * nom;
  k_mwm_q0<<<(unsigned)((n + 127) / 128), 128, 0, (cudaStream_t)stream>>>(
      (const double2*)minm, nk, nb1, nb2, npb, off, nom, (const double2*)head, (const double2*)epsw1,
      (const double2*)epsw2, coefs1, coefs2, (double2*)mwm);
  pg_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? PG_OK : PG_ECUDA;
}

extern "C" size_t pg_selfc_convolution_workspace(int nk, int nb1, int nb2, int nom, int n_dense, int nl) {
  if (nk <= 0 || nb1 <= 0 || nb2 <= 0 || nom <= 0) return 0;
  size_t b = 256;
  if (n_dense > 0) b += al256(sizeof(double2) * (size_t)nk * nb1 * nb2 * n_dense);
  if (nl > 0) b += al256(sizeof(double2) * (size_t)nk * nl * nb2 * nom);
  return b;
}

extern "C" int pg_selfc_convolution(const void* mwm, int nk, int nb1, int nb2, int nom, const double* enk,
                                    const double* omega, const double* womeg, int n_dense, const double* omega_dense,
                                    const double* womeg_dense, const double* spline, void* work, size_t work_bytes,
                                    void* sc, void* stream) {
  if (!mwm || !enk || !omega || !sc || nk <= 0 || nb1 <= 0 || nb2 <= 0 || nom <= 0 || n_dense < 0) return PG_EARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (nk > 65535) return PG_ETOOBIG;
  const double2* m = (const double2*)mwm;
  if (n_dense == 0) {
    if (!womeg) return PG_EARG;
    if (nom > 65535) return PG_ETOOBIG;
    k_fr_conv<<<dim3((unsigned)nom, (unsigned)nk), 256, 0, s>>>(m, m, enk, omega, omega, womeg, nk, nb1, nb2, nom,
                                                                nom, (double2*)sc);
    pg_count_launches(1);
    return cudaGetLastError() == cudaSuccess ? PG_OK : PG_ECUDA;
  }
  if (!omega_dense || !womeg_dense || !spline || !work) return PG_EARG;
  if (work_bytes < pg_selfc_convolution_workspace(nk, nb1, nb2, nom, n_dense, 0)) return PG_EWORKSPACE;
  double2* f = (double2*)work;
  const int P = nb1 * nb2;
  const long long ni = (long long)nk * P * n_dense;
  k_interp<<<(unsigned)((ni + 127) / 128), 128, 0, s>>>(m, spline, omega, omega_dense, nk, P, nom, n_dense, f);
  if (nom > 65535) return PG_ETOOBIG;
  k_fr_conv<<<dim3((unsigned)nom, (unsigned)nk), 256, 0, s>>>(m, f, enk, omega, omega_dense, womeg_dense, nk, nb1, nb2,
                                                              nom, n_dense, (double2*)sc);
  pg_count_launches(2);
  return cudaGetLastError() == cudaSuccess ? PG_OK : PG_ECUDA;
}

extern "C" int pg_selfc_convolution_svd(const void* mwm, int nk, int nb1, int nb2, int nl, int nom, const double* enk,
                                        const void* Ul, const double* omega, const double* womeg, void* work,
                                        size_t work_bytes, void* sc, void* stream) {
  if (!mwm || !enk || !Ul || !omega || !womeg || !work || !sc || nk <= 0 || nb1 <= 0 || nb2 <= 0 || nl <= 0 ||
      nom <= 0)
    return PG_EARG;
  if (work_bytes < pg_selfc_convolution_workspace(nk, nb1, nb2, nom, 0, nl)) return PG_EWORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  double2* cnl = (double2*)work;
  const long long nc = (long long)nk * nl * nb2 * nom;
  k_many_conv<<<(unsigned)((nc + 127) / 128), 128, 0, s>>>((const double2*)Ul, enk, omega, womeg, nk, nl, nb2, nom, cnl);
  const long long n = (long long)nk * nb1 * nom;
  k_svd_sc<<<(unsigned)((n + 127) / 128), 128, 0, s>>>((const double2*)mwm, cnl, nk, nb1, nb2, nl, nom, (double2*)sc);
  pg_count_launches(2);
  return cudaGetLastError() == cudaSuccess ? PG_OK : PG_ECUDA;
}
