/* pygw_gb300 — C-ABI of the GB300 (sm_103a) polarization path.
 *
 * Plain pointers and sizes only.  Every array argument is a DEVICE pointer
 * (allocated by the caller, e.g. as a torch CUDA tensor) unless stated
 * otherwise; `stream` is a cudaStream_t (NULL = legacy default stream).
 * Calls are stream-ordered and asynchronous: they enqueue kernels and return.
 * Return value: PG_OK (0) or a negative PG_E* code (pygw_gb300/csrc/pygw_status.h).
 * No entry point allocates memory; scratch space is passed in as `work`,
 * sized by the matching *_workspace() query.
 *
 * Layouts follow the reference's arrays (Fortran order where the reference
 * uses Fortran-ordered numpy arrays):
 *   enk  [nbnd, nkp]              float64, enk[b + nbnd*k]
 *   tetc [4, ntet]                int32, 0-based k indices
 *   kqid [nkp]                    int32, 0-based (column iq of KQmesh.kqid)
 *   kcw  [nb1, nb2, nkp, nom]     float64, nb1 = ncg+nomx+1, nb2 = nbnd-ncg-numin
 *   minm [nk_chunk][P][N]         complex128 (interleaved re, im), P = nb1*nb2,
 *                                 p = ie1*nb2 + ie2 — the per-k `minm2` blocks
 *   eps  [N, N, nom]              complex128, eps[I + N*J + N*N*w]
 *   epsw1, epsw2 [nom][N]         complex128; head [nom] complex128
 */
#ifndef PYGW_GB300_H
#define PYGW_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ weights
 * Replaces the f2py call
 *     kcw = ft.bz_calcqdepw_par2(enk, ef, kqid, ncg, nomx, numin, omega, tetc)
 * made by Polarization_weights (pygw.py:3443), i.e. the Fortran subroutine
 * bz_calcqdepw_par2 (for_tetrahedra.f90:390-464) with its callees
 * (for_tetrahedra3.f90:3-743, for_tetrahedra2.f90:1688-2773).
 * Requires ntet == 6*nkp (tetrahedron 6*ik+t links to 6*kqid[ik]+t,
 * for_tetrahedra.f90:426-432).  kcw is fully overwritten.
 * nom_chunk > 0 bounds the scratch: frequencies are processed in chunks of
 * that size (0 = all at once).  d_status (device, 1 uint, may be NULL)
 * receives PG_ERR_* bits OR-ed in; d_counters (device, PG_NCOUNTERS uint64,
 * may be NULL) receives PG_CNT_* counts added in (the per-polyhedron counts
 * once per frequency chunk).  The reference stops the
 * process on the PG_ERR_* conditions; here the affected (tetrahedron, band
 * pair) contributes zero and the bit is set. */
size_t pg_bz_calcqdepw_par2_workspace(int nbnd, int nkp, int ncg, int nomx, int numin, int nom, int ntet,
                                      int nom_chunk);
int pg_bz_calcqdepw_par2(const double* enk, int nbnd, int nkp, double ef, const int* kqid, int ncg, int nomx,
                         int numin, const double* omega, int nom, const int* tetc, int ntet, double* kcw, void* work,
                         size_t work_bytes, int nom_chunk, unsigned* d_status, unsigned long long* d_counters,
                         void* stream);

/* SVD frequency basis (iopfreq = 5): replaces
 *     kcw = ft.bz_calcqdepw_par3(enk, ef, kqid, ncg, nomx, numin, dUl, omega, tetc)
 * (pygw.py:3441; for_tetrahedra.f90:466-542).  The corner weights of every
 * (tetrahedron, band pair) are projected on dUl (device, (nom, nl) Fortran
 * order, nom·nl ≤ 6144) before they are accumulated; kcw is
 * (nb1, nb2, nkp, nl).  All frequencies are evaluated in one pass. */
size_t pg_bz_calcqdepw_par3_workspace(int nbnd, int nkp, int ncg, int nomx, int numin, int nom, int ntet, int nl);
int pg_bz_calcqdepw_par3(const double* enk, int nbnd, int nkp, double ef, const int* kqid, int ncg, int nomx,
                         int numin, const double* dUl, int nl, const double* omega, int nom, const int* tetc, int ntet,
                         double* kcw, void* work, size_t work_bytes, unsigned* d_status,
                         unsigned long long* d_counters, void* stream);

/* Same computation for callers that cannot allocate device memory (a Fortran
 * or C host program reaching the library through a foreign-function layer
 * with no device allocator, or a service held to a fixed memory budget).  No
 * counterpart in the reference.  Takes no workspace: its scratch is a
 * file-scope device array of pg_bz_calcqdepw_par2_noalloc_capacity() bytes
 * (256 MiB) that each GPU using the library holds until the process exits;
 * frequencies are processed in chunks that fit.  Returns PG_ETOOBIG when the
 * k lists plus one frequency of scratch (4*ntet*nb1*nb2 doubles) do not fit.
 * All calls share that array: calls that overlap on the GPU race and must be
 * serialised.  The first call in a device context looks up the array's
 * device address and caches it under the context's id (a reset device or a
 * new context gets a fresh lookup); make that call before any stream
 * capture. */
size_t pg_bz_calcqdepw_par2_noalloc_capacity(void);
int pg_bz_calcqdepw_par2_noalloc(const double* enk, int nbnd, int nkp, double ef, const int* kqid, int ncg,
                                 int nomx, int numin, const double* omega, int nom, const int* tetc, int ntet,
                                 double* kcw, unsigned* d_status, unsigned long long* d_counters, void* stream);

/* --------------------------------------------------------- χ0, plain FP64
 * Replaces the k loop of MatrixElements2Band.calc_eps (pygw.py:3083-3200):
 *     eps[:, :, w] += (minm2ᵀ·coef ⊙ kcw[:, :, k, w].ravel()) @ conj(minm2)
 *     epsw1[:, w]  += (minm2ᵀ·coef ⊙ kcw[:, :, k, w].ravel()) @ pm       (q = 0)
 * for the k-points k0 .. k0+nk_chunk-1 whose minm blocks are passed.
 * Accumulates into eps/epsw1 (caller zeroes them before the first chunk).
 * Only tiles on or above the diagonal are accumulated; call
 * pg_chi0_mirror_f64 once after the last chunk to fill the rest.
 * coef = -fspin = -2 in the reference.  pm/epsw1 both NULL for q != 0. */
int pg_chi0_accumulate_f64(const void* minm, int nk_chunk, int k0, const double* kcw, int nb1, int nb2, int nkp,
                           int nom, int npb, double coef, void* eps, const void* pm, void* epsw1, void* stream);
int pg_chi0_mirror_f64(void* eps, int npb, int nom, void* stream);
/* The q→0 wings alone (epsw1 += tmat @ pm, pygw.py:3192-3195), for use with
 * the split-precision χ0 below. */
int pg_wings_f64(const void* minm, int nk_chunk, int k0, const double* kcw, int nb1, int nb2, int nkp, int nom,
                 int npb, double coef, const void* pm, void* epsw1, void* stream);

/* ------------------------------------------------- χ0, split precision
 * Same sum as pg_chi0_accumulate_f64 over ALL k at once (minm holds every
 * k: [nkp][P][N]), on the tensor cores: the matrix elements and the weighted
 * matrix elements are split into five 8-bit digits per value with one
 * exponent per row, digit products are summed exactly (tcgen05 MMA into
 * FP32 tensor memory, renormalised every 896 K-values), and only digit pairs
 * below 2^-40 are dropped.  Writes the full Hermitian χ0 to eps (no mirror
 * needed).  omega_batch frequencies share one set of weighted digits
 * (workspace grows with it); kb_split > 0 caps the K-blocks per CTA
 * (0 = automatic).  d_status receives PG_ERR_TIMEOUT if a pipeline wait
 * expired (the result is then invalid).  gemm_events (may be NULL) holds
 * 2·ceil(nom/omega_batch) created cudaEvent_t handles; event 2b and 2b+1 are
 * recorded on `stream` just before and after batch b's digit-GEMM launch, so
 * a caller can time that kernel alone. */
size_t pg_chi0_mixed_workspace(int nb1, int nb2, int nkp, int npb, int omega_batch, int kb_split);
int pg_chi0_mixed(const void* minm, int nkp, const double* kcw, int nb1, int nb2, int nom, int npb, double coef,
                  void* eps, void* work, size_t work_bytes, int omega_batch, int kb_split, unsigned* d_status,
                  void* stream, void* const* gemm_events);
/* The same contraction for the k-points k0 .. k0+nk_chunk-1 only (minm holds
 * their blocks, [nk_chunk][P][N]; kcw covers all nkp points), so the matrix
 * elements can be streamed in k-chunks as the reference builds them one k at a
 * time (pygw.py:3096-3185): eps = (accumulate ? eps : 0) + χ0 of the chunk.
 * Each chunk is split with its own row exponents; chunk sums add in FP64.
 * Ragged band windows: with kstart (device, nk_chunk+1 row offsets into minm)
 * and knb2 (device, nk_chunk) point i contributes the nb1·knb2[i] pairs of its
 * first knb2[i] unoccupied bands, pair index ie1·knb2[i] + ie2, nK rows in all
 * (kstart = NULL: every point has the full nb1·nb2 window).
 * Workspace: pg_chi0_mixed_workspace with nkp = nk_chunk. */
int pg_chi0_mixed_accumulate(const void* minm, int nk_chunk, int k0, const int* kstart, const int* knb2, long long nK,
                             const double* kcw, int nb1, int nb2, int nkp, int nom, int npb, double coef, void* eps,
                             int accumulate, void* work, size_t work_bytes, int omega_batch, int kb_split,
                             unsigned* d_status, void* stream, void* const* gemm_events);
/* Workspace layout (byte offsets and sizes) for inspection by tests. */
int pg_chi0_mixed_layout(int nb1, int nb2, int nkp, int npb, int omega_batch, int kb_split, size_t* offs,
                         long long* dims);

/* ----------------------------------------------------- ε and ε⁻¹, FP64
 * Replaces pygw.py:3229-3271: symmetrise, +1, invert (scipy.linalg.inv),
 * q = 0 head/wings update, -1.  On return eps holds ε⁻¹ − 1; epsw1, epsw2,
 * head are updated in place when epsw1 != NULL (q = 0). */
size_t pg_eps_inverse_f64_workspace(int npb, int nom);
int pg_eps_inverse_f64(void* eps, int npb, int nom, void* epsw1, void* epsw2, void* head, void* work,
                       size_t work_bytes, void* stream);

/* Basis change along the leading index of complex arrays (frequency ↔ SVD
 * basis, pygw.py:3208, 3226, 3276-3280): out[nout][nelem] = in[nin][nelem]·U
 * with U real (nin, nout), Fortran order, nin·nout ≤ 6144; in ≠ out.  eps
 * [ω][N][N] has nelem = N·N, the wings [ω][N] nelem = N, the head nelem = 1. */
int pg_basis_change(const void* in, int nin, void* out, int nout, const double* U, long long nelem, void* stream);

/* ------------------------------------------- ε and ε⁻¹, mixed precision
 * Same contract as pg_eps_inverse_f64 (pygw.py:3229-3271).  The inverse is
 * computed in FP32 (complex Gauss–Jordan, partial pivoting) and refined
 * `iters` times (0, 1 or 2) by X ← X + X·(I − A·X) with the residual formed on
 * the tensor cores from six 8-bit digits per value (≈ 2^-48 relative to the
 * row scales) and the sum in FP64; the q = 0 head/wings update stays FP64.
 * omega_batch frequencies are inverted together (0 = all of them; the
 * workspace grows with it).  d_status receives PG_ERR_TIMEOUT if a pipeline
 * wait of the tensor-core kernel expired. */
size_t pg_eps_inverse_mixed_workspace(int npb, int nom, int omega_batch);
int pg_eps_inverse_mixed(void* eps, int npb, int nom, void* epsw1, void* epsw2, void* head, void* work,
                         size_t work_bytes, int omega_batch, int iters, unsigned* d_status, void* stream);

/* ------------------------------------------------ synthetic inputs
 * Matrix elements of the measured synthetic workloads, drawn on the device
 * for the k-points k0 .. k0+nk-1 of one q: out[rows][N] complex128,
 *   M = z·√(1/2)/(1 + |E_n(k) − E_m(k−q)|)·√v_I,  z ~ CN(0,1) keyed by (seed, q, k, n, m, I),
 * rows = nk·nb1·nb2, or nrows with ragged windows (kstart/knb2 as in
 * pg_chi0_mixed_accumulate).  enk [nbnd][nkp] (weights layout), kqid (nkp,
 * this q's k−q indices), sqv (N) √v_I.  No counterpart in the reference
 * (its matrix elements come from the LAPW code); used by the large
 * benchmarks, which stream M per k-chunk without holding it all. */
int pg_synth_minm(int nk, int k0, int iq, const double* enk, int nbnd, const int* kqid, int ncg, int numin, int nb1,
                  int nb2, const int* kstart, const int* knb2, long long nrows, const double* sqv, int npb,
                  unsigned long long seed, void* out, void* stream);

/* ---------------------------------------------- correlation self-energy
 * Replaces the mwm loop of MatrixElements2Band.calc_selfc (pygw.py:3352-3364):
 *   mwm[k][ω][p] = wkq · Σ_{I,J} conj(M[k][p][I]) · W[ω](I,J) · M[k][p][J]
 * for the nk k-points of minm [nk][P][N] (P = nb1·nb2 band pairs, row-major
 * p = ib1·nb2 + ib2) and the nom frequencies (or SVD functions) of
 * W [nom][N][N] = ε⁻¹ − 1 as returned by pg_eps_inverse_* (column-major per
 * frequency).  mixed = 0: FP64 (no workspace); mixed = 1: the split-precision
 * tensor-core GEMM (five 8-bit digits per value, omega_batch frequencies per
 * launch, workspace from the query).  d_status as for pg_chi0_mixed. */
size_t pg_selfc_mwm_workspace(int nk, int P, int npb, int omega_batch, int mixed);
int pg_selfc_mwm(const void* minm, int nk, int P, int npb, const void* eps, int nom, double wkq, void* mwm, int mixed,
                 int omega_batch, void* work, size_t work_bytes, unsigned* d_status, void* stream);

/* q = 0 terms of the same loop (pygw.py:3358-3363): for every row ie1 < nb1,
 * mwm[k][ω][ie1, ie1 + off] += coefs2·head[ω] + coefs1·Σ_I M·epsw2[ω][I]
 *                             + coefs1·Σ_I conj(M)·epsw1[ω][I],
 * off = ibgw + ncg_c; head [nom], epsw1/epsw2 [nom][N] complex128. */
int pg_selfc_mwm_q0(const void* minm, int nk, int nb1, int nb2, int npb, int off, int nom, const void* head,
                    const void* epsw1, const void* epsw2, double coefs1, double coefs2, void* mwm, void* stream);

/* Matsubara convolution of Compute_selfc_inside (mcommon.py:80-165):
 * sc[k][ie1][iom] = Σ_ie2 fr_convolution2(enk[k][ie2], mwm[k][·][ie1,ie2], …)
 * (all_fr_convolutions, fnc.f90:156-177) with enk [nk][nb2] the energies at
 * k−q (core first).  n_dense > 0 selects the iopfreq 4 branch: mwm·(ω²+1) is
 * interpolated to the dense mesh (omega_dense, womeg_dense) by the cubic-spline
 * matrix spline [n_dense][nom] (row-major) and convolved there
 * (few_fr_convolutions); womeg may then be null.  Workspace only for
 * n_dense > 0. */
size_t pg_selfc_convolution_workspace(int nk, int nb1, int nb2, int nom, int n_dense, int nl);
int pg_selfc_convolution(const void* mwm, int nk, int nb1, int nb2, int nom, const double* enk, const double* omega,
                         const double* womeg, int n_dense, const double* omega_dense, const double* womeg_dense,
                         const double* spline, void* work, size_t work_bytes, void* sc, void* stream);

/* SVD basis (mcommon.py:115-121): mwm [nk][nl][P] in the basis, Ul [nl][nom]
 * complex128; sc[k][ie1][iom] = Σ_l Σ_ie2 mwm[k][l][ie1,ie2]·Cnl[k][l][ie2][iom]
 * with Cnl from many_fr_convolutions (fnc.f90:139-154).  Workspace from
 * pg_selfc_convolution_workspace(nk, nb1, nb2, nom, 0, nl). */
int pg_selfc_convolution_svd(const void* mwm, int nk, int nb1, int nb2, int nl, int nom, const double* enk,
                             const void* Ul, const double* omega, const double* womeg, void* work, size_t work_bytes,
                             void* sc, void* stream);

/* ------------------------------------------------------------ bookkeeping
 * Number of kernels this library has enqueued since it was loaded (all entry
 * points, all streams).  No counterpart in the reference. */
unsigned long long pg_launch_count(void);

/* Limit, in nanoseconds of the GPU's global timer, of one pipeline wait
 * inside the split-precision digit GEMM (pg_chi0_mixed*, the refinement of
 * pg_eps_inverse_mixed, pg_selfc_mwm in split precision), for every launch
 * enqueued after the call; process-wide; 0 restores the default of 5 s.  When
 * a wait expires the launch sets PG_ERR_TIMEOUT in its status word, leaves
 * NaN in the tiles it did not finish and returns with its in-flight copies
 * and MMAs completed, so the context stays usable.  No counterpart in the
 * reference, whose equivalent failures stop the process
 * (for_tetrahedra2.f90:1777-1781). */
void pg_set_wait_limit_ns(unsigned long long ns);
unsigned long long pg_wait_limit_ns(void);

/* Frequencies whose B digit planes pg_chi0_mixed* prepares per pass over the
 * A digit planes (process-wide; read by every workspace query and call after
 * it is set, so set it before sizing a workspace).  A pass reads the five A
 * planes once and writes five B planes per frequency: a longer pass reads
 * less per frequency and needs one more set of B planes of workspace per
 * frequency.  The pass is rounded up to a whole number of omega_batch
 * launches.  n in [0, 64]; 0 restores the default, 4; returns PG_EARG
 * otherwise.  No counterpart in the reference (an implementation detail of
 * the split-precision contraction). */
int pg_set_chi0_prep_batch(int n);
int pg_chi0_prep_batch(void);

/* How the weights of 7- and 8-node polyhedra (two halves, pentahedra or
 * prisms) are combined, for every later pg_bz_calcqdepw_par2/par3 call
 * (process-wide).  0 (default): the two halves' weights are added at every
 * frequency.  1: the reference's own addressing is reproduced — its
 * convw1t_par keeps the halves in wtemp(4,2,nom) but addresses that array as
 * (4,nom,2) (for_tetrahedra3.f90:36, 100-120), so as compiled without bounds
 * checks the first half's weights are replaced, from the third frequency on,
 * by the second half's two frequencies earlier; with 1 the results equal the
 * reference's statements at every entry.  Returns PG_OK. */
int pg_set_weights_reference_layout(int on);
int pg_weights_reference_layout(void);

#ifdef __cplusplus
}
#endif

#endif /* PYGW_GB300_H */
