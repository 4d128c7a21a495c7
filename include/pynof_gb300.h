/*
 * libpynof_gb300 -- C ABI of the GB300 (sm_103a) RI / full-ERI JK and
 * MO-integral path of PyNOF.
 *
 * Conventions shared by every entry point
 * ---------------------------------------
 * - Every pointer is a DEVICE pointer unless stated otherwise; every array is
 *   row-major (numpy C order) float64, laid out exactly like the reference's
 *   numpy arrays:
 *       C      [nbf][nbf]            column p = MO p
 *       H      [nbf][nbf]
 *       b      [nbf][nbf][naux]      b[m][n][Q], symmetric in (m, n)
 *       I      [nbf][nbf][nbf][nbf]  I[m][n][s][l] = (mn|sl), 8-fold symmetric
 *       J, K   [nbf5][nbf][nbf]
 *       n      [nbf5];  cj12, ck12 [nbf5][nbf5]
 * - nbf5 <= nbf.  Sizes are in elements.
 * - `stream` is a cudaStream_t (NULL = legacy default stream).  Calls are
 *   asynchronous with respect to the host; results are valid once the stream
 *   has been synchronised.
 * - Scratch memory comes from the caller: `workspace` must hold at least the
 *   number of bytes the matching *_workspace_* query returns.  The library
 *   allocates no device memory and never frees caller memory.
 * - The return value is a GB_* status; gb_last_error() returns the message of
 *   the last failing call on the calling thread.
 * - The RI entry points use the (m, n) symmetry of b: J is computed on the
 *   pairs n >= m and mirrored.  PyNOF's b_mnl is symmetric by construction
 *   (pynof/integrals.py:39-49 builds it from the (P|mn) integrals);
 *   gb_check_symmetric_f64 verifies a buffer.
 */
#ifndef PYNOF_GB300_H
#define PYNOF_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GB_OK 0
#define GB_ERR_INVALID_ARG 1
#define GB_ERR_BAD_SHAPE 2
#define GB_ERR_WORKSPACE 3
#define GB_ERR_CUDA 4
#define GB_ERR_TIMEOUT 5
#define GB_ERR_NONFINITE 6
#define GB_ERR_UNSUPPORTED 7

/* Message of the last failing call on this thread ("" if none). */
const char* gb_last_error(void);
/* Library version, major * 10000 + minor * 100 + patch. */
int gb_version(void);

/* Launch profiler.  While enabled, every kernel the library launches is
 * bracketed by two CUDA events on its stream.  gb_profile_stop synchronises on
 * those events and writes a JSON object {"kernel": [launches, total_ms], ...}
 * into out (host buffer of out_len bytes). */
int gb_profile_start(void);
int gb_profile_stop(char* out, size_t out_len);

/* Maximum |b[m][n][l] - b[n][m][l]| over the tensor, written to *max_abs_diff
 * (a DEVICE pointer to one double). */
int gb_check_symmetric_f64(const double* b, int nbf, int naux, double* max_abs_diff, void* stream);

/* ------------------------------------------------------------------------
 * A1  computeJKj, RI.  Replaces JKj_RI_GPU (pynof/integrals.py:234-245),
 *     dispatched from computeJKj (pynof/integrals.py:172-191).
 *     J[q][m][n] = sum_l (sum_n' C[n'][q] (sum_m' C[m'][q] b[m'][n'][l])) b[m][n][l]
 *     K[q][m][n] = sum_l T[q][m][l] T[q][n][l],  T[q][n][l] = sum_m' C[m'][q] b[m'][n][l]
 *     for q < nbf5.
 * ---------------------------------------------------------------------- */
size_t gb_jkj_ri_workspace_f64(int nbf, int nbf5, int naux);
int gb_jkj_ri_f64(const double* C, const double* b, int nbf, int nbf5, int naux, double* J, double* K,
                  void* workspace, size_t workspace_bytes, void* stream);

/* Same build as gb_jkj_ri_f64 for callers that cannot allocate device memory
 * (their HBM is owned by another allocator or a fixed arena, or they run in a
 * loop where cudaMalloc/cudaFree would synchronise the device).  No counterpart
 * in the reference: PyNOF always lets cupy allocate.  Scratch comes from a
 * built-in device array of GB_NOALLOC_SCRATCH_BYTES, reserved on every GPU that
 * loads this library until the process exits; problems whose workspace
 * (gb_jkj_ri_workspace_f64) exceeds it are rejected with GB_ERR_WORKSPACE.
 * The first call on a device looks the array's address up (make it before any
 * stream capture; after a cudaDeviceReset the next call looks it up again).
 * All calls share the array: calls that overlap on the GPU race and must be
 * serialised on one stream. */
#define GB_NOALLOC_SCRATCH_BYTES (64u * 1024u * 1024u)
int gb_jkj_ri_noalloc_f64(const double* C, const double* b, int nbf, int nbf5, int naux, double* J, double* K,
                          void* stream);

/* ------------------------------------------------------------------------
 * A3  computeJKH_MO, RI.  Replaces JKH_MO_RI_GPU (pynof/integrals.py:383-399),
 *     dispatched from computeJKH_MO (pynof/integrals.py:307-326).
 *     J_MO[p][q] = (pp|qq), K_MO[p][q] = (pq|pq), H_core[p] = C_p^T H C_p.
 * ---------------------------------------------------------------------- */
size_t gb_jkh_mo_ri_workspace_f64(int nbf, int nbf5, int naux);
int gb_jkh_mo_ri_f64(const double* C, const double* H, const double* b, int nbf, int nbf5, int naux,
                     double* J_MO, double* K_MO, double* H_core, void* workspace, size_t workspace_bytes,
                     void* stream);

/* ------------------------------------------------------------------------
 * A5  Integrals_MO_RI.  Replaces Integrals_MO_RI_GPU (pynof/integrals.py:709-714),
 *     dispatched from JKH_MO_tmp (pynof/integrals.py:665-682).
 *     Hmat[i][j] = (C^T H C)[i][j] (j < nbf5),  bMO[a][q][l] = sum_mn C[m][a] C[n][q] b[m][n][l].
 *     Hmat is [nbf][nbf5], bMO is [nbf][nbf5][naux].
 * ---------------------------------------------------------------------- */
size_t gb_mo_ri_workspace_f64(int nbf, int nbf5, int naux);
int gb_mo_ri_f64(const double* C, const double* H, const double* b, int nbf, int nbf5, int naux, double* Hmat,
                 double* bMO, void* workspace, size_t workspace_bytes, void* stream);

/* ------------------------------------------------------------------------
 * A5  computeLagrange2, RI, closed shell (MSpin == 0).  Replaces the GPU
 *     branch of computeLagrange2 (pynof/utils.py:262-327).  elag is [nbf][nbf]
 *     (columns >= nbf5 are zero), Hmat [nbf][nbf5].  The diagonals of cj12 and
 *     ck12 are ignored (the reference zeroes them, utils.py:269-270).
 * ---------------------------------------------------------------------- */
size_t gb_lagrange2_ri_workspace_f64(int nbf, int nbf5, int naux);
int gb_lagrange2_ri_f64(const double* C, const double* H, const double* b, const double* n,
                        const double* cj12, const double* ck12, int nbf, int nbf5, int naux, int nbeta,
                        int nalpha, double* elag, double* Hmat, void* workspace, size_t workspace_bytes,
                        void* stream);

/* ------------------------------------------------------------------------
 * A2  computeJKj, full ERI.  Replaces JKj_Full_GPU (pynof/integrals.py:221-231).
 *     J_i[m][n] = sum_sl D_i[s][l] (mn|sl),  K_i[m][s] = sum_nl D_i[n][l] (mn|sl),
 *     D_i = C_i C_i^T.  I is [nbf]^4 (8-fold symmetric).
 * ---------------------------------------------------------------------- */
size_t gb_jkj_full_workspace_f64(int nbf, int nbf5);
int gb_jkj_full_f64(const double* C, const double* I, int nbf, int nbf5, double* J, double* K, void* workspace,
                    size_t workspace_bytes, void* stream);

/* A4  computeJKH_MO, full ERI.  Replaces JKH_MO_Full_GPU (pynof/integrals.py:365-380). */
size_t gb_jkh_mo_full_workspace_f64(int nbf, int nbf5);
int gb_jkh_mo_full_f64(const double* C, const double* H, const double* I, int nbf, int nbf5, double* J_MO,
                       double* K_MO, double* H_core, void* workspace, size_t workspace_bytes, void* stream);

/* A6  Integrals_MO_Full.  Replaces Integrals_MO_Full_GPU (pynof/integrals.py:693-698).
 *     Hmat [nbf][nbf5];  I_MO [nbf][nbf5][nbf5][nbf5] = (C^T, C_p^T, C_p^T, C_p^T) . I */
size_t gb_mo_full_workspace_f64(int nbf, int nbf5);
int gb_mo_full_f64(const double* C, const double* H, const double* I, int nbf, int nbf5, double* Hmat,
                   double* I_MO, void* workspace, size_t workspace_bytes, void* stream);

/* The RI factor from the three-centre integrals: b[m][n][l] = sum_k mnk[m][n][k]
 * M[k][l] with M = metric^(-1/2) [naux][naux] (symmetric).  Replaces the
 * einsum "mnk,kl->mnl" of compute_integrals (pynof/integrals.py:49); the
 * metric power itself (psi4's Matrix::power(-0.5, 1e-14), :45) stays on the
 * host in FP64.  The split-product form of the same contraction is
 * gb_dgemm_mixed(mnk, M, nbf*nbf, naux, naux, ...) (M symmetric). */
int gb_ri_factor_f64(const double* mnk, const double* M, int nbf, int naux, double* b, void* stream);

/* HF-JK helpers (pynof/integrals.py:490-562).
 * gb_density_hf_f64: D [nbf][nbf] = sum_{j0 <= j < j1} C[:, j] C[:, j]^T.
 *   Replaces computeD_HF (j in [0, nbeta), integrals.py:493-500) and
 *   computeDalpha_HF (j in [nbeta, nalpha), :503-510).
 * gb_jk_hf_full_f64: J[m][n] = sum_sl D[l][s] I[m][n][s][l],
 *   K[m][s] = sum_nl D[n][l] I[m][n][s][l], for a symmetric D (as the two
 *   density functions build it).  Replaces JK_HF_Full_GPU (:537-543) and,
 *   with the alpha density, JKalpha_HF_Full_GPU (:557-562). */
int gb_density_hf_f64(const double* C, int nbf, int j0, int j1, double* D, void* stream);
size_t gb_jk_hf_full_workspace_f64(int nbf);
int gb_jk_hf_full_f64(const double* D, const double* I, int nbf, double* J, double* K, void* workspace,
                      size_t workspace_bytes, void* stream);

/* Post-NOF four-index transforms from the 4-index tensor:
 *   out[p][q][r][t] = sum C[m][p0+p] C[n][q0+q] I[m][n][s][l] C[s][r0+r] C[l][t0+t],
 *   out [np][nq][nr][nt].  Replaces iajb_Full_GPU (pynof/integrals.py:626-638;
 *   i, j in [no1, nalpha), a, b in [nalpha, nbf)) and pqrt_Full_GPU (:657-660;
 *   every range [0, nbf)). */
size_t gb_mo4_full_workspace_f64(int nbf, int nq, int nr, int nt);
int gb_mo4_full_f64(const double* C, const double* I, int nbf, int p0, int np, int q0, int nq, int r0, int nr,
                    int t0, int nt, double* out, void* workspace, size_t workspace_bytes, void* stream);

/* A6  computeLagrange2, full ERI, closed shell (pynof/utils.py:302-326).  The
 *     diagonals of cj12 / ck12 are ignored. */
size_t gb_lagrange2_full_workspace_f64(int nbf, int nbf5);
int gb_lagrange2_full_f64(const double* C, const double* H, const double* I, const double* n, const double* cj12,
                          const double* ck12, int nbf, int nbf5, int nbeta, int nalpha, double* elag, double* Hmat,
                          void* workspace, size_t workspace_bytes, void* stream);

/* ------------------------------------------------------------------------
 * A8  computeF_RC (closed shell).  Replaces computeF_RC_GPU
 *     (pynof/utils.py:58-84).  F [nbf5][nbf][nbf];
 *     F_i = n_i H + n_i J_i [ini <= i < nbeta or nalpha <= i] + sum_j cj12_ij J_j
 *           - sum_j ck12_ij K_j, with ini = no1 if no1 > 1 else 0 and the
 *     diagonal entries (i, i), i >= ini, of cj12 / ck12 ignored.
 * ---------------------------------------------------------------------- */
size_t gb_fock_rc_workspace_f64(int nbf, int nbf5);
int gb_fock_rc_f64(const double* J, const double* K, const double* n, const double* H, const double* cj12,
                   const double* ck12, int nbf, int nbf5, int nbeta, int nalpha, int no1, double* F, void* workspace,
                   size_t workspace_bytes, void* stream);

/* A8  computeF_RO (restricted open shell).  Replaces computeF_RO_GPU
 *     (pynof/utils.py:172-246), reached from ENERGY1r when no1 > 0 and
 *     MSpin != 0 (pynof/utils.py:423-425).  Same arguments as
 *     gb_fock_rc_f64; with D = [0, nbeta) u [nalpha, nbf5) and the singly
 *     occupied O = [nbeta, nalpha):
 *     F_i = a_i H + sum_j A_ij J_j - sum_j B_ij K_j,  a_i = n_i (D), 1/2 (O);
 *     A_ij = cj12_ij (i, j in D) + n_i [i == j, ini <= i < nbeta or i >= nalpha]
 *          + n_i (i in D, j in O) + 1/2 (i != j in O) + n_j (i in O, j in D);
 *     B_ij = ck12_ij (i, j in D) + n_i / 2 (i in D, j in O) + 1/2 (i != j in O)
 *          + n_j / 2 (i in O, j in D); the diagonal entries (i, i), i >= ini,
 *     of cj12 / ck12 ignored. */
size_t gb_fock_ro_workspace_f64(int nbf, int nbf5);
int gb_fock_ro_f64(const double* J, const double* K, const double* n, const double* H, const double* cj12,
                   const double* ck12, int nbf, int nbf5, int nbeta, int nalpha, int no1, double* F, void* workspace,
                   size_t workspace_bytes, void* stream);

/* A8  computeLagrange (pynof/utils.py:249-259):
 *     elag[k][i] = sum_mn C[m][k] F_i[m][n] C[n][i] for k < noptorb, i < nbf5; 0 elsewhere. */
size_t gb_lagrange_workspace_f64(int nbf, int nbf5);
int gb_lagrange_f64(const double* F, const double* C, int nbf, int nbf5, int noptorb, double* elag,
                    void* workspace, size_t workspace_bytes, void* stream);

/* A7  computeE_elec (pynof/utils.py:385-402): *E (device scalar) =
 *     tr(elag[:nbf5, :nbf5]) + sum_i w_i C_i^T H C_i, w_i = n_i (1/2 for
 *     nbeta <= i < nalpha when high_spin). */
size_t gb_energy_elec_workspace_f64(int nbf, int nbf5);
int gb_energy_elec_f64(const double* elag, const double* C, const double* H, const double* n, int nbf, int nbf5,
                       int nbeta, int nalpha, int high_spin, double* E, void* workspace, size_t workspace_bytes,
                       void* stream);

/* Orbital rotation C' = C expm(Y) in FP64 on the device.  Replaces
 * rotate_orbital (utils.py:550-565), which builds Y on the host and calls
 * scipy.linalg.expm.  y: the packed step, nvar = nbf (nbf - 1) / 2 -
 * (nbf - nbf5) (nbf - nbf5 - 1) / 2 values over (i < nbf5, j > i) in row-major
 * order (Y[i][j] = y, Y[j][i] = -y); C, Cout: [nbf][nbf], Cout != C.
 * expm by scaling and squaring with a degree-16 Taylor polynomial; the number
 * of squarings follows from norm1, an upper bound of ||Y||_1 (max column sum
 * of |Y|) the caller knows from y.  norm1 < 0: the call measures ||Y||_1 on
 * the device and reads it back, synchronising the stream once.  With
 * norm1 >= 0 it launches only (it can be captured in a CUDA graph, which
 * then holds for every y whose bound needs the same number of squarings). */
size_t gb_rotate_orbital_workspace_f64(int nbf);
int gb_rotate_orbital_f64(const double* y, const double* C, int nbf, int nbf5, double norm1, double* Cout,
                          void* workspace, size_t workspace_bytes, void* stream);

/* A9  the occupation optimiser's function and gradient on the HOST (no GPU
 * work, no stream): E(gamma) of calcocce (pynof/pnof.py:994-1001, via
 * ocupacion_softmax, CJCKD8 and calce, pnof.py:770-809, 350-422, 905-929)
 * and, when grad != NULL, dE/dgamma of calcoccg (pnof.py:1004-1033, with
 * der_CJCKD8, pnof.py:425-525), in O(nbf5^2).  Closed shell without singly
 * occupied orbitals: gamma [ndoc ncwo], J_MO and K_MO [nbf5][nbf5], H_core
 * [nbf5], no1 + ndoc (1 + ncwo) <= nbf5.  Replaces the numpy evaluation that
 * scipy's CG repeats thousands of times per occupation step
 * (minimization.py:77-97). */
int gb_occ_energy_grad_f64(const double* gamma, const double* J_MO, const double* K_MO, const double* H_core,
                           int nbf5, int no1, int ndoc, int ncwo, double* energy, double* grad);

/* A9  calce (pynof/pnof.py:905-929) on the HOST for given coefficients
 * cj12, ck12 [nbf5][nbf5] (diagonals zeroed by the caller, as the reference
 * does in place), occupations n and H_core [nbf5], J_MO, K_MO [nbf5][nbf5].
 * Both this and gb_occ_energy_grad_f64 sum the energy with compensation
 * (Neumaier). */
int gb_calce_f64(const double* n, const double* cj12, const double* ck12, const double* J_MO, const double* K_MO,
                 const double* H_core, int nbf5, int nbeta, int nalpha, double* energy);

/* A9  occoptr's minimisation (pynof/minimization.py:77-97:
 * scipy.optimize.minimize(calcocce, gamma, jac=calcoccg, method="CG")) on the
 * DEVICE, with every argument pointer in device memory: J_MO, K_MO
 * [nbf5][nbf5], H_core [nbf5], gamma0 [ndoc ncwo] (closed shell, nsoc = 0,
 * no1 + ndoc (1 + ncwo) <= nbf5).  The energy and gradient are those of
 * gb_occ_energy_grad_f64 (softmax occupations, CJCKD8 and its derivative,
 * pnof.py:350-525, 770-809, 994-1033); the minimiser is scipy's CG
 * (Polak-Ribiere+ with the sufficient-descent check, More-Thuente line search
 * with c1 = 1e-4, c2 = 0.4), stopping at ||g||_inf <= gtol (scipy's 1e-5) or
 * after maxiter iterations (scipy's 200 ndoc ncwo).  Where scipy would try its
 * second line search it restarts from steepest descent once, then stops.
 * The whole loop is one CUDA graph on `stream` (a WHILE conditional node; no
 * host synchronisation): result[5] = {E, iterations, evaluations, success
 * (1, 0, or -1 when the evaluation cap 1 + 200 (maxiter + 1) was reached),
 * ||g||_inf}, gamma_out [ndoc ncwo] (may alias gamma0), and, when not null,
 * the occupations n_out [nbf5] (ocupacion_softmax) and C^J, C^K
 * [nbf5][nbf5] (CJCKD8, diagonals included) at the result.  `ws` is
 * 256-byte-aligned device memory of gb_occ_workspace_bytes bytes; one
 * minimisation at a time per workspace (the graph is cached per workspace
 * and context; gb_occ_release drops it).  Not capturable into another
 * graph. */
size_t gb_occ_workspace_bytes(int nbf5, int ndoc, int ncwo);
int gb_occ_minimize_dev(const double* gamma0, const double* J_MO, const double* K_MO, const double* H_core,
                        int nbf5, int no1, int ndoc, int ncwo, double gtol, int maxiter, double* gamma_out,
                        double* result, double* n_out, double* cj12_out, double* ck12_out, void* ws,
                        size_t ws_bytes, void* stream);
/* gb_occ_minimize_dev driven from the host: the same kernels and steps, as
 * replays of an ordinary graph of eight evaluations with the phase copied back
 * (one synchronisation of `stream` per replay) instead of the conditional
 * node; returns when the minimisation has ended (GB_ERR_TIMEOUT if it did not
 * within the evaluation cap). */
int gb_occ_minimize_dev_sync(const double* gamma0, const double* J_MO, const double* K_MO, const double* H_core,
                             int nbf5, int no1, int ndoc, int ncwo, double gtol, int maxiter, double* gamma_out,
                             double* result, double* n_out, double* cj12_out, double* ck12_out, void* ws,
                             size_t ws_bytes, void* stream);
/* One evaluation of E(gamma) and dE/dgamma on the device (calcocce +
 * calcoccg, pnof.py:994-1033): result[0] = E, result[4] = ||g||_inf, grad
 * [ndoc ncwo] (may be null); same workspace as gb_occ_minimize_dev. */
int gb_occ_energy_grad_dev(const double* gamma, const double* J_MO, const double* K_MO, const double* H_core,
                           int nbf5, int no1, int ndoc, int ncwo, double* result, double* grad, void* ws,
                           size_t ws_bytes, void* stream);
/* Drop the cached graphs of a workspace (before freeing it; a graph still in
 * flight is freed when it completes).  No call on the workspace may overlap. */
int gb_occ_release(const void* ws);

/* Plain FP64 GEMM C = A B^T with row-major A [M][K], B [N][K], C [M][N] on the
 * DMMA engine (the FP64 counterpart of gb_dgemm_mixed).  No counterpart in
 * the reference (numpy / cupy GEMMs); used e.g. for ERPA's (pq|sl) from b_pql
 * (pynof/postpnof.py:1404-1406). */
int gb_dgemm_f64(const double* A, const double* B, int M, int N, int K, double* C, void* stream);

/* Capture of the calling thread's work on a (non-default) stream into a CUDA
 * graph, thread-local capture mode: gb_graph_begin, then any of this
 * library's calls that neither allocate nor synchronise (preallocated
 * outputs and workspaces; gb_rotate_orbital_f64 with norm1 >= 0), then
 * gb_graph_end; gb_graph_launch replays.  No counterpart in the reference
 * (PyNOF issues every cupy call eagerly); used by the serving loop to make
 * one orbital step one launch. */
typedef struct gb_graph gb_graph;
int gb_graph_begin(void* stream);
int gb_graph_end(void* stream, gb_graph** graph);
int gb_graph_launch(gb_graph* graph, void* stream);
int gb_graph_destroy(gb_graph* graph);

/* ========================================================================
 * Split-product ("mixed") path on the tcgen05 tensor cores.
 *
 * FP64 operands are cut into nslices (1..6) balanced base-128 bf16 digit
 * slices with a power-of-two exponent per row; the slice products with
 * s + t <= nslices + 1 run as bf16 tcgen05 MMAs with FP32 accumulation in
 * TMEM, the leading product groups accumulated exactly.  nslices = 6 agrees
 * with FP64 to ~1e-12 normwise; nslices = 2 is the three-product bf16x3 split
 * (~1e-4).  nslices = GB_SPLIT_TF32X3 selects the three-product TF32 split
 * instead (hi = tf32(x), lo = tf32(x - hi); hi hi + hi lo + lo hi as tf32
 * tcgen05 MMAs, FP32 accumulation; ~1e-6).  Device status of these kernels:
 * gb_device_status.
 * ====================================================================== */

#define GB_SPLIT_TF32X3 32

/* Status word of the tensor-core kernels on the current device: 0, or the
 * first error one of them recorded -- GB_ERR_TIMEOUT when a bounded wait gave
 * up, GB_ERR_NONFINITE when an operand held a NaN or an infinity (digit
 * slices cannot represent it).  Once set, every later split-product GEMM
 * launch on the device returns without work until the word is cleared
 * (reset != 0), so every caller that reads it after its own work sees the
 * failure.  Synchronises the device.  No counterpart in the reference, which
 * has no device-side failure reporting. */
int gb_device_status(int reset, int* status);

/* Limit of every bounded wait inside the split-product kernels launched after
 * this call, in nanoseconds (0 restores the default of 2 s).  No counterpart
 * in the reference. */
int gb_set_wait_limit_ns(unsigned long long limit_ns);

/* Test hook for the timeout path, no counterpart in the reference: while
 * stage >= 0, the first CTA of every split-product GEMM launched afterwards
 * never issues the copy of that pipeline stage, so its wait for the stage
 * runs out (after the wait limit), the kernel gives up cleanly and
 * GB_ERR_TIMEOUT is recorded.  stage < 0 turns it off. */
int gb_test_withhold_stage(int stage);

/* Generic FP64-accurate GEMM on the tensor cores: C = A B^T with row-major
 * A [M][K], B [N][K], C [M][N].  No counterpart in the reference (PyNOF's
 * GEMMs go through numpy / cupy). */
size_t gb_dgemm_mixed_workspace(int M, int N, int K, int nslices);
int gb_dgemm_mixed(const double* A, const double* B, int M, int N, int K, int nslices, double* C, void* workspace,
                   size_t workspace_bytes, void* stream);

/* Slice the RI factor once (the resident operand of every build):
 * replaces the device copy made at the end of compute_integrals
 * (pynof/integrals.py:51-53) for the mixed path.  prep must hold
 * gb_ri_prepare_bytes_mixed bytes and stays valid while b is unchanged. */
size_t gb_ri_prepare_bytes_mixed(int nbf, int naux, int nslices);
int gb_ri_prepare_mixed(const double* b, int nbf, int naux, int nslices, void* prep, size_t prep_bytes,
                        void* stream);

/* A1  computeJKj, RI, on the tensor cores (same outputs as gb_jkj_ri_f64).
 *     Replaces JKj_RI_GPU (pynof/integrals.py:234-245). */
size_t gb_jkj_ri_workspace_mixed(int nbf, int nbf5, int naux, int nslices);
int gb_jkj_ri_mixed(const double* C, const void* prep, int nbf, int nbf5, int naux, int nslices, double* J,
                    double* K, void* workspace, size_t workspace_bytes, void* stream);

/* The same build in two parts, so that a caller can copy J to the host while
 * K is computed, and each range of K as soon as it is done (the drop-in
 * JKj_RI_GPU does this with a second stream).  No counterpart in the
 * reference, whose JKj_RI_GPU returns J and K from one call.
 * gb_jkj_ri_mixed_j forms J and leaves T in the workspace (same size as for
 * gb_jkj_ri_mixed); gb_jkj_ri_mixed_k then forms K[q] for q0 <= q < q1 from
 * it, on the same stream and workspace.  Results are bitwise those of
 * gb_jkj_ri_mixed. */
int gb_jkj_ri_mixed_j(const double* C, const void* prep, int nbf, int nbf5, int naux, int nslices, double* J,
                      void* workspace, size_t workspace_bytes, void* stream);
int gb_jkj_ri_mixed_k(int nbf, int nbf5, int naux, int nslices, int q0, int q1, double* K, void* workspace,
                      size_t workspace_bytes, void* stream);

/* The same build in finer parts, so that the copies of J and K to the host
 * can start soon after T is formed and run back to back (the drop-in
 * JKj_RI_GPU interleaves J and K ranges on one stream and copies each on a
 * second).  No counterpart in the reference.  gb_jkj_ri_mixed_t forms T and
 * d and leaves them (and T's slicing exponents) in the workspace;
 * gb_jkj_ri_mixed_jr then forms J[q] for q0 <= q < q1, q0 a multiple of 128,
 * and gb_jkj_ri_mixed_k K[q] for any range, in any order, on the same stream
 * and workspace.  Results are bitwise those of gb_jkj_ri_mixed. */
int gb_jkj_ri_mixed_t(const double* C, const void* prep, int nbf, int nbf5, int naux, int nslices, void* workspace,
                      size_t workspace_bytes, void* stream);
int gb_jkj_ri_mixed_jr(const void* prep, int nbf, int nbf5, int naux, int nslices, int q0, int q1, double* J,
                       void* workspace, size_t workspace_bytes, void* stream);

/* A3  computeJKH_MO, RI, on the tensor cores (same outputs as gb_jkh_mo_ri_f64).
 *     Replaces JKH_MO_RI_GPU (pynof/integrals.py:383-399). */
size_t gb_jkh_mo_ri_workspace_mixed(int nbf, int nbf5, int naux, int nslices);
int gb_jkh_mo_ri_mixed(const double* C, const double* H, const void* prep, int nbf, int nbf5, int naux, int nslices,
                       double* J_MO, double* K_MO, double* H_core, void* workspace, size_t workspace_bytes,
                       void* stream);

/* A5  computeLagrange2, RI, closed shell, on the tensor cores (same outputs as
 *     gb_lagrange2_ri_f64; relies on the (m, n) symmetry of b).  Replaces the
 *     GPU branch of computeLagrange2 (pynof/utils.py:262-327). */
size_t gb_lagrange2_ri_workspace_mixed(int nbf, int nbf5, int naux, int nslices);
int gb_lagrange2_ri_mixed(const double* C, const double* H, const void* prep, const double* n, const double* cj12,
                          const double* ck12, int nbf, int nbf5, int naux, int nbeta, int nalpha, int nslices,
                          double* elag, double* Hmat, void* workspace, size_t workspace_bytes, void* stream);

/* A3 + A5  computeJKH_MO and computeLagrange2 at the same orbitals in one call
 *     on the tensor cores: the outputs of gb_jkh_mo_ri_mixed and
 *     gb_lagrange2_ri_mixed.  The orbital optimiser evaluates both at every
 *     step (energy from J_MO, K_MO, H_core; gradient from elag: calcorbe /
 *     calcorbg, pynof/pnof.py:1103-1131, in orbopt_adam, pynof/minimization.py:
 *     200-253); one half transform and one MO transform bMO[a][q][l] = (aq|l)
 *     serve both, since J_MO = d d^T with d[p] = (pp|l) and
 *     K_MO[p][q] = sum_l (pq|l)^2 come from its first nbf5 rows.  Same
 *     workspace as gb_lagrange2_ri_mixed. */
size_t gb_jkh_lagrange2_ri_workspace_mixed(int nbf, int nbf5, int naux, int nslices);
int gb_jkh_lagrange2_ri_mixed(const double* C, const double* H, const void* prep, const double* n,
                              const double* cj12, const double* ck12, int nbf, int nbf5, int naux, int nbeta,
                              int nalpha, int nslices, double* J_MO, double* K_MO, double* H_core, double* elag,
                              double* Hmat, void* workspace, size_t workspace_bytes, void* stream);

/* ------------------------------------------------------------------------
 * Batched A1 (many molecules of different sizes) on the tensor cores.  No
 * counterpart in the reference, which builds one molecule per call.  The half
 * transform, J and K GEMMs of all molecules run as three grouped launches and
 * the whole build is captured into one CUDA graph.  tiles[0..1] choose the
 * tile configuration of the half-transform and J phases (0: orbitals on the
 * 128-row side; 1, 2, 3: operands swapped, orbitals on an N tile of 32, 64,
 * 128); NULL = {0, 0}.  Inputs per molecule: C (device), the prepared factor
 * of gb_ri_prepare_mixed; outputs J, K as for gb_jkj_ri_mixed.  The plan
 * captures work on `stream` at creation and replays it with gb_batch_launch;
 * the buffers must stay valid while the plan lives.
 * ---------------------------------------------------------------------- */
typedef struct gb_batch gb_batch;
size_t gb_jkj_batch_workspace_mixed(int nmol, const int* nbf, const int* nbf5, const int* naux, int nslices);
int gb_jkj_batch_create_mixed(int nmol, const double* const* C, const void* const* prep, const int* nbf,
                              const int* nbf5, const int* naux, int nslices, double* const* J, double* const* K,
                              const int* tiles, void* workspace, size_t workspace_bytes, void* stream,
                              gb_batch** plan);
int gb_batch_launch(gb_batch* plan, void* stream);
int gb_batch_destroy(gb_batch* plan);

#ifdef __cplusplus
}
#endif

#endif /* PYNOF_GB300_H */
