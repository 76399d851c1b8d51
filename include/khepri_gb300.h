/*
 * khepri_gb300.h — C ABI of libkhp, the GB300 (sm_103a) kernels of the Crystal RCWA solve.
 *
 * Conventions
 *   - Complex numbers are pairs of doubles (re, im): the memory layout of numpy / torch
 *     complex128.  A "complex pointer" below is a `double*` to such pairs.
 *   - Matrices are row-major and contiguous; batches are contiguous along the leading axis.
 *     n = 2 * nh, nh = px * py harmonics.  An S-matrix is [2][2][n][n] (S11, S12, S21, S22),
 *     the layout of the reference's np.array([[S11, S12], [S21, S22]]).
 *   - Every pointer is a DEVICE pointer.  Every call is asynchronous on `stream` (a
 *     cudaStream_t, NULL = legacy default stream) and returns 0 (KHP_OK) or an error code;
 *     khp_status_string() names it.  Per-problem status words (int32, OR-ed flags
 *     1 = singular pivot, 2 = eigensolver not converged, 4 = non-finite value, 8 = mixed-
 *     precision refinement not converged, 16 = per-problem input out of range) are written to
 *     device arrays and are never turned into traps.
 *   - No call allocates device memory: scratch comes from the caller through `workspace`
 *     (size from the matching *_workspace function, 256-byte aligned base).
 *   - Calls are reentrant per stream and hold no host-global state.  Calls on different
 *     streams may run concurrently on the device when each has its own workspace (kernels
 *     share no device globals; khp_star_product_noalloc's fixed scratch is the one exception):
 *     two chunks of a sweep in flight on two streams fill the SMs that one chunk's latency-
 *     bound stages leave idle.
 *
 * The reference (Kaeryv/Khepri) is a numpy library; each entry point below replaces the
 * reference function named beside it (file:line in that project).
 */
#ifndef KHEPRI_GB300_H
#define KHEPRI_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KHP_OK 0
#define KHP_ERR_INVALID_ARG 1
#define KHP_ERR_WORKSPACE 2
#define KHP_ERR_CUDA 3
#define KHP_ERR_SINGULAR 4
#define KHP_ERR_NOT_CONVERGED 5
#define KHP_ERR_NONFINITE 6
#define KHP_ERR_TOO_LARGE 7

/* Library version as major*10000 + minor*100 + patch. */
int khp_version(void);
/* Static description of an error code or of a per-problem status word. */
const char* khp_status_string(int code);

/*
 * Launch tuning, process-wide (no counterpart in the reference).  param KHP_TUNE_EIG_THREADS:
 * threads per CTA of the batched eigensolver (Hessenberg reduction and QR) for matrices of
 * size n (1 <= n <= 4096): a multiple of 32 up to 256, or 0 for the default (256).  The results
 * do not depend on it; the speed does (small matrices leave a 256-thread team mostly idle).  Set
 * it before the launches it should affect (it is read when a call enqueues its kernels).
 * khepri_gb300.autotune measures the choices and writes the table the Python API applies.
 * param KHP_TUNE_TF32_MIN_N (n ignored): the mixed solve's FP32 recursion products of size
 * n >= value run as 3xTF32 on the tensor cores (khp_cgemm_tf32x3's method), smaller ones on the
 * FP32 pipe; 0 = never (default 128).
 * param KHP_TUNE_MODE_DIGITS (n ignored): 7-bit digits per operand of the tensor-core products
 * M W inside the mixed solve's eigen-refinement steps: 8 (default; operands cut at 2^-56 of their
 * row / column maximum) or 6 (2^-42).  The final residual test and the products C W stay at 8.
 */
#define KHP_TUNE_EIG_THREADS 1
#define KHP_TUNE_TF32_MIN_N 2
#define KHP_TUNE_MODE_DIGITS 3
int khp_tune(int32_t param, int32_t n, int32_t value);

/*
 * Convolution (Toeplitz) matrices of pixmaps.  Replaces tools.convolution_matrix
 * (khepri/tools.py:33-56): C[r][c] = eps_hat(p_r - p_c, q_r - q_c) with r = q*px + p and
 * eps_hat(dx, dy) = (1/(nx*ny)) sum_{x,y} eps[x][y] exp(-2 pi i (dx x/nx + dy y/ny)),
 * the fftshift(fft2(eps))/(nx*ny) coefficients the reference gathers.
 *   eps:  complex [nmaps][nx][ny] (axis 0 = x);  conv: complex [nmaps][nh][nh].
 * Requires nx >= 2*px - 1 and ny >= 2*py - 1 (the reference's index range), ny <= 8192.
 */
size_t khp_convmat_workspace(int64_t nmaps, int32_t px, int32_t py);
int khp_convmat(int64_t nmaps, int64_t nx, int64_t ny, const double* eps, int32_t px, int32_t py, double* conv,
                void* workspace, size_t ws_bytes, void* stream);

/*
 * Convolution matrices of analytical layers (Layer.analytical, khepri/layer.py:161-168): closed-
 * form Fourier transforms of disc and rectangle islands in a host medium (fourier.py:23-58,
 * 145-159), then the same Toeplitz rule as khp_convmat.
 *   islands: device [nislands][8] doubles = map index, type (0 disc: center0, center1, radius;
 *     1 rectangle: ll0, ll1, ur0, ur1; in the reference's Drawing.islands() coordinates),
 *     eps re, eps im, params[4];  eps_host: device complex [nmaps];
 *   b1, b2: reciprocal basis (2 pi convention); cell_area: |a1 x a2|;  conv: complex [nmaps][nh][nh].
 */
size_t khp_convmat_islands_workspace(int64_t nmaps, int32_t px, int32_t py);
int khp_convmat_islands(int64_t nmaps, int32_t px, int32_t py, int32_t nislands, const double* islands,
                        const double* eps_host, double b1x, double b1y, double b2x, double b2y, double cell_area,
                        double* conv, void* workspace, size_t ws_bytes, void* stream);

/*
 * Per-structure preparation of a patterned layer (done once, reused for every wavelength and
 * k-point): ic = C^-1 (the reference's Layer.IC, khepri/layer.py:158) and the products
 * hx = C^-1 diag(gx) C, hy = C^-1 diag(gy) C that make P*Q assemble in O(n^2) per problem.
 *   conv, ic, hx, hy: complex [nmaps][nh][nh];  gx, gy: real [nh] (G vectors, absolute units).
 */
size_t khp_structure_prep_workspace(int64_t nmaps, int32_t nh);
int khp_structure_prep(int64_t nmaps, int32_t nh, const double* conv, const double* gx, const double* gy, double* ic,
                       double* hx, double* hy, int32_t* status, void* workspace, size_t ws_bytes, void* stream);

/*
 * Eigenmodes of patterned layers for a batch of problems.  Replaces
 * alternative.solve_structured_layer (khepri/alternative.py:158-178):
 * (lam^2, W) = eig(P Q), lam = principal sqrt(lam^2), V = Q W / lam.
 *   map_index: int32 [batch] structure of each problem (into conv/hx/hy, [nmaps][nh][nh]);
 *   kp: complex [batch][2] in-plane wavevector (absolute); k0: real [batch] = 2 pi / wavelength;
 *   W, V: complex [batch][n][n];  lam: complex [batch][n];  status: int32 [batch].
 */
size_t khp_layer_modes_workspace(int64_t batch, int32_t nh);
int khp_layer_modes(int64_t batch, int32_t nh, const int32_t* map_index, const double* conv, const double* hx,
                    const double* hy, const double* gx, const double* gy, const double* kp, const double* k0,
                    double* W, double* V, double* lam, int32_t* status, void* workspace, size_t ws_bytes,
                    void* stream);

/*
 * S-matrix of a layer of thickness depth[b] between free-space gaps.  Replaces
 * alternative.build_scatmat (khepri/alternative.py:181-195) with W0 = I and V0 the free-space
 * modes of alternative.free_space_eigenmodes (alternative.py:84-99).
 *   W, V: complex [batch][n][n];  lam: complex [batch][n];  depth, k0: real [batch];
 *   S: complex [batch][2][2][n][n].
 */
size_t khp_layer_smatrix_workspace(int64_t batch, int32_t nh);
int khp_layer_smatrix(int64_t batch, int32_t nh, const double* W, const double* V, const double* lam,
                      const double* depth, const double* gx, const double* gy, const double* kp, const double* k0,
                      double* S, int32_t* status, void* workspace, size_t ws_bytes, void* stream);

/*
 * Closed-form S-matrices of homogeneous media (per-harmonic 2x2 algebra, no dense solve).
 * kind 0: uniform layer (alternative.solve_uniform_layer + build_scatmat, alternative.py:130-156,
 *         181-195); kind 1: incidence half-space (alternative.scattering_reflection, :32-56);
 *         kind 2: emergence half-space (alternative.scattering_transmission, :59-82).
 *   eps: complex [batch];  depth: real [batch] (ignored for kinds 1, 2);
 *   S: complex [batch][2][2][n][n];  W, V: complex [batch][n][n] or NULL;  lam: complex [batch][n] or NULL.
 */
int khp_closed_form_smatrix(int64_t batch, int32_t nh, int32_t kind, const double* eps, const double* depth,
                            const double* gx, const double* gy, const double* kp, const double* k0, double* S,
                            double* W, double* V, double* lam, int32_t* status, void* stream);

/*
 * Redheffer star product S = SA * SB.  Replaces alternative.redheffer_product
 * (khepri/alternative.py:19-30).  One LU of D = I - SB11 SA22 serves all four blocks
 * (F^-1 = I + SA22 D^-1 SB11).  sa_stride / sb_stride: batch strides in complex elements
 * (0 broadcasts one matrix to the whole batch).  S must not alias SA or SB.
 */
size_t khp_star_product_workspace(int64_t batch, int32_t n);
int khp_star_product(int64_t batch, int32_t n, const double* SA, int64_t sa_stride, const double* SB,
                     int64_t sb_stride, double* S, int32_t* status, void* workspace, size_t ws_bytes, void* stream);

/*
 * Batched reflection and transmission of one layer stack for many problems, in one call.
 * Replaces the per-point loop Crystal.set_source -> solve -> poynting_flux_end
 * (khepri/crystal.py:180-206, 363-396; README.md:52-58) when only R and T are wanted: instead
 * of every layer's S-matrix and the four-block chain (alternative.py:19-30, 181-195;
 * layer.py:35-60) it runs a backward reflection-matrix recursion and a forward pass of the two
 * source columns (same continuity conditions; patterned layers handled in their mode basis).
 *   layer_kind, layer_map, layer_eps, layer_depth: HOST arrays [nlayers] from the incidence side;
 *     kind 0 = uniform (eps: complex pair), 1 = patterned (map index into conv/hx/hy);
 *     patterned layers with equal layer_map share their modes;
 *   problem_map, problem_depth: optional DEVICE arrays [nlayers][batch] (NULL = layer_map /
 *     layer_depth for every problem) giving each problem its own map index and depth per layer,
 *     so that one call solves many structures of one shape (one harmonic set and layer
 *     count); layers sharing a layer_map value must share the per-problem map too (the first
 *     such layer's entry is used).  A map index outside [0, nmaps) sets status bit 16 and is
 *     read as 0;
 *   conv, hx, hy: device complex [nmaps][nh][nh] from khp_convmat / khp_structure_prep;
 *   kp: complex [batch][2]; k0: [batch]; te, tm: complex [batch][npol] (npol polarisations
 *   share one recursion);  R, T: real [batch][npol].
 */
size_t khp_solve_batched_workspace(int64_t batch, int32_t nh, int32_t nlayers, const int32_t* layer_kind,
                                   const int32_t* layer_map);
int khp_solve_batched(int64_t batch, int32_t px, int32_t py, int32_t nlayers, const int32_t* layer_kind,
                      const int32_t* layer_map, const double* layer_eps, const double* layer_depth,
                      const int32_t* problem_map, const double* problem_depth, int64_t nmaps,
                      const double* conv, const double* hx, const double* hy, const double* gx, const double* gy,
                      double epsi_re, double epsi_im, double epse_re, double epse_im, const double* kp,
                      const double* k0, int32_t npol, const double* te, const double* tm, double* R, double* T,
                      int32_t* status, void* workspace, size_t ws_bytes, void* stream);

/*
 * Mixed-precision form of khp_solve_batched (same arguments plus refine_iters; at most 16
 * layers).  Every O(n^3) step runs in FP32; FP64 is used for three eigen-refinement steps per
 * patterned-layer eigensolve (residual M W - W mu) and for the residual of the whole stack's
 * interface equations, which refine_iters rounds of iterative refinement drive to near-FP64
 * accuracy through the FP32 factors (0 = FP32 answer only, at most 64; 2 is the default of the
 * Python API).  The residual's products run in double-float (FP32 pairs) in those rounds and in
 * FP64 in the up to 12 extra rounds of problems that have not converged by then.
 * A problem whose refinement has not converged (estimated error of its reflected or
 * transmitted amplitudes above 1e-9, e.g. an ill-conditioned system next to a Wood anomaly)
 * gets status bit 8; its R, T must then be recomputed, by khp_solve_batched_mixed_repair from
 * this call's refined modes (the Python API does this) or by khp_solve_batched.  After the
 * eigen-refinement every mode is checked in FP64: a problem with a mode whose relative residual
 * |M w - mu w| / (max|mu| |w|) exceeds 1e-8 gets status bit 32 and must be recomputed by
 * khp_solve_batched (its own FP64 eigensolve).
 */
size_t khp_solve_batched_mixed_workspace(int64_t batch, int32_t nh, int32_t nlayers, const int32_t* layer_kind,
                                         const int32_t* layer_map);
int khp_solve_batched_mixed(int64_t batch, int32_t px, int32_t py, int32_t nlayers, const int32_t* layer_kind,
                            const int32_t* layer_map, const double* layer_eps, const double* layer_depth,
                            const int32_t* problem_map, const double* problem_depth, int64_t nmaps,
                            const double* conv, const double* hx, const double* hy, const double* gx,
                            const double* gy, double epsi_re, double epsi_im, double epse_re, double epse_im,
                            const double* kp, const double* k0, int32_t npol, const double* te, const double* tm,
                            int32_t refine_iters, double* R, double* T, int32_t* status, void* workspace,
                            size_t ws_bytes, void* stream);

/*
 * FP64 re-solve of problems that khp_solve_batched_mixed flagged with status bit 8 (its stack
 * refinement did not converge), from that call's refined FP64 modes: the reflection-matrix
 * recursion of khp_solve_batched in FP64, without its FP64 eigensolve.  Replaces, like
 * khp_solve_batched, crystal.py:180-206 (layer.py:35-60, alternative.py:19-30, 181-195) and
 * crystal.py:363-396 for the problems it is given.
 *   The first arguments describe the problems to re-solve (batch of them: their kp, k0, te, tm,
 *   problem_map, problem_depth) exactly as for khp_solve_batched; mixed_index: device int32
 *   [batch], each problem's row in the earlier khp_solve_batched_mixed call of mixed_batch
 *   problems on the same stack (same nlayers, layer_kind, layer_map), whose workspace
 *   (mixed_workspace, mixed_ws_bytes) must be unchanged since.  Workspace:
 *   khp_solve_batched_workspace(batch, ...).  A bit-32 problem (modes that missed their own
 *   residual test) must go to khp_solve_batched instead.
 */
int khp_solve_batched_mixed_repair(int64_t batch, int32_t px, int32_t py, int32_t nlayers, const int32_t* layer_kind,
                                   const int32_t* layer_map, const double* layer_eps, const double* layer_depth,
                                   const int32_t* problem_map, const double* problem_depth, int64_t nmaps,
                                   const double* conv, const double* hx, const double* hy, const double* gx,
                                   const double* gy, double epsi_re, double epsi_im, double epse_re, double epse_im,
                                   const double* kp, const double* k0, int32_t npol, const double* te,
                                   const double* tm, int64_t mixed_batch, const int32_t* mixed_index,
                                   const void* mixed_workspace, size_t mixed_ws_bytes, double* R, double* T,
                                   int32_t* status, void* workspace, size_t ws_bytes, void* stream);

/*
 * Solve + gradient: khp_solve_batched_mixed and, in the same call, the gradient of
 *   L = sum_{b,p,g} dR[b][p][g] R_{b,p,g} + dT[b][p][g] T_{b,p,g}
 * (per-order reflected / transmitted powers, crystal.py:363-396 with only_total=False) with
 * respect to the convolution matrix of every map, by the adjoint method: one transposed solve
 * of the stack's interface equations per problem (FP64 residual, FP32 transposed sweep,
 * refine_iters + 3 rounds) and the Daleckii-Krein form of the eigen-decomposition's
 * derivative, which stays finite for degenerate modes.  No counterpart in the reference (it has
 * no gradient; its users take finite differences of whole solves).
 *   ic: device complex [nmaps][nh][nh] = C^-1 (khp_structure_prep);
 *   dR, dT: device real [batch][npol][nh] (NULL = 0);  R_orders, T_orders: device real
 *   [batch][npol][nh] out (NULL = not written);  dconv: device complex [nmaps][nh][nh] out, in
 *   the convention dL = Re sum(dconv o dC) (summed over the problems using each map; a problem
 *   returned with status bit 8 adds nothing to it: solve it again with more refine_iters and add
 *   its share, as the Python API does);
 *   refine_iters >= 1.  A problem whose forward refinement did not converge keeps status bit 8
 *   (no FP64 re-solve here).
 */
size_t khp_solve_batched_mixed_grad_workspace(int64_t batch, int32_t nh, int32_t nlayers, const int32_t* layer_kind,
                                              const int32_t* layer_map, int64_t nmaps);
int khp_solve_batched_mixed_grad(int64_t batch, int32_t px, int32_t py, int32_t nlayers, const int32_t* layer_kind,
                                 const int32_t* layer_map, const double* layer_eps, const double* layer_depth,
                                 const int32_t* problem_map, const double* problem_depth, int64_t nmaps,
                                 const double* conv, const double* ic, const double* hx, const double* hy,
                                 const double* gx, const double* gy, double epsi_re, double epsi_im, double epse_re,
                                 double epse_im, const double* kp, const double* k0, int32_t npol, const double* te,
                                 const double* tm, int32_t refine_iters, const double* dR, const double* dT, double* R,
                                 double* T, double* R_orders, double* T_orders, double* dconv, int32_t* status,
                                 void* workspace, size_t ws_bytes, void* stream);

/*
 * Adjoint of khp_convmat: deps = gradient with respect to the pixmaps, given dconv (both in
 * the convention dL = Re sum(d o delta)).  eps real: dL/deps = Re(deps).  Backward counterpart
 * of tools.py:33-56 (no counterpart in the reference).
 *   dconv: device complex [nmaps][nh][nh];  deps: device complex [nmaps][nx][ny].
 */
size_t khp_convmat_bwd_workspace(int64_t nmaps, int64_t ny, int32_t px, int32_t py);
int khp_convmat_bwd(int64_t nmaps, int64_t nx, int64_t ny, const double* dconv, int32_t px, int32_t py, double* deps,
                    void* workspace, size_t ws_bytes, void* stream);

/*
 * Twisted bilayers: R and T of an extended crystal over the product expansion e1 + e2
 * (khepri/expansion.py:52-73, khepri/extension.py:10-126, crystal.py:180-206, 363-396), from the
 * base-size chains.  s_left: device complex [batch][nbase][2][2][2 nbase][2 nbase], the chain
 * (incidence half-space * layers on e1 * uniform layers) solved on e1 at kp + g2[m] for every
 * harmonic m of e2; s_right: the chain (layers on e2 * emergence half-space) on e2 at kp + g1[m].
 * Only the final product is dense (n = 2 nbase^2): t = B21 (I - A22 B11)^-1 A21 c,
 * r = A11 c + A12 B11 (I - A22 B11)^-1 A21 c, with one FP64 LU per problem.
 *   gx, gy: the product expansion's G vectors [nbase^2] (index p nbase + q: e1 harmonic p,
 *   e2 harmonic q);  te, tm: complex [batch][npol];  R, T: [batch][npol];  rv, tv: optional
 *   complex [batch][2 nbase^2][2] out (reflected / transmitted amplitudes of the two unit
 *   sources, NULL = not kept).
 */
size_t khp_twisted_rt_workspace(int64_t batch, int32_t nbase);
int khp_twisted_rt(int64_t batch, int32_t nbase, const double* s_left, const double* s_right, const double* gx,
                   const double* gy, const double* kp, const double* k0, int32_t npol, const double* te,
                   const double* tm, double epsi_re, double epsi_im, double epse_re, double epse_im, double* R,
                   double* T, double* rv, double* tv, int32_t* status, void* workspace, size_t ws_bytes, void* stream);

/*
 * Star product without a caller-supplied workspace.  No counterpart in the reference: it
 * serves callers that cannot allocate or lend device memory (a host whose device memory is
 * fully partitioned up front, or a latency-critical loop where cudaMalloc, which may
 * synchronise the device, is not allowed).  Same arguments and result as khp_star_product
 * minus the workspace.  Its scratch is a fixed device array of KHP_NOALLOC_SCRATCH_BYTES
 * inside libkhp, held by every GPU that loads the library until the process exits; batches
 * whose khp_star_product_workspace(batch, n) exceeds it return KHP_ERR_TOO_LARGE.
 * The first call on a device looks up the array's device address (with that device current),
 * so make it before any stream capture.  The address is cached for the life of the process:
 * a cudaDeviceReset unloads the library's module and may move the array, so a process that
 * resets a device must not call this entry point on it afterwards.  All calls share the one
 * array and it keeps the last call's contents: calls that overlap on the GPU (other streams,
 * other host threads) race.
 */
#define KHP_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)
int khp_star_product_noalloc(int64_t batch, int32_t n, const double* SA, int64_t sa_stride, const double* SB,
                             int64_t sb_stride, double* S, int32_t* status, void* stream);

/*
 * Reflected and transmitted power.  Replaces Crystal.poynting_flux_end
 * (khepri/crystal.py:363-396) with the source vector of alternative.incident
 * (alternative.py:101-128) and alternative.poynting_fluxes (alternative.py:235-245).
 *   S: complex [batch][2][2][n][n] global S-matrix (s_stride: batch stride in complex elements);
 *   te, tm: complex [batch] polarisation weights;  epsi, epse: complex scalars (host values);
 *   R, T: real [batch];  r_orders, t_orders: real [batch][nh] or NULL.
 * Evanescent incidence (Re kz_inc = 0) yields NaN, as in the reference.
 */
int khp_flux(int64_t batch, int32_t px, int32_t py, const double* S, int64_t s_stride, const double* gx,
             const double* gy, const double* kp, const double* k0, const double* te, const double* tm, double epsi_re,
             double epsi_im, double epse_re, double epse_im, double* R, double* T, double* r_orders, double* t_orders,
             void* stream);

/*
 * Field reconstruction (Crystal.fields_coords_xy / fields_volume, khepri/crystal.py:234-343).
 *
 * khp_fields_amplitudes — one solved problem; for each of nlayers layers l (arrays of device
 * pointers, one entry per layer): forward-chain S at l (sl_ptrs, [2][2][n][n]), reverse-chain
 * S at l (sr_ptrs), the layer's W and V ([n][n]).  vref: V of the incidence half-space [n][n];
 * inc: complex [2n] incident (E; H) Fourier vector; kp: complex [2]; k0: real [1].
 * Output amps: complex [nlayers][2n] = RI^-1 R0 [c+; c-], with c+- from
 * fields.translate_mode_amplitudes (khepri/fields.py:18-27) and c1p from Crystal._fourier_fields
 * (crystal.py:259-264).  status: int32 [1], OR-ed flags.
 */
size_t khp_fields_amplitudes_workspace(int64_t nlayers, int32_t nh);
int khp_fields_amplitudes(int64_t nlayers, int32_t nh, const int64_t* sl_ptrs, const int64_t* sr_ptrs,
                          const int64_t* w_ptrs, const int64_t* v_ptrs, const double* vref, const double* inc,
                          const double* gx, const double* gy, const double* kp, const double* k0, double* amps,
                          int32_t* status, void* workspace, size_t ws_bytes, void* stream);

/*
 * Fourier-space fields at nz depths (khepri/fields.py:53-76): for depth z in slot s = slot_of_z[z],
 * f = RI (L o amps[s]) with L = [exp(lam zbar), exp(-lam zbar)] clamped to modulus <= 1e14,
 * then sz = -i IC (kx uy - ky ux), uz = -i (kx sy - ky sx).  ic_ptrs[s] points to the layer's
 * C^-1 ([nh][nh]) or is 0, in which case the complex scalar ic_scalar[s] (= 1/eps) is used.
 * zbar: real [nz] = k0 (depth - z_rel).  ff: complex [nz][6][nh] = (sx, sy, sz, ux, uy, uz).
 */
int khp_fields_fourier(int64_t nz, int32_t nh, const int32_t* slot_of_z, const double* zbar, const int64_t* w_ptrs,
                       const int64_t* v_ptrs, const int64_t* lam_ptrs, const int64_t* ic_ptrs, const double* ic_scalar,
                       const double* amps, const double* gx, const double* gy, const double* kp, const double* k0,
                       double* ff, void* stream);

/*
 * Inverse Fourier sum to real space, khepri/fourier.py:136-142 (idft):
 * out[r][p] = sum_g ff[r][g] exp(i ((kp_x + gx_g) x_p + (kp_y + gy_g) y_p)).
 * ff: complex [rows][nh]; x, y: real [npts]; kp: complex [2]; out: complex [rows][npts].
 */
int khp_fields_idft(int64_t rows, int32_t nh, const double* ff, const double* gx, const double* gy, const double* kp,
                    int64_t npts, const double* x, const double* y, double* out, void* stream);

/*
 * Band structure from a scattering matrix: the eigenpairs of the pencil (Sl, Sr) of
 * khepri/eigentricks.py:5-43 (scattering_splitlr, scattering_eigenvalues, scattering_det).
 *   S: complex [batch][4 ng][4 ng] dense, row-major, blocks [[S11, S12], [S21, S22]] of 2 ng
 *      (the reference's p = 0:2ng, m = 2ng:4ng); s_stride: batch stride in complex elements.
 *   w: complex [batch][4 ng] eigenvalues;  v: complex [batch][4 ng][4 ng] unit right
 *      eigenvectors (columns) or NULL;  det: complex [batch] = det(S11 - S12 S22^-1 S21) det(S22)
 *      or NULL.  Computed as the eigenpairs of Sr^-1 Sl (S22 is inverted once).
 *   status: int32 [batch], OR-ed: SINGULAR (S22 singular: an infinite pencil eigenvalue),
 *      NONFINITE (NaN / inf in S: the reference returns None), NOT_CONVERGED.
 */
size_t khp_scattering_eig_workspace(int64_t batch, int32_t ng);
int khp_scattering_eig(int64_t batch, int32_t ng, const double* S, int64_t s_stride, double* w, double* v,
                       double* det, int32_t* status, void* workspace, size_t ws_bytes, void* stream);

/*
 * Plane-wave amplitudes of a sampled beam over a Brillouin-zone-integration supercell
 * (khepri/beams.py:164-190, amplitudes_from_fields, with fourier.slow_dft, fourier.py:94-104).
 *   fields: complex [X][Y][2][3] (E, H; x, y, z) with X = bzs1 * ns, Y = bzs0 * ns;
 *   x, y: real [X][Y] sample coordinates; kp: complex [2] incident planar wavevector;
 *   gx, gy: real [ng] the expansion's g vectors;  out: complex [4][ng] for (Ex, Ey, Hx, Hy):
 *   sum over the bzs0 * bzs1 cells of the direct DFT of the fields divided by exp(i kp.r), over
 *   (cells * ns) — the reference's cell pairing of samples and coordinates included.
 *   Scratch: khp_bzi_amplitudes_workspace(bzs0, bzs1, ns) bytes.
 */
size_t khp_bzi_amplitudes_workspace(int32_t bzs0, int32_t bzs1, int32_t ns);
int khp_bzi_amplitudes(int32_t bzs0, int32_t bzs1, int32_t ns, const double* fields, const double* x, const double* y,
                       const double* kp, int32_t ng, const double* gx, const double* gy, double* out, void* workspace,
                       size_t ws_bytes, void* stream);

/*
 * tmat formulation of a patterned layer (khepri/tmat/scattering.py:25-51, matrices.py:126-212),
 * SI units, batched over (wavelength, kp) problems that share the Fourier coefficients.
 * khp_tmat_layer_smatrix:
 *   eps_g, epsinv_g: complex [nq0][nq1] coefficients of eps and 1/eps (tools.epsilon_g);
 *   gx, gy: real [px * py] g vectors of the harmonics in the reference's order (lattice.gx.T
 *   flattened: harmonic g = i1 + px * i2);  kp: real [batch][2];  wavelength: real [batch];
 *   u_blocks, v_blocks: complex [batch][16][px * py], the 4 x 4 blocks of diagonals of U and Vi
 *   (matrix_u, matrix_v; block (a, c) at a * 4 + c);  depth, slicing_pow as scattering_matrix.
 *   S: complex [batch][4 ng][4 ng] = multS^p(matrix_s(U expm(-A depth / 2^p) Vi)).
 *   A_out, E_out, T_out (each complex [batch][4 ng][4 ng] or NULL): A, the slice's expm, U E Vi.
 *   The exponential is one scaling and squaring for the batch (its largest 1-norm): the call
 *   synchronises the stream once to read that norm.
 * khp_tmat_multS: S = multS(S1, S2) (matrices.py:194-212), dense [4 ng][4 ng] each.
 * khp_tmat_matrix_s: S = matrix_s(T) (matrices.py:171-180), T and S [batch][4 ng][4 ng]
 *   contiguous; scratch: khp_tmat_multS_workspace(batch, ng) bytes.
 * status: int32 [batch], OR-ed (SINGULAR for a singular block inverse or solve).
 */
size_t khp_tmat_layer_workspace(int64_t batch, int32_t ng);
int khp_tmat_layer_smatrix(int64_t batch, int32_t px, int32_t py, int32_t nq0, int32_t nq1, const double* eps_g,
                           const double* epsinv_g, const double* gx, const double* gy, const double* kp,
                           const double* wavelength, const double* u_blocks, const double* v_blocks, double depth,
                           int32_t slicing_pow, double* S, double* A_out, double* E_out, double* T_out,
                           int32_t* status, void* workspace, size_t ws_bytes, void* stream);
size_t khp_tmat_multS_workspace(int64_t batch, int32_t ng);
int khp_tmat_matrix_s(int64_t batch, int32_t ng, const double* T, double* S, int32_t* status, void* workspace,
                      size_t ws_bytes, void* stream);
int khp_tmat_multS(int64_t batch, int32_t ng, const double* S1, int64_t s1_stride, const double* S2, int64_t s2_stride,
                   double* S, int32_t* status, void* workspace, size_t ws_bytes, void* stream);

/*
 * Diagnostics (no counterpart in the reference).
 * khp_launch_count: number of kernels libkhp has launched in this process (all entry points).
 * khp_probe_fp64_tflops: measured FP64 FMA throughput of the current device in TFLOP/s, the
 * denominator of FP64 roofline fractions; synchronises `stream`; scratch: device doubles,
 * at least 1024 * (number of SMs); returns a negative value on failure.
 */
long long khp_launch_count(void);
double khp_probe_fp64_tflops(double* scratch, int64_t scratch_doubles, void* stream);

/*
 * khp_probe_fp32_tflops: the same probe for the FP32 FMA pipe (scratch: floats, at least
 * 2048 * number of SMs).
 * khp_stage_timing(enable): with enable = 1, the mixed solve records CUDA events on its stream
 * around its stages (below) and sums their device time; 0 stops.  Either call discards what was
 * recorded.  khp_stage_timing_read(stage, ms, marks): total milliseconds and number of timed
 * intervals of a stage since the last khp_stage_timing call (synchronises the recorded events).
 * Off by default; meant for benchmarks, not for stream capture.
 */
#define KHP_STAGE_MODES 0       /* modes of the patterned layers: eigensolve, refinement, V, inverses */
#define KHP_STAGE_EIGENSOLVE 1  /* the FP32 eigensolver inside the modes stage */
#define KHP_STAGE_TC_PRODUCT 2  /* FP64-accurate tensor-core products (khp_zgemm_fp64_tc and internal uses) */
#define KHP_STAGE_RECURSION 3   /* FP32 reflection-matrix recursion with its kept factors */
#define KHP_STAGE_REFINE 4      /* FP64 iterative refinement of the stack equations and fluxes */
#define KHP_NUM_STAGES 5
double khp_probe_fp32_tflops(float* scratch, int64_t scratch_floats, void* stream);
int khp_stage_timing(int32_t enable);
int khp_stage_timing_read(int32_t stage, double* ms, int64_t* marks);

/*
 * FP64-accurate batched complex product on the bf16 tensor cores (no counterpart in the
 * reference; the mixed-precision solve forms its FP64 eigen-residuals and V = Q W this way).
 * C[b] = A[b] B[b]; A: complex [batch] m x k (row stride lda, batch stride bsA, in complex
 * elements), B: k x n, C: m x n.  Each operand is split exactly into signed digits per row (A)
 * or column (B): for k <= 288, eight 7-bit digits whose 36 leading products are accumulated per
 * level in tensor memory (tcgen05); above, seven 8-bit digits and 28 products on mma.sync with
 * FP32/int32 level sums.  The error per element is ~2^-55 * 2k * max|A row| * max|B column|, an
 * FP64 product's own bound.  k <= 4096.  Scratch: khp_zgemm_fp64_tc_workspace(batch, m, n, k)
 * bytes.
 */
size_t khp_zgemm_fp64_tc_workspace(int64_t batch, int32_t m, int32_t n, int32_t k);

/*
 * FP32-accurate batched complex product on the tcgen05 tensor cores by 3xTF32 (no counterpart
 * in the reference; the products of alternative.py:19-30 and 181-195, and of the mixed solve's
 * recursion, are of this kind).  C[b] = A[b] B[b]: A complex [batch] m x k (row stride lda,
 * batch stride a_stride, in complex elements), B k x n, C m x n, all FP32.  Every value is split
 * into a TF32 part and a TF32 remainder, and hi hi + hi lo + lo hi accumulate in FP32 in tensor
 * memory: the error per element is ~2^-21 * 2k * max|A row| * max|B column|.  Scratch:
 * khp_cgemm_tf32x3_workspace(batch, m, n, k) bytes (the split operands).
 */
size_t khp_cgemm_tf32x3_workspace(int64_t batch, int32_t m, int32_t n, int32_t k);
int khp_cgemm_tf32x3(int64_t batch, int32_t m, int32_t n, int32_t k, const float* A, int64_t lda, int64_t a_stride,
                     const float* B, int64_t ldb, int64_t b_stride, float* C, int64_t ldc, int64_t c_stride,
                     void* workspace, size_t ws_bytes, void* stream);
int khp_zgemm_fp64_tc(int64_t batch, int32_t m, int32_t n, int32_t k, const double* A, int64_t lda, int64_t bsA,
                      const double* B, int64_t ldb, int64_t bsB, double* C, int64_t ldc, int64_t bsC, void* workspace,
                      size_t ws_bytes, void* stream);

/*
 * Batched explicit inverse of complex n x n matrices, the reference's numpy.linalg.inv / solve
 * building block (khepri/alternative.py:24-27, 50-55, 164-165, 182-193; khepri/layer.py:158;
 * khepri/crystal.py:372): blocked LU with partial pivoting, then A^-1 = U^-1 L^-1 P.
 * precision: 0 = FP64 (A, Ainv complex128), 1 = FP32 (complex64).  A [batch] n x n row-major,
 * batch stride a_stride (complex elements), is overwritten by the LU factors; Ainv [batch] n x n,
 * batch stride inv_stride.  status: int32 [batch], OR-ed: SINGULAR (an exactly zero pivot
 * column) or NONFINITE (non-finite values in a pivot column); the inverse is then not meaningful.
 * Scratch: khp_inverse_workspace(batch, n) bytes.
 */
size_t khp_inverse_workspace(int64_t batch, int32_t n);
int khp_inverse(int64_t batch, int32_t n, int32_t precision, void* A, int64_t a_stride, void* Ainv,
                int64_t inv_stride, int32_t* status, void* workspace, size_t ws_bytes, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* KHEPRI_GB300_H */
