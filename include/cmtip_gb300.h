/*
 * cmtip_gb300 -- C ABI of the GB300 (sm_103a) reconstruction hot path of cartesian
 * MTIP: 3D type-1/type-2 NUFFT, the conjugate-gradient autocorrelation solve and
 * orientation matching.
 *
 * All array pointers are DEVICE pointers owned by the caller (PyTorch tensors in
 * the Python layer); every call is stream-ordered on the stream given at creation
 * (a cudaStream_t passed as void*, NULL = legacy default stream).  Objects own only
 * their workspace.  Every function returns a status code (CMT_OK = 0);
 * cmt_last_error() returns a thread-local description of the last failure.
 *
 * Reference interfaces replaced (paths inside the cmtip project):
 *   cmt_plan_create / cmt_set_pts / cmt_execute / cmt_plan_destroy
 *       -> cmtip/nufft/forward.py:45-82 forward_gpu (cufinufft type 2, isign -1,
 *          set_pts at :77-79, execute :79) and cmtip/nufft/adjoint.py:46-86
 *          adjoint_gpu (cufinufft type 1, isign +1, set_pts :74, execute :75,
 *          *support / .real / M**3 at :79-86), and the CPU twins forward_cpu
 *          (:13-42, finufft nufft3d2) / adjoint_cpu (:13-43, finufft nufft3d1).
 *   cmt_set_pts_quat / cmt_inverse_rotations
 *       -> cmtip/autocorrelation/autocorrelation.py:12-29 gen_nonuniform_positions and
 *          cmtip/alignment/align.py:50-57 (rotate pixel q-vectors by inv(R(q)), cast to
 *          float32, scale by pi / reciprocal_extent).
 *   cmt_execute_pair
 *       -> the data term of W in cmtip/autocorrelation/autocorrelation.py:150-155
 *          (core_problem_convolution, :32-63) applied as an explicit type-2 then
 *          type-1 pair instead of the Toeplitz embedding.
 *   cmt_cg_*
 *       -> cmtip/autocorrelation/autocorrelation.py:113-173 setup_linops and the
 *          scipy cg call of solve_ac (:234-239).
 *   cmt_match_*
 *       -> cmtip/alignment/align.py:68-132 match_orientations (compute_slices :39-65,
 *          std scaling :122-124, calc_eudist :27-36, argmin :131).
 */
#ifndef CMTIP_GB300_H
#define CMTIP_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define CMT_OK 0
#define CMT_ERR_ARG 1      /* bad argument (shape, type, size, null pointer) */
#define CMT_ERR_RANGE 2    /* a nonuniform point has |x| >= 3 pi (forward.py:27, adjoint.py:29) */
#define CMT_ERR_OOM 3      /* device allocation failed */
#define CMT_ERR_CUDA 4     /* CUDA runtime error */
#define CMT_ERR_TIMEOUT 5  /* a bounded device wait gave up */
#define CMT_ERR_CUFFT 6    /* cuFFT error */
#define CMT_ERR_STATE 7    /* call out of order (e.g. execute before set_pts) */

/* cmt_execute flags */
#define CMT_REAL_IN 1      /* type 1: strengths c are real; type 2: modes f are real */
#define CMT_REAL_OUT 2     /* type 1: write Re(f) (M^3 reals); type 2: write Re(c) (N reals) */
#define CMT_MODEORD_FFT 4  /* modes stored FFT-style (k at index k mod M) instead of centred */

typedef struct cmt_plan cmt_plan;

/* Create a cubic 3D NUFFT plan.
 * type   1 (nonuniform -> M^3 modes) or 2 (M^3 modes -> nonuniform)
 * M      modes per dimension; mode k in [-floor(M/2), (M-1)-floor(M/2)],
 *        stored centred (index k + floor(M/2)) unless CMT_MODEORD_FFT
 * prec   32 (float / complex64) or 64 (double / complex128)
 * eps    requested relative tolerance (sets kernel width); clamped to what prec can reach
 * isign  sign of the exponent: -1 for cmtip's forward, +1 for its adjoint
 * upsampfac  fine grid / M ratio (0 = automatic choice)
 * Replaces cufinufft(type, shape, isign=, eps=, dtype=, gpu_method=1) at forward.py:77 / adjoint.py:73. */
int cmt_plan_create(int type, int M, int prec, double eps, int isign, double upsampfac,
                    void *stream, cmt_plan **plan);

/* A plan (type, M modes, isign) on the points of src whose fine grid is exactly twice as
 * fine as src's: src's bin order and permutation apply unchanged, so no second sort and no
 * second copy of the points.  It follows src's current points at every execute; src must
 * outlive it.  The autocorrelation solve uses it for the Toeplitz kernel on 2M modes
 * (cmtip/autocorrelation/autocorrelation.py:141-147) over the points of the M-mode plan. */
int cmt_plan_create_derived(const cmt_plan *src, int type, int M, int isign, cmt_plan **plan);

/* Query the chosen fine-grid size, kernel width, ES shape parameter and bin size. */
int cmt_plan_info(const cmt_plan *plan, int *n_fine, int *width, double *beta, int *bin_size,
                  int64_t *n_subproblems);

/* Set nonuniform points from coordinate arrays (device, prec-typed, length N, radians,
 * |x| < 3 pi).  Points are counting-sorted into spatial bins of the fine grid; the plan
 * keeps the sorted coordinates and the permutation.  The sort's buffers come from the
 * device's default stream-ordered memory pool on the plan's stream; the library sets that
 * pool to keep freed memory, so repeated calls reuse it without new mappings.  Replaces
 * plan.set_pts (forward.py:77-79: cufinufft is given (L, K, H) so that H pairs with array
 * axis 0; here x pairs with axis 0). */
int cmt_set_pts(cmt_plan *plan, int64_t N, const void *x, const void *y, const void *z);

/* Set points from per-image inverse rotation matrices (device, n_img x 3 x 3 float64) and
 * detector q-vectors (device, 3 x n_pix float64): point (i, p) has coordinates
 * float32(inv_rot[i] . ppr[:, p]) * pi / reciprocal_extent, point index i * n_pix + p. */
int cmt_set_pts_quat(cmt_plan *plan, int64_t n_img, const double *inv_rot, int64_t n_pix,
                     const double *ppr, double reciprocal_extent);

/* Execute.  type 1: c (N strengths) -> f (M^3 modes); type 2: f -> c.
 * support  optional M^3 float mask multiplied into the modes (type 1: output; type 2: input)
 * scale    multiplies the output (cmtip's adjoint divides by M**3, adjoint.py:43)
 * flags    CMT_REAL_IN / CMT_REAL_OUT / CMT_MODEORD_FFT
 * For type 1 with CMT_REAL_IN, c may be NULL: all strengths are 1. */
int cmt_execute(cmt_plan *plan, void *c, void *f, const float *support, double scale, int flags);

/* Fused type-2 then type-1 pair on the plan's points (the normal operator A^H A):
 * f_out = scale * S . Re( sum_j e^{+i k.x_j} sum_k' e^{-i k'.x_j} (S . f_in)_k' )
 * with S the optional support.  f_in / f_out are real M^3 grids of the plan's precision. */
int cmt_execute_pair(cmt_plan *plan, const void *f_in, void *f_out, const float *support, double scale);

/* Release the plan.  Waits for the device first (cudaDeviceSynchronize): the sorted points
 * and the sort's buffers are stream-ordered pool allocations, which cudaFree would release
 * without waiting for launches still reading them. */
int cmt_plan_destroy(cmt_plan *plan);

/* Per-launch CUDA-event timing of the spread / interpolation kernels (enable 0/1), and
 * read-back of up to max recorded launches (ms, kinds: 1 spread, 2 interp) since the last
 * read.  Used by benchmarks; recording adds two event records per launch. */
int cmt_plan_profile(cmt_plan *plan, int enable);
int cmt_plan_profile_read(cmt_plan *plan, float *ms, int *kinds, int max, int *count);

/* Move the plan (its kernels and its cuFFT plans) to another stream. */
int cmt_plan_set_stream(cmt_plan *plan, void *stream);

/* Allocate the pair operator's workspace (second fine grid, C2C transform) now, so that a
 * later cmt_execute_pair allocates nothing (e.g. inside CUDA graph capture). */
int cmt_plan_prepare_pair(cmt_plan *plan);

/* Tuning of a plan (the autotuner's knobs): bin_size = fine cells per bin edge (2..32; the
 * shared-memory subgrid of a subproblem is (bin_size + w)^3), maxsub = points per
 * subproblem (one CTA; 256..2^20).  0 keeps a value.  Drops the plan's points (call
 * cmt_set_pts / cmt_set_pts_quat again).  CMT_ERR_ARG if the subgrid does not fit in shared
 * memory.  No counterpart in the reference (finufft picks its bins internally). */
int cmt_plan_set_tuning(cmt_plan *plan, int bin_size, int maxsub);
int cmt_plan_get_tuning(const cmt_plan *plan, int *bin_size, int *maxsub);

/* ---------------------------------------------------------------- data preparation
 * Detector binning and resolution clipping in one pass (cmtip/prep_data.py:181-212 bin_data,
 * :149-163 clip_data): in = (n_img, n_panels, px, py) values of precision prec (32 | 64);
 * each panel is averaged over bin x bin blocks in numpy's summation order (results equal
 * numpy's bit for bit), then the binned pixels keep[0 .. n_keep) (indices into the binned
 * (panel, x, y) order; NULL keeps all) are written to out = (n_img, n_keep).  Indices
 * outside the binned range give CMT_ERR_ARG (and zeros, never an out-of-range read).
 * Synchronises with the stream when keep is given. */
int cmt_bin_clip(int prec, const void *in, int64_t n_img, int n_panels, int px, int py, int bin,
                 const int64_t *keep, int64_t n_keep, void *out, void *stream);

/* ---------------------------------------------------------------- batches of plans
 * Many independent reconstructions in one launch per stage: a batch holds plans of one
 * type, precision, sign and kernel width (2..8, i.e. eps >= 1e-7) but its own modes M,
 * points, tuning and fine grid each.  cmt_batch_execute runs every plan's grid preparation,
 * ONE persistent spreading (type 1) or interpolation (type 2) kernel over the subproblems
 * of all plans, then every plan's FFT and deconvolution; c[i], f[i], support[i], scale[i]
 * mean what they mean for cmt_execute on plan i (support, scale may be NULL).  Plans are
 * borrowed (they must outlive the batch); a plan given new points or tuning is picked up
 * by the next execute.  Derived plans (cmt_plan_create_derived) may be batched; a batch of
 * derived plans only spreads through their extended register window, as a single derived
 * plan does.  Stream-ordered on the batch's stream.  No counterpart in the reference, which
 * reconstructs one particle per process. */
typedef struct cmt_batch cmt_batch;
int cmt_batch_create(int n_plans, cmt_plan *const *plans, void *stream, cmt_batch **batch);
int cmt_batch_execute(cmt_batch *batch, void *const *c, void *const *f, const float *const *support,
                      const double *scale, int flags);
int cmt_batch_profile(cmt_batch *batch, int enable);
int cmt_batch_last_ms(cmt_batch *batch, float *ms, int64_t *n_work);
int cmt_batch_destroy(cmt_batch *batch);

/* ---------------------------------------------------------------- CG solve
 * Solver of W x = d, W = alambda * S.conv(T, S x) + rlambda * x + flambda * S.Re(IFFT(FFT(S x).A))
 * (cmtip/autocorrelation/autocorrelation.py:113-173 setup_linops, :150-155 W_matvec) with
 * scipy's cg iteration (autocorrelation.py:239).  prec 32: float vectors, FP64 dots / norms /
 * alpha / beta; prec 64: all double.  op 0: Toeplitz data term on the (2M)^3 grid (the
 * reference's form); op 1: explicit fused type-2 then type-1 pair (cmt_execute_pair). */
typedef struct cmt_cg cmt_cg;

int cmt_cg_create(int M, int prec, int op, void *stream, cmt_cg **cg);

/* Toeplitz kernel: T_circ = (2M)^3 real grid (prec), FFT order, already / (2M)^3 as cmtip's
 * adjoint returns it (autocorrelation.py:141-147); stored as FFT(T_circ) / (2M)^3 (:148, :54). */
int cmt_cg_set_kernel(cmt_cg *cg, const void *t_circ);

/* mask_fft: ifftshift(gen_F_antisupport(M)) as float M^3 (autocorrelation.py:66-85, :105);
 * support: M^3 float; lambdas as in autocorrelation.py:223-225. */
int cmt_cg_set_operator(cmt_cg *cg, const float *mask_fft, const float *support, double alambda,
                        double rlambda, double flambda);

/* op 1: type-1 plan (M modes, same prec) whose points define A. */
int cmt_cg_set_pair_plan(cmt_cg *cg, cmt_plan *plan);

/* y = W x (M^3 vectors of the solver precision). */
int cmt_cg_matvec(cmt_cg *cg, const void *x, void *y);

/* x (in: x0, out: solution) after at most maxiter iterations; stops when
 * ||r|| < max(atol, rtol ||d||) (scipy semantics).  use_graph: replay a captured iteration.
 * iters / final_rho (optional, host) receive the iteration count and r.r. */
int cmt_cg_solve(cmt_cg *cg, const void *d, void *x, int maxiter, double rtol, double atol,
                 int use_graph, int *iters, double *final_rho);

/* The solves of n solvers (1..64, one precision, one device) at once: cgs[i] solves
 * W_i x_i = d_i from x_i as cmt_cg_solve does (d[i], x[i] device vectors of its precision),
 * each with its own operator, lambdas and stopping test.  One iteration of every solver is
 * captured as an independent branch of one CUDA graph, so the branches overlap on the GPU;
 * all run on the stream of cgs[0].  iters / final_rho: optional host arrays of n.  Replaces
 * the rank-parallel lambda scan of cmtip/autocorrelation/autocorrelation_mpi.py:139-155
 * (one scipy cg per MPI rank, each rank with its own rlambda / flambda). */
int cmt_cg_solve_many(int n, cmt_cg *const *cgs, const void *const *d, void *const *x, int maxiter, double rtol,
                      double atol, int *iters, double *final_rho);

int cmt_cg_destroy(cmt_cg *cg);

/* support = gaussian_filter(est, 0.5) > 1e-12 as 0/1 floats, and est *= support when
 * est_inplace (autocorrelation.py:217-220).  scratch: 2 M^3 floats. */
int cmt_support_from_estimate(float *est, int M, float *support, float *scratch, int est_inplace,
                              void *stream);

/* Largest grid edge accepted by cmt_support_from_estimate_noalloc. */
#define CMT_NOALLOC_MAX_M 128

/* cmt_support_from_estimate without the scratch argument and without any allocation, for
 * callers that cannot allocate device memory: a host whose own memory pool has reserved the
 * whole GPU (a cudaMalloc here would fail or fragment that pool), or a latency-bound caller
 * that cannot take the device-wide synchronisation a cudaMalloc / cudaFree may cause.  No
 * counterpart in the reference (cmtip computes the support on the host with scipy).  The
 * scratch is a fixed 2 * 128^3-float (16 MiB) device array that every GPU loading the
 * library keeps until the process exits; M > CMT_NOALLOC_MAX_M returns CMT_ERR_ARG.  The
 * first call on a device looks the array's device address up and caches it for that device
 * ordinal (the cache does not survive cudaDeviceReset): make that first call before any
 * stream capture.  All calls share the array, so calls that overlap on the GPU (other
 * streams, other host threads) race: order them on one stream. */
int cmt_support_from_estimate_noalloc(float *est, int M, float *support, int est_inplace, void *stream);

/* ---------------------------------------------------------------- orientation matching
 * Weighted euclidean distances between images and model slices with a fused running
 * top-k epilogue, then exact re-scoring of the candidates (cmtip/alignment/align.py:68-132:
 * std scaling :122-124, generate_weights :11-24, calc_eudist :27-36, argmin :131).
 * mode 0: BF16 operands on tcgen05 tensor cores (TMA + TMEM); 1: plain FP32; 2: plain FP64;
 * 3: BF16x3 (each operand split into two bf16 terms, hi.hi + hi.lo + lo.hi in one GEMM).
 * Both operands are centred on the mean weighted image (distances are shift invariant). */
typedef struct cmt_match cmt_match;

int cmt_match_create(int64_t n_pix, int mode, void *stream, cmt_match **match);

/* data: n_img x n_pix images (float for modes 0/1, double for 2), weights: n_pix float64.
 * The data pointer must stay valid until the last cmt_match_run. */
int cmt_match_set_data(cmt_match *match, int64_t n_img, const void *data, const double *weights);

/* model: n_ref x n_pix unscaled model slices (same type as data), split into nbatches equal
 * batches, each scaled by std(data) / std(batch).  The pointer must stay valid. */
int cmt_match_set_refs(cmt_match *match, int64_t n_ref, const void *model, int nbatches);

/* Per image: best_idx (int32), best_d / second_d (float64 distances after exact re-scoring),
 * near_tie (int32: best two within one FP32 rounding); n_near (host, optional) = count. */
int cmt_match_run(cmt_match *match, int *best_idx, double *best_d, double *second_d, int *near_tie,
                  int *n_near);

/* The tensor-core runs (modes 0 and 3) of n matchers -- one instance each, any image,
 * reference and pixel counts -- as one persistent launch per 16 matchers: their (image tile,
 * reference tile) units are concatenated and split over the SMs by cost, so small instances
 * do not leave the GPU idle; then each matcher's exact re-scoring, and one host
 * synchronisation.  Outputs per matcher as for cmt_match_run (arrays of n device pointers;
 * n_near: optional host array of n counts).  Runs on the stream of ms[0].  Replaces one
 * match_orientations call (cmtip/alignment/align.py:68-132) per reconstruction. */
int cmt_match_run_many(int n, cmt_match *const *ms, int *const *best_idx, double *const *best_d,
                       double *const *second_d, int *const *near_tie, int *n_near);

/* Tile of the tensor-core distance kernel (modes 0 / 3): references per tile bn (128 or
 * 256) and TMA ring stages (256: 3 or 4; 128: 4 or 6); default 256 x 4.  The autotuner
 * (tune.autotune_match) picks it per problem size; results do not depend on it.  No
 * counterpart in the reference. */
int cmt_match_set_tile(cmt_match *match, int bn, int stages);

/* Limit (seconds, 1e-3 .. 60; default 2) of every wait of the tensor-core pipeline.  A wait
 * that runs out unwinds the kernel (in-flight copies and MMAs drained, TMEM released) and
 * cmt_match_run returns CMT_ERR_TIMEOUT with the context still usable. */
int cmt_match_set_wait_limit(cmt_match *match, double seconds);

/* Test of that timeout path: while enabled (1) the tensor-core kernel's producer issues no
 * loads, so its consumers' waits run out; 0 restores normal runs.  No counterpart in the
 * reference. */
int cmt_match_stall_loads(cmt_match *match, int enable);

/* CUDA-event timing of a matcher's stages (enable 0/1), and read-back (ms, 4 values) of the
 * last set_data (image operands), set_refs (reference statistics and operands), distance
 * kernel and exact re-scoring.  Used by benchmarks; no counterpart in the reference. */
int cmt_match_profile(cmt_match *match, int enable);
int cmt_match_last_ms(cmt_match *match, float *ms);

/* host: the nbatches scale factors followed by std(data). */
int cmt_match_stats(cmt_match *match, double *host_out);

int cmt_match_destroy(cmt_match *match);

/* ---------------------------------------------------------------- phasing
 * Phase retrieval of an oversampled autocorrelation (cmtip/phasing/phase.py:11-219).  Arrays
 * are M^3 in C order; "FFT order" (the reference's trailing underscore) has the DC term at
 * the corner.  prec 64: density, amplitudes and transforms in double (the reference's
 * arithmetic); prec 32: float density, amplitudes and transforms, double reductions.
 * Supports and masks are uint8 (0 / nonzero), i.e. the bytes of a bool tensor.  The
 * phaser owns only its workspace (half spectrum, filter scratch, reduction partials,
 * cuFFT plans, the captured iteration graphs); every call is stream-ordered on its stream
 * with no host synchronisation. */
typedef struct cmt_phaser cmt_phaser;

int cmt_phase_create(int M, int prec, void *stream, cmt_phaser **phaser);
int cmt_phase_set_stream(cmt_phaser *phaser, void *stream);

/* phase.py:186-192: ac_filt_ = ifftshift(gaussian_filter(max(ac, 0), mode='constant')) and
 * amplitudes_ = sqrt(|fftn(ac_filt_)|) (prec).  ac: centred, double.  weights: the
 * 2 * radius + 1 normalised Gaussian taps (host), radius <= 8. */
int cmt_phase_amplitudes(cmt_phaser *phaser, const double *ac, const double *weights, int radius,
                         double *ac_filt_, void *amplitudes_);

/* create_support_ (phase.py:47-64): centred cube [Mquat, M - Mquat)^3, ifftshifted, and
 * ac_filt_ > 1e-2 * max(ac_filt_). */
int cmt_phase_create_support(cmt_phaser *phaser, const double *ac_filt_, int mquat, uint8_t *support_);

/* step_phase (phase.py:122-144): rho_mod_ = Re(ifftn(amplitude-replaced fftn(rho_))),
 * support_star_ = support_ & rho_mod_ > 0. */
int cmt_phase_step(cmt_phaser *phaser, const void *rho_, const void *amplitudes_, const uint8_t *amp_mask_,
                   const uint8_t *support_, void *rho_mod_, uint8_t *support_star_);

/* ER_loop / ER (phase.py:67-72, 83-99) and HIO_loop / HIO (:75-80, 102-119): n_loops
 * iterations updating rho_ in place.  amplitudes_ (prec) and amp_mask_ are full M^3 arrays
 * in FFT order.  rho_max: +inf for none (the reference's np.infty). */
int cmt_phase_er(cmt_phaser *phaser, void *rho_, const void *amplitudes_, const uint8_t *amp_mask_,
                 const uint8_t *support_, double rho_max, int n_loops);
int cmt_phase_hio(cmt_phaser *phaser, double beta, void *rho_, const void *amplitudes_, const uint8_t *amp_mask_,
                  const uint8_t *support_, double rho_max, int n_loops);

/* shrink_wrap (phase.py:147-162): support_ = gaussian_filter(|rho_|, mode='wrap') >
 * max|rho_| * cutoff.  weights / radius as for cmt_phase_amplitudes. */
int cmt_phase_shrink_wrap(cmt_phaser *phaser, double cutoff, const double *weights, int radius, const void *rho_,
                          uint8_t *support_);

/* center_of_mass sums (phase.py:20-22) into sums[4] (device, double): sum |rho_| hkl_a for
 * a = 0, 1, 2 and sum |rho_|.  hkl_: 3 x M^3 doubles, or NULL for recenter's grid
 * (phase.py:34-38). */
int cmt_phase_center_of_mass(cmt_phaser *phaser, const void *rho_, const double *hkl_, double *sums);

/* recenter's rolls (phase.py:41-44): np.roll(a, -s_axis, axis) on all three axes, in place,
 * for rho_ (prec) and support_ (either may be NULL). */
int cmt_phase_roll(cmt_phaser *phaser, void *rho_, uint8_t *support_, int s0, int s1, int s2);

/* phase.py:214-217: ac_phased = fftshift(|ifftn(|fftn(rho_)|^2)|), double, centred. */
int cmt_phase_autocorrelation(cmt_phaser *phaser, const void *rho_, double *ac_phased);

int cmt_phase_destroy(cmt_phaser *phaser);

/* inv(R(q)) for n float32 quaternions (w, x, y, z), skopi convention (element products
 * rounded to float32 as with float32 quaternions), into n x 3 x 3 float64. */
int cmt_inverse_rotations(const float *quat, int64_t n, double *inv_rot, void *stream);

const char *cmt_last_error(void);

/* library version string */
const char *cmt_version(void);

#ifdef __cplusplus
}
#endif

#endif /* CMTIP_GB300_H */
