/*
 * bldfm_gb300 -- C ABI of the GB300 steady-state advection-diffusion solve.
 *
 * Drop-in boundary for the reference's
 *   steady_state_transport_solver(srf_flx, z, profiles, domain, levels, modes,
 *                                 meas_pt, srf_bg_conc, footprint, analytic,
 *                                 halo, precision, cache)
 * (src/bldfm/solver.py:16-304).  The reference has no FFI: it is pure Python
 * and its callers import the function (src/bldfm/interface.py:15,115-128;
 * src/bldfm/__init__.py:3).  The Python module bldfm_gb300.solver binds these
 * entry points with ctypes and exposes the reference's signature.
 *
 * Conventions
 *  - Every entry point returns an int status (BLDFM_OK = 0 or a negative
 *    BLDFM_ERR_* code); bldfm_status_str() names it.
 *  - Arrays are C-contiguous, float64 unless stated.  Fields are row-major
 *    (ny rows of nx), level-major for 3D outputs: (nlvls, out_ny, out_nx).
 *  - "dev" pointers are CUDA device pointers on the current device; "host"
 *    pointers are ordinary host memory.  The z grid, the profiles and the
 *    level list are small (O(nz)) host arrays read during the call.
 *  - stream is a cudaStream_t passed as void* (NULL = legacy default stream).
 */
#ifndef BLDFM_GB300_H
#define BLDFM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define BLDFM_OK 0
#define BLDFM_ERR_ODD_MODES -1       /* ValueError("modes must consist of even numbers.")  solver.py:89-91 */
#define BLDFM_ERR_PRECISION -2       /* ValueError("precision must be single (default) or double.") solver.py:187-188 */
#define BLDFM_ERR_ARG -3             /* malformed descriptor / sizes / pointers */
#define BLDFM_ERR_SPECTRUM_SHAPE -4  /* truncated source spectrum does not match modes (reference raises IndexError) */
#define BLDFM_ERR_BROADCAST -5       /* analytic branch with >1 output level (reference raises ValueError) */
#define BLDFM_ERR_UNSUPPORTED -6     /* extended grid larger than the supported transform length */
#define BLDFM_ERR_WORKSPACE -7       /* workspace too small */
#define BLDFM_ERR_CUDA -8            /* a CUDA runtime call failed */
#define BLDFM_ERR_TIMEOUT -9         /* a bounded device wait ran out */
#define BLDFM_ERR_NONFINITE -10      /* non-finite values detected in the output */
#define BLDFM_ERR_PROFILE -11        /* z not strictly increasing, a non-finite z or profile value,
                                        Kz <= 0 or Kx, Ky < 0 (checked on the host before any work) */
#define BLDFM_ERR_HOST -12           /* host-side failure: memory allocation or thread start (a C++
                                        exception inside the library, caught at the entry point) */

/* ---- descriptor -------------------------------------------------------- */
#define BLDFM_PREC_SINGLE 0 /* reference precision="single": spectra stored as complex64 */
#define BLDFM_PREC_DOUBLE 1 /* reference precision="double" */

#define BLDFM_MODE_FP64 0 /* FP64 shooting sweep, rounding identical to the reference */
#define BLDFM_MODE_FP32 1 /* FP32 invariant-imbedding (Riccati) sweep, renormalised */
#define BLDFM_MODE_FP64R 2 /* FP64 invariant imbedding: the discrete solution without the
                              shooting method's cancellation (more accurate than the reference) */

typedef struct bldfm_desc {
    int32_t nx, ny;     /* srf_flx shape is (ny, nx)                          */
    int32_t nz;         /* len(z)                                             */
    int32_t nlx, nly;   /* requested Fourier modes (must be even)             */
    int32_t footprint;  /* reference footprint flag                           */
    int32_t analytic;   /* reference analytic flag                            */
    int32_t precision;  /* BLDFM_PREC_*                                       */
    int32_t mode;       /* BLDFM_MODE_*                                       */
    int32_t has_halo;   /* 0: halo = max(xmax, ymax) (reference halo=None)    */
    double xmax, ymax;  /* domain                                             */
    double halo;        /* metres, used when has_halo != 0                    */
    double meas_x, meas_y;
    double srf_bg_conc;
} bldfm_desc;

/* Sizes derived from a descriptor (solver.py:94-131, 264-290). */
typedef struct bldfm_plan_info {
    int32_t nxe, nye;       /* extended grid                        */
    int32_t nlx, nly;       /* modes after the clamp                */
    int32_t px, py;         /* halo pad in cells                    */
    int32_t nfx, nfy;       /* output transform size                */
    int32_t out_nx, out_ny; /* cropped output field                 */
    int64_t nsolved;        /* modes the sweep integrates           */
    int64_t workspace_bytes;
} bldfm_plan_info;

/* ---- entry points ------------------------------------------------------ */

/* Name of a status code. */
const char *bldfm_status_str(int status);

/* Library build string (arch, version). */
const char *bldfm_version(void);

/* Derived sizes and workspace bytes for bldfm_solve.
 * Replaces the grid arithmetic of solver.py:94-131. */
int bldfm_plan(const bldfm_desc *d, int nlvls, bldfm_plan_info *out);

/* Full solve on device buffers.  Replaces steady_state_transport_solver
 * (solver.py:16-304) for inputs already resident on the GPU.
 *   srf_flx_dev   (ny, nx) float64, ignored (may be NULL) when footprint != 0
 *   z_host        (nz,)
 *   prof_host     (5, nz): u, v, Kx, Ky, Kz  (the reference's profiles tuple)
 *   levels_host   (nlvls,) int64 indices into z
 *   conc_dev, flx_dev  (nlvls, out_ny, out_nx) float64 outputs
 *   workspace_dev bytes >= bldfm_plan().workspace_bytes, 256-byte aligned
 * Returns after the work is enqueued on stream.  In BLDFM_MODE_FP64 the
 * host computes the top eigenvalues with libm while the device sweeps. */
int bldfm_solve(const bldfm_desc *d, const double *srf_flx_dev,
                const double *z_host, const double *prof_host,
                const int64_t *levels_host, int32_t nlvls, double *conc_dev,
                double *flx_dev, void *workspace_dev, size_t workspace_bytes,
                void *stream);

/* Same solve on host buffers: copies srf_flx in and conc/flx out inside the
 * call and returns when the outputs are on the host (synchronous).  The
 * library keeps and reuses its own device and pinned buffers per device.
 * This is the entry point the reference-facing ctypes binding uses. */
int bldfm_solve_host(const bldfm_desc *d, const double *srf_flx_host,
                     const double *z_host, const double *prof_host,
                     const int64_t *levels_host, int32_t nlvls,
                     double *conc_host, double *flx_host);

/* Device evaluation of vertical_profiles (src/bldfm/pbl_model.py:8-204).
 * closure: 0 = MOST, 1 = CONSTANT, 2 = MOSTM, 3 = OAAHOC (tke <= 0 means the
 * reference's default 1.0).  For MOST/CONSTANT/MOSTM exactly one of ustar / z0
 * is > 0 (the other <= 0 means "derive it", pbl_model.py:64-77); OAAHOC needs
 * ustar.  domain_height / stretch <= 0 mean the reference's None.
 * Writes z_dev (nz) and prof_dev (5, nz): u, v, Kx, Ky, Kz.  nz_out (host)
 * receives len(z); call with z_dev == NULL to size the buffers first. */
int bldfm_vertical_profiles(int32_t n, double meas_height, double um, double vm,
                            double ustar, double z0, double mol, double prsc,
                            int32_t closure, double domain_height,
                            double stretch, double tke, int32_t *nz_out,
                            double *z_dev, double *prof_dev, void *stream);

/* Arguments of one vertical_profiles evaluation (meaning as for
 * bldfm_vertical_profiles). */
typedef struct bldfm_profile_params {
    int32_t n, closure;
    double meas_height, um, vm, ustar, z0, mol, prsc, domain_height, stretch, tke;
} bldfm_profile_params;

/* vertical_profiles for ncases parameter sets in one launch (one block per
 * case; no reference counterpart: the reference evaluates one case per call,
 * pbl_model.py:8-204).  nz_out[k] and zoff_out[k] (host) receive len(z) of
 * case k and its offset in the concatenated output; *ws_bytes_out the device
 * scratch the launch needs.  Call with z_dev == NULL to size everything.
 * Case k's z is z_dev[zoff[k] .. + nz[k]) and its five profile rows (u, v, Kx,
 * Ky, Kz, stride nz[k]) start at prof_dev + 5 zoff[k]. */
int bldfm_vertical_profiles_batch(int32_t ncases, const bldfm_profile_params *params, int32_t *nz_out,
                                  int64_t *zoff_out, size_t *ws_bytes_out, double *z_dev, double *prof_dev,
                                  void *ws_dev, size_t ws_bytes, void *stream);

/* Per-stage CUDA-event timers of bldfm_solve on the current device (no
 * counterpart in the reference, which only times whole runs with time.time,
 * runs/manuscript/low_level/comparison_analytic.py:43-49).  When enabled,
 * bldfm_stage_times() returns the mean milliseconds per stage over the
 * solves enqueued since the previous call (up to 1024): [0] forward transform,
 * [1] sweep, [2] k=0 mode / combination, [3] output transform.  It returns the
 * number of stages written and restarts the average.  Batches
 * (bldfm_solve_batch without a graph) record [0] upload and per-case forward
 * transforms, [1] the sweep, [2] the output transform, [3] the accuracy
 * check; surrogate batches [0] upload, [1] the serving kernel, [2] the exact
 * low band, [3] the accuracy guard, [4] the output transform. */
int bldfm_set_stage_timing(int enable);
int bldfm_stage_times(float *ms, int n);

/* Asynchronous copy of `bytes` between any two addresses the CUDA runtime
 * knows (cudaMemcpyDefault: device, pinned host) on `stream`.  No reference
 * counterpart: a convenience for hosts without a CUDA runtime binding (the
 * Python layer copies each batch's results and status into one pinned host
 * buffer with it). */
int bldfm_memcpy_async(void *dst, const void *src, size_t bytes, void *stream);

/* Algorithmic flops of the FP32 Riccati sweep for one solved mode (an FMA
 * counted as 2, MUL/ADD/RCP as 1) on the nz-level table of prof_host with
 * output levels levels_host: the steps above the highest output level update
 * only the ratio, the ones below also the flux product; isotropic profiles
 * (Kx == Ky, one wind direction) take the cheaper coefficient form.  The
 * numerator of the sweep roofline (no reference counterpart). */
int bldfm_sweep32_flops(int32_t nz, const double *prof_host, const int64_t *levels_host, int32_t nlvls,
                        double *flops_per_mode);

/* Measured FMA throughput of this GPU (flops/s, an FMA counted as 2): kind 0
 * scalar FP32, 1 FP64, 2 packed FP32 (f32x2 FMA, two per instruction).  The
 * pipe peak the sweep kernels are held against (no reference counterpart). */
int bldfm_fma_peak(int kind, double *flops_per_s, void *stream);

/* ---- batches ------------------------------------------------------------
 * Many cases (towers x timesteps), each with its own grid, modes, levels and
 * profiles, solved together in FP32 (BLDFM_MODE_FP32; analytic = 0).  Replaces
 * the reference's per-case loops and process pool around the solve
 * (src/bldfm/interface.py:141-326): one persistent sweep launch over every
 * (case, mode tile), one launch per transform pass, optionally replayed as a
 * CUDA graph (not on the legacy default stream). */
typedef struct bldfm_case {
    bldfm_desc desc;             /* mode must be BLDFM_MODE_FP32            */
    const double *srf_flx_dev;   /* (ny, nx) device, NULL in footprint mode */
    const double *z_host;        /* (nz)                                    */
    const double *prof_host;     /* (5, nz): u, v, Kx, Ky, Kz               */
    const int64_t *levels_host;  /* (nlvls)                                 */
    int32_t nlvls;
    int32_t pad;
    double *conc_dev, *flx_dev;  /* (nlvls, out_ny, out_nx) device outputs  */
} bldfm_case;

typedef struct bldfm_batch_opts {
    int32_t threads;     /* sweep CTA size: 128 or 256 (0: 256)            */
    int32_t ctas_per_sm; /* persistent sweep CTAs per SM (0: occupancy max) */
    int32_t use_graph;   /* capture the batch once, replay it afterwards   */
    int32_t xform_lines; /* output-transform passes: 1, 2 or 4 = shared-
                          * memory passes with that many lines per CTA
                          * (lowered to what fits the shared memory); 8 =
                          * register-resident passes where every case has
                          * the same supported line lengths; 16 or 0 = as
                          * 8, with the zoomed column pass where every
                          * case's band and kept window allow it           */
    int32_t skip_check;  /* 1: no accuracy check (the error sums from
                          * workspace byte 64 stay zero); 0: check      */
} bldfm_batch_opts;

/* Workspace bytes for a batch (256-byte aligned workspace required). */
int bldfm_batch_plan(const bldfm_case *cases, int32_t ncases,
                     const bldfm_batch_opts *opts, int64_t *workspace_bytes);

/* Enqueue a batch on stream; returns once enqueued.  The int32 at workspace
 * offset 0 holds the device status after completion.  A workspace smaller
 * than the batch needs gives BLDFM_ERR_WORKSPACE before anything is
 * enqueued, so a caller may solve first and plan only on that status.
 * Error statement (no reference counterpart): from workspace byte 64, four
 * floats per case, the weighted (sum |dXp|^2, sum |Xp|^2, sum |dXq|^2,
 * sum |Xq|^2) over the output levels of the FP32 spectra against
 * float-float (~48-bit) re-solves of a stratified sample of 32 modes (the
 * k = 0 mode, every mode with |kx|, |ky| <= 2, 19 equal slices of the mode
 * list); per field the estimated relative L2 error combines the square-root
 * ratio with the output transform's rounding, 2^-24 times
 * sqrt((sum |Xp|^2 + sum |Xq|^2) / sum |X|^2); the case's is the larger. */
int bldfm_solve_batch(const bldfm_case *cases, int32_t ncases,
                      const bldfm_batch_opts *opts, void *workspace,
                      size_t workspace_bytes, void *stream);

/* ---- surrogate building blocks ----------------------------------------- */

/* Check of the tcgen05 BF16 tensor-core GEMM the surrogate MLP runs on (no
 * reference counterpart): D (M x 256, FP32) = A (M x K) * B (256 x K)^T with
 * A, B row-major BF16 bit patterns on the host, M % 128 == 0, K % 16 == 0. */
int bldfm_tc_gemm_check(const uint16_t *A, const uint16_t *B, float *D,
                        int32_t M, int32_t K);

/* The surrogate MLP (no reference counterpart): inputs (8 features, rows of
 * 8 floats) -> 4 x 256 GELU hidden layers -> 4 outputs.  The three 256 x 256
 * layers run forward and backward on the tcgen05 tensor cores (BF16 operands,
 * FP32 accumulation in tensor memory); the last hidden layer and the output
 * layer stay FP32; FP32 master weights, Adam.  The handle owns device buffers
 * for up to `batch` samples (multiple of 256). */
int bldfm_surrogate_create(int32_t batch, uint64_t seed, void **handle);
int bldfm_surrogate_destroy(void *handle);
int bldfm_surrogate_nparams(void);
/* sample capacity of the handle */
int bldfm_surrogate_batch(void *handle);
/* get (host_out) and/or set (host_in) the FP32 parameter vector */
int bldfm_surrogate_params(void *handle, float *host_out, const float *host_in);
/* gradients and loss of the last training step */
int bldfm_surrogate_grads(void *handle, float *host_grads, float *host_loss);
/* one Adam step on n samples (device X [n][8], T [n][4], w [n][4]):
 * loss = sum w (y - t)^2 / n; lr = 0 computes the gradients only */
int bldfm_surrogate_train_step(void *handle, const float *X, const float *T,
                               const float *w, int32_t n, float lr,
                               void *stream);
/* Y [n][4] = MLP(X [n][8]), device pointers, n % 256 == 0 */
int bldfm_surrogate_forward(void *handle, const float *X, float *Y, int32_t n,
                            void *stream);

/* Footprint-weighted point measurement, replaces point_measurement
 * (src/bldfm/utils.py:80-92, np.sum(f * g)) for a batch: out[b] =
 * sum_{i < n} f[b * stride + i] * g[b * stride + i] in FP64 (Kahan-compensated,
 * deterministic order).  Device pointers; workspace of
 * bldfm_point_measurement_workspace(n, nbatch) bytes, 8-byte aligned. */
int64_t bldfm_point_measurement_workspace(int64_t n, int32_t nbatch);
int bldfm_point_measurement(const double *f_dev, const double *g_dev,
                            int64_t n, int64_t stride, int32_t nbatch,
                            double *out_dev, void *workspace_dev,
                            size_t workspace_bytes, void *stream);

/* Self-check of the failure detection (no reference counterpart): every
 * device wait of the library is bounded and reports BLDFM_ERR_TIMEOUT in the
 * status word instead of hanging or trapping.  This runs one kernel whose
 * mbarrier wait can never complete, polled `limit` times (1..2^20), and
 * returns its status in *status_host (BLDFM_ERR_TIMEOUT expected) and the
 * time the bounded wait took in *wait_ns_host. */
int bldfm_selftest_wait_timeout(int64_t limit, int32_t *status_host, int64_t *wait_ns_host);

/* Training data of the surrogate (no reference counterpart): a pool of
 * nondimensional MOST met cases (s1 = z_m / L, s2 = ln(z_m / z0)) on the
 * n-level stretched grid of vertical_profiles (src/bldfm/pbl_model.py:8-204,
 * default stretch and top), whose per-mode transfer at z_m the FP32
 * invariant-imbedding sweep evaluates on the device.  Targets per sample:
 * log|Tq| / (1 + k), arg Tq / (1 + k), log|R~|, arg R~ with Tq = q(z_m) / q(0),
 * R~ = U p(z_m) / q(z_m), k = |k| z_m. */
int bldfm_transfer_pool_create(const double *s1, const double *s2,
                               int32_t ncases, int32_t n, void **pool);
int bldfm_transfer_pool_destroy(void *pool);
/* u* / U and the level count of pool case c */
int bldfm_transfer_pool_case(void *pool, int32_t c, double *s3, int32_t *nz);
/* m random samples (case uniform, |k| log-uniform in [kmin, kmax], first
 * quadrant): X [m][8] features, T [m][4] targets, W [m][4] loss weights for
 * the footprint's relative L2 error given per-case energy reciprocals
 * norm [ncases][2] (flux, conc), or raw energies when norm is NULL;
 * cid [m] (optional) the case ids.  Device pointers. */
int bldfm_transfer_samples(void *pool, uint64_t seed, int32_t m, float kmin,
                           float kmax, const float *norm, float floor_w,
                           float *X, float *T, float *W, int32_t *cid,
                           void *stream);
/* targets of given samples (device cid [m], kpar [m], kperp [m] -> T [m][4]) */
int bldfm_transfer_eval(void *pool, const int32_t *cid, const float *kpar,
                        const float *kperp, float *T, int32_t m, void *stream);

/* Surrogate footprint solve (no reference counterpart; stands in for
 * steady_state_transport_solver, src/bldfm/solver.py:16-304, in footprint
 * mode with MOST profiles): the FP32 path with the per-mode sweep replaced
 * by the MLP's transfer at z_m, then the solver's own output transform.
 * Requires desc->mode == BLDFM_MODE_FP32, footprint, one output level at
 * z_m, Kx == Ky and one wind direction (else BLDFM_ERR_UNSUPPORTED).  The
 * caller decides whether the case lies in the network's training box. */
typedef struct bldfm_surrogate_case {
    double zm;        /* measurement height, a level of z */
    double wind;      /* wind speed at z_m */
    double s1, s2, s3; /* z_m / L, ln(z_m / z0), u* / wind */
    int32_t variant;  /* 0: fused features -> MLP -> spectra kernel;
                       * 1: transfer from the nondimensional FP32 sweep of
                       *    this case instead of the MLP (checks the serving
                       *    path; net may be NULL);
                       * 2: the MLP layer by layer (bldfm_surrogate_forward) */
    int32_t reserved;
    double exact_kz;  /* variants 0 and 2: the solved modes with |k| z_m <
                       * exact_kz (the footprint's low band, where its L2
                       * norm sits) take the exact FP32 sweep instead of the
                       * network, written over the served spectra before the
                       * output transform; 0: every mode from the network */
} bldfm_surrogate_case;
int bldfm_surrogate_plan(const bldfm_desc *d, int32_t nlvls,
                         int64_t *workspace_bytes);
/* Many surrogate footprints in one persistent launch plus the batched output
 * transform (the batch counterpart of bldfm_surrogate_solve; variant 0 only).
 * cases[k] as for bldfm_solve_batch (footprint, one level at z_m, FP32 mode),
 * mets[k] its met scalars; workspace of bldfm_surrogate_batch_plan bytes,
 * 256-byte aligned; the int32 at offset 0 holds the device status.
 * Accuracy guard: a stratified sample of each case (the k = 0 mode, the 12
 * solved modes with |kx|, |ky| <= 2, every 61st solved mode weighted 61) is
 * re-solved exactly (FP32 sweep) and compared with the served spectra; the last
 * (16 ncases + 255) & ~255 bytes of the planned workspace receive, per case,
 * four floats (sum |dXp|^2, sum |Xp|^2, sum |dXq|^2, sum |Xq|^2), an estimate
 * of the case's relative L2 error (no reference counterpart). */
int bldfm_surrogate_batch_plan(const bldfm_case *cases,
                               const bldfm_surrogate_case *mets, int32_t ncases,
                               int64_t *workspace_bytes);
int bldfm_surrogate_solve_batch(void *net, const bldfm_case *cases,
                                const bldfm_surrogate_case *mets, int32_t ncases,
                                void *workspace, size_t workspace_bytes,
                                void *stream);
int bldfm_surrogate_solve(void *net, const bldfm_desc *d,
                          const bldfm_surrogate_case *met, const double *z_host,
                          const double *prof_host, const int64_t *levels_host,
                          int32_t nlvls, double *conc_dev, double *flx_dev,
                          void *workspace_dev, size_t workspace_bytes,
                          void *stream);

/* Allocation-free FP32 solve.  No counterpart in the reference (which never
 * touches a GPU).  For callers that may not allocate device memory while they
 * solve: hosts that reserve all device memory up front and treat any later
 * cudaMalloc as a failure, and plugin hosts whose allocator policy forbids
 * cudaMalloc from libraries.  Same arguments as bldfm_solve minus the
 * workspace: every intermediate lives in one static device array of 16 MiB
 * that each GPU loading this library holds until exit.
 *  - BLDFM_MODE_FP32 only, analytic == 0, nz >= 2; larger problems return
 *    BLDFM_ERR_WORKSPACE (the 512^2 footprint with 512^2 modes needs ~7 MiB).
 *  - status_dev (device int32, may be NULL) receives the call's device
 *    status once the stream reaches the end of the call: 0, BLDFM_ERR_TIMEOUT
 *    (a bounded device wait ran out) or BLDFM_ERR_NONFINITE.
 *  - The first call on a device looks up the array's address with that
 *    device current.
 *  - Not for CUDA stream capture: each call copies its small host tables
 *    (level tables, slot map, band map) from one static pageable host buffer,
 *    which the next call rewrites; a captured graph would replay whatever
 *    that buffer holds then.  Use bldfm_solve_batch (use_graph) for graphs.
 *  - All calls share the array: calls whose GPU work overlaps race; order
 *    them on one stream.
 *  - Calls no cudaMalloc/cudaFree/cudaHostAlloc; host staging is static. */
int bldfm_solve_noalloc(const bldfm_desc *d, const double *srf_flx_dev,
                        const double *z_host, const double *prof_host,
                        const int64_t *levels_host, int32_t nlvls,
                        double *conc_dev, double *flx_dev, int32_t *status_dev,
                        void *stream);

#ifdef __cplusplus
}
#endif

#endif /* BLDFM_GB300_H */
