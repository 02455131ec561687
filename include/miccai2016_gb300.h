/*
 * miccai2016_gb300.h -- C ABI of the GB300 tubular-segmentation kernels.
 *
 * Every entry point is extern "C", takes plain pointers and sizes, returns an
 * int status (M16_OK = 0) and never throws.  Unless a comment says "host",
 * pointers are CUDA device pointers owned by the caller.  Scratch memory comes
 * from a caller-provided workspace whose size the matching *_workspace_bytes()
 * function reports; the library itself calls no allocator.  `stream` is a
 * cudaStream_t passed as void*; all work is enqueued on it.
 *
 * Volumes are C-ordered float32 arrays of shape (d0, d1, d2) with d2 the
 * fastest axis, exactly the numpy layout the reference's Python modules take.
 * Squeezed quaternions are (d0, d1, d2, 3) interleaved triples as produced by
 * the reference's qsqueeze() (src/clcode/quaternion_math.h:20-39).
 *
 * Each declaration cites the reference interface it replaces.
 */
#ifndef MICCAI2016_GB300_H
#define MICCAI2016_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define M16_OK 0
#define M16_ERR_BAD_SHAPE 1     /* a dimension is < 1, or the volume is too large */
#define M16_ERR_BAD_ARG 2       /* a NULL pointer, a non-finite or out-of-range parameter */
#define M16_ERR_WORKSPACE 3     /* workspace NULL, misaligned or smaller than required */
#define M16_ERR_CUDA 4          /* a CUDA runtime call failed */
#define M16_ERR_TIMEOUT 5       /* a bounded device-side wait gave up */
#define M16_ERR_TOO_LARGE 6     /* the request exceeds a fixed capacity: the scratch of m16_maxflow_solve_static
                                   or the work table of a server (max_work_items) */

/* Longest Gaussian derivative kernel (taps = 2 * radius + 1) the Frangi entry points take. */
#define M16_MAX_TAPS 127

/* Human-readable name of a status code (static string). */
const char *m16_status_string(int status);

/* Version of this ABI; bumped on any incompatible change. */
int m16_abi_version(void);

/* ---- continuous max-flow with anisotropic TV ------------------------------
 * Replaces CmfCutQAnisotropicGpu.CutParameters
 * (src/processing/continuous_cut_anisotropic_gpu.py:38-49).               */
typedef struct m16_cut_params {
    double cc;          /* augmented-Lagrangian step (CutParameters.cc, 0.2) */
    double steps;       /* gradient-ascent step (CutParameters.steps, 0.11) */
    double error_bound; /* stop when the residual falls below (CutParameters.error_bound) */
    int32_t num_iter;   /* maximum number of iterations (CutParameters.num_iter) */
    int32_t update;     /* check the residual every `update` iterations (>= 1) */
    double scaling[3];  /* voxel size [mm/voxel] per axis, the `scaling` argument */
} m16_cut_params;

/* Workspace bytes m16_maxflow_solve needs for a (d0, d1, d2) volume. */
size_t m16_maxflow_workspace_bytes(int32_t d0, int32_t d1, int32_t d2, const m16_cut_params *params);

/*
 * One continuous max-flow solve (paper Alg. 1.1), replacing
 * CmfCutQAnisotropicGpu.execute(img, quats, eigs, alpha, cs, ct, labels, scaling)
 * (src/processing/continuous_cut_anisotropic_gpu.py:143-344) and its kernels
 * update_p / update_u / update_tmp (src/clcode-anisotropic/update_qp.cl:150-316).
 *
 *   img        N      image; u starts as img / (max(img) + FLT_MIN)
 *   quat3      N x 3  squeezed quaternions of the anisotropy's eigenvectors
 *   sqevals3   host, 3 doubles: square roots of constant eigenvalues, or NULL
 *   sqeigs     N x 3  per-voxel square roots of the eigenvalues (when sqevals3 == NULL)
 *   alpha      N      TV weight per voxel, or NULL to use alpha_scalar everywhere
 *   cs, ct     N      source / sink capacities
 *   labels     N      uint8 seeds (1 foreground, 2 background) for the supervised
 *                     variant, or NULL for the unsupervised cut
 *   u          N      output: the relaxed labelling (not clipped to [0, 1])
 *   iterations host   output: iterations run (the reference's loop counter + 1 at a break)
 *   residuals  host   optional: the residual of every check, up to residuals_cap values;
 *                     n_residuals (host, optional) receives how many were checked
 *
 * The residual is cc * mean|div(hp) - p_s + p_t| checked before the u-update of
 * every iteration i with i % update == 0; the solve stops at the first check
 * that is NaN or below error_bound, exactly as the reference's loop does.
 * The call returns after the solve completed on `stream` (it synchronizes
 * `stream` to read the stopping state); it never synchronizes the device.
 */
int m16_maxflow_solve(const float *img, const float *quat3, const double *sqevals3,
                      const float *sqeigs, const float *alpha, float alpha_scalar,
                      const float *cs, const float *ct, const uint8_t *labels,
                      int32_t d0, int32_t d1, int32_t d2, const m16_cut_params *params,
                      float *u, int32_t *iterations, double *residuals, int32_t residuals_cap,
                      int32_t *n_residuals, void *workspace, size_t workspace_bytes, void *stream);

/* Iteration paths of the single solve: a flow launch, then a label launch
 * per iteration (DEFAULT and TWO_SWEEPS are the same path).  The values 2
 * and 3 (one launch per iteration; two iterations per launch) were measured
 * slower than the two sweeps at every volume size on sm_103a and were
 * removed: they return M16_ERR_BAD_ARG. */
#define M16_PATH_DEFAULT 0
#define M16_PATH_TWO_SWEEPS 1

/* Counters of one solve, for benchmarks and tracing. */
typedef struct m16_solve_stats {
    int32_t time_kernels;  /* in: 1 brackets every flow/label kernel launch with CUDA events */
    int32_t launches;      /* out: kernels the call launched */
    int32_t p_launches;    /* out: flow (P) kernel launches that ran */
    int32_t u_launches;    /* out: label (U) kernel launches that ran */
    double p_ms;           /* out: summed device time of the P launches (time_kernels only) */
    double u_ms;           /* out: summed device time of the U launches (time_kernels only) */
    int32_t path;          /* in: M16_PATH_* -- how an iteration is launched */
    int32_t flags;         /* in: M16_BATCH_* options of m16_batch_solve (0 elsewhere) */
    int32_t blocks_per_sm; /* out (m16_batch_solve): the sweeps' tile shape in use at the end, as the
                              target blocks per SM its z-chunk was chosen for; in, with
                              M16_BATCH_NO_TUNE: 8, 16 or 32 fixes that shape (0: the default) */
    int32_t pair_launches; /* reserved (0): kept for the layout of ABI versions 3 and 4 */
    double pair_ms;        /* reserved (0) */
    int32_t pair_zc;       /* reserved (0) */
    int32_t reserved;
} m16_solve_stats;

/* m16_solve_stats.flags: launch every iteration directly instead of replaying
 * CUDA graphs of whole check intervals (timed solves always launch directly). */
#define M16_BATCH_NO_GRAPH 1
/* m16_solve_stats.flags: use the default tile shape.  Without it the
 * sweeps' tile shape is tuned: a batch of a shape not seen before in this
 * process times the candidate shapes on its first check intervals (real
 * iterations of the solve) and keeps the fastest, later batches of that shape
 * reuse it.  Timed solves and batches too small to matter use the default. */
#define M16_BATCH_NO_TUNE 2
/* m16_solve_stats.flags: launch the single solve's sweeps in plain stream
 * order instead of with programmatic dependent launch (where each sweep's grid
 * is scheduled while the previous one drains and waits for it on the device). */
#define M16_SOLVE_NO_PDL 4

/* m16_maxflow_solve with counters; stats (host) may be NULL. */
int m16_maxflow_solve_ex(const float *img, const float *quat3, const double *sqevals3,
                         const float *sqeigs, const float *alpha, float alpha_scalar,
                         const float *cs, const float *ct, const uint8_t *labels,
                         int32_t d0, int32_t d1, int32_t d2, const m16_cut_params *params,
                         float *u, int32_t *iterations, double *residuals, int32_t residuals_cap,
                         int32_t *n_residuals, void *workspace, size_t workspace_bytes, void *stream,
                         m16_solve_stats *stats);

/*
 * m16_maxflow_solve for callers that cannot allocate device memory.
 *
 * No counterpart in the reference: it is an addition of this library.  Some
 * callers have no way to obtain device memory -- a plugin whose host owns all
 * device memory and gives it no allocator, a foreign-language binding that
 * needs a fixed footprint known at load time, a service that must not
 * allocate while serving.  This entry point takes inputs and outputs like
 * m16_maxflow_solve but no workspace: its scratch is a fixed 11 MiB array
 * inside the library that every GPU loading the library reserves until the
 * process exits.  Nothing is allocated by the call (no cudaMalloc, no
 * allocating library routine).
 *
 * Limits: at most 262,144 voxels (e.g. 64 x 64 x 64) and at most 4,096
 * residual checks (num_iter / update + 2 <= 4096); larger requests return
 * M16_ERR_TOO_LARGE before any GPU work.  Every call looks the array's
 * device address up on the calling device, so the address stays right after
 * a device reset.  With lazy module loading (the CUDA default) the array is
 * reserved when the library's max-flow module first loads on a device --
 * often this entry point's first call there -- and that call returns
 * M16_ERR_CUDA if the device has no room left for it: make one warm-up call
 * on each device before serving and before any stream capture.  All calls share the one
 * array: calls that overlap on the GPU (other streams, other host threads)
 * race and must be serialised by the caller.  The solve initialises every
 * scratch word it reads, so one call's leftovers never reach the next.
 */
int m16_maxflow_solve_static(const float *img, const float *quat3, const double *sqevals3,
                             const float *sqeigs, const float *alpha, float alpha_scalar,
                             const float *cs, const float *ct, const uint8_t *labels,
                             int32_t d0, int32_t d1, int32_t d2, const m16_cut_params *params,
                             float *u, int32_t *iterations, double *residuals, int32_t residuals_cap,
                             int32_t *n_residuals, void *stream);

/* ---- batched max-flow -------------------------------------------------------
 * Replaces the reference's one-execute()-per-grid-point loop
 * (src/phantom_experiment.py:350-368) by one batch: instances over any set of
 * volumes, each with its own (weighting, decay) or alpha field and its own
 * constant eigenvalues, advanced together and stopped one by one.          */
typedef struct m16_batch_volume {
    int32_t d0, d1, d2, reserved;
    const float *img;     /* N: u of every instance starts as img / (max(img) + FLT_MIN) */
    const float *quat3;   /* N x 3 squeezed quaternions */
    const float *grad2;   /* N: |grad img|^2 for alpha = weighting * exp(-grad2 / decay^2), or NULL */
    const float *cs;      /* N source capacities */
    const float *ct;      /* N sink capacities */
    double scaling[3];    /* voxel size [mm/voxel] */
} m16_batch_volume;

typedef struct m16_batch_instance {
    int32_t volume;       /* index into the volume array */
    int32_t reserved;
    double weighting;     /* alpha = weighting * exp(-grad2 / decay^2) (phantom_experiment.py:359) ... */
    double decay;
    const float *alpha;   /* ... unless this per-voxel alpha (N) is given */
    double sqevals[3];    /* square roots of the constant eigenvalues, e.g. ATV (1, 10^-0.75, 10^-0.75) */
    float *u;             /* N output */
} m16_batch_instance;

/* Workspace bytes of m16_batch_solve (0 when the descriptors are invalid). */
size_t m16_batch_workspace_bytes(const m16_batch_volume *vols, int32_t nvol, const m16_batch_instance *inst,
                                 int32_t ninst);

/*
 * Solve every instance as m16_maxflow_solve would (same iteration, same
 * residual and stopping rule from params; params->scaling is ignored, each
 * volume carries its own).  iterations and residuals (host, ninst each,
 * optional) receive each instance's iteration count and last residual.
 * stats (host, optional) counts launches and, with time_kernels, the summed
 * device time of the batched flow/label launches.  Synchronizes `stream`.
 */
int m16_batch_solve(const m16_batch_volume *vols, int32_t nvol, const m16_batch_instance *inst, int32_t ninst,
                    const m16_cut_params *params, int32_t *iterations, double *residuals, void *workspace,
                    size_t workspace_bytes, void *stream, m16_solve_stats *stats);

/*
 * The same batch as a sequence of steps.  m16_batch_begin prepares the batch
 * on `stream` (descriptors, set-up kernels, the default tile shape, a work
 * list over every group; nothing is synchronised) and returns a handle.
 * m16_batch_iterate enqueues `count` iterations (not past num_iter), with a
 * residual check on every iteration index that is a multiple of update, and
 * does nothing else: no synchronisation, allocation or copy, so a caller may
 * capture it into a CUDA graph.  A graph captured from a call that starts at
 * a multiple of update and runs update iterations replays one check interval.
 * Instances stop at their residual bound on the device (their lanes are
 * masked).  m16_batch_end scatters every instance's u to its output, reports
 * iterations (at the stop, else the iterations that ran) and the last
 * residuals, and frees the handle; it synchronizes `stream`.  The three calls
 * take the same stream (or the caller orders them).  The workspace
 * (m16_batch_workspace_bytes) and the inputs must stay valid until the end.
 * Graph replays are not bounded by num_iter: the caller replays at most the
 * check intervals num_iter allows.
 */
typedef struct m16_batch m16_batch;
int m16_batch_begin(const m16_batch_volume *vols, int32_t nvol, const m16_batch_instance *inst, int32_t ninst,
                    const m16_cut_params *params, void *workspace, size_t workspace_bytes, void *stream,
                    m16_batch **out);
int m16_batch_iterate(m16_batch *b, int32_t count, void *stream);
int m16_batch_end(m16_batch *b, int32_t *iterations, double *residuals, void *stream);

/* ---- serving: continuous batching of max-flow requests ----------------------
 * No reference interface: the reference solves one CmfCutQAnisotropicGpu at a
 * time.  A server owns one caller workspace; requests (each its own volume)
 * are admitted while the workspace has room, their inputs are uploaded on a
 * copy stream, and every m16_server_step advances all resident requests by
 * params->update iterations (one residual check each, at the request's own
 * iterations 0, update, 2 update, ...), so a request's iterations, residuals
 * and u are the same as those of m16_maxflow_solve on its inputs alone.  A
 * request retires at the residual bound (or NaN) or at params->num_iter; its
 * u is then copied to the request's host buffer and the memory is reused. */
typedef struct m16_server m16_server;

typedef struct m16_serve_request {
    int32_t d0, d1, d2, reserved;
    const float *img;     /* host, N: u starts as img / (max(img) + FLT_MIN) */
    const float *quat3;   /* host, N x 3 squeezed quaternions */
    const float *grad2;   /* host, N: |grad img|^2 for alpha = weighting * exp(-grad2 / decay^2) ... */
    const float *alpha;   /* ... or host, N per-voxel alpha (then grad2 is ignored) */
    const float *cs;      /* host, N source capacities */
    const float *ct;      /* host, N sink capacities */
    double scaling[3];
    double weighting, decay;
    double sqevals[3];    /* square roots of the constant eigenvalues */
    float *u;             /* host, N output, written when the request retires */
    int64_t tag;          /* caller's identifier, returned by m16_server_poll */
} m16_serve_request;

typedef struct m16_server_info {
    int32_t resident;     /* admitted and iterating */
    int32_t draining;     /* retired, u on its way to the host */
    int32_t free_slots;
    int32_t reserved;
    int64_t free_bytes;   /* workspace not held by requests */
    int64_t largest_free; /* largest request allocation that fits now */
    int64_t steps;        /* m16_server_step calls that ran iterations */
    int64_t voxel_iterations; /* iterations run by the requests, times their voxels (useful work) */
    double gpu_ms;        /* device time of the steps' kernels (CUDA events) */
} m16_server_info;

/* Workspace bytes a request of d0 x d1 x d2 voxels holds while resident. */
size_t m16_server_request_bytes(int32_t d0, int32_t d1, int32_t d2, int32_t has_alpha);

/* Workspace bytes the server keeps for its tables (the rest holds requests). */
size_t m16_server_table_bytes(int32_t max_slots, int32_t max_work_items);

/* params->num_iter must be a multiple of params->update.  workspace: device,
 * 256-byte aligned; stream: the compute stream (requests upload and download
 * on a stream of the server's own). */
int m16_server_create(const m16_cut_params *params, int32_t max_slots, int32_t max_work_items, void *workspace,
                      size_t workspace_bytes, void *stream, m16_server **out);

/* *admitted = 1 when the request got a slot and memory, else 0 (try again
 * after requests retire).  The host buffers must stay valid until the
 * request has been returned by m16_server_poll. */
int m16_server_admit(m16_server *s, const m16_serve_request *req, int32_t *admitted);

/* params->update iterations of every resident request, then retirement. */
int m16_server_step(m16_server *s);

/* Requests whose u has reached the host since the last call: tags,
 * iteration counts and last residuals (host arrays of cap entries). */
int m16_server_poll(m16_server *s, int64_t *tags, int32_t *iterations, double *residuals, int32_t cap, int32_t *n);

int m16_server_get_info(const m16_server *s, m16_server_info *info);

/* Waits for the server's work and frees its host resources. */
int m16_server_destroy(m16_server *s);

/* ---- gradient vector flow --------------------------------------------------
 * Workspace bytes of m16_gvf_run; has_response says whether a response field
 * will be passed, mags_cap bounds the convergence log (maxiter / update + 1). */
size_t m16_gvf_workspace_bytes(int32_t d0, int32_t d1, int32_t d2, int32_t has_response, int32_t mags_cap);

/*
 * Explicit GVF iterations g <- g - dt * (r (g - v) - mu * lap(g)), replacing
 * GvfGpu(vfield, params, voxel_size, response).execute()
 * (src/processing/gradient_vector_flow.py:68-253) and its kernels gvfDelta,
 * gvfUpdate, magDelta, gvfNormalize and response (src/clcode/gvf.cl:44-253).
 *
 *   v3           N x 3  the vector field (z, y, x, 3), the `vfield` argument
 *   response     N      fidelity weight, or NULL for |v|^2 (the `response` argument)
 *   voxel_size   host, 3 doubles [mm/voxel]
 *   mu, dt       GvfParameters.mu and time_step_for(voxel_size, mu, 3)
 *   first_iter   0 starts a new flow (g = 0); k > 0 continues one whose first k
 *                iterations ran in earlier calls with the same workspace
 *   n_iters      iterations to run in this call (GvfParameters.maxiter in one call)
 *   update, tol  every iteration i with i % update == 0 computes mean|delta| and
 *                stops the flow when it is below tol (tol = 0 never stops)
 *   normalize    1 normalises the returned vectors to unit length (GvfParameters.normalize)
 *   g3           N x 3  output: the current field
 *   iterations, stopped, mags, n_mags   host outputs (all optional): iterations run in
 *                total, whether tol stopped the flow, and the mean|delta| log
 * Synchronizes `stream` before returning.
 */
int m16_gvf_run(const float *v3, const float *response, int32_t d0, int32_t d1, int32_t d2,
                const double *voxel_size, double mu, double dt, int32_t first_iter, int32_t n_iters,
                int32_t update, double tol, int32_t normalize, float *g3, int32_t *iterations,
                int32_t *stopped, double *mags, int32_t mags_cap, int32_t *n_mags, void *workspace,
                size_t workspace_bytes, void *stream);

/* ---- Frangi vesselness -------------------------------------------------------
 * Taps layout (host float32): for scale s, axis a (0 = z, 1 = y, 2 = x) and
 * derivative order o in {0, 1, 2}, the 2*radius[s][a]+1 taps of the Gaussian
 * derivative kernel, already multiplied by sigma**o, start at
 * taps[((s * 3 + a) * 3 + o) * M16_MAX_TAPS].  They are the kernels of
 * GaussianFilter3D._gauss_kernel_with (src/processing/qfrangi_gpu.py:158-185).
 * radius (host int32) is nscales x 3.                                        */
size_t m16_frangi_workspace_bytes(int32_t d0, int32_t d1, int32_t d2, int32_t nscales);

/*
 * Multi-scale Frangi vesselness, replacing VesselnessCalculation.execute /
 * FeatureFilter.execute_for (src/processing/qfrangi_gpu.py:511-580, 696-753)
 * with GaussianFilter3D + Hessian (:30-271, convolve_naive.cl), Eigendecomposition
 * (qeigs.cl, eigenvalues ascending by absolute value) and VesselnessUpdate
 * (frangi.cl, max.cl).
 *   img      N        image (float32)
 *   alpha, beta       Frangi weights (VesselnessCalculation.Parameters.alpha/.beta)
 *   c        >= 0: the structureness weight; < 0: half the maximum Hessian norm
 *            of each scale, as the reference does for c = None
 *   bright   1 bright tubes on dark background, 0 dark on bright
 *   val      N        output: maximum vesselness over the scales (-inf where no
 *                     scale gave a number)
 *   quat3    N x 3    output: squeezed quaternion of the eigenvectors (columns) at
 *                     the maximising scale (0 where no scale gave a number)
 *   c_used   host, nscales floats, optional: the c of every scale
 */
int m16_frangi(const float *img, int32_t d0, int32_t d1, int32_t d2, int32_t nscales, const float *taps,
               const int32_t *radius, float alpha, float beta, float c, int32_t bright, float *val,
               float *quat3, float *c_used, void *workspace, size_t workspace_bytes, void *stream);

/* One scale's Hessian (N x 6: 00, 11, 22, 01, 02, 12), replacing
 * Hessian.execute (qfrangi_gpu.py:208-271); taps/radius of one scale as above;
 * workspace of m16_frangi_workspace_bytes(d0, d1, d2, 1). */
int m16_hessian(const float *img, int32_t d0, int32_t d1, int32_t d2, const float *taps,
                const int32_t *radius, float *h6, void *workspace, size_t workspace_bytes, void *stream);

/* Jacobi eigendecomposition of n symmetric 3x3 matrices (N x 6 in the order
 * above) into [l1, l2, l3 ascending by |l|, squeezed quaternion], replacing
 * Eigendecomposition.execute / eigs (qeigs.cl:146-256); NaN x 6 where 50
 * sweeps do not converge.  h6 and out6 may be the same buffer. */
int m16_eigs(const float *h6, int64_t n, float *out6, void *stream);

/* ---- direction sign adjustment and transformation completion ------------------ */

/* Ridge candidates of a vesselness response: 1 where resp > threshold and resp
 * exceeds its 8 trilinearly sampled neighbours in the plane of the 2nd and 3rd
 * eigenvectors (outside the volume counts -1), else 0.  Replaces RawRidgeDetector
 * (src/processing/ridge_detection.py:12-77) and detectRidges (detect_ridges.cl:34-102).
 * resp N, quat3 N x 3 squeezed quaternions, ridge N output.  d0 <= 65535. */
int m16_detect_ridges(const float *resp, const float *quat3, int32_t d0, int32_t d1, int32_t d2,
                      double threshold, float *ridge, void *stream);

/* m16_detect_ridges and m16_extract_main_directions in one pass over the
 * quaternions (their double-precision expansion is evaluated once): ridge
 * (N) and dirs3 (N x 3) as the two calls give them.  dirs3 may be quat3 (each
 * voxel reads only its own quaternion).  d0 <= 65535.  Replaces the pair
 * RawRidgeDetector.execute + AdvancedAdjuster._qeigs_to_main_dirs
 * (ridge_detection.py:45-77, adjust_directions.py:341-362). */
int m16_detect_ridges_main_directions(const float *resp, const float *quat3, int32_t d0, int32_t d1, int32_t d2,
                                      double threshold, float *ridge, float *dirs3, void *stream);

/* Main direction (first eigenvector column) of each squeezed quaternion,
 * replacing extractMainDirections (adjust_directions.cl:29-43) as used by
 * AdvancedAdjuster._qeigs_to_main_dirs (adjust_directions.py:341-362).
 * quat3 and dirs3 (n x 3) may be the same buffer. */
int m16_extract_main_directions(const float *quat3, int64_t n, float *dirs3, void *stream);

/* Completion of each vector to a right-handed orthonormal frame, converted to a
 * squeezed quaternion, replacing TransformationCompleter.complete
 * (adjust_directions.py:486-504) / completeTransformations (adjust_directions.cl:68-100).
 * dirs3 and quat3 (n x 3) may be the same buffer. */
int m16_complete_transformations(const float *dirs3, int64_t n, float *quat3, void *stream);

/* Sign of every direction flipped where its dot product with the direction of
 * the nearest ridge point (squared distance scaled by `scaling3`, ties to the
 * lowest index) is negative, in place.  Replaces
 * AdvancedAdjuster._adjust_all_directions (adjust_directions.py:419-446) /
 * adjustNonRidgeSigns (adjust_directions.cl:182-246); the ridge list is given
 * as plain device arrays (coords num_ridge x 3 uint16 in axis order 0, 1, 2;
 * rdirs num_ridge x 3 float32) instead of 8192-wide images.  scaling3 host. */
int m16_adjust_nonridge_signs(float *dirs3, int32_t d0, int32_t d1, int32_t d2, const uint16_t *coords,
                              const float *rdirs, int64_t num_ridge, const double *scaling3, void *stream);

/* Workspace bytes of m16_adjust_nonridge_signs_indexed (0 for invalid sizes). */
size_t m16_adjust_nonridge_signs_workspace_bytes(int32_t d0, int32_t d1, int32_t d2, int64_t num_ridge);

/* The same sign flips as m16_adjust_nonridge_signs -- bit for bit, the same
 * nearest ridge point with the same lowest-index tie-break -- found through a
 * cell index of the ridge points built in the workspace, so the cost grows
 * with the points near each voxel instead of with N x num_ridge.  Replaces the
 * same reference interface (adjust_directions.py:419-446,
 * adjust_directions.cl:182-246).  d0 <= 65535, num_ridge <= 2^31 - 1;
 * coordinates beyond the volume are allowed. */
int m16_adjust_nonridge_signs_indexed(float *dirs3, int32_t d0, int32_t d1, int32_t d2, const uint16_t *coords,
                                      const float *rdirs, int64_t num_ridge, const double *scaling3,
                                      void *workspace, size_t workspace_bytes, void *stream);

/* ---- ridge minimum spanning tree, local phase --------------------------------- */

/* Workspace bytes of m16_ridge_mst_local (0 for invalid sizes). */
size_t m16_ridge_mst_workspace_bytes(int64_t num_points, const int32_t *box_dims3, int32_t n_offsets);

/*
 * The local phase of the ridge-point minimum spanning tree that replaces
 * minimum_spanning_tree(squareform(pdist(...))) of
 * AdvancedAdjuster._adjust_ridge_directions (adjust_directions.py:374-379):
 * the minimum spanning forest, in the total order (weight, i, j) of edges
 * (i < j), of the candidate edges between points whose offset is one of
 * `offsets3` (n_offsets x 3, each lexicographically positive, host) and whose
 * float64 length is <= r.  Lengths are computed as
 * sqrt((d0 d0 + d1 d1) + d2 d2) with d = p_i * voxel_size - p_j * voxel_size,
 * every step rounded, as numpy computes them.  Boruvka rounds on the device;
 * the forest is unique, so the edges are exactly those of Kruskal's algorithm
 * in that order.
 *   pts3        num_points x 3 int32 (device), distinct points inside the box
 *   box_lo3, box_dims3   host: the box holding every point
 *   voxel_size3 host
 *   edges       device, 2 x (num_points - 1) int32 (output pairs i < j)
 *   n_edges     host: number of edges written
 * Points outside the box or two points on one cell return M16_ERR_BAD_ARG.
 * Synchronizes `stream`.
 */
int m16_ridge_mst_local(const int32_t *pts3, int64_t num_points, const int32_t *box_lo3, const int32_t *box_dims3,
                        const double *voxel_size3, const int32_t *offsets3, int32_t n_offsets, double r,
                        int32_t *edges, int64_t *n_edges, void *workspace, size_t workspace_bytes, void *stream);

/*
 * Host function (no device work): the signs of the ridge directions along the
 * tree of AdvancedAdjuster._adjust_ridge_directions (adjust_directions.py:382-415).
 * order (host, n_order entries): the points in visiting order, each parent
 * before its children; pred (host, n): each point's parent in that visit;
 * e (host, n): per point the sign of np.dot(its direction, its parent's
 * unadjusted direction): 1, -1, 0 (zero: keeps its direction, as does a
 * restart point such as the root) or 2 (NaN: negated).  s (host, n int8):
 * output, the final sign of every visited point: 1 where e is 0, -1 where e
 * is 2, else the parent's sign times e.
 */
int m16_compose_signs(int64_t n, const int32_t *order, int64_t n_order, const int32_t *pred, const int8_t *e,
                      int8_t *s);

/*
 * Host function (no device work): per segment label l (0 .. num_labels - 1)
 * the sums over the points with point_label[i] == l (host int32,
 * num_points) of dirs3[i][k] * voxel_size3[k] (dirs3 host float32,
 * num_points x 3), taken in point order and in double, each product rounded
 * before it is added; sums3 (host, num_labels x 3 doubles) is overwritten.
 * The per-segment summed directions that the ridge cleaning of
 * AdvancedAdjuster._do_clean_ridge (adjust_directions.py:319-337) ranks its
 * segments by, with np.bincount's order and rounding.  A label outside
 * 0 .. num_labels - 1 returns M16_ERR_BAD_ARG.
 */
int m16_segment_direction_sums(const int32_t *point_label, const float *dirs3, int64_t num_points,
                               const double *voxel_size3, int32_t num_labels, double *sums3);

/*
 * Host function (no device work): the visiting order of that propagation over
 * an undirected forest of n points (n_edges edges ea[k] -- eb[k], host):
 * breadth first from `root`, then every other tree from its lowest-index
 * point, as the reference hangs the rest of a forest off the root.  order
 * (host, n): every point once, parents before children; pred (host, n): each
 * point's parent, -1 for the root and the other trees' first points.
 */
int m16_tree_order(int64_t n, const int32_t *ea, const int32_t *eb, int64_t n_edges, int32_t root, int32_t *order,
                   int32_t *pred);

/*
 * The same propagation on the device, in two calls.  Replaces the visit of
 * AdvancedAdjuster._adjust_ridge_directions (src/processing/adjust_directions.py:382-415)
 * from root point 0; every other tree of a forest starts at its lowest-index
 * point.
 *
 * m16_ridge_edge_codes: per edge (edges_a[k] -- edges_b[k], device int32,
 * num_edges < num_points) the sign code of the float32 dot product of the two
 * points' directions (dirs3: device float32, num_points x 3): 1, -1, 0, 2
 * (NaN), 3 where the float32 rounding of the dot could decide the sign (the
 * caller evaluates those with the reference's own np.dot and writes 1, -1 or
 * 0), 4 for an endpoint outside [0, num_points).  codes: device int8.
 */
int m16_ridge_edge_codes(const float *dirs3, int64_t num_points, const int32_t *edges_a, const int32_t *edges_b,
                         int64_t num_edges, int8_t *codes, void *stream);

/* Workspace bytes of m16_ridge_signs (0 for invalid sizes). */
size_t m16_ridge_signs_workspace_bytes(int64_t num_points, int64_t num_edges);

/*
 * m16_ridge_signs: the final sign (device int8, num_points) of every point's
 * direction, from the edges of a forest and their codes (each 1, -1, 0 or 2;
 * anything else returns M16_ERR_BAD_ARG): a parity union-find over the 1 / -1
 * edges on the device, the pieces between zero and NaN edges ordered on the
 * host.  Equal to m16_tree_order + m16_compose_signs from root 0.
 * Synchronizes `stream`.
 */
int m16_ridge_signs(int64_t num_points, const int32_t *edges_a, const int32_t *edges_b, const int8_t *codes,
                    int64_t num_edges, int8_t *signs, void *workspace, size_t workspace_bytes, void *stream);

/* Workspace bytes of m16_ridge_forest_joins (0 for invalid sizes). */
size_t m16_ridge_forest_joins_workspace_bytes(int64_t num_points);

/*
 * The global phase of the ridge-point tree on the device for unit voxel size:
 * the edges that join the trees of a forest (its local phase, from
 * m16_ridge_mst_local) the way Kruskal over all pairs in (weight, i, j)
 * order joins them -- the tree of minimum_spanning_tree(squareform(pdist(...)))
 * in AdvancedAdjuster._adjust_ridge_directions (src/processing/adjust_directions.py:374-379).
 * pts3: device int32 num_points x 3, coordinates in [0, 32767]; edges_a,
 * edges_b: device int32, the forest.  The least point pair of every two trees
 * is found exactly (integer squared distances, ties to the lowest indices);
 * the search compares every tree's points with those of the trees ranked
 * below it by size, and returns M16_ERR_TOO_LARGE, writing nothing, when that
 * takes more than max_pair_evaluations distance evaluations.  join_a, join_b
 * (host int32, capacity num_points - 1), *num_joins (host): the joining
 * edges, the lower index first.  Synchronizes `stream`.
 */
int m16_ridge_forest_joins(const int32_t *pts3, int64_t num_points, const int32_t *edges_a, const int32_t *edges_b,
                           int64_t num_edges, int64_t max_pair_evaluations, int32_t *join_a, int32_t *join_b,
                           int64_t *num_joins, void *workspace, size_t workspace_bytes, void *stream);

/* ---- 26-connected labelling ------------------------------------------------------ */

/* Workspace bytes of m16_label26 (0 for invalid sizes). */
size_t m16_label26_workspace_bytes(int32_t d0, int32_t d1, int32_t d2);

/*
 * Connected components of a binary volume (mask: uint8, nonzero = foreground)
 * under 26-connectivity, numbered 1, 2, ... in the raster order of each
 * component's first voxel and 0 on the background -- exactly the labels and
 * count of scipy.ndimage.label(mask, structure=np.ones((3, 3, 3))), which the
 * sign adjustment runs for its hysteresis (ridge_detection.py:80-131) and its
 * ridge cleaning (adjust_directions.py:290-339).  d0 * d1 * d2 < 2^31.
 * labels: int32 (device); n_labels: host.  Synchronizes `stream`.
 */
int m16_label26(const uint8_t *mask, int32_t d0, int32_t d1, int32_t d2, int32_t *labels, int32_t *n_labels,
                void *workspace, size_t workspace_bytes, void *stream);

/* Workspace bytes of m16_label (the same as m16_label26's). */
size_t m16_label_workspace_bytes(int32_t d0, int32_t d1, int32_t d2);

/*
 * m16_label26 with a choice of connectivity: 26 (a 3 x 3 x 3 structure of
 * ones) or 6 (scipy.ndimage.label's default cross).  The same numbering as
 * scipy.ndimage.label with that structure.  Synchronizes `stream`.
 */
int m16_label(const uint8_t *mask, int32_t d0, int32_t d1, int32_t d2, int32_t connectivity, int32_t *labels,
              int32_t *n_labels, void *workspace, size_t workspace_bytes, void *stream);

/* Workspace bytes of m16_hysteresis (0 for invalid sizes). */
size_t m16_hysteresis_workspace_bytes(int32_t d0, int32_t d1, int32_t d2);

/*
 * The hysteresis of the sign adjustment (ridge_detection.py:80-131): out = the
 * voxels of the 26-connected components of (cand | sure) that hold a sure
 * voxel -- the union of the reference's flood fills from every sure voxel.
 * cand, sure, out: uint8 (device), nonzero = set.  Synchronizes `stream`.
 */
int m16_hysteresis(const uint8_t *cand, const uint8_t *sure, int32_t d0, int32_t d1, int32_t d2, uint8_t *out,
                   void *workspace, size_t workspace_bytes, void *stream);

/* ---- Dice of the largest connected component ---------------------------------------- */

/* Workspace bytes of m16_dice_largest (0 for invalid sizes). */
size_t m16_dice_largest_workspace_bytes(int32_t d0, int32_t d1, int32_t d2);

/*
 * The experiment's Dice (phantom_experiment.py:52-103, select_largest and
 * dice_for): seg >= threshold, its 6-connected components, the largest one
 * (the lowest label among equal sizes), then 2 |largest & truth| /
 * (|largest| + |truth|) in double.  seg: float32 (device); truth: uint8
 * (device), nonzero = inside.  dice, largest_size, n_components: host
 * (largest_size and n_components may be NULL).  With no foreground the Dice
 * is 0 and largest_size 0 (the reference fails there).  d0 * d1 * d2 < 2^31 - 1.
 * Synchronizes `stream`.
 */
int m16_dice_largest(const float *seg, const uint8_t *truth, int32_t d0, int32_t d1, int32_t d2, float threshold,
                     double *dice, int64_t *largest_size, int32_t *n_components, void *workspace,
                     size_t workspace_bytes, void *stream);

/* ---- per-volume cut inputs and scoring --------------------------------------- */

/*
 * Source / sink capacities and |grad img|^2 of a volume, replacing the
 * experiment's host steps PhantomExperiment._calculate_bgfg_weights_for
 * (src/phantom_experiment.py:280-301) and
 * np.linalg.norm(np.gradient(img), axis=0) ** 2 (:345).  Evaluated in float64
 * in the host code's operation order and rounded to float32:
 *   r  = log((normpdf(img, 1, s^2) + eps) / (normpdf(img, 0, s^2) + eps))
 *   cs = rq * max(r, 0)   (the foreground weights, the cut's source capacities)
 *   ct = rq * max(-r, 0)  (the background weights, the sink capacities)
 * with s = noise_level and rq = 1 / log((1 / sqrt(2 pi s^2) + eps) / eps);
 * grad2 uses central differences inside and one-sided ones at the ends of
 * each axis (every axis needs >= 2 voxels).  Any of cs, ct, grad2 may be NULL.
 * d0 <= 65535.
 */
int m16_capacities(const float *img, int32_t d0, int32_t d1, int32_t d2, double noise_level, double eps, float *cs,
                   float *ct, float *grad2, void *stream);

/* Workspace bytes of m16_fast_dice for ninst segmentations. */
size_t m16_fast_dice_workspace_bytes(int32_t ninst);

/*
 * Fast Dice of ninst segmentations against one ground truth, replacing
 * fast_dice_for (src/phantom_experiment.py:38-49):
 * 2 sum((u >= 0.5) * truth) / (sum(u >= 0.5) + sum(truth)), sums in float64.
 *   u       host array of ninst device pointers, each to n floats
 *   truth   n floats (0 / 1, or any weights as in the reference)
 *   dice    host, ninst doubles (output)
 * Synchronizes `stream`.
 */
int m16_fast_dice(const float *const *u, int32_t ninst, int64_t n, const float *truth, double *dice, void *workspace,
                  size_t workspace_bytes, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* MICCAI2016_GB300_H */
