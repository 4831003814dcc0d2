/*
 * sssi_gb300.h -- C ABI of libsssi_gb300, a GB300 (sm_103a) implementation of
 * SSSI's finite-difference time-domain core: acoustic propagation with a
 * convolutional perfectly matched layer (CPML) and with a sponge boundary,
 * elastic propagation with a simplified PML, the stand-alone staggered
 * derivative, and the reverse-time-migration imaging condition.
 *
 * Conventions shared by every entry point
 *   - Arrays are column-major (MATLAB order) double precision unless stated:
 *     v[z + x*nz], source[z + x*nz + t*nz*nx], data[x + t*nx],
 *     snapshot[z + x*nz + t*nz*nx]; 3D adds y after x.
 *   - nz, nx (, ny) are the sizes of the model handed over, i.e. already padded
 *     by extBoundary (src/extBoundary.m:22-39): nBoundary damping cells on the
 *     bottom, left and right (and front/rear); the top is a free surface.
 *   - Pointers may be host memory or device memory of the current CUDA device;
 *     the library detects which.  Host inputs are copied in and host outputs
 *     copied back inside the call.  Optional outputs may be NULL.
 *   - Every function returns SSSI_OK (0) or an SSSI_ERR_* code;
 *     sssi_last_error() gives the message of the calling thread's last failure.
 *   - Calls are synchronous: outputs are complete when the call returns.
 */
#ifndef SSSI_GB300_H
#define SSSI_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define SSSI_OK 0
#define SSSI_ERR_ARG 1      /* invalid argument (sizes, orders, pointers) */
#define SSSI_ERR_CUDA 2     /* CUDA runtime error, or no usable GPU */
#define SSSI_ERR_NOMEM 3    /* device or host allocation failed */
#define SSSI_ERR_UNSTABLE 4 /* the wavefield became non-finite (CFL violated) */
#define SSSI_ERR_BUSY 5     /* admission refused: not enough device memory now */
#define SSSI_ERR_INTERNAL 6  /* e.g. a step's tile copy did not arrive within the wait limit */
#define SSSI_ERR_CANCELLED 7 /* the shot was cancelled (sssi_cancel) */

/* ---- arithmetic modes ---- */
/* FP64 with the reference's rounding sequence (no fused multiply-add,
 * c_k*(a-b)/d per term): results are bit-identical to the reference C
 * gateways compiled without contraction. */
#define SSSI_MODE_FP64_STRICT 0
/* FP64 with folded coefficients w_k = c_k/d and fused multiply-adds:
 * same algorithm, rounding differs from the reference at the 1e-16 level. */
#define SSSI_MODE_FP64 1
/* FP32 wavefield, FP64 CPML memory variables and FP64 imaging sums. */
#define SSSI_MODE_FP32 2

/* Message of the calling thread's last failure ("" after a success). */
const char *sssi_last_error(void);

/* Library version as 10000*major + 100*minor + patch. */
int sssi_version(void);

/* Number of CUDA kernels this library has launched so far in this process. */
int64_t sssi_launch_count(void);

/* Releases device and pinned host buffers cached between calls. */
int sssi_release_cache(void);

/* Stream the library launches on (a cudaStream_t; NULL = legacy default). */
int sssi_set_stream(void *stream);

/* Phase timing with CUDA events on the launching stream.  When enabled, each
 * propagation call records an event at every phase boundary (RTM shot:
 * forward modelling of both models, reverse propagation with imaging, image
 * finish; forward/reverse calls: one propagation phase).  After the call,
 * sssi_last_timing reports each phase's device time in milliseconds and the
 * number of kernels launched in it. */
int sssi_enable_timing(int on);
int sssi_last_timing(double *phase_ms, int64_t *phase_launches, int max_phases, int *n_phases);

/* No counterpart in the reference: a measurement helper.  FP64 fused
 * multiply-adds per second this GPU sustains (eight independent chains per
 * thread, every SM busy); the FP64 stencil kernels are bound by this rate. */
int sssi_measure_fp64_rate(double *fma_per_s);

/* ---- host-side building blocks ---- */

/* Staggered-grid first-derivative coefficients of half-order `order`
 * (1..8): solves A c = e1 with A_ij = (2j-1)^(2i-1) by LU with partial
 * pivoting.  Replaces dCoef(order, "s"), src/fd_cmex/finiteDifference.c:24-82,
 * which calls MATLAB's mldivide. */
int sssi_dCoef(int order, double *coeff);

/* CPML damping d = -(3v)/(2L) * ln(1e-6) * (u/L)^2 for `count` cells.
 * Replaces dampPml, src/fd_cmex/finiteDifference.c:253-280. */
int sssi_dampPml(const double *u, const double *v, int64_t count, double L, double *d);

/* Staggered first derivative of a column-major 2D (ndims = 2) or 3D array
 * (dims[0..ndims-1]) along dimension dim (1-based):
 *     out(m) = sum_k coeff[k] * (data(m + order + k) - data(m + order - 1 - k)) / dist
 * for k = 0..order-1, where m runs over the output, whose size along dim is
 * dims[dim-1] - (2*order - 1) (the other sizes unchanged).  data / out may be
 * host or device memory.  SSSI_MODE_FP64_STRICT rounds as the reference
 * (bit-identical results); SSSI_MODE_FP64 folds coeff/dist and fuses.
 * Replaces diffOperator_mex, src/fd_cmex/diffOperator_mex.c:29-213. */
int sssi_diffOperator(const double *data, int ndims, const int64_t *dims, const double *coeff, int order, double dist,
                      int dim, double *out, int mode);

/* ---- drop-in propagators (the MEX gateways' work, plain pointers) ---- */

/* 2D forward modelling.  v: nz x nx; source: nz x nx x nt (dense, as the
 * MEX takes it); outputs data: nx x nt (top interior row of every step),
 * snapshot: nz x nx x nt (interior of every step), either may be NULL.
 * Replaces fwdTimeCpmlFor2dAw_mex, src/fd_cmex/fwdTimeCpmlFor2dAw_mex.c:39-290. */
int sssi_fwdTimeCpmlFor2dAw(const double *v, const double *source, int64_t nz, int64_t nx, int64_t nt,
                            int nDiffOrder, int nBoundary, double dz, double dx, double dt, double *data,
                            double *snapshot, int mode);

/* 2D reverse propagation: data (nx x nt) injected on the top interior row
 * with time running nt-1..0.  model: (nz+2l) x (nx+2l), l = 2*nDiffOrder-1,
 * the padded wavefield one step before the last one computed (as the
 * reference returns it); snapshot: nz x nx x nt.
 * Replaces rvsTimeCpmlFor2dAw_mex, src/fd_cmex/rvsTimeCpmlFor2dAw_mex.c:38-287. */
int sssi_rvsTimeCpmlFor2dAw(const double *v, const double *data, int64_t nz, int64_t nx, int64_t nt,
                            int nDiffOrder, int nBoundary, double dz, double dx, double dt, double *model,
                            double *snapshot, int mode);

/* ---- native forms (sparse sources, fused imaging) ---- */

/* 2D forward modelling with point sources: source s sits at interior cell
 * (src_iz[s], src_ix[s]) with amplitude wavelets[s*nt + t] at step t.
 * data / snapshot as sssi_fwdTimeCpmlFor2dAw (either may be NULL). */
int sssi_fwdTimeCpmlFor2dAwPoint(const double *v, int64_t nz, int64_t nx, int64_t nt, int nDiffOrder,
                                  int nBoundary, double dz, double dx, double dt, int nsrc,
                                  const int64_t *src_iz, const int64_t *src_ix, const double *wavelets,
                                  double *data, double *snapshot, int mode);

/* 3D forward modelling: [data, snapshot] = fwdTimeCpmlFor3dAw(v, source,
 * nDiffOrder, nBoundary, dz, dx, dy, dt) of src/fwdTimeCpmlFor3dAw.m:1-163
 * (MATLAB only in the reference; this is the MEX it would call).
 * v: nz x nx x ny; source: nz x nx x ny x nt (may be NULL: no source);
 * data: nx x ny x nt, the top interior face after each step (NULL: not
 * returned); snapshot: nz x nx x ny x nt (NULL: not returned).  Damping as
 * that file computes it: profiles in cell units, x and z profiles from the
 * y = 0 slice of v, y profiles from its top row (src/fwdTimeCpmlFor3dAw.m:45-70).
 * SSSI_MODE_FP64_STRICT runs as SSSI_MODE_FP64 (there is no C reference to
 * reproduce bit for bit). */
int sssi_fwdTimeCpmlFor3dAw(const double *v, const double *source, int64_t nz, int64_t nx, int64_t ny,
                            int64_t nt, int nDiffOrder, int nBoundary, double dz, double dx, double dy,
                            double dt, double *data, double *snapshot, int mode);

/* The same with nsrc (<= 8) point sources instead of the dense source volume:
 * wavelets is nsrc x nt (row s at wavelets + s * nt); source s adds
 * wavelets[s * nt + t] at interior cell (src_iz[s], src_ix[s], src_iy[s]) in step t. */
int sssi_fwdTimeCpmlFor3dAwPoint(const double *v, int64_t nz, int64_t nx, int64_t ny, int64_t nt,
                                 int nDiffOrder, int nBoundary, double dz, double dx, double dy, double dt,
                                 int nsrc, const int64_t *src_iz, const int64_t *src_ix, const int64_t *src_iy,
                                 const double *wavelets, double *data, double *snapshot, int mode);

/* One reverse-time-migration shot, the work of
 * applications/rtm_2d_acoustic/mainRtmTimeCpmlFor2dAw.m:156-166,252-275,315
 * done on the device: forward modelling of the point source in v (true
 * model) and vs (migration model), reverse propagation of
 * dataTrue - dataSmooth in v, and the zero-lag imaging condition
 *     image = M ./ s2,  M = sum_t f_t .* r_t,  s2 = epsilon + sum_t f_t.^2
 * with f the forward field in vs and r the reverse field.
 * SSSI_MODE_FP64_STRICT / SSSI_MODE_FP64 keep every forward snapshot in FP64
 * and image every step.  SSSI_MODE_FP32 stores the forward field every
 * `snap_stride` steps in FP16 with one power-of-two scale per snapshot and
 * images those steps (sums scaled by snap_stride), with FP64 accumulators.
 * image: nz x nx; data_true / data_smooth: nx x nt (may be NULL). */
int sssi_rtmTimeCpmlFor2dAw(const double *v, const double *vs, int64_t nz, int64_t nx, int64_t nt,
                            int nDiffOrder, int nBoundary, double dz, double dx, double dt,
                            const double *wavelet, int64_t src_iz, int64_t src_ix, double epsilon, int mode,
                            int snap_stride, double *image, double *data_true, double *data_smooth);

/* ---- sponge absorbing boundary (second-order five-point propagator) ----
 *
 * The MATLAB propagators src/fwdTimeSpongeFor2dAw.m and
 * src/rvsTimeSpongeFor2dAw.m (and the RTM shot of
 * applications/rtm_2d_acoustic/mainRtmTimeSpongeFor2dAw.m) on the device:
 * zero-bordered field, fdm3 = b.*p - past + ax.*(right+left) + az.*(down+up)
 * - vdtSq.*source, then the sponge factors
 * boundary(k) = exp(-(0.015 (nB-k+1))^2)^10 on the new past and present
 * (left/right columns above the bottom band, bottom rows across).  Note the
 * minus sign on the source term, as in the reference.
 * SSSI_MODE_FP64_STRICT rounds as the MATLAB expressions are written (no fused
 * multiply-add); SSSI_MODE_FP64 fuses; SSSI_MODE_FP32 keeps the field in FP32.
 * nBoundary must be in 0..min(nz, nx). */

/* [data, snapshot] = fwdTimeSpongeFor2dAw(v, source, nBoundary, dz, dx, dt):
 * v nz x nx, source nz x nx x nt, data nx x nt (row 0 after every step),
 * snapshot nz x nx x nt (either output may be NULL).
 * Replaces src/fwdTimeSpongeFor2dAw.m:1-101. */
int sssi_fwdTimeSpongeFor2dAw(const double *v, const double *source, int64_t nz, int64_t nx, int64_t nt,
                              int nBoundary, double dz, double dx, double dt, double *data, double *snapshot,
                              int mode);

/* The same with nsrc (<= 64) point sources: cell (src_iz[s], src_ix[s]) takes
 * wavelets[s*nt + t] at step t (sources on one cell add up). */
int sssi_fwdTimeSpongeFor2dAwPoint(const double *v, int64_t nz, int64_t nx, int64_t nt, int nBoundary, double dz,
                                   double dx, double dt, int nsrc, const int64_t *src_iz, const int64_t *src_ix,
                                   const double *wavelets, double *data, double *snapshot, int mode);

/* [model, snapshot] = rvsTimeSpongeFor2dAw(v, data, nBoundary, dz, dx, dt):
 * data nx x nt enters row 0 with time running nt-1..0; snapshot nz x nx x nt;
 * model nz x nx is the field after the last step (t = 0) -- the reference
 * declares this output but never assigns it.
 * Replaces src/rvsTimeSpongeFor2dAw.m:1-103. */
int sssi_rvsTimeSpongeFor2dAw(const double *v, const double *data, int64_t nz, int64_t nx, int64_t nt,
                              int nBoundary, double dz, double dx, double dt, double *model, double *snapshot,
                              int mode);

/* One sponge RTM shot (mainRtmTimeSpongeFor2dAw.m:160-161,247-268,310):
 * forward modelling of the point source in v and vs, reverse propagation of
 * dataTrue - dataSmooth in v, image = M ./ s2 with M = sum_t f_t .* r_t,
 * s2 = epsilon + sum_t f_t.^2 (f: forward field in vs).  FP64 modes only:
 * strict keeps both snapshot volumes and sums in the reference's order;
 * SSSI_MODE_FP64 accumulates inside the reverse step. */
int sssi_rtmTimeSpongeFor2dAw(const double *v, const double *vs, int64_t nz, int64_t nx, int64_t nt, int nBoundary,
                              double dz, double dx, double dt, const double *wavelet, int64_t src_iz, int64_t src_ix,
                              double epsilon, int mode, double *image, double *data_true, double *data_smooth);

/* ---- 2D elastic propagation (simplified PML) ----
 *
 * [snapshotVzp, snapshotVxp, snapshotVzs, snapshotVxs] =
 *     fwdTimeSpmlFor2dEw(vp, vs, source, nDiffOrder, nBoundary, dz, dx, dt)
 * of src/fwdTimeSpmlFor2dEw.m:1-103 (MATLAB only in the reference): the
 * velocity split into P and S parts through two potentials, staggered
 * derivatives of half-order nDiffOrder (diffOperator), damping from dampPml in
 * cell units on the side columns (x) and bottom rows (z), the source added to
 * both P components.  vp, vs: nz x nx; source: nz x nx x nt; each snapshot
 * nz x nx x nt (any may be NULL).  nBoundary must be in 0..min(nz, nx/2).
 * SSSI_MODE_FP64_STRICT rounds as the MATLAB file and diffOperator_mex do;
 * SSSI_MODE_FP64 folds c_k/d and fuses; SSSI_MODE_FP32 is the fused form in FP32. */
int sssi_fwdTimeSpmlFor2dEw(const double *vp, const double *vs, const double *source, int64_t nz, int64_t nx,
                            int64_t nt, int nDiffOrder, int nBoundary, double dz, double dx, double dt,
                            double *snapshotVzp, double *snapshotVxp, double *snapshotVzs, double *snapshotVxs,
                            int mode);

/* The same with nsrc (<= 64) point sources: cell (src_iz[s], src_ix[s]) takes
 * wavelets[s*nt + t] at step t (sources on one cell add up). */
int sssi_fwdTimeSpmlFor2dEwPoint(const double *vp, const double *vs, int64_t nz, int64_t nx, int64_t nt,
                                 int nDiffOrder, int nBoundary, double dz, double dx, double dt, int nsrc,
                                 const int64_t *src_iz, const int64_t *src_ix, const double *wavelets,
                                 double *snapshotVzp, double *snapshotVxp, double *snapshotVzs, double *snapshotVxs,
                                 int mode);

/* [snapshotVzp, snapshotVxp, snapshotVyp, snapshotVzs, snapshotVxs, snapshotVys] =
 *     fwdTimeSpmlFor3dEw(vp, vs, source_x, source_y, source_z, nDiffOrder, nBoundary, dz, dx, dy, dt)
 * of src/fwdTimeSpmlFor3dEw.m:1-236 (MATLAB only in the reference): the 3D
 * form of the above, damping profiles as that file takes them (x and z from
 * the y = 1 slice of vp, y from its top row).  vp, vs: nz x nx x ny; each
 * source nz x nx x ny x nt (NULL: none); each snapshot nz x nx x ny x nt (NULL:
 * not returned).  nBoundary must be in 0..min(nz, nx/2, ny/2). */
int sssi_fwdTimeSpmlFor3dEw(const double *vp, const double *vs, const double *source_x, const double *source_y,
                            const double *source_z, int64_t nz, int64_t nx, int64_t ny, int64_t nt, int nDiffOrder,
                            int nBoundary, double dz, double dx, double dy, double dt, double *snapshotVzp,
                            double *snapshotVxp, double *snapshotVyp, double *snapshotVzs, double *snapshotVxs,
                            double *snapshotVys, int mode);

/* The same with nsrc (<= 64) point sources: cell (src_iz[s], src_ix[s],
 * src_iy[s]) takes wavelets[s*nt + t] into the component src_component[s]
 * (0: x, 1: y, 2: z) at step t. */
int sssi_fwdTimeSpmlFor3dEwPoint(const double *vp, const double *vs, int64_t nz, int64_t nx, int64_t ny, int64_t nt,
                                 int nDiffOrder, int nBoundary, double dz, double dx, double dy, double dt, int nsrc,
                                 const int64_t *src_iz, const int64_t *src_ix, const int64_t *src_iy,
                                 const int *src_component, const double *wavelets, double *snapshotVzp,
                                 double *snapshotVxp, double *snapshotVyp, double *snapshotVzs, double *snapshotVxs,
                                 double *snapshotVys, int mode);

/* ---- MAT-file persistence ----
 *
 * The applications save seismograms, snapshots and images with MATLAB's
 * save and read them back with load
 * (applications/rtm_2d_acoustic/mainRtmTimeCpmlFor2dAw.m:170-183,250-266,348-351).
 * These write and read Level-5 MAT-files (what save(..., '-v6') writes and
 * every MATLAB load reads): real double arrays of 1 to 8 dimensions, each at
 * most 4 GiB, streamed from / to host or device memory through a bounded
 * staging buffer.  Compressed (v7) and HDF5 (v7.3) files are refused with a
 * message. */

/* Writes nvars variables to path (created or truncated): variable v is
 * names[v] (1..63 characters), arrays[v] (column-major doubles, host or device)
 * of ndims[v] dimensions dims[v][0..ndims[v]-1]. */
int sssi_mat_write(const char *path, int nvars, const char *const *names, const double *const *arrays,
                   const int *ndims, const int64_t *const *dims);

/* Reads variable `name` of path: *ndims and dims[0..7] receive its shape; with
 * out != NULL its values (converted to double from the stored type) go to out
 * (host or device), which must hold `capacity` elements. */
int sssi_mat_read(const char *path, const char *name, double *out, int64_t capacity, int *ndims, int64_t *dims);

/* ---- batched and served shots: the plan API ----
 *
 * The reference runs one shot per MEX call and loops over shots in MATLAB
 * (applications/rtm_2d_acoustic/mainRtmTimeCpmlFor2dAw.m:156-166,252-275) or
 * over MPI ranks (applications/rtm_2d_acoustic_mpi/mainRtmTimeCpmlFor2dAwOpenMPI.m:94-113).
 * A plan keeps many shots resident on one GPU and advances all of them with
 * one launch per time step: 2D forward-modelling and RTM shots of any grid
 * size share the batched step kernel, 3D forward shots run alongside.  Shots
 * are admitted first come first served while their estimated device memory
 * fits the plan's budget, join the running batch at the next step boundary
 * (continuous batching) and leave it when they finish, so their memory serves
 * the next ones.  A worker thread with its own CUDA stream does all GPU work;
 * submit, poll and wait are safe to call from any host thread.
 *
 * Results are identical to the single-shot entry points of the same mode
 * (the per-cell arithmetic does not depend on which shots share a launch). */
typedef struct sssi_plan sssi_plan;

#define SSSI_SHOT_FWD2D 0 /* forward modelling: data = top interior row, nx x nt */
#define SSSI_SHOT_RTM2D 1 /* one RTM shot: image nz x nx (as sssi_rtmTimeCpmlFor2dAw) */
#define SSSI_SHOT_FWD3D 2 /* 3D forward modelling: data = top interior face, nx x ny x nt */

#define SSSI_SHOT_QUEUED 0
#define SSSI_SHOT_RUNNING 1
#define SSSI_SHOT_DONE 2
#define SSSI_SHOT_FAILED 3

typedef struct {
    int mode;            /* SSSI_MODE_FP32 or SSSI_MODE_FP64 (FP64_STRICT runs as FP64) */
    int nDiffOrder;      /* shared by every shot of the plan */
    double dz, dx, dy;   /* grid spacing shared by every shot (dy: 3D shots) */
    size_t device_bytes; /* device memory the plan may hold for admitted shots;
                            0: three quarters of the memory free at creation */
    int steps_per_round; /* time steps between admissions; 0: 64 */
} sssi_plan_config;

typedef struct {
    int kind;              /* SSSI_SHOT_* */
    const double *v;       /* velocity, nz x nx (x ny), host or device, padded by extBoundary */
    const double *vs;      /* RTM: migration (smoothed) velocity, nz x nx */
    int64_t nz, nx, ny, nt; /* ny: 3D only */
    int nBoundary;
    double dt;
    int nsrc;              /* point sources (<= 8); RTM: exactly one */
    const int64_t *src_iz, *src_ix, *src_iy; /* interior indices; src_iy: 3D only */
    const double *wavelets; /* nsrc x nt, row s at wavelets + s * nt */
    double epsilon;        /* RTM: imaging stabiliser */
    int snap_stride;       /* RTM in FP32 plans: forward field stored every snap_stride steps (0: 4) */
    double *data;          /* receivers (FWD2D, FWD3D), dataTrue (RTM, may be NULL); host or device */
    double *image;         /* RTM image, nz x nx; host or device (may be NULL when stacked) */
    int64_t stack;         /* RTM: a stack of the plan (sssi_plan_stack_create) the image is added to, or 0 */
    int64_t stack_z0, stack_x0; /* position of the shot's grid in the stack's grid */
} sssi_shot_desc;

typedef struct {
    int state;     /* SSSI_SHOT_* state */
    int status;    /* SSSI_OK, or the SSSI_ERR_* code of a failed shot */
    double submit_s, start_s, done_s; /* seconds since plan creation (start: admission) */
    int64_t cell_updates; /* grid cells advanced by one step, summed over the shot's propagations */
} sssi_shot_info;

typedef struct {
    int64_t queued, running, done, failed;
    size_t device_bytes_in_use, device_bytes_budget;
    int64_t batch_steps;      /* launches of the batched 2D step */
    double cell_updates;      /* all shots, all propagations */
    /* host time of the plan's threads, seconds: admitting shots (allocation,
     * model conversion, uploads), rounds (launches, schedules, events), of
     * which waiting for the GPU, and copying outputs out */
    double admit_s, round_s, gpu_wait_s, deliver_s;
    /* device time of the batched 2D steps (events around each round's
     * launches) and the cell-updates made in it */
    double batch2d_gpu_s, batch2d_cell_updates;
    /* the batched step's tile shape in use (0: 64 x 32, 1: 32 x 32, 2: 128 x 16
     * cells in FP32; FP64 has 32 x 32 only) and the tuner's last timing of each
     * (milliseconds for its trial steps; 0: not timed) */
    int batch2d_tile_shape;
    double batch2d_tune_ms[3];
} sssi_plan_stats;

/* Creates a plan on the current device.  Native form of the submit/poll/wait
 * API sketched for the batched and served workloads; no counterpart in the
 * reference. */
int sssi_plan_create(const sssi_plan_config *config, sssi_plan **plan);
/* Shots still queued or running fail with SSSI_ERR_INTERNAL ("plan destroyed"). */
int sssi_plan_destroy(sssi_plan *plan);
/* Checks the shot, copies its inputs (v, vs, wavelets, source indices) and
 * queues it; outputs are written when the shot completes, so data / image
 * must stay valid until then.  *ticket identifies the shot. */
int sssi_shot_submit(sssi_plan *plan, const sssi_shot_desc *shot, int64_t *ticket);
/* A stacked image held on the device by the plan: the sum of the images of
 * the RTM shots submitted with this stack, each added at its (stack_z0,
 * stack_x0) window as it completes, as the reference stacks its shots
 * (Stacked = Stacked + M ./ s2, mainRtmTimeCpmlFor2dAw.m:315).  nz x nx
 * doubles, zero at creation, counted against the plan's device budget. */
int sssi_plan_stack_create(sssi_plan *plan, int64_t nz, int64_t nx, int64_t *stack);
/* Waits until every shot submitted to the stack so far has finished (done,
 * failed or cancelled: a failed shot adds nothing) and copies the stack to
 * out (nz x nx, host or device). */
int sssi_plan_stack_get(sssi_plan *plan, int64_t stack, double *out);
/* Cancels a shot: a queued shot leaves the queue at once, a running one at
 * the plan's next round boundary (its device memory then returns to the
 * budget); either ends SSSI_SHOT_FAILED with status SSSI_ERR_CANCELLED and
 * writes no outputs.  Finished shots are left as they are.  No counterpart in
 * the reference (its shot loops run to completion). */
int sssi_cancel(sssi_plan *plan, int64_t ticket);
/* Current state of a shot (never blocks). */
int sssi_poll(sssi_plan *plan, int64_t ticket, sssi_shot_info *info);
/* Blocks until the shot is done or failed; returns its status (message in
 * sssi_last_error()).  info may be NULL.  A shot whose receiver row becomes
 * non-finite (a time step beyond the stability limit) fails alone with
 * SSSI_ERR_UNSTABLE; a step whose tile copy does not arrive in time fails
 * every 2D shot that was advancing in it (SSSI_ERR_INTERNAL), and the plan
 * goes on with the next ones. */
int sssi_wait(sssi_plan *plan, int64_t ticket, sssi_shot_info *info);
int sssi_plan_stats_get(sssi_plan *plan, sssi_plan_stats *stats);

/* ---- test support ---- */

/* No counterpart in the reference: a test knob of the batched 2D step.  At
 * batch step `step` (counted from 0 in every call or plan that starts after
 * this one) the first block withholds the tile copies of its first tile, so
 * that tile's bounded wait runs out after `wait_limit` polls (0: the default
 * limit) and the failure path is taken: the call returns SSSI_ERR_INTERNAL, a
 * plan fails the shots of that step, and the device stays usable.  step < 0
 * turns the knob off. */
int sssi_debug_withhold_copy(int step, unsigned wait_limit);

/* No counterpart in the reference: a test knob of the batched 2D step.  With
 * shape >= 0, batches built after this call use that tile shape (0: 64 x 32,
 * 1: 32 x 32, 2: 128 x 16 cells; a shape the element type lacks is ignored)
 * instead of timing the shapes; shape < 0 hands the choice back to the tuner.
 * Results do not depend on the shape: the tests use this to show it. */
int sssi_debug_tile_shape(int shape);

/* No counterpart in the reference: what the 3D propagator's schedule tuner
 * chose.  A 3D propagation of at least 64 steps times four candidate
 * work-item schedules on its first steps (0: even chunks along y, about three
 * items per resident block; 1, 2, 3: chunks cut by estimated cost, about three,
 * two or four items per resident block) and keeps the fastest; this reports
 * the choice of the last one to finish tuning in *schedule (-1 before any) and
 * the four timed runs in ms[0..3] (ms). */
int sssi_debug_schedule3d(int* schedule, float* ms);

/* No counterpart in the reference: a test entry of the division the strict
 * FP64 forms use for their per-term division by the grid spacing (a
 * reciprocal, a correction and an exact check, the IEEE division otherwise).
 * For each of the n dividends a[k] (host or device memory) it writes that
 * quotient by d to fast[k] and the IEEE quotient to ieee[k]; the two must
 * agree bit for bit. */
int sssi_debug_divide(const double* a, int64_t n, double d, double* fast, double* ieee);

/* ---- forward modelling without any allocation ---- */

/* Size of the fixed working array behind sssi_fwdTimeCpmlFor2dAwNoAlloc. */
#define SSSI_NOALLOC_SCRATCH_BYTES (32u << 20)

/* No counterpart in the reference: an addition for callers that must not
 * allocate memory while they run, such as a service whose GPU memory already
 * belongs to its own pool (an extra cudaMalloc would fail), a latency-bound
 * loop that cannot pay for the device-wide synchronisation of cudaMalloc and
 * cudaFree, or a host program that forbids heap use after start-up.
 *
 * Same inputs, outputs and results as sssi_fwdTimeCpmlFor2dAw in the FP64
 * modes (bit-identical in SSSI_MODE_FP64_STRICT), but every pointer must be
 * device memory owned by the caller, and all working state lives in one array
 * of SSSI_NOALLOC_SCRATCH_BYTES compiled into the library.  The function calls
 * no allocating routine.  nz and nx must be below 2^30 and nt below 2^31;
 * grids whose state does not fit the array (beyond about 620 x 1240 at
 * nDiffOrder 4) are refused with SSSI_ERR_ARG and a message giving the size
 * needed.
 *
 * The array is reserved on a GPU when the library's module is first loaded
 * there, which with CUDA's lazy module loading is the first call of this
 * function on that GPU, and is then held until the process exits: a caller
 * that gives all free GPU memory to its own pool should make one call (nt = 0
 * is enough) before doing so.  The device address of the array is looked up
 * on every call for the calling thread's current device.
 *
 * All calls share that one array: calls whose work overlaps on the GPU (from
 * two streams) corrupt each other and must be serialised by the caller; calls
 * from several host threads are serialised inside the function.  Each call
 * clears the state that has to start at zero.  The call blocks until its
 * work is done, so it must not be made while a stream of the calling thread
 * is being captured into a CUDA graph. */
int sssi_fwdTimeCpmlFor2dAwNoAlloc(const double *v, const double *source, int64_t nz, int64_t nx, int64_t nt,
                                   int nDiffOrder, int nBoundary, double dz, double dx, double dt, double *data,
                                   double *snapshot, int mode);

#ifdef __cplusplus
}
#endif

#endif /* SSSI_GB300_H */
