/* ctgb.h - C ABI of the GB300 distance-driven CT operators (libctgb.so).
 *
 * Drop-in boundary for CTLIB's pybind11 module `ctlib` (src/ctlib.cpp:106-114):
 * the five operators below replace projection / projection_t / backprojection /
 * backprojection_t / fbp with the same tensor layouts (B x 1 x H x W images,
 * B x 1 x V x D sinograms, contiguous, fp32 or fp64) and the same options
 * vector semantics, but take plain device pointers, a caller-provided scratch
 * buffer and a CUDA stream, and return a status code instead of terminating
 * the process on a bad scan_type (src/ctlib.cpp:26).
 *
 * The options vector is decoded once into a plan (ctgb_plan_create) instead of
 * on every call through blocking .item() reads of a device tensor
 * (src/ctlib.cpp:18, src/fan_ed_kernel.cu:1165-1181).
 *
 * All functions are thread-safe with respect to distinct plans; one plan may
 * be used from several threads/streams concurrently (it is read-only after
 * creation). Errors: CTGB_OK (0) on success, otherwise a CTGB_ERR_* code and a
 * message retrievable with ctgb_last_error() on the calling thread.
 */
#ifndef CTGB_H
#define CTGB_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ctgb_plan ctgb_plan;

enum {
  CTGB_OK = 0,
  CTGB_ERR_INVALID = 1,   /* bad options, sizes, pointers or dtype */
  CTGB_ERR_CUDA = 2,      /* a CUDA runtime call or launch failed */
  CTGB_ERR_WORKSPACE = 3  /* scratch buffer smaller than ctgb_workspace_size() */
};

enum { CTGB_FLOAT32 = 0, CTGB_FLOAT64 = 1 };

enum {
  CTGB_OP_PROJECTION = 0,
  CTGB_OP_PROJECTION_T = 1,
  CTGB_OP_BACKPROJECTION = 2,
  CTGB_OP_BACKPROJECTION_T = 3,
  CTGB_OP_FBP = 4,
  CTGB_OP_BACKPROJECTION_SV = 5,
  CTGB_OP_DATA_GRADIENT = 6 /* for ctgb_workspace_size only */
};

/* Decode an options vector (host array, the reference's layout: fan
 * [views, dets, width, height, dImg, dDet, Ang0, dAng, s2r, d2r, binshift,
 * scan_type], parallel [views, dets, width, height, dImg, dDet, Ang0, dAng,
 * binshift, ..., scan_type]; src/fan_ed_kernel.cu:1165-1175,
 * src/para_kernel.cu:687-695) and upload the per-view geometry tables to
 * `device`. Replaces the option decoding of every reference host wrapper. */
int ctgb_plan_create(ctgb_plan** plan, const double* options, int n_options, int dtype, int device);
int ctgb_plan_destroy(ctgb_plan* plan);

/* views, dets, width, height, scan_type, dtype of a plan (any may be NULL) */
int ctgb_plan_info(const ctgb_plan* plan, int* views, int* dets, int* width, int* height,
                   int* scan_type, int* dtype);

/* Schedule of one operator on a plan, as picked by the autotuner
 * (ctlib_gb300/tune.py): the largest number of batch slices one thread carries
 * (1, 2, 4, 8, 16; 0 = default: 16 for fp32, 4 for fp64) and the warps per CTA
 * of the gather kernel (4 or 8; 0 = default 8). Changes the workspace size.
 * No counterpart in the reference (its launch shape is fixed, 256 threads per
 * (slice, view, 256-bin block), src/fan_ed_kernel.cu:1179-1185). */
int ctgb_plan_set_schedule(ctgb_plan* plan, int op, int slices_per_thread, int warps_per_cta);

/* Straight-line steps of one operator's gather loop (2 or 3; 0 = default 3):
 * the overlapped pixels per detector cell (projection, backprojection_t) or
 * cells per pixel (projection_t, backprojection, fbp) evaluated without a
 * branch before a remainder loop takes any further ones. 2 pays when few cells
 * (pixels) span three pixels (cells); fp32 only, fp64 always uses 3.
 * Results do not depend on it. No counterpart
 * in the reference (its merge walk has no fixed step count). */
int ctgb_plan_set_unroll(ctgb_plan* plan, int op, int steps);

/* Limit, in nanoseconds, of every bounded wait in the staged image gather
 * (projection_t, backprojection, fbp, backprojection_sv) on this plan:
 * 1000000000 (1 s) by default, at most 10 s. A wait that runs out makes its
 * CTA finish on global loads, with the same results, and is counted by
 * ctgb_wait_timeouts. 0 makes every wait give up unless its copy has already
 * landed at the first look, which takes the fallback path on purpose (for
 * tests of it). No counterpart in the reference, whose kernels do not wait. */
int ctgb_plan_set_wait_limit(ctgb_plan* plan, unsigned long long limit_ns);

/* Summation order of one plan's operators: compensated = 1 (the default) sums
 * each output's terms over lines (projection, backprojection_t), views
 * (projection_t, backprojection, fbp) and filter taps (fbp) in plain fp32
 * blocks of 32 (16 taps) folded into a Kahan-compensated total; compensated = 0
 * keeps one plain fp32 running sum per output instead, as the reference's walk
 * does (src/fan_ed_kernel.cu:360-401 accumulates each pixel and bin straight
 * into an fp32 value). The plain form exists to measure what compensation
 * buys: float32 plans only (CTGB_ERR_INVALID for float64), applied by the five
 * operators (ctgb_data_gradient and ragged batches always compensate), with
 * three straight-line steps whatever the schedule. Results of either form do
 * not depend on the schedule. No counterpart in the reference. */
int ctgb_plan_set_summation(ctgb_plan* plan, int compensated);

/* Ramp filter of fbp on this plan: window 0 = Ram-Lak (the reference's kernel,
 * the default), 1 = Shepp-Logan, 2 = Ram-Lak under a Hann window; ea_exact != 0
 * (equal-angle fans only) scales each tap by (n dDet / sin(n dDet))^2, which
 * makes the kernel exact on equiangular samples where the reference applies the
 * parallel-beam kernel in angle units (src/fan_ea_kernel.cu:1074-1093).
 * Synchronises the plan's device and rewrites the plan's taps; a ragged batch
 * uses the filters its plans had when it was created. Only (0, 0) has a
 * counterpart in the reference (rlfilter, src/fan_ed_kernel.cu:926-943). */
int ctgb_plan_set_filter(ctgb_plan* plan, int window, int ea_exact);

/* Measurement hook: when both are non-null, every later operator call on this
 * plan records `start_event` right before its gather kernel and `stop_event`
 * right after it, on the call's stream (cudaEvent_t handles created with
 * timing enabled), so cudaEventElapsedTime gives that kernel's own duration;
 * NULL, NULL turns it off. Not thread-safe against concurrent calls on the same
 * plan. No counterpart in the reference. */
int ctgb_plan_set_kernel_events(ctgb_plan* plan, void* start_event, void* stop_event);

/* Scratch bytes `op` needs for `batch` slices (0 is a valid answer). */
size_t ctgb_workspace_size(const ctgb_plan* plan, int op, int batch);

/* A: image (B x 1 x H x W) -> sinogram (B x 1 x V x D).
 * Replaces projection(): src/ctlib.cpp:56-69, prj_{fan_ed,fan_ea,para}_cuda
 * (src/fan_ed_kernel.cu:1163-1195, src/fan_ea_kernel.cu:923-955,
 *  src/para_kernel.cu:685-714). */
int ctgb_projection(const ctgb_plan* plan, const void* image, void* sino, int batch, void* workspace,
                    size_t workspace_bytes, void* stream);

/* A^T: sinogram -> image. Replaces projection_t(): src/ctlib.cpp:71-84,
 * prj_t_*_cuda (src/fan_ed_kernel.cu:1197-1229, src/fan_ea_kernel.cu:957-989,
 * src/para_kernel.cu:716-745). */
int ctgb_projection_t(const ctgb_plan* plan, const void* sino, void* image, int batch, void* workspace,
                      size_t workspace_bytes, void* stream);

/* B (weighted backprojector): sinogram -> image. Replaces backprojection():
 * src/ctlib.cpp:30-43, bprj_*_cuda (src/fan_ed_kernel.cu:1265-1297,
 * src/fan_ea_kernel.cu:1025-1057, src/para_kernel.cu:778-807). */
int ctgb_backprojection(const ctgb_plan* plan, const void* sino, void* image, int batch, void* workspace,
                        size_t workspace_bytes, void* stream);

/* B^T: image -> sinogram. Replaces backprojection_t(): src/ctlib.cpp:15-28,
 * bprj_t_*_cuda (src/fan_ed_kernel.cu:1231-1263, src/fan_ea_kernel.cu:991-1023,
 * src/para_kernel.cu:747-776). */
int ctgb_backprojection_t(const ctgb_plan* plan, const void* image, void* sino, int batch,
                          void* workspace, size_t workspace_bytes, void* stream);

/* RL-filtered backprojection: sinogram -> image. Replaces fbp():
 * src/ctlib.cpp:86-99, fbp_*_cuda (src/fan_ed_kernel.cu:1333-1382,
 * src/fan_ea_kernel.cu:1059-1107, src/para_kernel.cu:809-849). The ramp
 * filter runs in fp32/fp64 FMA arithmetic (the reference's cuDNN convolution
 * runs in TF32 unless the caller disables it). */
int ctgb_fbp(const ctgb_plan* plan, const void* sino, void* image, int batch, void* workspace,
             size_t workspace_bytes, void* stream);

/* Single-view backprojection, equal-distance fan beams only: sinogram
 * B x 1 x V x D -> B x V x H x W, image v holding view v's term of
 * backprojection (the same overlaps and U^2 weights, no sum over views), so that
 * summing over views gives ctgb_backprojection. Replaces backprojection_sv():
 * src/ctlib.cpp:45-54, bprj_sv_fan_ed_cuda and bprj_sv_fan_ed
 * (src/fan_ed_kernel.cu:946-1161, 1299-1331). Other scan types return
 * CTGB_ERR_INVALID (the reference exits the process). Workspace as for
 * CTGB_OP_BACKPROJECTION_SV in ctgb_workspace_size. */
int ctgb_backprojection_sv(const ctgb_plan* plan, const void* sino, void* images, int batch, void* workspace,
                           size_t workspace_bytes, void* stream);

/* Gradient of the data term 0.5*||A x - y||^2 for iterative reconstruction:
 * grad = A^T (A x - y), image B x 1 x H x W and measured sinogram y
 * B x 1 x V x D in, grad B x 1 x H x W out; `residual` (B x 1 x V x D, may be
 * NULL) receives A x - y, from which the caller forms the loss. The same values
 * as projection, a subtraction and projection_t, without a separate subtraction
 * or sinogram re-layout: the projection kernel writes the residual straight into
 * the backprojection's input planes. Uses the schedules set for
 * CTGB_OP_PROJECTION (its first kernel) and CTGB_OP_PROJECTION_T (its second);
 * workspace: ctgb_workspace_size(plan, CTGB_OP_DATA_GRADIENT, batch). No single
 * counterpart in the reference: a caller composes it from projection and
 * projection_t (src/ctlib.cpp:56-84).
 * A convenience entry with no speed claim: it runs the same two gathers as the
 * composed calls, and on the 16-slice 512^2 fan-ED batch it takes the same time
 * (5.30 against 5.29 ms). What fusion saves is the subtraction pass and the
 * sinogram re-layout, about 0.1 GB of memory traffic (tens of microseconds);
 * the two gathers, bound by their instruction issue, are the other 99%. */
int ctgb_data_gradient(const ctgb_plan* plan, const void* image, const void* sino, void* residual, void* grad,
                       int batch, void* workspace, size_t workspace_bytes, void* stream);

/* A (as ctgb_projection) for callers that cannot allocate device memory.
 * No counterpart in the reference. Some callers of these operators may not
 * call cudaMalloc, cudaFree or any allocating routine at run time: a C or
 * embedded host program linked against this library alone has no caching
 * allocator, where every cudaMalloc/cudaFree can synchronise the device and
 * stall other streams; a reconstruction service that reserves all of its
 * device memory at start-up treats a later allocation as a fault. This entry
 * point takes only the input and output buffers and uses instead a fixed
 * static scratch array of ctgb_projection_noalloc_max_bytes() bytes (64 MiB)
 * inside this library, reserved on every GPU that loads it until process exit.
 * A batch whose scratch (ctgb_workspace_size for CTGB_OP_PROJECTION) exceeds
 * that size fails with CTGB_ERR_WORKSPACE. The first call on a device (and the
 * first after its context is destroyed and created again, e.g. by
 * cudaDeviceReset) looks up the array's device address; make that first call
 * before any stream capture. All calls share the one array, which keeps the
 * last call's contents (nothing in it needs clearing between calls): calls
 * whose work overlaps on the GPU (other streams, other threads) race on it and
 * must be serialised by the caller. */
int ctgb_projection_noalloc(const ctgb_plan* plan, const void* image, void* sino, int batch, void* stream);

/* Size in bytes of the static scratch array used by ctgb_projection_noalloc. */
size_t ctgb_projection_noalloc_max_bytes(void);

/* Ragged batches: n slices (1..128), each with its own plan (image size, views,
 * detectors, geometry; all plans fp32 or all fp64), processed together: every
 * stage of an operator is one launch over a task list built here, longest tasks
 * first. The image gather's tasks are CTAs of the staged per-slice kernel (one
 * per slice, pixel tile and view part), so the results equal per-slice calls
 * bit for bit.
 * A run takes host arrays of n device pointers (slice i: 1 x 1 x H_i x W_i or
 * 1 x 1 x V_i x D_i) and needs no host-to-device copy, so it can be captured in
 * a CUDA graph. The plans must outlive the ragged object. No counterpart in the
 * reference (one launch per call and geometry, src/ctlib.cpp:15-99). */
typedef struct ctgb_ragged ctgb_ragged;
int ctgb_ragged_create(ctgb_ragged** ragged, const ctgb_plan* const* plans, int n_slices, int device);
int ctgb_ragged_destroy(ctgb_ragged* ragged);
size_t ctgb_ragged_workspace_size(const ctgb_ragged* ragged, int op);
int ctgb_ragged_run(const ctgb_ragged* ragged, int op, const void* const* in, void* const* out, void* workspace,
                    size_t workspace_bytes, void* stream);

/* Message of the last failed call on this thread ("" if none). */
const char* ctgb_last_error(void);

/* Number of bounded waits in the staged image gather (A^T, B, fbp) that ran out
 * on `device` since the library was loaded or last reset (`reset` != 0 zeroes
 * it after reading). Each such event makes the affected CTA finish on global
 * loads, so results stay correct; a non-zero count means a copy pipeline stalled
 * for over a second. Synchronises the device. Diagnostics only: no counterpart
 * in the reference. */
int ctgb_wait_timeouts(int device, unsigned long long* count, int reset);

/* kNN graph adjacency (replaces `laplacian`, src/ctlib.cpp:101-104 and
 * src/laplacian_cuda_kernel.cu:46-128). `points` is an n x dim row-major device
 * array of `dtype`. For every point i the k smallest squared distances
 * |x_i|^2 + |x_j|^2 - 2 <x_i, x_j> (i itself included, ties to the smaller j)
 * are weighted exp(-d / m), m the lower median of all n*k selected distances,
 * and normalised to sum 1 per row. Output, the reference's COO layout:
 * indices[0][i*k + e] = i, indices[1][i*k + e] = j_e (int64, 2 x n*k) and
 * values[i*k + e] (float32 for either dtype, as the reference's sparse tensor),
 * neighbours in increasing distance. 1 <= k <= min(n, 256), and for fp64 at
 * most what fits a CTA's shared memory (about 140; CTGB_ERR_INVALID beyond);
 * runs on the current device. The n x n distance matrix is never formed. */
size_t ctgb_laplacian_workspace_size(int n, int dim, int k, int dtype);
int ctgb_laplacian(const void* points, int n, int dim, int k, int dtype, long long* indices, float* values,
                   void* workspace, size_t workspace_bytes, void* stream);

/* ABI version, bumped on incompatible changes. */
int ctgb_version(void);

/* Host-side geometry of an options vector without touching a GPU (for tests
 * and tooling). `what`: 0 flags (V ints as doubles: bit0 row lines, bit1
 * flipped), 1 detector boundaries (V*(D+1)), 2 A/A^T factors (V*D),
 * 3 line maps (V*L*2: alpha, sigma), 4 inverse seeds (V*5), 5 fbp pre-weight (D),
 * 6 ramp taps (2D-1), 7 the image gather's split line maps as stored for `dtype`
 * (V*L*4: alpha hi, alpha lo, sigma hi, sigma lo, each rounded to the type; the
 * high parts make alpha_hi + sigma_hi*k exact for every pixel edge k of the
 * line). Returns the element count, or -1 on error. */
long ctgb_geometry_query(const double* options, int n_options, int dtype, int what, double* out,
                         size_t n_out);

#ifdef __cplusplus
}
#endif

#endif /* CTGB_H */
