/*
 * cpab_gb300.h -- C ABI of the GB300 (sm_103a) CPAB integration library.
 *
 * Plain pointers and sizes only.  Every pointer argument named like a tensor
 * is a CUDA device pointer to contiguous float32 (or int32) memory on the
 * current device; `nc`, `size` and `outsize` are host arrays of `ndim` ints.
 * `stream` is a cudaStream_t (NULL = legacy default stream).  Work is only
 * enqueued: no entry point synchronises the host except cpab_device_status
 * and the autotuners (cpab_*_tune).
 *
 * Every entry point returns CPAB_OK (0) or an error code; the message for
 * the last error of the calling thread is returned by cpab_last_error().
 * Nothing here terminates the process (the reference calls exit() on a CUDA
 * error: libcpab/pytorch/transformer_cuda.cu:8-16).
 *
 * Tensor layouts are the reference's (libcpab/pytorch/transformer_cuda.cpp:
 * 17-70, libcpab/pytorch/interpolation.py):
 *   points  [ndim, nP] (shared by all theta, broadcast=0) or
 *           [n_theta, ndim, nP] (one grid per theta, broadcast=1)
 *   tables  [n_theta, nC, ndim, ndim+1]  (A, T or E; row-major affine maps)
 *   basis   [D, d] with D = nC * ndim * (ndim+1), float32
 *   theta   [n_theta, d]
 *   data    [nb, C, size[0] (, size[1] (, size[2]))]
 *   images  [nb, C, outsize[0] (, outsize[1] (, outsize[2]))]
 * nC = nc[0] (1D), 4*nc[0]*nc[1] (2D), 5*nc[0]*nc[1]*nc[2] (3D).
 */
#ifndef CPAB_GB300_H
#define CPAB_GB300_H

#include <stddef.h>

#if defined(__GNUC__)
#define CPAB_API __attribute__((visibility("default")))
#else
#define CPAB_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define CPAB_OK 0
#define CPAB_ERR_ARGUMENT 1     /* invalid size, pointer or option        */
#define CPAB_ERR_CUDA 2         /* a CUDA runtime call or launch failed   */
#define CPAB_ERR_UNSUPPORTED 3  /* configuration beyond a kernel's limits */
#define CPAB_ERR_WORKSPACE 4    /* workspace missing or too small         */

/* Gradient modes of cpab_backward / cpab_transform_data_backward (and of the
 * ragged and no-alloc backward entry points). */
#define CPAB_GRAD_REFERENCE 0   /* the reference's midpoint-rule analytic gradient,
                                   along the reference's own midpoint trajectory  */
#define CPAB_GRAD_EXACT 1       /* exact derivative of the forward map             */
#define CPAB_GRAD_REFERENCE_MAP 2 /* the reference's gradient formula along the
                                   trajectory of the per-cell midpoint map (one
                                   affine map per step, fewer instructions); its
                                   cells can differ from the reference's where a
                                   step lands within rounding of a cell boundary */

/* Bits reported by cpab_device_status. */
#define CPAB_DEV_TMA_TIMEOUT 1u /* a bulk copy to shared memory did not complete */
#define CPAB_DEV_BAD_CELL 2u    /* reserved (every lookup returns a valid cell)  */
#define CPAB_DEV_BAD_OFFSETS 8u /* a ragged series had invalid offsets (skipped) */
#define CPAB_DEV_ITER_LIMIT 16u /* an exact-flow trajectory hit its step limit     */

/* Message of the calling thread's last error ("" if none). */
CPAB_API const char *cpab_last_error(void);

/* ABI version (major*10000 + minor*100 + patch). */
CPAB_API int cpab_version(void);

/*
 * Number of cells for a tessellation (nC), or -1 for invalid arguments.
 */
CPAB_API int cpab_num_cells(int ndim, const int *nc);

/*
 * Per-(theta, cell) tables from theta: A = B theta (reshaped), and the step
 * maps T = expm(dT [A;0]) (top ndim rows) and E = T - I, dT = 1/nsteps.
 * Any of A, T, E may be NULL.  E is computed in compensated form (no I + small
 * cancellation).
 * Replaces libcpab/pytorch/transformer.py:146-155 (B copied host->device per
 * call, As = B theta^T, expm of libcpab/pytorch/expm.py with its host sync).
 */
CPAB_API int cpab_cell_tables(int ndim, const int *nc, int nsteps, const float *theta, int n_theta,
                     int d, const float *basis, float *A, float *T, float *E, void *stream);

/*
 * Forward integration with the reference's own step maps:
 * nsteps times { c = cell(p); p = T_c [p;1] }.  out is [n_theta, ndim, nP].
 * Drop-in for cpab_gpu.forward(points, trels, nstepsolver, nc)
 * (libcpab/pytorch/transformer_cuda.cpp:17-41, kernels
 * libcpab/core/cpab_ops.cu:268-388).
 */
CPAB_API int cpab_forward(int ndim, const int *nc, int nsteps, const float *points, int broadcast,
                 long long nP, const float *trels, int n_theta, float *out, void *stream);

/*
 * Forward integration with compensated increments: p = p + E_c [p;1].
 * The arithmetic used by Cpab.transform_grid.  ties (device counter, may be
 * NULL) is incremented once per cell lookup resolved by the FP64 path.
 */
CPAB_API int cpab_integrate(int ndim, const int *nc, int nsteps, const float *points, int broadcast,
                   long long nP, const float *E, int n_theta, float *out,
                   unsigned long long *ties, void *stream);

/*
 * cpab_integrate that also records the cell used at every step,
 * cells [n_theta, nP, nsteps] int32 (diagnostics: boundary-tie analysis).
 * No counterpart in the reference.
 */
CPAB_API int cpab_integrate_trace(int ndim, const int *nc, int nsteps, const float *points,
                                  int broadcast, long long nP, const float *E, int n_theta,
                                  float *out, int *cells, void *stream);

/*
 * Workspace bytes needed by cpab_backward for this problem on the current
 * device (0 on invalid arguments; see cpab_last_error): the per-CTA partial
 * cell gradients and, for large tessellations where that fits more warps per
 * SM, the per-warp cell-gradient tables (L2-resident; e.g. 84 MB for 8 x 128^3
 * points at [4,4,4]).  Plans are cached per problem shape and device.
 */
CPAB_API size_t cpab_backward_workspace(int ndim, const int *nc, int nsteps, long long nP, int n_theta);

/*
 * dL/dtheta [n_theta, d] (and optionally dL/dpoints [n_theta, ndim, nP]) from
 * grad_out = dL/d(out) [n_theta, ndim, nP].
 *   mode CPAB_GRAD_REFERENCE: the reference's analytic gradient (midpoint-rule
 *     sensitivity, libcpab/core/cpab_ops.cu:390-697) computed in reverse mode
 *     along the reference's midpoint trajectory in its own arithmetic
 *     (libcpab/core/cpab_ops.cpp:306-365); needs A.
 *   mode CPAB_GRAD_REFERENCE_MAP: the same gradient along the trajectory of
 *     the collapsed per-cell midpoint map; needs A.
 *   mode CPAB_GRAD_EXACT: exact adjoint of cpab_integrate; needs A and E.
 * Replaces cpab_gpu.backward (libcpab/pytorch/transformer_cuda.cpp:43-70) and
 * the contraction gradient.mul_(grad).sum(dim=(2,3))
 * (libcpab/pytorch/transformer.py:186-202), without the [d, n_theta, ndim, nP]
 * intermediate.  The result is deterministic (no floating-point atomics).
 */
CPAB_API int cpab_backward(int ndim, const int *nc, int nsteps, int mode, const float *points,
                  int broadcast, long long nP, const float *A, const float *E, int n_theta,
                  const float *basis, int d, const float *grad_out, float *dtheta,
                  float *dpoints, void *workspace, size_t workspace_bytes,
                  unsigned long long *ties, void *stream);

/*
 * cpab_backward for callers that cannot allocate device memory (a host
 * runtime that owns all device memory through its own pool, or code running
 * where allocation is not allowed) and so cannot supply a workspace.  No
 * counterpart in the reference.
 *
 * Same arguments and results as cpab_backward minus the workspace.  Its
 * scratch is a fixed 8 MiB array (2,097,152 floats) in the library's device
 * memory, reserved on every GPU that loads the library until the process
 * exits; problems with n_theta * nC * ndim * (ndim+1) above 2,097,152 are
 * rejected with CPAB_ERR_WORKSPACE.  The first call on a device looks up the
 * array's address (cudaGetSymbolAddress) with that device current: make it
 * before capturing a stream.  All calls share the array (each call writes
 * what it reads, no clearing needed); calls that may overlap on the GPU race
 * and must be serialised by the caller.  It calls no cudaMalloc, cudaFree or
 * allocating library routine.
 */
CPAB_API int cpab_backward_noalloc(int ndim, const int *nc, int nsteps, int mode,
                                   const float *points, int broadcast, long long nP,
                                   const float *A, const float *E, int n_theta,
                                   const float *basis, int d, const float *grad_out,
                                   float *dtheta, float *dpoints, unsigned long long *ties,
                                   void *stream);

/*
 * Linear / bilinear / trilinear sampling with clamp-to-edge.  grid is
 * [nb, ndim, prod(outsize)] with the meshgrid's x fastest; out is the image
 * layout above.  Replaces libcpab/pytorch/interpolation.py:12-172.
 */
CPAB_API int cpab_interpolate(int ndim, const float *data, int nb, int C, const int *size,
                     const float *grid, const int *outsize, float *out, void *stream);

/*
 * Backward of cpab_interpolate: ddata (overwritten, may be NULL) and dgrid
 * (overwritten, may be NULL) from grad_out (image layout).  ddata is a
 * scatter-add with float atomics, like the reference's autograd.
 */
CPAB_API int cpab_interpolate_backward(int ndim, const float *data, int nb, int C, const int *size,
                              const float *grid, const int *outsize, const float *grad_out,
                              float *ddata, float *dgrid, void *stream);

/*
 * Fused transform_data forward: meshgrid -> cpab_integrate -> interpolate in
 * one kernel.  lin holds the meshgrid's per-axis coordinates, concatenated
 * (outsize[0] + ... + outsize[ndim-1] floats, e.g. torch.linspace(0,1,n)).
 * E is [nb, nC, ndim, ndim+1].  grid_out (may be NULL) receives the
 * transformed points as [nb, ndim, prod(outsize)] in image order (last axis
 * fastest), for cpab_transform_data_backward in reference mode.
 * Replaces libcpab/cpab.py:304-331 (uniform_meshgrid, transform_grid,
 * interpolate as separate passes).
 */
CPAB_API int cpab_transform_data(int ndim, const int *nc, int nsteps, const float *lin,
                        const int *outsize, const float *E, int nb, const float *data, int C,
                        const int *size, float *out, float *grid_out,
                        unsigned long long *ties, void *stream);

/*
 * The two halves of cpab_transform_data, for callers whose images are still
 * arriving (e.g. a host-to-device copy on another stream) while the
 * trajectories are integrated.  cpab_transform_grid_image writes the
 * transformed meshgrid as [nb, ndim, prod(outsize)] in image order (the
 * grid_out of cpab_transform_data; it needs no image); cpab_sample_grid then
 * samples data at that grid into out (image layout).  Together they give
 * cpab_transform_data's output bit for bit.  No counterpart in the
 * reference (its transform_data, libcpab/cpab.py:304-331, runs
 * uniform_meshgrid, transform_grid and interpolate as separate passes in
 * meshgrid order).
 */
CPAB_API int cpab_transform_grid_image(int ndim, const int *nc, int nsteps, const float *lin,
                                       const int *outsize, const float *E, int nb,
                                       float *grid_out, unsigned long long *ties, void *stream);

CPAB_API int cpab_sample_grid(int ndim, const float *data, int nb, int C, const int *size,
                              const float *grid, const int *outsize, float *out, void *stream);

/* Workspace bytes needed by cpab_transform_data_backward (as cpab_backward_workspace). */
CPAB_API size_t cpab_transform_data_backward_workspace(int ndim, const int *nc, int nsteps, int mode,
                                              const int *outsize, int nb);

/*
 * Fused transform_data backward from grad_out = dL/d(out) (image layout):
 * ddata (overwritten, may be NULL) and dtheta [nb, d].  Mode
 * CPAB_GRAD_REFERENCE and CPAB_GRAD_REFERENCE_MAP need A and grid_saved (from
 * cpab_transform_data); CPAB_GRAD_EXACT needs A and E.
 */
CPAB_API int cpab_transform_data_backward(int ndim, const int *nc, int nsteps, int mode,
                                 const float *lin, const int *outsize, const float *A,
                                 const float *E, const float *grid_saved, int nb,
                                 const float *data, int C, const int *size, const float *basis,
                                 int d, const float *grad_out, float *ddata, float *dtheta,
                                 void *workspace, size_t workspace_bytes,
                                 unsigned long long *ties, void *stream);

/*
 * Exact-flow scheme (opt-in; no counterpart in the reference, whose
 * integrator is the fixed-step scheme of cpab_forward / cpab_integrate,
 * libcpab/core/cpab_ops.cu:268-388): each point follows the true flow of the
 * continuous piecewise-affine field for time 1.  A: velocity tables
 * [n_theta, nC, ndim, ndim+1] (cpab_cell_tables).  1D in closed form, 2D/3D
 * by certified in-cell steps of the analytic cell flow.  steps (device
 * uint64, may be NULL) accumulates the in-cell steps taken.  Its gradient:
 * cpab_backward_exact.
 */
CPAB_API int cpab_integrate_exact(int ndim, const int *nc, const float *points, int broadcast,
                                  long long nP, const float *A, int n_theta, float *out,
                                  unsigned long long *ties, unsigned long long *steps,
                                  void *stream);

/*
 * Backward of cpab_integrate_exact (no counterpart in the reference): dtheta
 * [n_theta, d] (overwritten; deterministic) and dL/dpoints [n_theta, ndim, nP]
 * (overwritten, may be NULL) from grad_out = dL/d(out), where out
 * [n_theta, ndim, nP] is cpab_integrate_exact's result for the same A.  The
 * flow is integrated backwards from out in certified in-cell sub-steps; per
 * sub-step the cotangent is carried back through the in-cell flow and dL/dA
 * gathers the adjoint Frechet derivative of its exponential.  The field is
 * continuous across faces, so the crossing times add no term.  workspace:
 * cpab_backward_exact_workspace() bytes of device memory.
 */
CPAB_API size_t cpab_backward_exact_workspace(int ndim, const int *nc, long long nP,
                                              int n_theta);
CPAB_API int cpab_backward_exact(int ndim, const int *nc, const float *out, long long nP,
                                 const float *A, int n_theta, const float *basis, int d,
                                 const float *grad_out, float *dtheta, float *dpoints,
                                 void *workspace, size_t workspace_bytes,
                                 unsigned long long *ties, void *stream);

/*
 * Composition T_K o ... o T_1 (1 <= K <= 4 transformations of the same ndim):
 * the fused form of CpabSequential.transform_data (libcpab/sequential.py:
 * 109-128), which there is one transform_grid call per transformation and an
 * interpolation of the final grid.  nc holds K*ndim ints (stage k at
 * nc + k*ndim), nsteps K ints, E a HOST array of K device pointers to each
 * stage's compensated tables [nb, nC_k, ndim, ndim+1].  lin, outsize, data,
 * out and grid_out (may be NULL; the final grid) as in cpab_transform_data.
 */
CPAB_API int cpab_sequential_transform_data(int ndim, int K, const int *nc, const int *nsteps,
                                            const float *lin, const int *outsize,
                                            const float *const *E, int nb, const float *data,
                                            int C, const int *size, float *out, float *grid_out,
                                            unsigned long long *ties, void *stream);

/*
 * Backward of cpab_sequential_transform_data with the reference's gradient
 * semantics: its transform_grid gives the points no gradient
 * (libcpab/pytorch/transformer.py:202), so of the thetas only the last
 * transformation's gets one (dtheta_last [nb, d_last]); ddata as in
 * cpab_transform_data_backward.  A_last, basis_last: the last stage's A tables
 * and basis; grid_saved: the final grid (reference mode).  workspace:
 * cpab_transform_data_backward_workspace() of the last stage.
 */
CPAB_API int cpab_sequential_transform_data_backward(int ndim, int K, const int *nc,
                                                     const int *nsteps, int mode,
                                                     const float *lin, const int *outsize,
                                                     const float *const *E, const float *A_last,
                                                     const float *grid_saved, int nb,
                                                     const float *data, int C, const int *size,
                                                     const float *basis_last, int d_last,
                                                     const float *grad_out, float *ddata,
                                                     float *dtheta_last, void *workspace,
                                                     size_t workspace_bytes,
                                                     unsigned long long *ties, void *stream);

/*
 * Cell index of every point ([ndim, nP] -> int32 [nP]), bit-identical to the
 * reference's C++/CUDA lookup (libcpab/core/cpab_ops.cpp:26-190).
 */
CPAB_API int cpab_findcellidx(int ndim, const int *nc, const float *points, long long nP, int *out,
                     unsigned long long *ties, void *stream);

/*
 * Ragged batched 1D series.  No single reference entry point: the reference
 * processes each series as its own Cpab.transform_data call (libcpab/cpab.py:
 * 304-331) with outsize [L_s], i.e. grid = torch.linspace(0, 1, L_s)
 * (libcpab/pytorch/functions.py:102-108), transform_grid with that series'
 * theta (libcpab/pytorch/transformer.py:72-87, the cpab_gpu.forward /
 * cpab_gpu.backward pair of libcpab/pytorch/transformer_cuda.cpp:17-70) and
 * linear interpolation (libcpab/pytorch/interpolation.py:18-60).  These
 * entry points run all S series in one persistent launch.
 *
 * Series s owns values[offsets[s] .. offsets[s+1]) (L_s = offsets[s+1] -
 * offsets[s] points, 0 <= L_s < 2^22); offsets is a DEVICE array of S + 1
 * int64 (a series with invalid offsets is skipped and raises
 * CPAB_DEV_BAD_OFFSETS).  total = number of value elements; total + 128*S
 * must be below 2^31.  A and E are [S, nC, 1, 2] (one theta per series, from
 * cpab_cell_tables); basis is [2*nC, d]; dtheta is [S, d].  workspace is
 * device memory of cpab_ragged1d_workspace() bytes (warp-tile prefix, the
 * deterministic partial sums and, for nc <= 128, the adjoint's per-lane cell
 * sums: 256 * nc bytes per resident warp, 32 warps per SM); the calls do not
 * synchronise and can be captured in a CUDA graph.
 */
CPAB_API size_t cpab_ragged1d_workspace(int nc, int nsteps, int S);

/* out[offsets[s] + j] = interp(values_s, T_s(linspace(0, 1, L_s)[j])). */
CPAB_API int cpab_ragged1d_forward(int nc, int nsteps, const float *E, int S,
                                   const long long *offsets, long long total,
                                   const float *values, float *out, void *workspace,
                                   size_t workspace_bytes, unsigned long long *ties,
                                   void *stream);

/*
 * Backward of cpab_ragged1d_forward from grad_out = dL/d(out): dtheta [S, d]
 * (overwritten) and dvalues [total] (overwritten, may be NULL; scatter-add
 * with float atomics like the reference's autograd).  Mode as in
 * cpab_backward.
 */
CPAB_API int cpab_ragged1d_backward(int nc, int nsteps, int mode, const float *A, const float *E,
                                    int S, const long long *offsets, long long total,
                                    const float *basis, int d, const float *values,
                                    const float *grad_out, float *dtheta, float *dvalues,
                                    void *workspace, size_t workspace_bytes,
                                    unsigned long long *ties, void *stream);

/*
 * Forward, squared-error loss and backward in one launch (plus the prefix
 * and finalize kernels): out (may be NULL) as cpab_ragged1d_forward, sse[s] =
 * sum_j (out - target)^2 over series s, and the gradients of
 * L = sum_s loss_scale/2 * sse[s] (loss_scale = 2/total gives the mean
 * squared error): dtheta [S, d] and dvalues (may be NULL).
 */
CPAB_API int cpab_ragged1d_mse(int nc, int nsteps, int mode, const float *A, const float *E, int S,
                               const long long *offsets, long long total, const float *basis,
                               int d, const float *values, const float *target, float loss_scale,
                               float *out, float *sse, float *dtheta, float *dvalues,
                               void *workspace, size_t workspace_bytes,
                               unsigned long long *ties, void *stream);

/*
 * Autotuner: times the launch shapes (threads per block 64/128/256 x points
 * per lane 1/2/4) of the ragged forward (kind 0) or adjoint (kind 1, timed
 * as cpab_ragged1d_mse) kernels on these inputs, keeps the fastest for later
 * calls with the same (device, kind, mode, nc, nsteps, S, total), and leaves
 * the outputs of the chosen shape in out (kind 0) or out/sse/dtheta/dvalues
 * (kind 1).  force (may be NULL): {threads, points per lane} to keep without
 * timing.  shape (may be NULL) receives {threads, points per lane};
 * best_ms (may be NULL) the fastest time.  Synchronises the stream; refuses
 * to run while the stream is being captured.
 */
CPAB_API int cpab_ragged1d_tune(int kind, int nc, int nsteps, int mode, const float *A,
                                const float *E, int S, const long long *offsets, long long total,
                                const float *basis, int d, const float *values,
                                const float *target, float loss_scale, float *out, float *sse,
                                float *dtheta, float *dvalues, void *workspace,
                                size_t workspace_bytes, const int *force, int *shape,
                                float *best_ms, void *stream);

/*
 * Ragged point sets: S sets of ndim-dimensional points, each moved by its
 * own theta, in one persistent launch.  Replaces one transform_grid call per
 * (theta, point set) pair (libcpab/cpab.py:276-302 ->
 * libcpab/pytorch/transformer.py:72-87, the cpab_gpu.forward /
 * cpab_gpu.backward pair of libcpab/pytorch/transformer_cuda.cpp:17-70), or
 * one call on sets padded to a common size.  No counterpart in the reference.
 *
 * points is [ndim, total] (coordinate-major like cpab_integrate's points);
 * set s owns the columns offsets[s] .. offsets[s+1] (L_s points,
 * 0 <= L_s < 2^22); offsets is a DEVICE array of S + 1 int64 (a set with
 * invalid offsets is skipped and raises CPAB_DEV_BAD_OFFSETS).
 * total + 128*S must be below 2^31.  A and E are [S, nC, ndim, ndim+1] (one
 * theta per set, from cpab_cell_tables); basis is [nC*ndim*(ndim+1), d];
 * dtheta is [S, d].  Each set's result equals cpab_integrate / cpab_backward
 * on that set alone (same arithmetic, same lookups; dtheta up to the order of
 * the float sums).  workspace is device memory of
 * cpab_ragged_points_workspace() bytes; the calls do not synchronise and can
 * be captured in a CUDA graph.  Warps are most efficient when nearby points
 * of a set start in the same cell (e.g. points sorted by starting cell).
 */
CPAB_API size_t cpab_ragged_points_workspace(int ndim, const int *nc, int S);

/* out [ndim, total]: set s's points integrated with its table E[s]. */
CPAB_API int cpab_ragged_points_forward(int ndim, const int *nc, int nsteps, const float *E,
                                        int S, const long long *offsets, long long total,
                                        const float *points, float *out, void *workspace,
                                        size_t workspace_bytes, unsigned long long *ties,
                                        void *stream);

/*
 * Backward of cpab_ragged_points_forward from grad_out = dL/d(out)
 * [ndim, total]: dtheta [S, d] (overwritten; deterministic) and dpoints
 * [ndim, total] (overwritten, may be NULL).  Mode as in cpab_backward
 * (CPAB_GRAD_REFERENCE and CPAB_GRAD_REFERENCE_MAP need A; CPAB_GRAD_EXACT needs A and E).
 */
CPAB_API int cpab_ragged_points_backward(int ndim, const int *nc, int nsteps, int mode,
                                         const float *A, const float *E, int S,
                                         const long long *offsets, long long total,
                                         const float *basis, int d, const float *points,
                                         const float *grad_out, float *dtheta, float *dpoints,
                                         void *workspace, size_t workspace_bytes,
                                         unsigned long long *ties, void *stream);

/*
 * Ragged images: S images of mixed sizes (each with its own size and
 * outsize, same C and ndim) sampled in one launch.  Replaces a loop of
 * libcpab/pytorch/interpolation.py:12-172 calls (one data size and one
 * outsize per call, :39-40), i.e. the sampling half of a loop of
 * transform_data calls (libcpab/cpab.py:304-331) over images of different
 * sizes; no counterpart in the reference.
 *
 * cpab_ragged_images_plan (host only, no CUDA call) fills plan, a HOST array
 * of (S + 1) * CPAB_IMAGE_PLAN_FIELDS int64: row s = [data_off, pts_off,
 * tile_off, size[3], outsize[3], 0] with the extents padded with 1, and row
 * S = [data_points, total, tiles, 0, ...].  sizes and outsizes are host
 * [S, ndim] (outsizes NULL: each image keeps its size).  totals[3] receives
 * data_points (sum of prod(size)), total (sum of prod(outsize), below 2^31)
 * and tiles.  The caller copies the plan to the device once and passes it
 * with those totals to the calls below (the kernels check the rows they use
 * and raise CPAB_DEV_BAD_OFFSETS on a row that does not fit them).
 *
 * Layout: data packs the [C, size_s] blocks (image s at C * data_off[s]);
 * grid is [ndim, total] with image s in the columns pts_off[s] ..
 * pts_off[s] + prod(outsize_s) in meshgrid order (x fastest), e.g. the
 * output of cpab_ragged_points_forward with offsets = the plan's pts_off
 * column; out packs the [C, outsize_s] blocks (image s at C * pts_off[s]).
 * Each image's output is bit-identical to cpab_interpolate on that image.
 */
#define CPAB_IMAGE_PLAN_FIELDS 10
CPAB_API int cpab_ragged_images_plan(int ndim, int S, const int *sizes, const int *outsizes,
                                     long long *plan, long long *totals);

CPAB_API int cpab_interpolate_ragged(int ndim, int S, int C, const long long *plan,
                                     long long data_points, long long total, long long tiles,
                                     const float *data, const float *grid, float *out,
                                     void *stream);

/*
 * Backward of cpab_interpolate_ragged from grad_out (out's layout): ddata
 * (overwritten, may be NULL; scatter-add with float atomics like
 * cpab_interpolate_backward) and dgrid [ndim, total] (overwritten, may be
 * NULL).
 */
CPAB_API int cpab_interpolate_ragged_backward(int ndim, int S, int C, const long long *plan,
                                              long long data_points, long long total,
                                              long long tiles, const float *data,
                                              const float *grid, const float *grad_out,
                                              float *ddata, float *dgrid, void *stream);

/*
 * Autotuner.  Each *_tune call takes the arguments of the call it tunes
 * (cpab_integrate, cpab_backward, cpab_transform_data,
 * cpab_transform_data_backward, cpab_ragged_points_forward / _backward),
 * times that kernel's launch shapes on them -- one warm-up launch, then the
 * best of three timed with CUDA events on the stream -- and keeps the fastest
 * for every later call on the same problem: the same device, tessellation,
 * nsteps, gradient mode (backward kernels other than cpab_backward, whose
 * shape serves all modes) and sizes (points and theta count; image count,
 * output size and C; set count and total points).  It then runs the chosen
 * shape once more, leaving the outputs of a plain call.  Candidates:
 *   forward kernels: 64 / 128 / 256 threads per CTA x 1 / 2 points per
 *     thread (1 / 2 / 4 for the ragged point sets);
 *   adjoint kernels: 64 / 128 / 256 threads x per-warp tables in shared or
 *     (2D, 3D) global memory x the planner's CTA count per theta or image,
 *     half of it and twice it (the ragged point-set adjoint: threads only).
 * force (may be NULL) names one shape to keep instead of timing: it is
 * validated, stored and run (a way to restore shapes saved from an earlier
 * tuning run).  shape (may be NULL) receives the kept shape as
 * CPAB_SHAPE_FIELDS ints {threads per CTA, points per thread (0: not used),
 * CTAs per theta or image (0: not used), table staging (0 shared, 1 global,
 * -1: not used)}; best_ms (may be NULL) its time (0 when forced).
 *
 * A shape only redistributes work over threads and CTAs: every point follows
 * the same arithmetic, so point outputs (out, dpoints) are identical for all
 * shapes and sums over points (dtheta, d(data)) differ only in the order of
 * their float additions.  The backward tuners allocate their own workspace;
 * after tuning, the *_workspace queries return the size for the kept shape.
 * Tuning synchronises the stream and refuses to run while it is captured.
 */
#define CPAB_SHAPE_FIELDS 4

CPAB_API int cpab_integrate_tune(int ndim, const int *nc, int nsteps, const float *points,
                                 int broadcast, long long nP, const float *E, int n_theta,
                                 float *out, const int *force, int *shape, float *best_ms,
                                 void *stream);

CPAB_API int cpab_backward_tune(int ndim, const int *nc, int nsteps, int mode,
                                const float *points, int broadcast, long long nP, const float *A,
                                const float *E, int n_theta, const float *basis, int d,
                                const float *grad_out, float *dtheta, float *dpoints,
                                const int *force, int *shape, float *best_ms, void *stream);

CPAB_API int cpab_transform_data_tune(int ndim, const int *nc, int nsteps, const float *lin,
                                      const int *outsize, const float *E, int nb,
                                      const float *data, int C, const int *size, float *out,
                                      float *grid_out, const int *force, int *shape,
                                      float *best_ms, void *stream);

CPAB_API int cpab_transform_data_backward_tune(int ndim, const int *nc, int nsteps, int mode,
                                               const float *lin, const int *outsize,
                                               const float *A, const float *E,
                                               const float *grid_saved, int nb,
                                               const float *data, int C, const int *size,
                                               const float *basis, int d, const float *grad_out,
                                               float *ddata, float *dtheta, const int *force,
                                               int *shape, float *best_ms, void *stream);

/* kind 0: cpab_ragged_points_forward (E, points -> out); kind 1:
 * cpab_ragged_points_backward (A, E, points, grad_out -> dtheta, dpoints). */
CPAB_API int cpab_ragged_points_tune(int kind, int ndim, const int *nc, int nsteps, int mode,
                                     const float *A, const float *E, int S,
                                     const long long *offsets, long long total,
                                     const float *basis, int d, const float *points,
                                     const float *grad_out, float *out, float *dtheta,
                                     float *dpoints, const int *force, int *shape,
                                     float *best_ms, void *stream);

/* Forget every kept launch shape (all kinds, all devices) except those of
 * cpab_ragged1d_tune; later calls use the built-in heuristics again. */
CPAB_API void cpab_tune_reset(void);

/*
 * Synchronise the current device and report the device error word (the
 * CPAB_DEV_* bits raised by kernels since the last clear).  clear != 0 resets
 * it.  Returns CPAB_OK, or CPAB_ERR_CUDA if the device reported an error.
 */
CPAB_API int cpab_device_status(unsigned *flags, int clear);

#ifdef __cplusplus
}
#endif

#endif /* CPAB_GB300_H */
