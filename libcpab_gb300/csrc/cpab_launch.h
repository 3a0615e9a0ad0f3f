// Internal launch interface between the C-ABI layer (cpab_capi.cu) and the
// kernel translation units.  Not part of the public ABI (see include/).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <array>

#include "cpab_common.cuh"

namespace cpab {

// ------------------------------- autotuner ----------------------------------
// Launch shapes picked by the autotuner entry points (cpab_integrate_tune,
// cpab_transform_data_tune, cpab_ragged_points_tune), cached per device,
// kernel family and problem shape.  A launcher takes the cached shape when
// there is one and its own heuristic otherwise; `force` (the candidates the
// tuner times) overrides both.  Fields left at their defaults mean "the
// heuristic's choice".
struct LaunchShape {
    int block = 0;      // threads per CTA
    int ppt = 0;        // points per thread (forward kernels)
    int parts = 0;      // CTAs per theta or image (fused backward)
    int staging = -1;   // fused backward: per-warp tables in shared (0) / global (1) memory
};
enum TuneKind : int {
    kTuneIntegrate = 1,
    kTuneFusedForward = 2,
    kTuneFusedBackward = 3,
    kTunePointsForward = 4,
    kTunePointsBackward = 5,
    kTuneAdjoint = 6
};
using TuneKey = std::array<long long, 8>;
TuneKey tune_key(const Tess &t, int nsteps, int mode, long long a, long long b, long long c);
bool tuned_get(int kind, const TuneKey &key, LaunchShape *shape);
void tuned_set(int kind, const TuneKey &key, const LaunchShape &shape);
void tuned_clear();

// Per-(theta, cell) tables from theta and the basis B [D, d] (fp32):
// A = B theta, T = expm(dt [A;0]) (rows 0..ndim-1), E = T - I.
cudaError_t launch_cell_tables(const Tess &t, int nsteps, const float *theta, int n_theta, int d,
                               const float *basis, float *A, float *T, float *E,
                               cudaStream_t s);

// Forward integration.  `table` holds T (compensated=false, p <- T p~) or
// E (compensated=true, p <- p + E p~).  trace (nullable) receives the cell of
// every step, [n_theta, nP, nsteps].
cudaError_t launch_integrate(const Tess &t, int nsteps, const float *points, int broadcast,
                             long long nP, const float *table, bool compensated, int n_theta,
                             float *out, int *trace, unsigned long long *ties, unsigned *err,
                             cudaStream_t s, const LaunchShape *force = nullptr);

cudaError_t launch_findcellidx(const Tess &t, const float *points, long long nP, int *out,
                               unsigned long long *ties, cudaStream_t s);

// Adjoint (backward) of the integration.
//   mode 0: transpose of the reference's midpoint-rule sensitivity
//           (table = A);
//   mode 1: exact discrete adjoint of p <- p + E p~ (table = E).
// Writes per-CTA partial cell gradients to `partials`
// ([n_theta, parts, nC*ndim*(ndim+1)] floats) and optionally dL/dpoints
// per theta ([n_theta, ndim, nP]).
struct AdjointPlan {
    int block;           // threads per CTA
    int parts;           // CTAs per theta
    int tiles;           // point tiles per theta
    size_t smem;         // dynamic shared memory bytes
    size_t partial_floats;
    size_t gw_floats;    // per-warp cell tables in the workspace (0: in shared memory)
    // workspace layout: partials [partial_floats], then (64-float aligned) the
    // per-warp tables [n_theta][parts][warps][round4(G)]
    size_t gw_offset() const { return (partial_floats + 63) & ~(size_t)63; }
    size_t ws_floats() const { return gw_floats ? gw_offset() + gw_floats : partial_floats; }
};
bool plan_adjoint(const Tess &t, int nsteps, long long nP, int n_theta, AdjointPlan *plan,
                  bool allow_global_gw = true, const LaunchShape *force = nullptr);
bool plan_adjoint_mode(const Tess &t, int nsteps, int mode, long long nP, int n_theta,
                       AdjointPlan *plan, bool allow_global_gw = true,
                       const LaunchShape *force = nullptr);
cudaError_t launch_adjoint(const Tess &t, int nsteps, int mode, const AdjointPlan &plan,
                           const float *points, int broadcast, long long nP, const float *table,
                           int n_theta, const float *gout, float *dpoints, float *partials,
                           unsigned long long *ties, unsigned *err, cudaStream_t s);

// Sum the partials (fixed order), map cell gradients to dL/dA (mode 1: through
// the adjoint Frechet derivative of expm), and contract with the basis:
// dtheta[theta, k] = sum_i B[i, k] dA[i].
// mode kFinalizeDirect: the partials are dL/dA (the exact-flow adjoint).
constexpr int kFinalizeDirect = 3;
cudaError_t launch_finalize(const Tess &t, int nsteps, int mode, const float *partials, int parts,
                            const float *A, const float *basis, int d, int n_theta,
                            float *dtheta, cudaStream_t s);

// Linear / bilinear / trilinear sampling (libcpab/pytorch/interpolation.py).
// err: device error word (a timed-out grid-tile copy of the 3D kernel).
cudaError_t launch_interpolate(int ndim, const float *data, int nb, int C, const int *size,
                               const float *grid, const int *outsize, float *out,
                               unsigned *err, cudaStream_t s);
cudaError_t launch_interpolate_backward(int ndim, const float *data, int nb, int C,
                                        const int *size, const float *grid, const int *outsize,
                                        const float *gout, float *ddata, float *dgrid,
                                        cudaStream_t s);

// Fused transform_data: meshgrid -> integrate (E) -> sample.  lin holds the
// per-axis meshgrid coordinates (outsize[0] + outsize[1] + ... floats).
// grid_out (nullable) receives the transformed grid [nb, ndim, nP].
cudaError_t launch_transform_data(const Tess &t, int nsteps, const float *lin, const int *outsize,
                                  const float *E, int nb, const float *data, int C,
                                  const int *size, float *out, float *grid_out,
                                  unsigned long long *ties, unsigned *err, cudaStream_t s,
                                  const LaunchShape *force = nullptr);

bool plan_transform_data_backward(const Tess &t, int nsteps, int mode, long long nP, int nb,
                                  AdjointPlan *plan, const LaunchShape *force = nullptr);

// Transformations applied to the grid before the one being differentiated
// (a composition T_K o ... o T_1 differentiated in theta_K only): their
// compensated tables E_k [nb, nC_k, N, N+1] are read from global memory.
constexpr int kMaxPre = 3;
struct PreStages {
    int K;
    Tess t[kMaxPre];
    int nsteps[kMaxPre];
    const float *E[kMaxPre];
};

// Composition of up to kMaxPre + 1 transformations of one dimension: the grid
// passes through all of them in one kernel, then data is sampled
// (cpab_sequential.cu).  stages.E[k] are the compensated tables of stage k.
struct SeqStages {
    int K;
    Tess t[kMaxPre + 1];
    int nsteps[kMaxPre + 1];
    const float *E[kMaxPre + 1];
};
cudaError_t launch_sequential_transform_data(const SeqStages &sq, const float *lin,
                                             const int *outsize, int nb, const float *data,
                                             int C, const int *size, float *out,
                                             float *grid_out, unsigned long long *ties,
                                             unsigned *err, cudaStream_t s);

// Fused transform_data backward: given dL/dout, produce d(data) (accumulated)
// and the partial cell gradients for launch_finalize.
cudaError_t launch_transform_data_backward(const Tess &t, int nsteps, int mode,
                                           const AdjointPlan &plan, const float *lin,
                                           const int *outsize, const float *table,
                                           const float *grid_saved, int nb, const float *data,
                                           int C, const int *size, const float *gout,
                                           float *ddata, float *partials,
                                           unsigned long long *ties, unsigned *err,
                                           cudaStream_t s, const PreStages *pre = nullptr);

// Exact-flow integration (cpab_exact.cu): the true flow of the continuous
// piecewise-affine field for time 1 (table A: velocity maps).  steps
// (nullable) accumulates the number of in-cell steps taken.
cudaError_t launch_integrate_exact(const Tess &t, const float *points, int broadcast,
                                   long long nP, const float *A, int n_theta, float *out,
                                   unsigned long long *ties, unsigned *err,
                                   unsigned long long *steps, cudaStream_t s);

// Reverse-mode derivative of the exact flow (cpab_exact.cu): from the forward
// result out [n_theta, ndim, nP] and dL/d(out), per-CTA partial dL/dA for
// launch_finalize(kFinalizeDirect) and dL/dpoints (may be NULL).
bool plan_adjoint_exact(const Tess &t, long long nP, int n_theta, AdjointPlan *plan);
cudaError_t launch_adjoint_exact(const Tess &t, const AdjointPlan &plan, const float *out,
                                 long long nP, const float *A, int n_theta, const float *gout,
                                 float *dpoints, float *partials, unsigned long long *ties,
                                 unsigned *err, cudaStream_t s);

// Ragged batched 1D series (cpab_ragged.cu).  Series s has the points
// torch.linspace(0, 1, L_s) and the values values[off[s] .. off[s+1]).
constexpr long long kRaggedMaxLen = 1ll << 22;   // per-series length limit

struct RaggedBwd;
size_t ragged_workspace_bytes(const Tess &t, int S);
size_t ragged_adjoint_smem_for(const Tess &t, int nsteps, int mode, int block);
bool ragged_get_tuned(int kind, int mode, const Tess &t, int nsteps, int S, long long total,
                      int *block, int *ppt);
void ragged_set_tuned(int kind, int mode, const Tess &t, int nsteps, int S, long long total,
                      int block, int ppt);
cudaError_t launch_ragged_forward(const Tess &t, int nsteps, int block, int ppt, int S,
                                  const long long *off, long long total, const float *E,
                                  const float *values, float *out, void *ws,
                                  unsigned long long *ties, unsigned *err, cudaStream_t s);

struct RaggedBwd {
    const float *A;        // [S][nC][2]   (mode 0 trajectory table, finalize)
    const float *E;        // [S][nC][2]
    const float *values;   // [total]
    const float *target;   // [total] (fused MSE) or null
    const float *gout;     // [total] (plain backward) or null
    float loss_scale;      // fused MSE: dL/d(out) = loss_scale * (out - target)
    float *out;            // [total] (fused MSE, optional)
    float *dvalues;        // [total] (optional, accumulated)
    float *partials;       // [(TW + S)][nC * 2]  (set from the workspace)
    float *sse_partials;   // [(TW + S)]          (set from the workspace)
    float *lane_slots;     // [TW][nC][2][32] per-lane cell sums, nC <= kLaneSlotCells
                           // (set from the workspace)
};
// fused = true: dL/d(out) from the MSE residual against `target`, per-series
// sum of squared residuals into sse[S]; fused = false: dL/d(out) = gout.
cudaError_t launch_ragged_adjoint(const Tess &t, int nsteps, int mode, bool fused, int block,
                                  int ppt, int S, const long long *off, long long total,
                                  const RaggedBwd &a, const float *basis, int d, float *dtheta,
                                  float *sse, void *ws, unsigned long long *ties, unsigned *err,
                                  cudaStream_t s);

// Ragged point sets of any dimension (cpab_ragged_points.cu): set s owns the
// columns offsets[s] .. offsets[s+1] of points [ndim, total] and has its own
// cell tables (E, A: [S, nC, ndim, ndim+1]).
size_t ragged_points_workspace_bytes(const Tess &t, int S);
cudaError_t launch_ragged_points_forward(const Tess &t, int nsteps, int S, const long long *off,
                                         long long total, const float *E, const float *points,
                                         float *out, void *ws, unsigned long long *ties,
                                         unsigned *err, cudaStream_t s,
                                         const LaunchShape *force = nullptr);
cudaError_t launch_ragged_points_backward(const Tess &t, int nsteps, int mode, int S,
                                          const long long *off, long long total, const float *A,
                                          const float *E, const float *points,
                                          const float *gout, float *dpoints, const float *basis,
                                          int d, float *dtheta, void *ws,
                                          unsigned long long *ties, unsigned *err,
                                          cudaStream_t s,
                                          const LaunchShape *force = nullptr);

cudaError_t launch_sample_grid(int ndim, const float *grid, int nb, const float *data, int C,
                               const int *size, const int *outsize, float *out, cudaStream_t s);

// Ragged images of mixed sizes (cpab_interp_ragged.cu).  Plan row s (int64):
// [data_off, pts_off, tile_off, size[3], outsize[3], 0] (extents padded with
// 1); row S holds the three totals.  Tiles of 256 points (1D) or 8 x-rows x
// 32 last-axis columns (2D, and 3D at one y).
constexpr int kImagePlanFields = 10;
__host__ __device__ inline long long image_tile_count(int ndim, const int *outsize) {
    if (ndim == 1) return (outsize[0] + 255ll) / 256;
    const long long ta = (outsize[0] + 7ll) / 8, tz = (outsize[ndim - 1] + 31ll) / 32;
    return ndim == 2 ? ta * tz : ta * tz * outsize[1];
}
cudaError_t launch_interpolate_ragged(int ndim, int S, const long long *plan,
                                      long long data_points, const float *data, int C,
                                      long long total, long long tiles, const float *grid,
                                      float *out, unsigned *err, cudaStream_t s);
cudaError_t launch_interpolate_ragged_backward(int ndim, int S, const long long *plan,
                                               long long data_points, const float *data, int C,
                                               long long total, long long tiles,
                                               const float *grid, const float *gout,
                                               float *ddata, float *dgrid, unsigned *err,
                                               cudaStream_t s);

int num_sms();

}  // namespace cpab
