// Backward of the integration: dL/dtheta (and dL/dpoints) from dL/d(out).
//
// The reference (libcpab/core/cpab_ops.cu:390-697, launched from
// libcpab/pytorch/transformer_cuda.cu:66-119) runs one thread per
// (point, theta, basis index k), integrates the midpoint-rule sensitivity
// q_k = d p / d theta_k for every k, writes the full [d, n_theta, ndim, nP]
// tensor (read-modify-written at each of the nsteps steps) and contracts it
// with the cotangent in Python (libcpab/pytorch/transformer.py:201).  Its cost
// grows with d and its memory is d * n_theta * ndim * nP floats.
//
// Here one thread owns one trajectory and pushes the cotangent backwards
// through the visited cells (reverse mode), so the cost is independent of d:
//
//   mode 0 ("reference"): the transpose of the reference's own recurrence.
//     The reference integrates, along the midpoint trajectory
//     pMid = p + h/2 A[p;1],  p' = p + h A[pMid;1],
//     q' = M q + h B_k [pMid;1] + h^2/2 A B_k [p;1],  M = I + hA + h^2/2 A^2,
//     so with lambda_N = dL/dp_N and lambda_n = M^T lambda_{n+1}:
//     dL/dtheta_k = sum_n < B_k,c_n , G_n >,
//     G_n = h lambda_{n+1} [pMid_n;1]^T + h^2/2 (A^T lambda_{n+1}) [p_n;1]^T.
//     G_n is linear in S_n = lambda_{n+1} [p_n;1]^T with cell-constant
//     coefficients ([pMid;1] = (I + h/2 [A;0]) [p;1]), so the reverse pass only
//     sums S per cell and propagates lambda with the per-cell D = M - I;
//     k_finalize applies G = h S (I + h/2 [A;0])^T + h^2/2 A_lin^T S once per
//     cell.  The result is the reference's analytic gradient up to rounding.
//     The forward sweep steps the trajectory with the reference's own
//     operation order (ref_mid_step: float affine products, the h updates
//     in emulated double), so its cells are the reference's; the reverse
//     sweep rebuilds segment positions from those checkpoints with the
//     equivalent single affine map p' = p + (h A~ + h^2/2 A~^2)[p;1] per
//     cell (A~ = [A;0]; build_dtab, mid_map_step).
//   mode 1 ("exact"): exact discrete adjoint of the forward map
//     p' = p + E_c [p;1]:  dL/dT_c += lambda_{n+1} [p_n;1]^T,
//     lambda_n = lambda_{n+1} + E_lin^T lambda_{n+1}; dL/dA then follows from
//     the adjoint Frechet derivative of expm (k_finalize).
//
// No per-step state goes to global memory: the forward pass logs each step's
// cell (1 or 2 bytes) and a checkpoint every kSeg steps in shared memory; the
// reverse pass rebuilds each segment's positions from its checkpoint with the
// logged cells (no cell lookups) into a shared-memory segment buffer.
//
// Deterministic reduction: a thread accumulates S for its current cell in
// registers.  At each step the lanes that leave a cell add their S into the
// warp's own copy of the cell-gradient table in one pass; lanes leaving the
// same cell at the same step are first summed in lane order (match.any and
// shuffles), so each table element receives at most one add per step, in
// step order.  At the end the warp copies are summed in warp order into one
// partial per CTA, and k_finalize sums the partials in CTA order.  No
// floating-point atomics are used, so the result is bit-reproducible for a
// given GPU and input.  In 1D, where the lanes of a sorted grid sit in
// non-decreasing cells, the lane groups are found without match.any
// (warp_flush_1d).  For large tessellations the per-warp tables live in the
// workspace instead of shared memory when that fits more warps per SM
// (adjoint_shape, carve_adjoint).
#include "cpab_adjoint.cuh"

namespace cpab {

template <int N, int MODE, typename CT, bool GWG>
__global__ void __launch_bounds__(256)
    k_adjoint(Tess t, int nsteps, Steps st, const float *__restrict__ points, int broadcast,
              long long nP, const float *__restrict__ table, int parts, int tiles,
              const float *__restrict__ gout, float *__restrict__ dpoints,
              float *__restrict__ partials, float *gw_ext, unsigned long long *ties,
              unsigned *err) {
    extern __shared__ float4 smem4[];
    __shared__ uint64_t bar;
    const int B = blockDim.x, tid = threadIdx.x;
    const int G = t.nC * N * (N + 1);
    const int th = blockIdx.y, part = blockIdx.x;
    float *gw = GWG ? gw_ext + ((size_t)th * parts + part) * (B / 32) * round4(G) : nullptr;
    const AdjSmem<N, CT> sm =
        carve_adjoint<N, CT, GWG>(reinterpret_cast<float *>(smem4), t.nC, nsteps, gw);

    if (!adjoint_prologue<N, MODE, CT>(sm, table + (long long)th * G, t.nC, st, &bar, err)) return;
    float *warp_tab = sm.gw + (size_t)(tid >> 5) * round4(G);
    const float *src = points + (broadcast ? (long long)th * N * nP : 0ll);

    for (int tile = part; tile < tiles; tile += parts) {
        const long long idx = (long long)tile * B + tid;
        const bool live = idx < nP;
        float p[N], lam[N];
#pragma unroll
        for (int r = 0; r < N; ++r) p[r] = live ? __ldg(src + r * nP + idx) : 0.5f;
        logged_forward<N, MODE, CT>(sm, t, nsteps, st, p, ties, err);
#pragma unroll
        for (int r = 0; r < N; ++r) lam[r] = live ? __ldg(gout + ((long long)th * N + r) * nP + idx) : 0.f;
        reverse_sweep<N, MODE, CT>(sm, nsteps, st, live, lam, warp_tab);
        if (dpoints && live) {
#pragma unroll
            for (int r = 0; r < N; ++r) dpoints[((long long)th * N + r) * nP + idx] = lam[r];
        }
    }
    adjoint_epilogue<N, CT>(sm, t.nC, partials + ((long long)th * parts + part) * G);
}

// ------------------------------ planning -------------------------------------
template <int N, int MODE, typename CT>
static bool plan_t(const Tess &t, int nsteps, long long nP, int n_theta, AdjointPlan *plan,
                   bool allow_global, const LaunchShape &sh) {
    int block = 0, per_sm = 0;
    bool global_gw = false;
    size_t smem = 0;
    // global per-warp tables in 2D and 3D, where the tables can be large
    decltype(&k_adjoint<N, MODE, CT, false>) kg = nullptr;
    if constexpr (N >= 2)
        if (allow_global) kg = k_adjoint<N, MODE, CT, true>;
    if (!adjoint_shape<N, CT>(k_adjoint<N, MODE, CT, false>, kg, t.nC, nsteps, &block,
                              &global_gw, &smem, &per_sm, sh.block, sh.staging))
        return false;
    const long long tiles = (nP + block - 1) / block;
    const long long target = 2ll * num_sms() * per_sm;
    long long parts = sh.parts > 0 ? sh.parts : (target + n_theta - 1) / n_theta;
    if (parts > tiles) parts = tiles;
    if (parts < 1) parts = 1;
    plan->block = block;
    plan->tiles = (int)tiles;
    plan->parts = (int)parts;
    plan->smem = smem;
    plan->partial_floats = (size_t)n_theta * parts * t.nC * N * (N + 1);
    plan->gw_floats = global_gw ? (size_t)n_theta * parts * (block / 32) * round4(t.nC * N * (N + 1))
                                : 0;
    return true;
}

static bool plan_adjoint_mode_uncached(const Tess &t, int nsteps, int mode, long long nP,
                                       int n_theta, AdjointPlan *plan, bool allow_global,
                                       const LaunchShape &sh) {
    const bool small = t.nC <= 256;
#define CPAB_PLAN(N)                                                                               \
    if (mode != 1)                                                                                 \
        return small ? plan_t<N, 0, uint8_t>(t, nsteps, nP, n_theta, plan, allow_global, sh)       \
                     : plan_t<N, 0, uint16_t>(t, nsteps, nP, n_theta, plan, allow_global, sh);     \
    return small ? plan_t<N, 1, uint8_t>(t, nsteps, nP, n_theta, plan, allow_global, sh)           \
                 : plan_t<N, 1, uint16_t>(t, nsteps, nP, n_theta, plan, allow_global, sh);
    switch (t.ndim) {
        case 1: { CPAB_PLAN(1) }
        case 2: { CPAB_PLAN(2) }
        default: { CPAB_PLAN(3) }
    }
#undef CPAB_PLAN
}

// The tuned shape (cpab_backward_tune) applies to plans that may stage the
// per-warp tables in global memory; the no-allocation entry point plans with
// shared-memory tables only and keeps the heuristic shape.
bool plan_adjoint_mode(const Tess &t, int nsteps, int mode, long long nP, int n_theta,
                       AdjointPlan *plan, bool allow_global, const LaunchShape *force) {
    if (force) return plan_adjoint_mode_uncached(t, nsteps, mode, nP, n_theta, plan,
                                                 allow_global, *force);
    LaunchShape sh;
    const bool tuned = allow_global &&
                       tuned_get(kTuneAdjoint, tune_key(t, nsteps, 0, nP, n_theta, 0), &sh);
    const int flag = (allow_global ? 1 : 0) +
                     (tuned ? 2 * (1 + (sh.staging + 1) + 4 * (sh.block / 32) + 64 * sh.parts) : 0);
    static PlanCache cache;
    return cache.get(0, t, nsteps, mode, nP, n_theta, flag, plan, [&](AdjointPlan *p) {
        return plan_adjoint_mode_uncached(t, nsteps, mode, nP, n_theta, p, allow_global, sh);
    });
}

bool plan_adjoint(const Tess &t, int nsteps, long long nP, int n_theta, AdjointPlan *plan,
                  bool allow_global, const LaunchShape *force) {
    // All modes share the shared-memory layout; plan with the larger register
    // footprint (mode 0) so the plan is valid for any of them.
    return plan_adjoint_mode(t, nsteps, 0, nP, n_theta, plan, allow_global, force);
}

template <int N, int MODE, typename CT>
static cudaError_t launch_adjoint_t(const Tess &t, int nsteps, const AdjointPlan &plan,
                                    const float *points, int broadcast, long long nP,
                                    const float *table, int n_theta, const float *gout,
                                    float *dpoints, float *partials, unsigned long long *ties,
                                    unsigned *err, cudaStream_t s) {
    auto kern = k_adjoint<N, MODE, CT, false>;
    if constexpr (N >= 2)
        if (plan.gw_floats) kern = k_adjoint<N, MODE, CT, true>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)plan.smem);
    if (e != cudaSuccess) return e;
    const Steps st = make_steps(nsteps);
    if (n_theta == 0) return cudaSuccess;
    if (n_theta > 65535) return cudaErrorInvalidConfiguration;   // theta on grid y
    const dim3 grid((unsigned)plan.parts, (unsigned)n_theta);
    float *gw = plan.gw_floats ? partials + plan.gw_offset() : nullptr;
    kern<<<grid, plan.block, plan.smem, s>>>(t, nsteps, st, points, broadcast, nP, table,
                                                       plan.parts, plan.tiles, gout, dpoints,
                                                       partials, gw, ties, err);
    return cudaGetLastError();
}

cudaError_t launch_adjoint(const Tess &t, int nsteps, int mode, const AdjointPlan &plan,
                           const float *points, int broadcast, long long nP, const float *table,
                           int n_theta, const float *gout, float *dpoints, float *partials,
                           unsigned long long *ties, unsigned *err, cudaStream_t s) {
    const bool small = t.nC <= 256;
#define CPAB_ADJ(N)                                                                             \
    if (mode == 0)                                                                              \
        return small ? launch_adjoint_t<N, 0, uint8_t>(t, nsteps, plan, points, broadcast, nP,  \
                                                       table, n_theta, gout, dpoints, partials, \
                                                       ties, err, s)                            \
                     : launch_adjoint_t<N, 0, uint16_t>(t, nsteps, plan, points, broadcast, nP, \
                                                        table, n_theta, gout, dpoints,          \
                                                        partials, ties, err, s);                \
    if (mode == 2)                                                                              \
        return small ? launch_adjoint_t<N, 2, uint8_t>(t, nsteps, plan, points, broadcast, nP,  \
                                                       table, n_theta, gout, dpoints, partials, \
                                                       ties, err, s)                            \
                     : launch_adjoint_t<N, 2, uint16_t>(t, nsteps, plan, points, broadcast, nP, \
                                                        table, n_theta, gout, dpoints,          \
                                                        partials, ties, err, s);                \
    return small ? launch_adjoint_t<N, 1, uint8_t>(t, nsteps, plan, points, broadcast, nP,      \
                                                   table, n_theta, gout, dpoints, partials,     \
                                                   ties, err, s)                                \
                 : launch_adjoint_t<N, 1, uint16_t>(t, nsteps, plan, points, broadcast, nP,     \
                                                    table, n_theta, gout, dpoints, partials,    \
                                                    ties, err, s);
    switch (t.ndim) {
        case 1: { CPAB_ADJ(1) }
        case 2: { CPAB_ADJ(2) }
        default: { CPAB_ADJ(3) }
    }
#undef CPAB_ADJ
}

// ------------------------------ finalize -------------------------------------
template <int N, int MODE>
__global__ void __launch_bounds__(256)
    k_finalize(int nC, Steps st, const float *__restrict__ partials, int parts,
               const float *__restrict__ A, const float *__restrict__ basis, int d,
               float *__restrict__ dtheta) {
    constexpr int P = N * (N + 1);
    extern __shared__ float4 smem4[];
    float *g = reinterpret_cast<float *>(smem4);
    const int th = blockIdx.x, tid = threadIdx.x, B = blockDim.x;
    const int G = nC * P;
    const float *src = partials + (long long)th * parts * G;
    for (int i = tid; i < G; i += B) {
        // four interleaved sums (loads in flight), combined in a fixed order
        float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
        int q = 0;
        for (; q + 4 <= parts; q += 4) {
            s0 += __ldg(src + (long long)q * G + i);
            s1 += __ldg(src + (long long)(q + 1) * G + i);
            s2 += __ldg(src + (long long)(q + 2) * G + i);
            s3 += __ldg(src + (long long)(q + 3) * G + i);
        }
        for (; q < parts; ++q) s0 += __ldg(src + (long long)q * G + i);
        g[i] = (s0 + s1) + (s2 + s3);
    }
    __syncthreads();
    finish_theta<N, MODE>(g, g + round4(G), A + (long long)th * G, nC, st, basis, d,
                          dtheta + (long long)th * d);
}

cudaError_t launch_finalize(const Tess &t, int nsteps, int mode, const float *partials, int parts,
                            const float *A, const float *basis, int d, int n_theta,
                            float *dtheta, cudaStream_t s) {
    if (n_theta == 0) return cudaSuccess;
    const int P = t.ndim * (t.ndim + 1);
    const int block = 256;
    const size_t smem = ((size_t)round4(t.nC * P) + block) * sizeof(float);
    const Steps st = make_steps(nsteps);
#define CPAB_FIN(N, M)                                                                         \
    {                                                                                          \
        auto kern = k_finalize<N, M>;                                                          \
        if (smem > 48 * 1024) {                                                                \
            cudaError_t e = cudaFuncSetAttribute(                                              \
                kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);                 \
            if (e != cudaSuccess) return e;                                                    \
        }                                                                                      \
        kern<<<n_theta, block, smem, s>>>(t.nC, st, partials, parts, A, basis, d, dtheta);     \
        return cudaGetLastError();                                                             \
    }
    if (mode == kFinalizeDirect) {   // the partials are dL/dA (exact-flow adjoint)
        switch (t.ndim) {
            case 1: CPAB_FIN(1, 3)
            case 2: CPAB_FIN(2, 3)
            default: CPAB_FIN(3, 3)
        }
    }
    if (mode != 1) {   // modes 0 and 2: the midpoint sensitivity's cell map
        switch (t.ndim) {
            case 1: CPAB_FIN(1, 0)
            case 2: CPAB_FIN(2, 0)
            default: CPAB_FIN(3, 0)
        }
    }
    switch (t.ndim) {
        case 1: CPAB_FIN(1, 1)
        case 2: CPAB_FIN(2, 1)
        default: CPAB_FIN(3, 1)
    }
#undef CPAB_FIN
}

}  // namespace cpab
