// Fused transform_data: meshgrid -> integrate -> sample, and its backward.
//
// The reference's transform_data (libcpab/cpab.py:304-331) is
// uniform_meshgrid -> transform_grid -> interpolate: the transformed grid
// round-trips through global memory between two separate launches (and the
// interpolation itself is ~30 PyTorch launches).  Here one kernel builds each
// grid point from the per-axis meshgrid coordinates (the same torch.linspace
// values the reference uses), integrates it with exactly the arithmetic of
// k_integrate (compensated update), and samples every channel in registers.
// Threads are laid out in output order (last axis fastest), so the output
// writes are coalesced and neighbouring threads read neighbouring pixels.
//
// Backward: one kernel per (image, point) that (1) obtains the final position
// p_N (recomputed along the logged forward pass in "exact" mode, or read back
// from the forward's saved grid in "reference" mode, whose sensitivity is
// taken along the midpoint trajectory), (2) applies the interpolation adjoint
// (scatter into d(data), dL/dp_N through the lerp weights) and (3) runs the
// trajectory adjoint of cpab_adjoint.cuh, emitting per-CTA partial cell
// gradients that launch_finalize contracts with the basis.
#include "cpab_adjoint.cuh"
#include "cpab_interp.cuh"

namespace cpab {

// Axis indices of output element o (last axis fastest) and its grid point.
template <int N>
__device__ __forceinline__ void grid_point(int o, const Geo &g, const float *lin, float (&p)[N]) {
    unsigned idx[N];
    unsigned r = (unsigned)o;
#pragma unroll
    for (int j = N - 1; j >= 0; --j) {
        const unsigned q = fast_div(r, g.dout[j]);
        idx[j] = r - q * g.outsize[j];
        r = q;
    }
    int off = 0;
#pragma unroll
    for (int j = 0; j < N; ++j) {
        p[j] = __ldg(lin + off + idx[j]);
        off += g.outsize[j];
    }
}

template <int N, int PPT>
__global__ void __launch_bounds__(256)
    k_transform_data(Tess t, int nsteps, Geo g, const float *__restrict__ lin,
                     const float *__restrict__ E, int C, const float *__restrict__ data,
                     float *__restrict__ out, float *__restrict__ grid_out, int tiles,
                     unsigned long long *ties, unsigned *err) {
    constexpr int P = N * (N + 1);
    extern __shared__ float4 smem4[];
    __shared__ uint64_t bar;
    float *tab = reinterpret_cast<float *>(smem4);
    const int b = blockIdx.y, tile = blockIdx.x;
    const int G = t.nC * P;
    if (!stage_table(tab, E + (long long)b * G, G, &bar, err)) return;
    float p[PPT][N];
    int o[PPT];
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
        o[j] = (tile * PPT + j) * (int)blockDim.x + (int)threadIdx.x;
        if (o[j] < g.nP) grid_point<N>(o[j], g, lin, p[j]);
        else {
#pragma unroll
            for (int r = 0; r < N; ++r) p[j][r] = 0.5f;
        }
    }
    for (int s = 0; s < nsteps; ++s) {
#pragma unroll
        for (int j = 0; j < PPT; ++j) {
            int c = find_cell<N>(p[j], t, ties);
            float M[P], y[N];
            load_cell<N>(tab, c, M);
            affine_apply<N>(M, p[j], y);
#pragma unroll
            for (int r = 0; r < N; ++r) p[j][r] += y[r];
        }
    }
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
        if (o[j] >= g.nP) continue;
        if (C > 0) {   // C == 0: integrate only (grid_out), sampled later by k_sample_grid
            const Corner<N> cr = corners<N>(p[j], g);
            for (int c = 0; c < C; ++c)
                out[((long long)b * C + c) * g.nP + o[j]] =
                    lerp_corners<N>(data + ((long long)b * C + c) * g.nD, cr);
        }
        if (grid_out) {
#pragma unroll
            for (int r = 0; r < N; ++r) grid_out[((long long)b * N + r) * g.nP + o[j]] = p[j][r];
        }
    }
}

// Sampling half of a split transform_data forward: the epilogue of
// k_transform_data applied to a grid saved in image order (grid_out of a
// C = 0 launch), so that the images can arrive while the trajectories are
// integrated.  Same arithmetic as the fused epilogue: bit-identical output.
template <int N>
__global__ void __launch_bounds__(256)
    k_sample_grid(Geo g, const float *__restrict__ grid, int C, const float *__restrict__ data,
                  float *__restrict__ out) {
    const int b = blockIdx.y;
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= g.nP) return;
    float p[N];
#pragma unroll
    for (int r = 0; r < N; ++r) p[r] = __ldg(grid + ((long long)b * N + r) * g.nP + o);
    const Corner<N> cr = corners<N>(p, g);
    for (int c = 0; c < C; ++c)
        out[((long long)b * C + c) * g.nP + o] =
            lerp_corners<N>(data + ((long long)b * C + c) * g.nD, cr);
}

cudaError_t launch_sample_grid(int ndim, const float *grid, int nb, const float *data, int C,
                               const int *size, const int *outsize, float *out, cudaStream_t s) {
    const Geo g = make_geo(ndim, size, outsize);
    if ((long long)nb * g.nP == 0) return cudaSuccess;
    if (nb > 65535) return cudaErrorInvalidConfiguration;
    const dim3 grid_dim((unsigned)((g.nP + 255) / 256), (unsigned)nb);
    switch (ndim) {
        case 1: k_sample_grid<1><<<grid_dim, 256, 0, s>>>(g, grid, C, data, out); break;
        case 2: k_sample_grid<2><<<grid_dim, 256, 0, s>>>(g, grid, C, data, out); break;
        default: k_sample_grid<3><<<grid_dim, 256, 0, s>>>(g, grid, C, data, out); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_transform_data(const Tess &t, int nsteps, const float *lin, const int *outsize,
                                  const float *E, int nb, const float *data, int C,
                                  const int *size, float *out, float *grid_out,
                                  unsigned long long *ties, unsigned *err, cudaStream_t s,
                                  const LaunchShape *force) {
    const Geo g = make_geo(t.ndim, size, outsize);
    if ((long long)nb * g.nP == 0) return cudaSuccess;
    // Default: 256 threads, two points per thread once there is enough work
    // to fill the GPU twice; or the autotuned / forced shape.
    LaunchShape sh;
    if (force) {
        sh = *force;
    } else if (!tuned_get(kTuneFusedForward, tune_key(t, nsteps, 0, g.nP, nb, C), &sh)) {
        sh.block = 256;
        sh.ppt = (long long)nb * g.nP >= (long long)num_sms() * 2048 * 2 ? 2 : 1;
    }
    if (sh.block < 32 || sh.block > 256 || sh.block % 32 || (sh.ppt != 1 && sh.ppt != 2))
        return cudaErrorInvalidConfiguration;
    const int block = sh.block;
    const bool two = sh.ppt == 2;
    const int ppt = sh.ppt;
    const long long per = (long long)block * ppt;
    const int tiles = (int)((g.nP + per - 1) / per);
    if (nb > 65535) return cudaErrorInvalidConfiguration;   // images on grid y
    const dim3 grid((unsigned)tiles, (unsigned)nb);
    const size_t smem = (size_t)t.nC * t.ndim * (t.ndim + 1) * sizeof(float);
#define CPAB_TD(N, PP)                                                                         \
    {                                                                                          \
        auto kern = k_transform_data<N, PP>;                                                   \
        if (smem > 48 * 1024) {                                                                \
            cudaError_t e = cudaFuncSetAttribute(                                              \
                kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);                 \
            if (e != cudaSuccess) return e;                                                    \
        }                                                                                      \
        kern<<<grid, block, smem, s>>>(t, nsteps, g, lin, E, C, data, out, grid_out, \
                                                 tiles, ties, err);                            \
        return cudaGetLastError();                                                             \
    }
    switch (t.ndim) {
        case 1: if (two) CPAB_TD(1, 2) else CPAB_TD(1, 1)
        case 2: if (two) CPAB_TD(2, 2) else CPAB_TD(2, 1)
        default: if (two) CPAB_TD(3, 2) else CPAB_TD(3, 1)
    }
#undef CPAB_TD
}

template <int N, int MODE, typename CT, bool GWG>
__global__ void __launch_bounds__(256)
    k_transform_data_backward(Tess t, int nsteps, Steps st, Geo g, PreStages pre,
                              const float *__restrict__ lin, const float *__restrict__ table,
                              const float *__restrict__ grid_saved, int C,
                              const float *__restrict__ data, const float *__restrict__ gout,
                              float *__restrict__ ddata, float *__restrict__ partials,
                              float *gw_ext, int parts, int tiles, unsigned long long *ties,
                              unsigned *err) {
    extern __shared__ float4 smem4[];
    __shared__ uint64_t bar;
    const int B = blockDim.x, tid = threadIdx.x;
    const int G = t.nC * N * (N + 1);
    const int b = blockIdx.y, part = blockIdx.x;
    float *gw = GWG ? gw_ext + ((size_t)b * parts + part) * (B / 32) * round4(G) : nullptr;
    const AdjSmem<N, CT> sm =
        carve_adjoint<N, CT, GWG>(reinterpret_cast<float *>(smem4), t.nC, nsteps, gw);

    if (!adjoint_prologue<N, MODE, CT>(sm, table + (long long)b * G, t.nC, st, &bar, err)) return;
    float *warp_tab = sm.gw + (size_t)(tid >> 5) * round4(G);

    for (int tile = part; tile < tiles; tile += parts) {
        const int o = tile * B + tid;
        const bool live = o < g.nP;
        float p[N], pN[N], lam[N];
        if (live) grid_point<N>(o, g, lin, p);
        else {
#pragma unroll
            for (int r = 0; r < N; ++r) p[r] = 0.5f;
        }
        // composition: the transformations before this one move the grid first
#pragma unroll
        for (int k = 0; k < kMaxPre; ++k) {
            if (k >= pre.K) break;
            e_sweep<N>(pre.E[k] + (long long)b * pre.t[k].nC * (N * (N + 1)), pre.t[k],
                       pre.nsteps[k], p, ties, err);
        }
        logged_forward<N, MODE, CT>(sm, t, nsteps, st, p, ties, err);
#pragma unroll
        for (int r = 0; r < N; ++r) {
            if constexpr (MODE == 1) pN[r] = p[r];
            else pN[r] = live ? __ldg(grid_saved + ((long long)b * N + r) * g.nP + o) : 0.5f;
        }
        float gf[N];
#pragma unroll
        for (int r = 0; r < N; ++r) gf[r] = 0.f;
        if (live) {
            const Corner<N> cr = corners<N>(pN, g);
            for (int c = 0; c < C; ++c) {
                const long long plane = ((long long)b * C + c);
                const float w = __ldg(gout + plane * g.nP + o);
                lerp_grads<N>(data + plane * g.nD, cr, w, ddata ? ddata + plane * g.nD : nullptr,
                              gf);
            }
        }
#pragma unroll
        for (int r = 0; r < N; ++r) lam[r] = gf[r] * (float)(g.size[r] - 1);
        reverse_sweep<N, MODE, CT>(sm, nsteps, st, live, lam, warp_tab);
    }
    adjoint_epilogue<N, CT>(sm, t.nC, partials + ((long long)b * parts + part) * G);
}

template <int N, int MODE, typename CT>
static bool plan_td_t(const Tess &t, int nsteps, long long nP, int nb, AdjointPlan *plan,
                      const LaunchShape &sh) {
    int block = 0, per_sm = 0;
    bool global_gw = false;
    size_t smem = 0;
    // global per-warp tables in 2D and 3D, where the tables can be large
    decltype(&k_transform_data_backward<N, MODE, CT, false>) kg = nullptr;
    if constexpr (N >= 2) kg = k_transform_data_backward<N, MODE, CT, true>;
    if (!adjoint_shape<N, CT>(k_transform_data_backward<N, MODE, CT, false>, kg, t.nC, nsteps,
                              &block, &global_gw, &smem, &per_sm, sh.block, sh.staging))
        return false;
    const long long tiles = (nP + block - 1) / block;
    const long long target = 2ll * num_sms() * per_sm;
    long long parts = sh.parts > 0 ? sh.parts : (target + nb - 1) / nb;
    if (parts > tiles) parts = tiles;
    if (parts < 1) parts = 1;
    plan->block = block;
    plan->tiles = (int)tiles;
    plan->parts = (int)parts;
    plan->smem = smem;
    plan->partial_floats = (size_t)nb * parts * t.nC * N * (N + 1);
    plan->gw_floats = global_gw ? (size_t)nb * parts * (block / 32) * round4(t.nC * N * (N + 1))
                                : 0;
    return true;
}

static bool plan_td_uncached(const Tess &t, int nsteps, int mode, long long nP, int nb,
                             AdjointPlan *plan, const LaunchShape &sh) {
    const bool small = t.nC <= 256;
#define CPAB_PLAN(N)                                                                               \
    if (mode != 1)                                                                                 \
        return small ? plan_td_t<N, 0, uint8_t>(t, nsteps, nP, nb, plan, sh)                       \
                     : plan_td_t<N, 0, uint16_t>(t, nsteps, nP, nb, plan, sh);                     \
    return small ? plan_td_t<N, 1, uint8_t>(t, nsteps, nP, nb, plan, sh)                           \
                 : plan_td_t<N, 1, uint16_t>(t, nsteps, nP, nb, plan, sh);
    switch (t.ndim) {
        case 1: { CPAB_PLAN(1) }
        case 2: { CPAB_PLAN(2) }
        default: { CPAB_PLAN(3) }
    }
#undef CPAB_PLAN
}

bool plan_transform_data_backward(const Tess &t, int nsteps, int mode, long long nP, int nb,
                                  AdjointPlan *plan, const LaunchShape *force) {
    LaunchShape sh;
    if (force) return plan_td_uncached(t, nsteps, mode, nP, nb, plan, *force);
    const bool tuned = tuned_get(kTuneFusedBackward, tune_key(t, nsteps, mode, nP, nb, 0), &sh);
    // the cache key carries the tuned shape (0: the planner's own)
    const int flag = tuned ? 1 + (sh.staging + 1) + 4 * (sh.block / 32) + 64 * sh.parts : 0;
    static PlanCache cache;
    return cache.get(1, t, nsteps, mode, nP, nb, flag, plan, [&](AdjointPlan *p) {
        return plan_td_uncached(t, nsteps, mode, nP, nb, p, sh);
    });
}

template <int N, int MODE, typename CT>
static cudaError_t launch_td_bwd_t(const Tess &t, int nsteps, const AdjointPlan &plan,
                                   const Geo &g, const PreStages &pre, const float *lin,
                                   const float *table,
                                   const float *grid_saved, int nb, const float *data, int C,
                                   const float *gout, float *ddata, float *partials,
                                   unsigned long long *ties, unsigned *err, cudaStream_t s) {
    auto kern = k_transform_data_backward<N, MODE, CT, false>;
    if constexpr (N >= 2)
        if (plan.gw_floats) kern = k_transform_data_backward<N, MODE, CT, true>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)plan.smem);
    if (e != cudaSuccess) return e;
    const Steps st = make_steps(nsteps);
    if (nb == 0) return cudaSuccess;
    if (nb > 65535) return cudaErrorInvalidConfiguration;   // images on grid y
    const dim3 grid((unsigned)plan.parts, (unsigned)nb);
    float *gw = plan.gw_floats ? partials + plan.gw_offset() : nullptr;
    kern<<<grid, plan.block, plan.smem, s>>>(t, nsteps, st, g, pre, lin, table, grid_saved, C,
                                                       data, gout, ddata, partials, gw, plan.parts,
                                                       plan.tiles, ties, err);
    return cudaGetLastError();
}

cudaError_t launch_transform_data_backward(const Tess &t, int nsteps, int mode,
                                           const AdjointPlan &plan, const float *lin,
                                           const int *outsize, const float *table,
                                           const float *grid_saved, int nb, const float *data,
                                           int C, const int *size, const float *gout,
                                           float *ddata, float *partials,
                                           unsigned long long *ties, unsigned *err,
                                           cudaStream_t s, const PreStages *pre_in) {
    const Geo g = make_geo(t.ndim, size, outsize);
    PreStages pre;
    pre.K = 0;
    if (pre_in) pre = *pre_in;
    const bool small = t.nC <= 256;
#define CPAB_TDB(N)                                                                             \
    if (mode == 0)                                                                              \
        return small ? launch_td_bwd_t<N, 0, uint8_t>(t, nsteps, plan, g, pre, lin, table,           \
                                                      grid_saved, nb, data, C, gout, ddata,     \
                                                      partials, ties, err, s)                   \
                     : launch_td_bwd_t<N, 0, uint16_t>(t, nsteps, plan, g, pre, lin, table,          \
                                                       grid_saved, nb, data, C, gout, ddata,    \
                                                       partials, ties, err, s);                 \
    if (mode == 2)                                                                              \
        return small ? launch_td_bwd_t<N, 2, uint8_t>(t, nsteps, plan, g, pre, lin, table,           \
                                                      grid_saved, nb, data, C, gout, ddata,     \
                                                      partials, ties, err, s)                   \
                     : launch_td_bwd_t<N, 2, uint16_t>(t, nsteps, plan, g, pre, lin, table,          \
                                                       grid_saved, nb, data, C, gout, ddata,    \
                                                       partials, ties, err, s);                 \
    return small ? launch_td_bwd_t<N, 1, uint8_t>(t, nsteps, plan, g, pre, lin, table, grid_saved,   \
                                                  nb, data, C, gout, ddata, partials, ties,     \
                                                  err, s)                                       \
                 : launch_td_bwd_t<N, 1, uint16_t>(t, nsteps, plan, g, pre, lin, table, grid_saved,  \
                                                   nb, data, C, gout, ddata, partials, ties,    \
                                                   err, s);
    switch (t.ndim) {
        case 1: { CPAB_TDB(1) }
        case 2: { CPAB_TDB(2) }
        default: { CPAB_TDB(3) }
    }
#undef CPAB_TDB
}

}  // namespace cpab
