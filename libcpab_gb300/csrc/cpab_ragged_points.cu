// Ragged point sets of any dimension: S sets of points (SoA [ndim, total],
// set s = columns offsets[s] .. offsets[s+1]), each moved by its own theta --
// transform_grid of many (theta, point set) pairs with uneven sizes in one
// persistent launch.  The reference has no such entry point: it needs one
// transform_grid call per set (libcpab/pytorch/transformer.py:72-87), or one
// call on sets padded to a common size.
//
// Same structure as the 1D series kernels (cpab_ragged.cuh): warp tiles of one
// set, the set's tables restaged into the warp's own shared-memory slice when
// the set changes, per-(warp, set) partial slots for a deterministic dtheta.
// The forward integrates PPT points per lane with the compensated update of
// k_integrate; the backward runs the trajectory adjoint of cpab_adjoint.cuh
// (logged forward, segment rebuild, reverse sweep with warp flushes) and
// returns dtheta per set and, optionally, dL/dpoints.  Warp coherence comes
// from the caller's point order; the Python layer can bucket each set's
// points by starting cell (a stable sort) before the launch.
#include "cpab_ragged.cuh"

namespace cpab {

template <int N, int PPT>
__global__ void __launch_bounds__(256)
    k_ragged_points_forward(Tess t, int nsteps, int S, const long long *__restrict__ off,
                            const int *__restrict__ tile_off, const float *__restrict__ E,
                            long long total, const float *__restrict__ points,
                            float *__restrict__ out, unsigned long long *ties, unsigned *err) {
    constexpr int P = N * (N + 1);
    constexpr int TPW = 32 * PPT;
    extern __shared__ float4 smem4[];
    const int G = t.nC * P, Gr = round4(G);
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    float *tab = reinterpret_cast<float *>(smem4) + (size_t)wib * Gr;
    const int TW = gridDim.x * (blockDim.x >> 5);
    const int w = blockIdx.x * (blockDim.x >> 5) + wib;
    const int TT = __ldg(tile_off + S);
    const int K = (TT + TW - 1) / TW;
    const long long t0 = (long long)w * K;
    const int t1 = (int)min(t0 + K, (long long)TT);
    if (t0 >= t1) return;
    int s = find_series(tile_off, S, (int)t0);
    int s_end = __ldg(tile_off + s + 1);
    bool staged = false;
    for (int tl = (int)t0; tl < t1; ++tl) {
        if (tl >= s_end || !staged) {
            while (tl >= s_end) s_end = __ldg(tile_off + (++s) + 1);
            __syncwarp();
            for (int i = lane; i < G; i += 32) tab[i] = __ldg(E + (long long)s * G + i);
            __syncwarp();
            staged = true;
        }
        const long long base = __ldg(off + s);
        const int L = (int)(__ldg(off + s + 1) - base);
        const int j0 = (tl - __ldg(tile_off + s)) * TPW;
        float p[PPT][N];
        int j[PPT];
#pragma unroll
        for (int k = 0; k < PPT; ++k) {
            j[k] = j0 + k * 32 + lane;
#pragma unroll
            for (int r = 0; r < N; ++r)
                p[k][r] = (j[k] < L) ? __ldg(points + r * total + base + j[k]) : 0.5f;
        }
        for (int st = 0; st < nsteps; ++st) {
#pragma unroll
            for (int k = 0; k < PPT; ++k) {
                int c = find_cell<N>(p[k], t, ties);
                float M[P], y[N];
                load_cell<N>(tab, c, M);
                affine_apply<N>(M, p[k], y);
#pragma unroll
                for (int r = 0; r < N; ++r) p[k][r] += y[r];
            }
        }
#pragma unroll
        for (int k = 0; k < PPT; ++k) {
            if (j[k] >= L) continue;
#pragma unroll
            for (int r = 0; r < N; ++r) out[r * total + base + j[k]] = p[k][r];
        }
    }
}

// Per-warp slice (floats): tab [Gr] (A in mode 0, E in mode 1), dtab, gw [Gr].
template <int N>
__host__ __device__ inline int points_warp_floats(int nC) {
    const int Gr = round4(nC * N * (N + 1));
    return 2 * Gr + dtab_floats<N>(nC);
}

template <int N, typename CT>
__host__ __device__ inline size_t points_adjoint_smem(int nC, int nsteps, int block) {
    const int nseg = (nsteps + kSeg - 1) / kSeg;
    const size_t b = (size_t)(block / 32) * points_warp_floats<N>(nC) * 4 +
                     (size_t)nseg * N * block * 4 + (size_t)kSeg * N * block * 4 +
                     (size_t)nsteps * block * sizeof(CT);
    return (b + 15) & ~(size_t)15;
}

template <int N, int MODE, typename CT>
__global__ void __launch_bounds__(256, 3)
    k_ragged_points_adjoint(Tess t, int nsteps, Steps st, int S, const long long *__restrict__ off,
                            const int *__restrict__ tile_off, int ppt,
                            const float *__restrict__ table, long long total,
                            const float *__restrict__ points, const float *__restrict__ gout,
                            float *__restrict__ dpoints, float *__restrict__ partials,
                            unsigned long long *ties, unsigned *err) {
    constexpr int P = N * (N + 1);
    extern __shared__ float4 smem4[];
    const int B = blockDim.x, W = B / 32;
    const int G = t.nC * P, Gr = round4(G);
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int nseg = (nsteps + kSeg - 1) / kSeg;
    float *base_f = reinterpret_cast<float *>(smem4);
    float *mine = base_f + (size_t)wib * points_warp_floats<N>(t.nC);
    AdjSmem<N, CT> sm;
    sm.tab = mine;
    sm.gw = mine + Gr;
    sm.dtab = sm.gw + Gr;
    sm.mtab = mtab_of<N>(sm.dtab, t.nC);
    sm.ck = base_f + (size_t)W * points_warp_floats<N>(t.nC);
    sm.pb = sm.ck + (size_t)nseg * N * B;
    sm.cl = reinterpret_cast<CT *>(sm.pb + (size_t)kSeg * N * B);

    const int TW = gridDim.x * W;
    const int w = blockIdx.x * W + wib;
    const int TT = __ldg(tile_off + S);
    const int K = (TT + TW - 1) / TW;
    const long long t0 = (long long)w * K;
    const int t1 = (int)min(t0 + K, (long long)TT);
    if (t0 >= t1) return;   // warp-uniform; no block-level barrier follows
    const int tpw = 32 * ppt;
    int s = find_series(tile_off, S, (int)t0);
    int s_end = __ldg(tile_off + s + 1);

    auto stage = [&](int sid) {
        __syncwarp();
        const float *src = table + (long long)sid * G;
        for (int i = lane; i < G; i += 32) sm.tab[i] = __ldg(src + i);
        for (int i = lane; i < Gr; i += 32) sm.gw[i] = 0.f;
        __syncwarp();
        build_dtab<N, MODE>(sm.tab, sm.dtab, t.nC, st, lane, 32);
        __syncwarp();
    };
    auto finish = [&](int sid) {
        __syncwarp();
        const long long slot = (long long)w + sid;
        for (int i = lane; i < G; i += 32) partials[slot * G + i] = sm.gw[i];
    };

    stage(s);
    for (int tl = (int)t0; tl < t1; ++tl) {
        if (tl >= s_end) {
            finish(s);
            while (tl >= s_end) s_end = __ldg(tile_off + (++s) + 1);
            stage(s);
        }
        const long long base = __ldg(off + s);
        const int L = (int)(__ldg(off + s + 1) - base);
        const int j0 = (tl - __ldg(tile_off + s)) * tpw;
#pragma unroll 1
        for (int k = 0; k < ppt; ++k) {
            const int j = j0 + k * 32 + lane;
            const bool live = j < L;
            float p[N], lam[N];
#pragma unroll
            for (int r = 0; r < N; ++r) {
                p[r] = live ? __ldg(points + r * total + base + j) : 0.5f;
                lam[r] = live ? __ldg(gout + r * total + base + j) : 0.f;
            }
            logged_forward<N, MODE, CT>(sm, t, nsteps, st, p, ties, err);
            reverse_sweep<N, MODE, CT>(sm, nsteps, st, live, lam, sm.gw);
            if (dpoints && live) {
#pragma unroll
                for (int r = 0; r < N; ++r) dpoints[r * total + base + j] = lam[r];
            }
        }
    }
    finish(s);
}

// ------------------------------- host side -----------------------------------
size_t ragged_points_workspace_bytes(const Tess &t, int S) {
    const size_t tiles = ((size_t)(S + 1) * 4 + 255) & ~(size_t)255;
    const size_t slots = (size_t)num_sms() * 64 + (size_t)S;
    const size_t P = (size_t)t.ndim * (t.ndim + 1);
    return tiles + ((slots * t.nC * P * 4 + 255) & ~(size_t)255);
}

static void points_carve(int S, void *ws, int **tile_off, float **partials) {
    char *p = static_cast<char *>(ws);
    const size_t tiles = ((size_t)(S + 1) * 4 + 255) & ~(size_t)255;
    *tile_off = reinterpret_cast<int *>(p);
    *partials = reinterpret_cast<float *>(p + tiles);
}

template <int N, int PPT>
static cudaError_t launch_rpf_t(const Tess &t, int nsteps, int S, const long long *off,
                                const int *tile_off, const float *E, long long total,
                                const float *points, float *out, unsigned long long *ties,
                                unsigned *err, cudaStream_t s, int block) {
    auto kern = k_ragged_points_forward<N, PPT>;
    const size_t smem = (size_t)(block / 32) * round4(t.nC * N * (N + 1)) * 4;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
    }
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, smem);
    if (per_sm <= 0) return cudaErrorInvalidConfiguration;
    kern<<<num_sms() * per_sm, block, smem, s>>>(t, nsteps, S, off, tile_off, E, total, points,
                                                  out, ties, err);
    return cudaGetLastError();
}

template <int N>
static cudaError_t launch_rpf_n(int ppt, const Tess &t, int nsteps, int S, const long long *off,
                                const int *tile_off, const float *E, long long total,
                                const float *points, float *out, unsigned long long *ties,
                                unsigned *err, cudaStream_t s, int block) {
    switch (ppt) {
        case 1: return launch_rpf_t<N, 1>(t, nsteps, S, off, tile_off, E, total, points, out, ties, err, s, block);
        case 2: return launch_rpf_t<N, 2>(t, nsteps, S, off, tile_off, E, total, points, out, ties, err, s, block);
        default: return launch_rpf_t<N, 4>(t, nsteps, S, off, tile_off, E, total, points, out, ties, err, s, block);
    }
}

cudaError_t launch_ragged_points_forward(const Tess &t, int nsteps, int S, const long long *off,
                                         long long total, const float *E, const float *points,
                                         float *out, void *ws, unsigned long long *ties,
                                         unsigned *err, cudaStream_t s, const LaunchShape *force) {
    int *tile_off;
    float *partials;
    points_carve(S, ws, &tile_off, &partials);
    if (S == 0) return cudaSuccess;
    // Default: 256 threads, 2 points per lane; or the autotuned / forced shape.
    LaunchShape sh;
    if (force) {
        sh = *force;
    } else if (!tuned_get(kTunePointsForward, tune_key(t, nsteps, 0, S, total, 0), &sh)) {
        sh.block = 256;
        sh.ppt = 2;
    }
    if (sh.block < 32 || sh.block > 256 || sh.block % 32 ||
        (sh.ppt != 1 && sh.ppt != 2 && sh.ppt != 4))
        return cudaErrorInvalidConfiguration;
    cudaError_t e = launch_ragged_plan(S, off, total, 32 * sh.ppt, tile_off, err, s);
    if (e != cudaSuccess) return e;
    switch (t.ndim) {
        case 1: return launch_rpf_n<1>(sh.ppt, t, nsteps, S, off, tile_off, E, total, points, out, ties, err, s, sh.block);
        case 2: return launch_rpf_n<2>(sh.ppt, t, nsteps, S, off, tile_off, E, total, points, out, ties, err, s, sh.block);
        default: return launch_rpf_n<3>(sh.ppt, t, nsteps, S, off, tile_off, E, total, points, out, ties, err, s, sh.block);
    }
}

// Largest block size whose shared memory fits (0: none).
// force_block > 0: that block size if it fits, else 0.
template <int N, typename CT>
static int points_block(const Tess &t, int nsteps, int force_block) {
    int dev = 0, max_optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (max_optin <= 0) max_optin = 48 * 1024;
    const int cands[3] = {256, 128, 64};
    for (int i = 0; i < 3; ++i) {
        if (force_block > 0 && cands[i] != force_block) continue;
        if (points_adjoint_smem<N, CT>(t.nC, nsteps, cands[i]) <= (size_t)max_optin)
            return cands[i];
    }
    return 0;
}

template <int N, int MODE, typename CT>
static cudaError_t launch_rpa_t(const Tess &t, int nsteps, int S, const long long *off,
                                const int *tile_off, const float *A, const float *E,
                                long long total, const float *points, const float *gout,
                                float *dpoints, float *partials, const float *basis, int d,
                                float *dtheta, unsigned long long *ties, unsigned *err,
                                cudaStream_t s, int force_block) {
    const int block = points_block<N, CT>(t, nsteps, force_block);
    if (!block) return cudaErrorInvalidConfiguration;
    auto kern = k_ragged_points_adjoint<N, MODE, CT>;
    const size_t smem = points_adjoint_smem<N, CT>(t.nC, nsteps, block);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, smem);
    if (per_sm <= 0) return cudaErrorInvalidConfiguration;
    const int W = block / 32;
    // partial slots are sized for at most 64 resident warps per SM
    const int grid = min(num_sms() * per_sm, num_sms() * 64 / W);
    const Steps st = make_steps(nsteps);
    kern<<<grid, block, smem, s>>>(t, nsteps, st, S, off, tile_off, 1,
                                   MODE == 1 ? E : A, total, points, gout, dpoints, partials,
                                   ties, err);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (d == 0 || !dtheta) return cudaSuccess;
    auto fin = k_ragged_finalize<N, MODE>;
    const size_t fsmem = ((size_t)round4(t.nC * N * (N + 1)) + 256) * sizeof(float);
    if (fsmem > 48 * 1024) {
        e = cudaFuncSetAttribute(fin, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fsmem);
        if (e != cudaSuccess) return e;
    }
    fin<<<S, 256, fsmem, s>>>(t.nC, st, S, tile_off, grid * W, partials, nullptr, A, basis, d,
                              dtheta, nullptr);
    return cudaGetLastError();
}

cudaError_t launch_ragged_points_backward(const Tess &t, int nsteps, int mode, int S,
                                          const long long *off, long long total, const float *A,
                                          const float *E, const float *points,
                                          const float *gout, float *dpoints, const float *basis,
                                          int d, float *dtheta, void *ws,
                                          unsigned long long *ties, unsigned *err,
                                          cudaStream_t s, const LaunchShape *force) {
    int *tile_off;
    float *partials;
    points_carve(S, ws, &tile_off, &partials);
    if (S == 0) return cudaSuccess;
    // Default: the largest block whose shared memory fits; or the autotuned /
    // forced block size (64, 128 or 256 threads).
    LaunchShape sh;
    if (force) sh = *force;
    else tuned_get(kTunePointsBackward, tune_key(t, nsteps, mode, S, total, 0), &sh);
    if (sh.block != 0 && sh.block != 64 && sh.block != 128 && sh.block != 256)
        return cudaErrorInvalidConfiguration;
    const int fb = sh.block;
    cudaError_t e = launch_ragged_plan(S, off, total, 32, tile_off, err, s);
    if (e != cudaSuccess) return e;
    const bool small = t.nC <= 256;
#define CPAB_RPA(N)                                                                                \
    if (mode == 0)                                                                                 \
        return small ? launch_rpa_t<N, 0, uint8_t>(t, nsteps, S, off, tile_off, A, E, total,       \
                                                   points, gout, dpoints, partials, basis, d,      \
                                                   dtheta, ties, err, s, fb)                       \
                     : launch_rpa_t<N, 0, uint16_t>(t, nsteps, S, off, tile_off, A, E, total,      \
                                                    points, gout, dpoints, partials, basis, d,     \
                                                    dtheta, ties, err, s, fb);                     \
    if (mode == 2)                                                                                 \
        return small ? launch_rpa_t<N, 2, uint8_t>(t, nsteps, S, off, tile_off, A, E, total,       \
                                                   points, gout, dpoints, partials, basis, d,      \
                                                   dtheta, ties, err, s, fb)                       \
                     : launch_rpa_t<N, 2, uint16_t>(t, nsteps, S, off, tile_off, A, E, total,      \
                                                    points, gout, dpoints, partials, basis, d,     \
                                                    dtheta, ties, err, s, fb);                     \
    return small ? launch_rpa_t<N, 1, uint8_t>(t, nsteps, S, off, tile_off, A, E, total, points,   \
                                               gout, dpoints, partials, basis, d, dtheta, ties,    \
                                               err, s, fb)                                         \
                 : launch_rpa_t<N, 1, uint16_t>(t, nsteps, S, off, tile_off, A, E, total,          \
                                                points, gout, dpoints, partials, basis, d,         \
                                                dtheta, ties, err, s, fb);
    switch (t.ndim) {
        case 1: { CPAB_RPA(1) }
        case 2: { CPAB_RPA(2) }
        default: { CPAB_RPA(3) }
    }
#undef CPAB_RPA
}

}  // namespace cpab
