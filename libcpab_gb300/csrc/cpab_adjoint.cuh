// Device helpers shared by the adjoint kernels (cpab_adjoint.cu) and the
// fused transform_data backward (cpab_fused.cu).  The scheme is described at
// the top of cpab_adjoint.cu.
#pragma once
#include <map>
#include <mutex>
#include <tuple>

#include "cpab_launch.h"
#include "cpab_midpoint.cuh"

namespace cpab {

constexpr int kSeg = 10;

// The per-cell adjoint table (build_dtab) is two arrays: the N x N
// propagators D (row stride dtab_stride, 16-byte aligned rows for the vector
// loads in 2D and 3D), then the N-float translations of the midpoint maps
// (row stride mtab_stride) starting at mtab_of.
template <int N>
__host__ __device__ constexpr int dtab_stride() { return N == 1 ? 1 : (N == 2 ? 4 : 12); }
template <int N>
__host__ __device__ constexpr int mtab_stride() { return N == 1 ? 1 : (N == 2 ? 2 : 4); }

__host__ __device__ inline int round4(int x) { return (x + 3) & ~3; }

template <int N>
__host__ __device__ inline int dtab_floats(int nC) {
    return round4(nC * dtab_stride<N>()) + round4(nC * mtab_stride<N>());
}
template <int N>
__host__ __device__ inline float *mtab_of(float *dtab, int nC) {
    return dtab + round4(nC * dtab_stride<N>());
}

// The midpoint step of an affine field is itself affine,
// p + h A~(p~ + h/2 A~ p~) = p + (h A~ + h^2/2 A~^2) p~ (A~ = [A; 0]): one map
// per cell.  The reverse sweep rebuilds segment positions with it (from the
// exactly stepped checkpoints of the forward sweep: positions within a few
// ulp of the reference's, which only the sums of lambda p~^T see).
template <int N>
__device__ __forceinline__ void load_dtab(const float *dtab, int c, float (&D)[N * N]);

template <int N>
__device__ __forceinline__ void mid_map_step(const float *dtab, const float *mtab, int c,
                                             float (&p)[N]) {
    float D[N * N], m[N];
    load_dtab<N>(dtab, c, D);
    const float *ms = mtab + c * mtab_stride<N>();
    if constexpr (N == 1) {
        m[0] = ms[0];
    } else if constexpr (N == 2) {
        const float2 b = *reinterpret_cast<const float2 *>(ms);
        m[0] = b.x; m[1] = b.y;
    } else {
        const float4 b = *reinterpret_cast<const float4 *>(ms);
        m[0] = b.x; m[1] = b.y; m[2] = b.z;
    }
    float y[N];
#pragma unroll
    for (int r = 0; r < N; ++r) {
        float acc = m[r];
#pragma unroll
        for (int k = 0; k < N; ++k) acc = fmaf(D[r * N + k], p[k], acc);
        y[r] = acc;
    }
#pragma unroll
    for (int r = 0; r < N; ++r) p[r] += y[r];
}

// One forward step of the trajectory that the adjoint differentiates: the
// reference's midpoint rule in modes 0 and 2 (tab holds A), the compensated
// step p += E [p; 1] of k_integrate in mode 1 (tab holds E).  Mode 2's
// logged forward takes the collapsed midpoint map instead (forward_step).
template <int N, int MODE>
__device__ __forceinline__ void traj_step(const float *tab, int c, const Steps &st,
                                          float (&p)[N]) {
    if constexpr (MODE == 0) {
        float A[N * (N + 1)];
        load_cell<N>(tab, c, A);
        ref_mid_step<N>(A, st, p);
    } else {
        constexpr int P = N * (N + 1);
        float M[P], y[N];
        load_cell<N>(tab, c, M);
        affine_apply<N>(M, p, y);
#pragma unroll
        for (int r = 0; r < N; ++r) p[r] += y[r];
    }
}

// The step the reverse sweep uses to rebuild a segment from its checkpoint:
// the midpoint map from dtab in mode 0, the compensated step in mode 1.
template <int N, int MODE>
__device__ __forceinline__ void rebuild_step(const float *tab, const float *dtab,
                                             const float *mtab, int c, const Steps &st,
                                             float (&p)[N]) {
    if constexpr (MODE != 1) mid_map_step<N>(dtab, mtab, c, p);
    else traj_step<N, 1>(tab, c, st, p);
}

// Per-cell adjoint table: row c of D at dtab[c * dtab_stride<N>()], the N x N
// propagator (row-major) with lambda_n = lambda_{n+1} + D^T lambda_{n+1}:
//     modes 0, 2: D = h A_lin + h^2/2 A_lin^2  (M - I of the midpoint sensitivity)
//     mode 1:     D = E_lin                     (the linear part of T - I)
// and, in modes 0 and 2, row c of mtab = mtab_of(dtab, nC), the translation of the
// midpoint map h a + h^2/2 A_lin a (a = the cell's translation column;
// mid_map_step).  tab keeps A (modes 0, 2) or E (mode 1).  Cells are split over
// the calling threads (first, first + stride, ...); the caller synchronises.
template <int N, int MODE>
__device__ __forceinline__ void build_dtab(const float *tab, float *dtab, int nC, const Steps &st,
                                           int first, int stride) {
    float *mtab = mtab_of<N>(dtab, nC);
    for (int c = first; c < nC; c += stride) {
        const float *a = tab + c * (N * (N + 1));
        float *d = dtab + c * dtab_stride<N>();
        float *m = mtab + c * mtab_stride<N>();
        if constexpr (MODE == 1) {
#pragma unroll
            for (int r = 0; r < N; ++r)
#pragma unroll
                for (int k = 0; k < N; ++k) d[r * N + k] = a[r * (N + 1) + k];
        } else {
#pragma unroll
            for (int r = 0; r < N; ++r)
#pragma unroll
                for (int k = 0; k <= N; ++k) {
                    float s = 0.f;
#pragma unroll
                    for (int q = 0; q < N; ++q) s = fmaf(a[r * (N + 1) + q], a[q * (N + 1) + k], s);
                    const float v = fmaf(st.h, a[r * (N + 1) + k], st.hh2 * s);
                    if (k < N) d[r * N + k] = v;
                    else m[r] = v;
                }
            if constexpr (N == 3) m[3] = 0.f;
        }
    }
}

template <int N>
__device__ __forceinline__ void load_dtab(const float *dtab, int c, float (&D)[N * N]) {
    const float *src = dtab + c * dtab_stride<N>();
    if constexpr (N == 1) {
        D[0] = src[0];
    } else if constexpr (N == 2) {
        const float4 a = *reinterpret_cast<const float4 *>(src);
        D[0] = a.x; D[1] = a.y; D[2] = a.z; D[3] = a.w;
    } else {
        const float4 a = reinterpret_cast<const float4 *>(src)[0];
        const float4 b = reinterpret_cast<const float4 *>(src)[1];
        D[0] = a.x; D[1] = a.y; D[2] = a.z; D[3] = a.w;
        D[4] = b.x; D[5] = b.y; D[6] = b.z; D[7] = b.w;
        D[8] = src[8];
    }
}

// One reverse step: S_c += lambda_{n+1} [p_n;1]^T, then lambda_n from
// lambda_{n+1}.  Both modes accumulate the same outer product; the mode-0
// cell gradient G_c is a fixed linear map of S_c applied in k_finalize.
template <int N>
__device__ __forceinline__ void adjoint_step(const float *dtab, int c, const float (&p)[N],
                                             float (&lam)[N], float (&acc)[N * (N + 1)]) {
    float D[N * N];
    load_dtab<N>(dtab, c, D);
#pragma unroll
    for (int r = 0; r < N; ++r) {
#pragma unroll
        for (int k = 0; k < N; ++k) acc[r * (N + 1) + k] = fmaf(lam[r], p[k], acc[r * (N + 1) + k]);
        acc[r * (N + 1) + N] += lam[r];
    }
    float nl[N];
#pragma unroll
    for (int k = 0; k < N; ++k) {
        float s = lam[k];
#pragma unroll
        for (int r = 0; r < N; ++r) s = fmaf(D[r * N + k], lam[r], s);
        nl[k] = s;
    }
#pragma unroll
    for (int k = 0; k < N; ++k) lam[k] = nl[k];
}

// Shared memory carve-up for the adjoint kernels (floats unless noted):
//   tab   [round4(G)]            cell table of this theta (TMA destination)
//   dtab  [dtab_floats(nC)]      per-cell propagators D and midpoint-map translations
//   gw    [W][round4(G)]         per-warp cell-gradient tables (or in global memory, see
//                                carve_adjoint)
//   ck    [nseg][N][block]       checkpoints (position every kSeg steps)
//   pb    [kSeg][N][block]       positions of the segment being reversed
//   cl    [nsteps][block] (CT)   per-step cells
// Per-thread arrays are indexed [...][block] by thread, so warps access
// consecutive words (no bank conflicts).
template <int N, typename CT>
__host__ __device__ inline size_t adjoint_smem_bytes(int nC, int nsteps, int block,
                                                     bool gw_in_smem = true) {
    constexpr int P = N * (N + 1);
    const int G = round4(nC * P);
    const int Dn = dtab_floats<N>(nC);
    const int W = gw_in_smem ? block / 32 : 0;
    const int nseg = (nsteps + kSeg - 1) / kSeg;
    size_t b = (size_t)G * 4 + (size_t)Dn * 4 + (size_t)W * G * 4 +
               (size_t)nseg * N * block * 4 + (size_t)kSeg * N * block * 4 +
               (size_t)nsteps * block * sizeof(CT);
    return (b + 15) & ~(size_t)15;
}

// Host: the launch shape of an adjoint kernel with the most resident warps per
// SM among 256/128/64 threads per CTA and per-warp tables in shared memory
// (kern_shared) or in global memory (kern_global, may be nullptr; see
// carve_adjoint).  Ties keep shared memory and the larger CTA.  force_block
// (> 0) and force_staging (0 shared, 1 global; -1 either) restrict the
// candidates (the autotuner's shapes).
template <int N, typename CT, typename K>
inline bool adjoint_shape(K kern_shared, K kern_global, int nC, int nsteps, int *block,
                          bool *global_gw, size_t *smem, int *per_sm, int force_block = 0,
                          int force_staging = -1) {
    const bool allow_global = kern_global != nullptr;
    int dev = 0, max_optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (max_optin <= 0) max_optin = 48 * 1024;
    const int cands[3] = {256, 128, 64};
    int best = 0;
    for (int g = 0; g < (allow_global ? 2 : 1); ++g) {
        if (force_staging >= 0 && g != force_staging) continue;
        for (int ci = 0; ci < 3; ++ci) {
            const int b = cands[ci];
            if (force_block > 0 && b != force_block) continue;
            const size_t sm = adjoint_smem_bytes<N, CT>(nC, nsteps, b, g == 0) + 64;
            if (sm > (size_t)max_optin) continue;
            const K kern = g == 0 ? kern_shared : kern_global;
            if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)sm) != cudaSuccess)
                return false;
            int n = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, b, sm);
            if (n * (b / 32) > best) {
                best = n * (b / 32);
                *block = b;
                *global_gw = g == 1;
                *smem = sm;
                *per_sm = n;
            }
        }
    }
    return best > 0;
}

// Host: launch plans are computed once per problem shape and device (the
// occupancy queries behind a plan cost tens of microseconds, on the critical
// path of an eager training step).
struct PlanCache {
    using Key = std::tuple<int, int, int, int, int, int, int, long long, int, int, int>;
    std::mutex mu;
    std::map<Key, AdjointPlan> plans;

    template <typename F>
    bool get(int kind, const Tess &t, int nsteps, int mode, long long nP, int n, int flag,
             AdjointPlan *plan, F compute) {
        int dev = 0;
        cudaGetDevice(&dev);
        const Key key(dev, kind, t.ndim, t.nc[0], t.nc[1], t.nc[2], nsteps, nP, n, mode, flag);
        {
            std::lock_guard<std::mutex> lock(mu);
            auto it = plans.find(key);
            if (it != plans.end()) {
                *plan = it->second;
                return true;
            }
        }
        if (!compute(plan)) return false;
        std::lock_guard<std::mutex> lock(mu);
        if (plans.size() > 4096) plans.clear();
        plans[key] = *plan;
        return true;
    }
};

template <int N, typename CT>
struct AdjSmem {
    float *tab, *dtab, *mtab, *gw, *ck, *pb;
    CT *cl;
};

// GWG: gw_ext is this CTA's W per-warp tables in global memory (L2-resident;
// each warp owns its table, so the flush stays a plain read-add-write), else
// the tables are in shared memory.  Global tables free shared memory for more
// resident warps when the tables are large (3D, hundreds of cells).
template <int N, typename CT, bool GWG = false>
__device__ __forceinline__ AdjSmem<N, CT> carve_adjoint(float *base, int nC, int nsteps,
                                                        float *gw_ext = nullptr) {
    constexpr int P = N * (N + 1);
    const int B = blockDim.x, W = B / 32;
    const int Gr = round4(nC * P);
    const int nseg = (nsteps + kSeg - 1) / kSeg;
    AdjSmem<N, CT> s;
    s.tab = base;
    s.dtab = s.tab + Gr;
    s.mtab = mtab_of<N>(s.dtab, nC);
    float *after = s.dtab + dtab_floats<N>(nC);
    if constexpr (GWG) {   // a template choice keeps the shared-memory path's
        s.gw = gw_ext;     // flushes on shared-memory instructions
        s.ck = after;
    } else {
        s.gw = after;
        s.ck = after + (size_t)W * Gr;
    }
    s.pb = s.ck + (size_t)nseg * N * B;
    s.cl = reinterpret_cast<CT *>(s.pb + (size_t)kSeg * N * B);
    return s;
}

// Sum each contiguous lane run [lo, hi] of sum[] into lane lo (five fixed
// shuffle rounds) and add it there.  All lanes of m call it; runs lie in m.
template <int P>
__device__ __forceinline__ void add_runs(unsigned m, int lo, int hi, float (&sum)[P], float *dst) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
#pragma unroll
        for (int i = 0; i < P; ++i) {
            const float u = __shfl_down_sync(m, sum[i], off);
            if (lane + off <= hi) sum[i] += u;
        }
    }
    if (lane == lo) {
#pragma unroll
        for (int i = 0; i < P; ++i) dst[i] += sum[i];
    }
}

// Add the accumulators of the lanes in m (the lanes leaving a cell at this
// step; called by exactly those lanes) into the warp's cell table.  Lanes that
// leave the same cell at the same step are first summed into their lowest
// lane (a fixed shuffle tree when every group is a contiguous run of more than
// four lanes, else a lane-order chain), so every table element receives at
// most one add per step, in step order, and the summation order depends only
// on the inputs: the sums are reproducible.  In the common case (no two lanes
// share a cell) all lanes add in one pass.
template <int P>
__device__ __forceinline__ void flush_cells(unsigned m, int cell, const float (&acc)[P],
                                            float *warp_tab) {
    const int lane = threadIdx.x & 31;
    float *dst = warp_tab + cell * P;
    const unsigned grp = __match_any_sync(m, cell);
    const unsigned gmax = __reduce_max_sync(m, (unsigned)__popc(grp));
    if (gmax == 1u) {
#pragma unroll
        for (int i = 0; i < P; ++i) dst[i] += acc[i];
        return;
    }
    float sum[P];
#pragma unroll
    for (int i = 0; i < P; ++i) sum[i] = acc[i];
    const int lo = __ffs(grp) - 1;
    const unsigned run = grp >> lo;
    if (gmax > 4u && __all_sync(m, (run & (run + 1u)) == 0u)) {
        // Every group is a contiguous run of lanes [lo, hi] (typical when
        // neighbouring points cross a face together): tree reduction towards
        // the lowest lane in five fixed shuffle rounds.
        add_runs<P>(m, lo, 31 - __clz(grp), sum, dst);
        return;
    }
    unsigned rest = grp & (grp - 1u);        // the other members, lowest first
    for (unsigned k = 1; k < gmax; ++k) {
        const int src = rest ? __ffs(rest) - 1 : lane;
#pragma unroll
        for (int i = 0; i < P; ++i) {
            const float u = __shfl_sync(m, acc[i], src);
            if (rest) sum[i] += u;
        }
        rest &= rest - 1u;
    }
    if (lane == __ffs(grp) - 1) {
#pragma unroll
        for (int i = 0; i < P; ++i) dst[i] += sum[i];
    }
}

// Warp-level flush: lanes with flush = true add their accumulators for
// `cell`.  Called by all lanes of the warp.
template <int P>
__device__ __forceinline__ void warp_flush(bool flush, int cell, const float (&acc)[P],
                                           float *warp_tab) {
    const unsigned m = __ballot_sync(0xffffffffu, flush);
    if (m) {
        if (flush) flush_cells<P>(m, cell, acc, warp_tab);
        __syncwarp();
    }
}

// 1D variant of warp_flush.  A 1D flow keeps the order of points, so the
// lanes of a warp holding consecutive points of a sorted grid (the ragged
// series) sit in non-decreasing cells: equal cells form contiguous lane runs.
// Then every lane takes part in a fixed five-round shuffle tree over its run
// (non-flushing lanes add zeros) and the run's lowest lane adds the sum if
// any lane of the run flushes: the same one-add-per-element-per-step
// discipline as flush_cells, without match.any.  Unsorted warps use
// warp_flush.  Called by all lanes of the warp.
template <int P>
__device__ __forceinline__ void warp_flush_1d(bool flush, int cell, const float (&acc)[P],
                                              float *warp_tab) {
    const unsigned fm = __ballot_sync(0xffffffffu, flush);
    if (!fm) return;
    const int lane = threadIdx.x & 31;
    const int prev = __shfl_up_sync(0xffffffffu, cell, 1);
    if (__any_sync(0xffffffffu, lane > 0 && prev > cell)) {
        warp_flush<P>(flush, cell, acc, warp_tab);
        return;
    }
    const unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || prev != cell);
    const unsigned le = 0xffffffffu >> (31 - lane);            // lanes <= lane
    const int lo = 31 - __clz(heads & le);
    const unsigned above = heads & ~le;
    const int hi = above ? __ffs(above) - 2 : 31;
    float sum[P];
#pragma unroll
    for (int i = 0; i < P; ++i) sum[i] = flush ? acc[i] : 0.f;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
#pragma unroll
        for (int i = 0; i < P; ++i) {
            const float u = __shfl_down_sync(0xffffffffu, sum[i], off);
            if (lane + off <= hi) sum[i] += u;
        }
    }
    const unsigned run = (hi == 31 ? 0xffffffffu : ((1u << (hi + 1)) - 1u)) & ~((1u << lo) - 1u);
    if (lane == lo && (fm & run)) {
        float *dst = warp_tab + cell * P;
#pragma unroll
        for (int i = 0; i < P; ++i) dst[i] += sum[i];
    }
    __syncwarp();
}

// Where reverse_sweep puts a lane's accumulated dL/dA of a cell when the lane
// leaves it: the warp's cell table, through warp_flush / warp_flush_1d
// (called by all lanes of the warp).
template <int N>
struct WarpTabSink {
    float *warp_tab;
    template <int P>
    __device__ __forceinline__ void operator()(bool flush, int cell,
                                               const float (&acc)[P]) const {
        if constexpr (N == 1) warp_flush_1d<P>(flush, cell, acc, warp_tab);
        else warp_flush<P>(flush, cell, acc, warp_tab);
    }
};

// Reverse sweep of one trajectory whose cells are logged in cl and whose
// checkpoints are in ck; lam holds dL/dp_N on entry and dL/dp_0 on exit.
// Each segment's positions are rebuilt from its checkpoint with the logged
// cells (no lookups) into pb, then walked backwards.  The loops are not
// unrolled: the body stays small enough for the instruction cache.
// Executed by all lanes of the warp (uniform trip counts); sink(flush, cell,
// acc) receives each lane's sum over a run of steps in one cell.
template <int N, int MODE, typename CT, typename Sink>
__device__ __forceinline__ void reverse_sweep_to(const AdjSmem<N, CT> &sm, int nsteps,
                                                 const Steps &st, bool live, float (&lam)[N],
                                                 Sink &sink) {
    constexpr int P = N * (N + 1);
    const int B = blockDim.x, tid = threadIdx.x;
    const int nseg = (nsteps + kSeg - 1) / kSeg;
    float acc[P];
#pragma unroll
    for (int i = 0; i < P; ++i) acc[i] = 0.f;
    int gcell = -1;
    for (int seg = nseg - 1; seg >= 0; --seg) {
        const int n0 = seg * kSeg;
        const int len = min(kSeg, nsteps - n0);
        float x[N];
#pragma unroll
        for (int r = 0; r < N; ++r) x[r] = sm.ck[(seg * N + r) * B + tid];
#pragma unroll 1
        for (int s = 0; s < len; ++s) {
#pragma unroll
            for (int r = 0; r < N; ++r) sm.pb[(s * N + r) * B + tid] = x[r];
            rebuild_step<N, MODE>(sm.tab, sm.dtab, sm.mtab, (int)sm.cl[(n0 + s) * B + tid], st,
                                  x);
        }
#pragma unroll 1
        for (int s = len - 1; s >= 0; --s) {
            const int c = (int)sm.cl[(n0 + s) * B + tid];
            const bool change = c != gcell;
            sink(change && gcell >= 0 && live, gcell, acc);
            if (change) {
                gcell = c;
#pragma unroll
                for (int i = 0; i < P; ++i) acc[i] = 0.f;
            }
            float p[N];
#pragma unroll
            for (int r = 0; r < N; ++r) p[r] = sm.pb[(s * N + r) * B + tid];
            adjoint_step<N>(sm.dtab, c, p, lam, acc);
        }
    }
    sink(gcell >= 0 && live, gcell, acc);
}

template <int N, int MODE, typename CT>
__device__ __forceinline__ void reverse_sweep(const AdjSmem<N, CT> &sm, int nsteps,
                                              const Steps &st, bool live, float (&lam)[N],
                                              float *warp_tab) {
    WarpTabSink<N> sink{warp_tab};
    reverse_sweep_to<N, MODE, CT>(sm, nsteps, st, live, lam, sink);
}

// Sweep with the arithmetic of k_integrate's compensated path,
// p <- p + E_c [p;1], nsteps times.  tabE may be in shared or global memory.
template <int N>
__device__ __forceinline__ void e_sweep(const float *tabE, const Tess &t, int nsteps,
                                        float (&p)[N], unsigned long long *ties, unsigned *err) {
    constexpr int P = N * (N + 1);
    for (int s = 0; s < nsteps; ++s) {
        int c = find_cell<N>(p, t, ties);
        float M[P], y[N];
        load_cell<N>(tabE, c, M);
        affine_apply<N>(M, p, y);
#pragma unroll
        for (int r = 0; r < N; ++r) p[r] += y[r];
    }
}

// Forward sweep that logs cells and checkpoints; p holds p_0 on entry and
// p_N on exit.
template <int N, int MODE, typename CT>
__device__ __forceinline__ void logged_forward(const AdjSmem<N, CT> &sm, const Tess &t,
                                               int nsteps, const Steps &st, float (&p)[N],
                                               unsigned long long *ties, unsigned *err) {
    const int B = blockDim.x, tid = threadIdx.x;
    for (int n0 = 0, seg = 0; n0 < nsteps; n0 += kSeg, ++seg) {
#pragma unroll
        for (int r = 0; r < N; ++r) sm.ck[(seg * N + r) * B + tid] = p[r];
        const int end = min(n0 + kSeg, nsteps);
        for (int n = n0; n < end; ++n) {
            int c = find_cell<N>(p, t, ties);
            sm.cl[n * B + tid] = (CT)c;
            if constexpr (MODE == 2) mid_map_step<N>(sm.dtab, sm.mtab, c, p);
            else traj_step<N, MODE>(sm.tab, c, st, p);
        }
    }
}

// Kernel prologue: stage the cell table, build the propagators and clear the
// per-warp tables.  Returns false (block exits) if staging failed.
template <int N, int MODE, typename CT>
__device__ __forceinline__ bool adjoint_prologue(const AdjSmem<N, CT> &sm, const float *table,
                                                 int nC, const Steps &st, uint64_t *bar,
                                                 unsigned *err) {
    constexpr int P = N * (N + 1);
    const int W = blockDim.x / 32, Gr = round4(nC * P);
    if (!stage_table(sm.tab, table, nC * P, bar, err)) return false;
    build_dtab<N, MODE>(sm.tab, sm.dtab, nC, st, threadIdx.x, blockDim.x);
    for (int i = threadIdx.x; i < W * Gr; i += blockDim.x) sm.gw[i] = 0.f;
    __syncthreads();
    return true;
}

// Kernel epilogue: write this CTA's partial (per-warp tables summed in warp
// order).
template <int N, typename CT>
__device__ __forceinline__ void adjoint_epilogue(const AdjSmem<N, CT> &sm, int nC, float *dst) {
    constexpr int P = N * (N + 1);
    const int B = blockDim.x, W = B / 32, G = nC * P, Gr = round4(G);
    __syncthreads();
    for (int i = threadIdx.x; i < G; i += B) {
        float s = 0.f;
        for (int w = 0; w < W; ++w) s += sm.gw[(size_t)w * Gr + i];
        dst[i] = s;
    }
}

// Frechet derivative of expm at Y in direction E, by a truncated Horner
// recursion on Y/2^s, E/2^s followed by s squarings:
//   R_{k-1} = I + (Y/k) R_k,  dR_{k-1} = (E/k) R_k + (Y/k) dR_k,
//   then  L <- L R + R L,  R <- R R.
// Rout receives R = expm(Y) (the overload without it drops R).
template <int K>
__device__ __forceinline__ void frechet_expm(const float (&Y0)[K][K], const float (&E0)[K][K],
                                             float (&L)[K][K], float (&Rout)[K][K]) {
    float norm = 0.f;
#pragma unroll
    for (int j = 0; j < K; ++j) {
        float s = 0.f;
#pragma unroll
        for (int i = 0; i < K; ++i) s += fabsf(Y0[i][j]);
        norm = fmaxf(norm, s);
    }
    int sq = 0;
    if (norm > 0.5f) sq = min(64, (int)ceilf(log2f(norm / 0.5f)));
    const float sc = ldexpf(1.f, -sq);
    float Y[K][K], E[K][K], R[K][K], D[K][K];
#pragma unroll
    for (int i = 0; i < K; ++i)
#pragma unroll
        for (int j = 0; j < K; ++j) {
            Y[i][j] = Y0[i][j] * sc;
            E[i][j] = E0[i][j] * sc;
            R[i][j] = (i == j) ? 1.f : 0.f;
            D[i][j] = 0.f;
        }
    for (int k = 12; k >= 1; --k) {
        const float r = 1.f / (float)k;
        float nR[K][K], nD[K][K];
#pragma unroll
        for (int i = 0; i < K; ++i)
#pragma unroll
            for (int j = 0; j < K; ++j) {
                float a = 0.f, b = 0.f;
#pragma unroll
                for (int m = 0; m < K; ++m) {
                    a = fmaf(Y[i][m], R[m][j], a);
                    b = fmaf(E[i][m], R[m][j], fmaf(Y[i][m], D[m][j], b));
                }
                nR[i][j] = fmaf(a, r, (i == j) ? 1.f : 0.f);
                nD[i][j] = b * r;
            }
#pragma unroll
        for (int i = 0; i < K; ++i)
#pragma unroll
            for (int j = 0; j < K; ++j) { R[i][j] = nR[i][j]; D[i][j] = nD[i][j]; }
    }
    for (int s = 0; s < sq; ++s) {
        float nR[K][K], nD[K][K];
#pragma unroll
        for (int i = 0; i < K; ++i)
#pragma unroll
            for (int j = 0; j < K; ++j) {
                float a = 0.f, b = 0.f;
#pragma unroll
                for (int m = 0; m < K; ++m) {
                    a = fmaf(R[i][m], R[m][j], a);
                    b = fmaf(D[i][m], R[m][j], fmaf(R[i][m], D[m][j], b));
                }
                nR[i][j] = a;
                nD[i][j] = b;
            }
#pragma unroll
        for (int i = 0; i < K; ++i)
#pragma unroll
            for (int j = 0; j < K; ++j) { R[i][j] = nR[i][j]; D[i][j] = nD[i][j]; }
    }
#pragma unroll
    for (int i = 0; i < K; ++i)
#pragma unroll
        for (int j = 0; j < K; ++j) L[i][j] = D[i][j];
#pragma unroll
    for (int i = 0; i < K; ++i)
#pragma unroll
        for (int j = 0; j < K; ++j) Rout[i][j] = R[i][j];
}

template <int K>
__device__ __forceinline__ void frechet_expm(const float (&Y0)[K][K], const float (&E0)[K][K],
                                             float (&L)[K][K]) {
    float R[K][K];
    frechet_expm<K>(Y0, E0, L, R);
}

// Per-theta tail of the finalize kernels, run by one block after the summed
// cell statistics are in g (shared memory, nC * N*(N+1) floats; red is
// blockDim.x floats of shared scratch): map them to
// dL/dA (mode 0: G = h S (I + h/2 [A;0])^T + h^2/2 A_lin^T S; mode 1: adjoint
// Frechet derivative of expm; mode 3, the exact-flow adjoint: already dL/dA)
// and contract with the basis, dtheta[k] = sum_i B[i, k] dA[i].
template <int N, int MODE>
__device__ __forceinline__ void finish_theta(float *g, float *red, const float *__restrict__ A_th,
                                             int nC, const Steps &st,
                                             const float *__restrict__ basis, int d,
                                             float *__restrict__ dth) {
    constexpr int P = N * (N + 1);
    const int tid = threadIdx.x, B = blockDim.x, G = nC * P;
    if constexpr (MODE == 3) {
        // the exact-flow adjoint's partials are dL/dA already
    } else if constexpr (MODE != 1) {
        // S_c = sum_n lambda_{n+1} [p_n;1]^T  ->
        // G_c = h S_c (I + h/2 [A_c;0])^T + h^2/2 A_lin^T S_c
        for (int c = tid; c < nC; c += B) {
            const float *a = A_th + (long long)c * P;
            float S[N][N + 1], Gc[N][N + 1];
#pragma unroll
            for (int i = 0; i < N; ++i)
#pragma unroll
                for (int j = 0; j <= N; ++j) S[i][j] = g[c * P + i * (N + 1) + j];
#pragma unroll
            for (int i = 0; i < N; ++i)
#pragma unroll
                for (int j = 0; j <= N; ++j) {
                    float x = 0.f, y = 0.f;
                    if (j < N) {
#pragma unroll
                        for (int k = 0; k <= N; ++k) x = fmaf(S[i][k], a[j * (N + 1) + k], x);
                    }
#pragma unroll
                    for (int r = 0; r < N; ++r) y = fmaf(a[r * (N + 1) + i], S[r][j], y);
                    Gc[i][j] = fmaf(st.h, fmaf(st.hh, x, S[i][j]), st.hh2 * y);
                }
#pragma unroll
            for (int i = 0; i < N; ++i)
#pragma unroll
                for (int j = 0; j <= N; ++j) g[c * P + i * (N + 1) + j] = Gc[i][j];
        }
        __syncthreads();
    } else {
        const float dt = st.h;
        // dL/dT_c (top N rows) -> dL/dA_c = dt * [L_exp(X^T, [dL/dT_c; 0])]_{top rows}
        for (int c = tid; c < nC; c += B) {
            const float *a = A_th + (long long)c * P;
            float Y[N + 1][N + 1], E[N + 1][N + 1], L[N + 1][N + 1];
#pragma unroll
            for (int i = 0; i <= N; ++i)
#pragma unroll
                for (int j = 0; j <= N; ++j) {
                    Y[j][i] = (i < N) ? dt * a[i * (N + 1) + j] : 0.f;   // Y = X^T
                    E[i][j] = (i < N) ? g[c * P + i * (N + 1) + j] : 0.f;
                }
            frechet_expm<N + 1>(Y, E, L);
#pragma unroll
            for (int i = 0; i < N; ++i)
#pragma unroll
                for (int j = 0; j <= N; ++j) g[c * P + i * (N + 1) + j] = dt * L[i][j];
        }
        __syncthreads();
    }
    if (d <= 0) return;
    if (d > B) {
        for (int k = tid; k < d; k += B) {
            float acc = 0.f;
            for (int i = 0; i < G; ++i) acc = fmaf(__ldg(basis + (long long)i * d + k), g[i], acc);
            dth[k] = acc;
        }
        return;
    }
    // d <= B: `groups` threads per basis column each take every groups-th row;
    // their partial sums are added in group order (red: B floats of shared
    // memory)
    const int groups = B / d;
    const int k = tid % d, gi = tid / d;
    if (gi < groups) {
        float acc = 0.f;
        for (int i = gi; i < G; i += groups)
            acc = fmaf(__ldg(basis + (long long)i * d + k), g[i], acc);
        red[tid] = acc;
    }
    __syncthreads();
    if (tid < d) {
        float acc = 0.f;
        for (int q = 0; q < groups; ++q) acc += red[q * d + tid];
        dth[tid] = acc;
    }
}

}  // namespace cpab
