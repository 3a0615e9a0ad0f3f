// Device helpers shared by the adjoint kernels (cpab_adjoint.cu) and the
// fused transform_data backward (cpab_fused.cu).  The scheme is described at
// the top of cpab_adjoint.cu.
#pragma once
#include "cpab_launch.h"

namespace cpab {

constexpr int kSeg = 10;
// Flush queue: entries per warp, and the row stride of its value array (odd,
// so that the draining lanes, one per component, hit distinct banks).
constexpr int kQueue = 40;
constexpr int kQueueStride = kQueue + 1;

struct Steps {
    float h, hh, hh2;   // 1/N, 1/(2N), 1/(2N^2)
};

// One forward step of the trajectory that the adjoint differentiates.
template <int N, int MODE>
__device__ __forceinline__ void traj_step(const float *tab, int c, const Steps &st,
                                          float (&p)[N]) {
    constexpr int P = N * (N + 1);
    float M[P], y[N];
    load_cell<N>(tab, c, M);
    affine_apply<N>(M, p, y);
    if constexpr (MODE == 1) {
#pragma unroll
        for (int r = 0; r < N; ++r) p[r] += y[r];
    } else {
        float pm[N], vm[N];
#pragma unroll
        for (int r = 0; r < N; ++r) pm[r] = fmaf(st.hh, y[r], p[r]);
        affine_apply<N>(M, pm, vm);
#pragma unroll
        for (int r = 0; r < N; ++r) p[r] = fmaf(st.h, vm[r], p[r]);
    }
}

// Row stride of the per-cell adjoint propagator table (16-byte aligned rows
// for the vector loads).
template <int N>
__host__ __device__ constexpr int dtab_stride() { return N == 1 ? 1 : (N == 2 ? 4 : 12); }

// Per-cell propagator of the adjoint, D with lambda_n = lambda_{n+1} + D^T lambda_{n+1}:
//   mode 0: D = h A_lin + h^2/2 A_lin^2  (M - I of the midpoint sensitivity)
//   mode 1: D = E_lin                     (the linear part of T - I)
// stored row-major, D[r][k] at dtab[c * stride + r * N + k].  Written by the
// whole block; the caller synchronises.
template <int N, int MODE>
__device__ __forceinline__ void build_dtab(const float *tab, float *dtab, int nC, const Steps &st) {
    constexpr int P = N * (N + 1);
    for (int c = threadIdx.x; c < nC; c += blockDim.x) {
        const float *a = tab + c * P;
        float *d = dtab + c * dtab_stride<N>();
#pragma unroll
        for (int r = 0; r < N; ++r)
#pragma unroll
            for (int k = 0; k < N; ++k) {
                if constexpr (MODE == 1) {
                    d[r * N + k] = a[r * (N + 1) + k];
                } else {
                    float s = 0.f;
#pragma unroll
                    for (int m = 0; m < N; ++m) s = fmaf(a[r * (N + 1) + m], a[m * (N + 1) + k], s);
                    d[r * N + k] = fmaf(st.h, a[r * (N + 1) + k], st.hh2 * s);
                }
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

template <typename CT>
__host__ __device__ constexpr int cell_bytes() { return (int)sizeof(CT); }

__host__ __device__ inline int round4(int x) { return (x + 3) & ~3; }

// Shared memory carve-up for the adjoint kernels (floats unless noted):
//   tab   [round4(G)]            cell table of this theta (TMA destination)
//   dtab  [round4(nC*stride)]    per-cell adjoint propagators D
//   gw    [W][round4(G)]         per-warp cell-gradient tables
//   qv    [W][P][kQueueStride]   per-warp flush queue, values
//   qc    [W][kQueue] (int)      per-warp flush queue, cells
//   ck    [nseg][N][block]       checkpoints (position every kSeg steps)
//   pb    [kSeg][N][block]       positions of the segment being reversed
//   cl    [nsteps][block] (CT)   per-step cells
// Per-thread arrays are indexed [...][block] by thread, so warps access
// consecutive words (no bank conflicts).
template <int N, typename CT>
__host__ __device__ inline size_t adjoint_smem_bytes(int nC, int nsteps, int block) {
    constexpr int P = N * (N + 1);
    const int G = round4(nC * P);
    const int Dn = round4(nC * dtab_stride<N>());
    const int W = block / 32;
    const int nseg = (nsteps + kSeg - 1) / kSeg;
    size_t b = (size_t)G * 4 + (size_t)Dn * 4 + (size_t)W * G * 4 +
               (size_t)W * (P * kQueueStride + kQueue) * 4 + (size_t)nseg * N * block * 4 +
               (size_t)kSeg * N * block * 4 + (size_t)nsteps * block * sizeof(CT);
    return (b + 15) & ~(size_t)15;
}

template <int N, typename CT>
struct AdjSmem {
    float *tab, *dtab, *gw, *qv, *ck, *pb;
    int *qc;
    CT *cl;
};

template <int N, typename CT>
__device__ __forceinline__ AdjSmem<N, CT> carve_adjoint(float *base, int nC, int nsteps) {
    constexpr int P = N * (N + 1);
    const int B = blockDim.x, W = B / 32;
    const int Gr = round4(nC * P);
    const int nseg = (nsteps + kSeg - 1) / kSeg;
    AdjSmem<N, CT> s;
    s.tab = base;
    s.dtab = s.tab + Gr;
    s.gw = s.dtab + round4(nC * dtab_stride<N>());
    s.qv = s.gw + (size_t)W * Gr;
    s.qc = reinterpret_cast<int *>(s.qv + (size_t)W * P * kQueueStride);
    s.ck = reinterpret_cast<float *>(s.qc + (size_t)W * kQueue);
    s.pb = s.ck + (size_t)nseg * N * B;
    s.cl = reinterpret_cast<CT *>(s.pb + (size_t)kSeg * N * B);
    return s;
}

// Per-warp flush queue.  A lane that leaves a cell appends (cell, S) in the
// order (step, lane); when fewer than 32 free entries remain the warp adds
// the entries into its cell-gradient table in queue order (one lane per
// component), so the sums are reproducible.  `n` is warp-uniform.
template <int P>
struct FlushQueue {
    float *qv;   // [P][kQueueStride]
    int *qc;     // [kQueue]
    float *tab;  // warp's cell-gradient table
    int n;
};

template <int P>
__device__ __forceinline__ void queue_drain(FlushQueue<P> &q) {
    __syncwarp();
    const int lane = threadIdx.x & 31;
    if (lane < P) {
        const float *src = q.qv + lane * kQueueStride;
        float *dst = q.tab + lane;
#pragma unroll 1
        for (int e = 0; e < q.n; ++e) dst[q.qc[e] * P] += src[e];
    }
    __syncwarp();
    q.n = 0;
}

// Append the accumulators of the lanes in m (warp-uniform mask; called by all
// lanes of the warp).
template <int P>
__device__ __forceinline__ void queue_push(FlushQueue<P> &q, unsigned m, int cell,
                                           const float (&acc)[P]) {
    const int lane = threadIdx.x & 31;
    if ((m >> lane) & 1u) {
        const int e = q.n + __popc(m & ((1u << lane) - 1u));
#pragma unroll
        for (int i = 0; i < P; ++i) q.qv[i * kQueueStride + e] = acc[i];
        q.qc[e] = cell;
    }
    q.n += __popc(m);
    if (q.n > kQueue - 32) queue_drain<P>(q);
}

// Reverse sweep of one trajectory whose cells are logged in cl and whose
// checkpoints are in ck; lam holds dL/dp_N on entry and dL/dp_0 on exit.
// Each segment's positions are rebuilt from its checkpoint with the logged
// cells (no lookups) into pb, then walked backwards.  The loops are not
// unrolled: the body stays small enough for the instruction cache.
// Executed by all lanes of the warp (uniform trip counts).
template <int N, int MODE, typename CT>
__device__ __forceinline__ void reverse_sweep(const AdjSmem<N, CT> &sm, int nsteps,
                                              const Steps &st, bool live, float (&lam)[N],
                                              FlushQueue<N * (N + 1)> &q) {
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
            traj_step<N, MODE>(sm.tab, (int)sm.cl[(n0 + s) * B + tid], st, x);
        }
#pragma unroll 1
        for (int s = len - 1; s >= 0; --s) {
            const int c = (int)sm.cl[(n0 + s) * B + tid];
            const bool change = c != gcell;
            const unsigned m = __ballot_sync(0xffffffffu, change && gcell >= 0 && live);
            if (m) queue_push<P>(q, m, gcell, acc);
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
    const unsigned m = __ballot_sync(0xffffffffu, gcell >= 0 && live);
    if (m) queue_push<P>(q, m, gcell, acc);
}

// Forward sweep that logs cells and checkpoints; p holds p_0 on entry and
// p_N on exit.
template <int N, int MODE, typename CT>
__device__ __forceinline__ void logged_forward(const AdjSmem<N, CT> &sm, const Tess &t,
                                               int nsteps, const Steps &st, float (&p)[N],
                                               unsigned long long *ties, unsigned *err) {
    const int B = blockDim.x, tid = threadIdx.x;
    for (int n = 0; n < nsteps; ++n) {
        if (n % kSeg == 0) {
#pragma unroll
            for (int r = 0; r < N; ++r) sm.ck[((n / kSeg) * N + r) * B + tid] = p[r];
        }
        int c = find_cell<N>(p, t, ties);
        if ((unsigned)c >= (unsigned)t.nC) {
            raise_error(err, kErrBadCell);
            c = 0;
        }
        sm.cl[n * B + tid] = (CT)c;
        traj_step<N, MODE>(sm.tab, c, st, p);
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
    build_dtab<N, MODE>(sm.tab, sm.dtab, nC, st);
    for (int i = threadIdx.x; i < W * Gr; i += blockDim.x) sm.gw[i] = 0.f;
    __syncthreads();
    return true;
}

template <int N, typename CT>
__device__ __forceinline__ FlushQueue<N * (N + 1)> warp_queue(const AdjSmem<N, CT> &sm, int nC) {
    constexpr int P = N * (N + 1);
    const int w = threadIdx.x >> 5;
    FlushQueue<P> q;
    q.qv = sm.qv + (size_t)w * P * kQueueStride;
    q.qc = sm.qc + (size_t)w * kQueue;
    q.tab = sm.gw + (size_t)w * round4(nC * P);
    q.n = 0;
    return q;
}

// Kernel epilogue: drain every warp's queue, then write this CTA's partial
// (per-warp tables summed in warp order).
template <int N, typename CT>
__device__ __forceinline__ void adjoint_epilogue(const AdjSmem<N, CT> &sm, FlushQueue<N * (N + 1)> &q,
                                                 int nC, float *dst) {
    constexpr int P = N * (N + 1);
    const int B = blockDim.x, W = B / 32, G = nC * P, Gr = round4(G);
    queue_drain<P>(q);
    __syncthreads();
    for (int i = threadIdx.x; i < G; i += B) {
        float s = 0.f;
        for (int w = 0; w < W; ++w) s += sm.gw[(size_t)w * Gr + i];
        dst[i] = s;
    }
}

}  // namespace cpab
