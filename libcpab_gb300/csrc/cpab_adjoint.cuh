// Device helpers shared by the adjoint kernels (cpab_adjoint.cu) and the
// fused transform_data backward (cpab_fused.cu).  The scheme is described at
// the top of cpab_adjoint.cu.
#pragma once
#include "cpab_launch.h"

namespace cpab {

constexpr int kSeg = 10;

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

// Add the flushing lanes' register accumulators into the warp's table.
// Called by exactly the lanes in `m` (all holding flush=true).
template <int P>
__device__ __forceinline__ void flush_group(unsigned m, int cell, const float (&acc)[P],
                                            float *warp_tab) {
    const unsigned grp = __match_any_sync(m, cell);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(grp) - 1;
    float *dst = warp_tab + cell * P;
    if (grp == 0xffffffffu) {
#pragma unroll
        for (int i = 0; i < P; ++i) {
            float v = acc[i];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
            if (lane == 0) dst[i] += v;
        }
    } else {
#pragma unroll
        for (int i = 0; i < P; ++i) {
            float v = 0.f;
            for (unsigned mm = grp; mm; mm &= mm - 1) v += __shfl_sync(grp, acc[i], __ffs(mm) - 1);
            if (lane == leader) dst[i] += v;
        }
    }
}

// One reverse step: accumulate this step's cell gradient into acc and move
// lambda from step n+1 to step n.  p is the position at step n.
template <int N, int MODE>
__device__ __forceinline__ void adjoint_step(const float *tab, int c, const Steps &st,
                                             const float (&p)[N], float (&lam)[N],
                                             float (&acc)[N * (N + 1)]) {
    constexpr int P = N * (N + 1);
    float M[P];
    load_cell<N>(tab, c, M);
    if constexpr (MODE == 1) {
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
            for (int r = 0; r < N; ++r) s = fmaf(M[r * (N + 1) + k], lam[r], s);
            nl[k] = s;
        }
#pragma unroll
        for (int k = 0; k < N; ++k) lam[k] = nl[k];
    } else {
        float v[N], pm[N], u[N], u2[N];
        affine_apply<N>(M, p, v);
#pragma unroll
        for (int r = 0; r < N; ++r) pm[r] = fmaf(st.hh, v[r], p[r]);
        // u = A_lin^T lambda, u2 = A_lin^T u
#pragma unroll
        for (int k = 0; k < N; ++k) {
            float s = 0.f;
#pragma unroll
            for (int r = 0; r < N; ++r) s = fmaf(M[r * (N + 1) + k], lam[r], s);
            u[k] = s;
        }
#pragma unroll
        for (int k = 0; k < N; ++k) {
            float s = 0.f;
#pragma unroll
            for (int r = 0; r < N; ++r) s = fmaf(M[r * (N + 1) + k], u[r], s);
            u2[k] = s;
        }
#pragma unroll
        for (int r = 0; r < N; ++r) {
            const float a = st.h * lam[r], b = st.hh2 * u[r];
#pragma unroll
            for (int k = 0; k < N; ++k)
                acc[r * (N + 1) + k] = fmaf(a, pm[k], fmaf(b, p[k], acc[r * (N + 1) + k]));
            acc[r * (N + 1) + N] += a + b;
        }
#pragma unroll
        for (int k = 0; k < N; ++k) lam[k] = fmaf(st.h, u[k], fmaf(st.hh2, u2[k], lam[k]));
    }
}

template <typename CT>
__host__ __device__ constexpr int cell_bytes() { return (int)sizeof(CT); }

__host__ __device__ inline int round4(int x) { return (x + 3) & ~3; }

// Shared memory carve-up for the adjoint kernels (floats unless noted):
//   tab   [round4(G)]            cell table of this theta (TMA destination)
//   gw    [W][round4(G)]         per-warp cell-gradient tables
//   ck    [nseg][N][block]       checkpoints (position every kSeg steps)
//   pb    [kSeg][N][block]       positions of the segment being reversed
//   cl    [nsteps][block] (CT)   per-step cells
// Every array is indexed [...][block] by thread, so warps access
// consecutive words (no bank conflicts).
template <int N, typename CT>
__host__ __device__ inline size_t adjoint_smem_bytes(int nC, int nsteps, int block) {
    const int G = round4(nC * N * (N + 1));
    const int W = block / 32;
    const int nseg = (nsteps + kSeg - 1) / kSeg;
    size_t b = (size_t)G * 4 + (size_t)W * G * 4 + (size_t)nseg * N * block * 4 +
               (size_t)kSeg * N * block * 4 + (size_t)nsteps * block * sizeof(CT);
    return (b + 15) & ~(size_t)15;
}

// Reverse sweep of one trajectory whose cells are logged in cl and whose
// checkpoints are in ck; lam holds dL/dp_N on entry and dL/dp_0 on exit.
// Each segment's positions are rebuilt from its checkpoint with the logged
// cells (no lookups) into pb, then walked backwards.  The loops are not
// unrolled: the body stays small enough for the instruction cache.
// Executed by all lanes of the warp (uniform trip counts).
template <int N, int MODE, typename CT>
__device__ __forceinline__ void reverse_sweep(const float *tab, const float *ck, const CT *cl,
                                              float *pb, int nsteps, const Steps &st,
                                              bool live, float (&lam)[N], float *warp_tab) {
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
        float q[N];
#pragma unroll
        for (int r = 0; r < N; ++r) q[r] = ck[(seg * N + r) * B + tid];
#pragma unroll 1
        for (int s = 0; s < len; ++s) {
#pragma unroll
            for (int r = 0; r < N; ++r) pb[(s * N + r) * B + tid] = q[r];
            traj_step<N, MODE>(tab, (int)cl[(n0 + s) * B + tid], st, q);
        }
#pragma unroll 1
        for (int s = len - 1; s >= 0; --s) {
            const int c = (int)cl[(n0 + s) * B + tid];
            const bool change = c != gcell;
            const unsigned m = __ballot_sync(0xffffffffu, change && gcell >= 0 && live);
            if (m) {
                if ((m >> (tid & 31)) & 1u) flush_group<P>(m, gcell, acc, warp_tab);
                __syncwarp();
            }
            if (change) {
                gcell = c;
#pragma unroll
                for (int i = 0; i < P; ++i) acc[i] = 0.f;
            }
            float p[N];
#pragma unroll
            for (int r = 0; r < N; ++r) p[r] = pb[(s * N + r) * B + tid];
            adjoint_step<N, MODE>(tab, c, st, p, lam, acc);
        }
    }
    const unsigned m = __ballot_sync(0xffffffffu, gcell >= 0 && live);
    if (m) {
        if ((m >> (tid & 31)) & 1u) flush_group<P>(m, gcell, acc, warp_tab);
        __syncwarp();
    }
}

// Forward sweep that logs cells and checkpoints; p holds p_0 on entry and
// p_N on exit.
template <int N, int MODE, typename CT>
__device__ __forceinline__ void logged_forward(const float *tab, const Tess &t, int nsteps,
                                               const Steps &st, float (&p)[N], float *ck, CT *cl,
                                               unsigned long long *ties, unsigned *err) {
    const int B = blockDim.x, tid = threadIdx.x;
    for (int n = 0; n < nsteps; ++n) {
        if (n % kSeg == 0) {
#pragma unroll
            for (int r = 0; r < N; ++r) ck[((n / kSeg) * N + r) * B + tid] = p[r];
        }
        int c = find_cell<N>(p, t, ties);
        if ((unsigned)c >= (unsigned)t.nC) {
            raise_error(err, kErrBadCell);
            c = 0;
        }
        cl[n * B + tid] = (CT)c;
        traj_step<N, MODE>(tab, c, st, p);
    }
}

}  // namespace cpab
