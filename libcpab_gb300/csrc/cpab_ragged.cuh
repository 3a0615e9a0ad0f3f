// Device pieces shared by the ragged kernels (cpab_ragged.cu: 1D series;
// cpab_ragged_points.cu: point sets of any dimension).
//
// Work is cut into warp tiles of consecutive points of one set.  k_ragged_plan
// builds the tile prefix tile_off[S+1] on the device; a warp of a persistent
// grid owns the contiguous tile range [w K, (w+1) K), K = ceil(tiles / warps),
// so set s is touched exactly by warps tile_off[s]/K .. (tile_off[s+1]-1)/K and
// each (warp, set) pair writes its own partial slot w + s: the finalize sums a
// set's slots in warp order (deterministic, no atomics).
#pragma once
#include "cpab_adjoint.cuh"

namespace cpab {

__device__ __forceinline__ bool series_ok(long long a, long long b, long long total) {
    return a >= 0 && b >= a && b <= total && b - a < kRaggedMaxLen;
}

// Largest s with tile_off[s] <= t (tile_off[0] = 0 <= t < tile_off[S]).
__device__ __forceinline__ int find_series(const int *tile_off, int S, int t) {
    int lo = 0, hi = S;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(tile_off + mid) <= t) lo = mid;
        else hi = mid;
    }
    return lo;
}


// Warp-tile prefix over sets (one block): tile_off[s] = sum_{s'<s} tiles(s'),
// tile_off[S] = total tiles (tpw points per tile).  Invalid sets count as
// empty and raise kErrBadOffsets.  Defined in cpab_ragged.cu.
cudaError_t launch_ragged_plan(int S, const long long *off, long long total, int tpw,
                               int *tile_off, unsigned *err, cudaStream_t s);

// ------------------------------- finalize ------------------------------------
// One block per series / point set: sum its partial slots in warp order, then
// the per-theta tail shared with k_finalize (sse: per-series squared error of
// the fused 1D MSE, may be NULL).
template <int N, int MODE>
__global__ void __launch_bounds__(256)
    k_ragged_finalize(int nC, Steps st, int S, const int *__restrict__ tile_off, int TW,
                      const float *__restrict__ partials, const float *__restrict__ sse_partials,
                      const float *__restrict__ A, const float *__restrict__ basis, int d,
                      float *__restrict__ dtheta, float *__restrict__ sse) {
    extern __shared__ float4 smem4[];
    float *g = reinterpret_cast<float *>(smem4);
    const int s = blockIdx.x, tid = threadIdx.x, B = blockDim.x;
    const int G = nC * N * (N + 1);
    const int TT = __ldg(tile_off + S);
    const int K = max(1, (TT + TW - 1) / TW);
    const int a = __ldg(tile_off + s), b = __ldg(tile_off + s + 1);
    const int w0 = a / K, w1 = (b > a) ? (b - 1) / K : w0 - 1;
    for (int i = tid; i < G; i += B) {
        float acc = 0.f;
        for (int w = w0; w <= w1; ++w) acc += __ldg(partials + ((long long)w + s) * G + i);
        g[i] = acc;
    }
    if (sse && tid == 0) {
        float acc = 0.f;
        for (int w = w0; w <= w1; ++w) acc += __ldg(sse_partials + (long long)w + s);
        sse[s] = acc;
    }
    __syncthreads();
    if (dtheta)
        finish_theta<N, MODE>(g, g + round4(G), A + (long long)s * G, nC, st, basis, d,
                              dtheta + (long long)s * d);
}

}  // namespace cpab
