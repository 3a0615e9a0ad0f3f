// Ragged batched 1D series: many theta, one series each, uneven lengths.
//
// The reference has no ragged entry point.  Its equivalent is one
// Cpab.transform_data call per series (libcpab/cpab.py:304-331) with outsize
// [L_s]: grid = torch.linspace(0, 1, L_s) (libcpab/pytorch/functions.py:102-108),
// transform_grid with that series' theta (libcpab/pytorch/transformer.py:72-87),
// then linear interpolation of the series' values
// (libcpab/pytorch/interpolation.py:18-60).  Here all series run in one
// persistent launch indexed by the series offsets:
//
//   * work unit = warp tile: 32 * ppt consecutive points of one series.  The
//     tile prefix over series (tile_off, S + 1 ints) is built on the device by
//     k_ragged_plan, so nothing waits for the host and the whole sequence can
//     be captured in a CUDA graph;
//   * each warp owns a contiguous range of K = ceil(tiles / warps) tiles; it
//     finds its first series by binary search in tile_off and walks forward,
//     restaging the series' cell table into its own slice of shared memory
//     when the series changes;
//   * a series' grid is monotone, so the lanes of a warp tile are already
//     bucketed by starting cell (neighbouring lanes start in the same or the
//     next cell) and no sort is needed;
//   * dtheta: a warp accumulates its series' cell statistics in its own table
//     (warp flush of cpab_adjoint.cuh) and, when it leaves the series, writes
//     them to partial slot (warp + series).  Warps own contiguous tile ranges,
//     so series s is touched exactly by warps tile_off[s]/K ..
//     (tile_off[s+1]-1)/K and the slots of all touched (warp, series) pairs
//     are distinct.  k_ragged_finalize sums a series' slots in warp order:
//     deterministic, no atomics.
//
// The trajectory arithmetic is that of the other kernels: compensated update
// p <- p + E [p;1] for the transformed grid (bit-identical to cpab_integrate
// on torch.linspace points), cell lookup of cpab_common.cuh, the adjoint of
// cpab_adjoint.cuh, and the interpolation of cpab_interp.cuh.
#include <map>
#include <mutex>
#include <tuple>

#include "cpab_ragged.cuh"
#include "cpab_interp.cuh"

namespace cpab {

// torch.linspace(0, 1, L)[j] in float32: step = 1/(L-1); the first half is
// step*j, the second half 1 - step*(L-1-j) (one rounding, as a fused
// multiply-add gives).  L == 1 gives 0.
__device__ __forceinline__ float linspace01(int j, int L, float step) {
    if (L == 1) return 0.f;
    return (j < (L >> 1)) ? __fmul_rn(step, (float)j) : fmaf(-step, (float)(L - 1 - j), 1.f);
}

// Warp-tile prefix over series (one block): tile_off[s] = sum_{s'<s} tiles(s'),
// tile_off[S] = total tiles.  Invalid series count as empty and raise
// kErrBadOffsets.
__global__ void __launch_bounds__(1024)
    k_ragged_plan(int S, const long long *__restrict__ off, long long total, int tpw,
                  int *__restrict__ tile_off, unsigned *err) {
    __shared__ long long wsum[32];
    const int tid = threadIdx.x, B = blockDim.x, lane = tid & 31, wid = tid >> 5;
    const int per = (S + B - 1) / B;
    const int s0 = min(tid * per, S), s1 = min(s0 + per, S);
    long long local = 0;
    for (int s = s0; s < s1; ++s) {
        const long long a = off[s], b = off[s + 1];
        if (!series_ok(a, b, total)) {
            raise_error(err, kErrBadOffsets);
            continue;
        }
        local += (b - a + tpw - 1) / tpw;
    }
    long long incl = local;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const long long v = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += v;
    }
    if (lane == 31) wsum[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        long long v = (lane < B / 32) ? wsum[lane] : 0;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const long long u = __shfl_up_sync(0xffffffffu, v, d);
            if (lane >= d) v += u;
        }
        wsum[lane] = v;   // inclusive prefix of warp totals
    }
    __syncthreads();
    long long run = incl - local + (wid > 0 ? wsum[wid - 1] : 0);
    for (int s = s0; s < s1; ++s) {
        tile_off[s] = (int)run;
        const long long a = off[s], b = off[s + 1];
        if (series_ok(a, b, total)) run += (b - a + tpw - 1) / tpw;
    }
    if (tid == B - 1) tile_off[S] = (int)run;
}

cudaError_t launch_ragged_plan(int S, const long long *off, long long total, int tpw,
                               int *tile_off, unsigned *err, cudaStream_t s) {
    k_ragged_plan<<<1, 1024, 0, s>>>(S, off, total, tpw, tile_off, err);
    return cudaGetLastError();
}

__device__ __forceinline__ Geo series_geo(int L) {
    Geo g;
    g.size[0] = L;
    g.sizem1[0] = (float)(L - 1);
    return g;
}

// ------------------------------- forward -------------------------------------
// out[off[s] + j] = interp(values_s, T_s(linspace(0,1,L_s)[j])).  Each lane
// integrates PPT points of its warp tile interleaved.
template <int PPT>
__global__ void __launch_bounds__(256)
    k_ragged_forward(Tess t, int nsteps, int S, const long long *__restrict__ off,
                     const int *__restrict__ tile_off, const float *__restrict__ E,
                     const float *__restrict__ values, float *__restrict__ out,
                     unsigned long long *ties, unsigned *err) {
    constexpr int TPW = 32 * PPT;
    extern __shared__ float4 smem4[];
    const int G = t.nC * 2, Gr = round4(G);
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
        const float step = (L > 1) ? 1.f / (float)(L - 1) : 0.f;
        const int j0 = (tl - __ldg(tile_off + s)) * TPW;
        float p[PPT][1];
        int j[PPT];
#pragma unroll
        for (int k = 0; k < PPT; ++k) {
            j[k] = j0 + k * 32 + lane;
            p[k][0] = (j[k] < L) ? linspace01(j[k], L, step) : 0.5f;
        }
        for (int st = 0; st < nsteps; ++st) {
#pragma unroll
            for (int k = 0; k < PPT; ++k) {
                const int c = cell_1d(p[k][0], t);
                const float2 m = *reinterpret_cast<const float2 *>(tab + 2 * c);
                p[k][0] += fmaf(m.x, p[k][0], m.y);
            }
        }
        const Geo g = series_geo(L);
#pragma unroll
        for (int k = 0; k < PPT; ++k) {
            if (j[k] >= L) continue;
            const Corner<1> cr = corners<1>(p[k], g);
            out[base + j[k]] = lerp_corners<1>(values + base, cr);
        }
    }
}

// ------------------------------- adjoint -------------------------------------
// Per-warp shared-memory slice (floats): tab (A in mode 0, E in mode 1),
// tabE (mode 0 only), dtab, gw.
template <int MODE>
__host__ __device__ inline int ragged_warp_floats(int nC) {
    const int Gr = round4(nC * 2);
    return Gr * (MODE != 1 ? 2 : 1) + dtab_floats<1>(nC) + Gr;
}

template <int MODE, typename CT>
__host__ __device__ inline size_t ragged_adjoint_smem(int nC, int nsteps, int block) {
    const int nseg = (nsteps + kSeg - 1) / kSeg;
    const size_t b = (size_t)(block / 32) * ragged_warp_floats<MODE>(nC) * 4 +
                     (size_t)nseg * block * 4 + (size_t)kSeg * block * 4 +
                     (size_t)nsteps * block * sizeof(CT);
    return (b + 15) & ~(size_t)15;
}

// The lane-slot sink of the reverse sweep (LS = true): a lane that leaves a
// cell adds its sum over the steps spent there into its own slots
// ls[cell][i][lane] with fire-and-forget global reductions, and widens the
// range [lo, hi] of cells it touched.  Each slot is written by one lane only,
// in program order, so its value does not depend on timing; the warp sums the
// 32 slots of each touched cell with a fixed shuffle tree when it finishes a
// series (reproducible dtheta).  Unlike the warp-table flush (a five-round
// shuffle tree over the run of lanes in a cell, executed by the whole warp at
// every step where any lane changes cell), a lane's flush is two reductions.
struct LaneSlotSink {
    float *ls;
    int lo, hi;
    template <int P>
    __device__ __forceinline__ void operator()(bool flush, int cell, const float (&acc)[P]) {
        if (flush) {
            float *q = ls + cell * (P * 32) + (threadIdx.x & 31);
#pragma unroll
            for (int i = 0; i < P; ++i) atomicAdd(q + i * 32, acc[i]);
            lo = min(lo, cell);
            hi = max(hi, cell);
        }
    }
};

template <int MODE, typename CT, bool FUSED, bool LS>
__global__ void __launch_bounds__(256)
    k_ragged_adjoint(Tess t, int nsteps, Steps st, int S, const long long *__restrict__ off,
                     const int *__restrict__ tile_off, int ppt, RaggedBwd a,
                     unsigned long long *ties, unsigned *err) {
    constexpr int P = 2;
    extern __shared__ float4 smem4[];
    const int B = blockDim.x, W = B / 32;
    const int G = t.nC * P, Gr = round4(G);
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int nseg = (nsteps + kSeg - 1) / kSeg;
    float *base_f = reinterpret_cast<float *>(smem4);
    float *mine = base_f + (size_t)wib * ragged_warp_floats<MODE>(t.nC);
    AdjSmem<1, CT> sm;
    sm.tab = mine;
    float *tabE = (MODE != 1) ? mine + Gr : mine;
    sm.dtab = mine + Gr * (MODE != 1 ? 2 : 1);
    sm.mtab = mtab_of<1>(sm.dtab, t.nC);
    sm.gw = sm.dtab + dtab_floats<1>(t.nC);
    sm.ck = base_f + (size_t)W * ragged_warp_floats<MODE>(t.nC);
    sm.pb = sm.ck + (size_t)nseg * B;
    sm.cl = reinterpret_cast<CT *>(sm.pb + (size_t)kSeg * B);

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
    float sse = 0.f;
    LaneSlotSink slots{LS ? a.lane_slots + (size_t)w * t.nC * (P * 32) : nullptr, INT_MAX, -1};
    if constexpr (LS) {
        float4 *z = reinterpret_cast<float4 *>(slots.ls);
        for (int i = lane; i < t.nC * (P * 8); i += 32) z[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }

    auto stage = [&](int sid) {
        __syncwarp();
        const float *src = (MODE != 1 ? a.A : a.E) + (long long)sid * G;
        for (int i = lane; i < G; i += 32) sm.tab[i] = __ldg(src + i);
        if (MODE != 1)
            for (int i = lane; i < G; i += 32) tabE[i] = __ldg(a.E + (long long)sid * G + i);
        for (int i = lane; i < Gr; i += 32) sm.gw[i] = 0.f;
        __syncwarp();
        build_dtab<1, MODE>(sm.tab, sm.dtab, t.nC, st, lane, 32);
        __syncwarp();
    };
    auto finish = [&](int sid) {
        __syncwarp();
        if constexpr (LS) {
            // cell sums of the series into gw; the slots are zeroed for the next one
            const int lo = __reduce_min_sync(0xffffffffu, slots.lo);
            const int hi = __reduce_max_sync(0xffffffffu, slots.hi);
            for (int c = lo; c <= hi; ++c) {
                float *q = slots.ls + c * (P * 32) + lane;
                float v[P];
#pragma unroll
                for (int i = 0; i < P; ++i) {
                    v[i] = __ldcg(q + i * 32);   // this lane's own reductions, in order
                    q[i * 32] = 0.f;
                }
#pragma unroll
                for (int d = 16; d > 0; d >>= 1)
#pragma unroll
                    for (int i = 0; i < P; ++i) v[i] += __shfl_xor_sync(0xffffffffu, v[i], d);
                if (lane == 0) {
#pragma unroll
                    for (int i = 0; i < P; ++i) sm.gw[c * P + i] = v[i];
                }
            }
            slots.lo = INT_MAX;
            slots.hi = -1;
            __syncwarp();
        }
        float v = sse;
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
        const long long slot = (long long)w + sid;
        if (FUSED && lane == 0) a.sse_partials[slot] = v;
        for (int i = lane; i < G; i += 32) a.partials[slot * G + i] = sm.gw[i];
        sse = 0.f;
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
        const float step = (L > 1) ? 1.f / (float)(L - 1) : 0.f;
        const int j0 = (tl - __ldg(tile_off + s)) * tpw;
        const Geo g = series_geo(L);
#pragma unroll 1
        for (int k = 0; k < ppt; ++k) {
            const int j = j0 + k * 32 + lane;
            const bool live = j < L;
            float p[1] = {live ? linspace01(j, L, step) : 0.5f};
            float pN[1] = {p[0]};
            if constexpr (MODE != 1) e_sweep<1>(tabE, t, nsteps, pN, ties, err);
            logged_forward<1, MODE, CT>(sm, t, nsteps, st, p, ties, err);
            if constexpr (MODE == 1) pN[0] = p[0];
            float lam[1] = {0.f};
            if (live) {
                const Corner<1> cr = corners<1>(pN, g);
                float wgt;
                if constexpr (FUSED) {
                    const float v = lerp_corners<1>(a.values + base, cr);
                    if (a.out) a.out[base + j] = v;
                    const float r = v - __ldg(a.target + base + j);
                    sse = fmaf(r, r, sse);
                    wgt = a.loss_scale * r;
                } else {
                    wgt = __ldg(a.gout + base + j);
                }
                float gf[1] = {0.f};
                lerp_grads<1>(a.values + base, cr, wgt, a.dvalues ? a.dvalues + base : nullptr,
                              gf);
                lam[0] = gf[0] * g.sizem1[0];
            }
            if constexpr (LS) reverse_sweep_to<1, MODE, CT>(sm, nsteps, st, live, lam, slots);
            else reverse_sweep<1, MODE, CT>(sm, nsteps, st, live, lam, sm.gw);
        }
    }
    finish(s);
}

// ------------------------------- planning ------------------------------------
namespace {
std::mutex g_tune_mu;
// (device, kind, mode, nC, nsteps, S, total) -> (block, ppt)
std::map<std::tuple<int, int, int, int, int, int, long long>, std::pair<int, int>> g_tuned;

}  // namespace

// Lane slots (the adjoint's per-lane cell sums, k_ragged_adjoint<..., true>)
// for tessellations of at most kLaneSlotCells cells, sized for at most
// kLaneSlotWarpsPerSM resident warps per SM (the kernel's grid is capped to it).
constexpr int kLaneSlotCells = 128, kLaneSlotWarpsPerSM = 32;

static size_t lane_slot_bytes(const Tess &t) {
    if (t.nC > kLaneSlotCells) return 0;
    return (size_t)num_sms() * kLaneSlotWarpsPerSM * t.nC * 2 * 32 * 4;
}

size_t ragged_workspace_bytes(const Tess &t, int S) {
    const size_t tiles = ((size_t)(S + 1) * 4 + 255) & ~(size_t)255;
    const size_t slots = (size_t)num_sms() * 64 + (size_t)S;
    const size_t part = (slots * t.nC * 2 * 4 + 255) & ~(size_t)255;
    const size_t sse = (slots * 4 + 255) & ~(size_t)255;
    return tiles + part + sse + lane_slot_bytes(t);
}

static void ragged_carve(const Tess &t, int S, void *ws, int **tile_off, float **partials,
                         float **sse_partials, float **lane_slots) {
    char *p = static_cast<char *>(ws);
    const size_t tiles = ((size_t)(S + 1) * 4 + 255) & ~(size_t)255;
    const size_t slots = (size_t)num_sms() * 64 + (size_t)S;
    const size_t part = (slots * t.nC * 2 * 4 + 255) & ~(size_t)255;
    const size_t sse = (slots * 4 + 255) & ~(size_t)255;
    *tile_off = reinterpret_cast<int *>(p);
    *partials = reinterpret_cast<float *>(p + tiles);
    *sse_partials = reinterpret_cast<float *>(p + tiles + part);
    *lane_slots = lane_slot_bytes(t) ? reinterpret_cast<float *>(p + tiles + part + sse) : nullptr;
}

bool ragged_get_tuned(int kind, int mode, const Tess &t, int nsteps, int S, long long total,
                      int *block, int *ppt) {
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tuned.find(std::make_tuple(dev, kind, mode, t.nC, nsteps, S, total));
    if (it == g_tuned.end()) return false;
    *block = it->second.first;
    *ppt = it->second.second;
    return true;
}

void ragged_set_tuned(int kind, int mode, const Tess &t, int nsteps, int S, long long total,
                      int block, int ppt) {
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tuned[std::make_tuple(dev, kind, mode, t.nC, nsteps, S, total)] = std::make_pair(block, ppt);
}

// ------------------------------- launchers -----------------------------------
template <int PPT>
static cudaError_t launch_rf_t(const Tess &t, int nsteps, int block, int S, const long long *off,
                               const int *tile_off, const float *E, const float *values,
                               float *out, unsigned long long *ties, unsigned *err,
                               cudaStream_t s) {
    auto kern = k_ragged_forward<PPT>;
    const size_t smem = (size_t)(block / 32) * round4(t.nC * 2) * 4;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
    }
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, smem);
    if (per_sm <= 0) return cudaErrorInvalidConfiguration;
    kern<<<num_sms() * per_sm, block, smem, s>>>(t, nsteps, S, off, tile_off, E, values, out,
                                                  ties, err);
    return cudaGetLastError();
}

cudaError_t launch_ragged_forward(const Tess &t, int nsteps, int block, int ppt, int S,
                                  const long long *off, long long total, const float *E,
                                  const float *values, float *out, void *ws,
                                  unsigned long long *ties, unsigned *err, cudaStream_t s) {
    int *tile_off;
    float *partials, *ssep, *lane_slots;
    ragged_carve(t, S, ws, &tile_off, &partials, &ssep, &lane_slots);
    if (S == 0) return cudaSuccess;
    k_ragged_plan<<<1, 1024, 0, s>>>(S, off, total, 32 * ppt, tile_off, err);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    switch (ppt) {
        case 1: return launch_rf_t<1>(t, nsteps, block, S, off, tile_off, E, values, out, ties, err, s);
        case 2: return launch_rf_t<2>(t, nsteps, block, S, off, tile_off, E, values, out, ties, err, s);
        default: return launch_rf_t<4>(t, nsteps, block, S, off, tile_off, E, values, out, ties, err, s);
    }
}

template <int MODE, typename CT, bool FUSED, bool LS>
static cudaError_t launch_ra_ls(const Tess &t, int nsteps, int block, int ppt, int S,
                                const long long *off, const int *tile_off, const RaggedBwd &a,
                                const float *basis, int d, float *dtheta, float *sse,
                                unsigned long long *ties, unsigned *err, cudaStream_t s) {
    auto kern = k_ragged_adjoint<MODE, CT, FUSED, LS>;
    const size_t smem = ragged_adjoint_smem<MODE, CT>(t.nC, nsteps, block);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, smem);
    if (per_sm <= 0) return cudaErrorInvalidConfiguration;
    // partial slots are sized for at most 64 resident warps per SM, lane slots
    // for kLaneSlotWarpsPerSM
    const int grid = min(num_sms() * per_sm,
                         num_sms() * (LS ? kLaneSlotWarpsPerSM : 64) / (block / 32));
    const Steps st = make_steps(nsteps);
    kern<<<grid, block, smem, s>>>(t, nsteps, st, S, off, tile_off, ppt, a, ties, err);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    auto fin = k_ragged_finalize<1, MODE>;
    const size_t fsmem = ((size_t)round4(t.nC * 2) + 256) * sizeof(float);
    if (fsmem > 48 * 1024) {
        e = cudaFuncSetAttribute(fin, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fsmem);
        if (e != cudaSuccess) return e;
    }
    fin<<<S, 256, fsmem, s>>>(t.nC, st, S, tile_off, grid * (block / 32), a.partials,
                              a.sse_partials, a.A, basis, d, dtheta, sse);
    return cudaGetLastError();
}

template <int MODE, typename CT, bool FUSED>
static cudaError_t launch_ra_t(const Tess &t, int nsteps, int block, int ppt, int S,
                               const long long *off, const int *tile_off, const RaggedBwd &a,
                               const float *basis, int d, float *dtheta, float *sse,
                               unsigned long long *ties, unsigned *err, cudaStream_t s) {
    if (a.lane_slots)
        return launch_ra_ls<MODE, CT, FUSED, true>(t, nsteps, block, ppt, S, off, tile_off, a,
                                                   basis, d, dtheta, sse, ties, err, s);
    return launch_ra_ls<MODE, CT, FUSED, false>(t, nsteps, block, ppt, S, off, tile_off, a,
                                                basis, d, dtheta, sse, ties, err, s);
}

// Shared-memory bytes of the adjoint kernel for this block size (0 if the
// configuration does not fit).
size_t ragged_adjoint_smem_for(const Tess &t, int nsteps, int mode, int block) {
    const bool small = t.nC <= 256;
    size_t b;
    if (mode != 1)
        b = small ? ragged_adjoint_smem<0, uint8_t>(t.nC, nsteps, block)
                  : ragged_adjoint_smem<0, uint16_t>(t.nC, nsteps, block);
    else
        b = small ? ragged_adjoint_smem<1, uint8_t>(t.nC, nsteps, block)
                  : ragged_adjoint_smem<1, uint16_t>(t.nC, nsteps, block);
    int dev = 0, max_optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (max_optin <= 0) max_optin = 48 * 1024;
    return b <= (size_t)max_optin ? b : 0;
}

cudaError_t launch_ragged_adjoint(const Tess &t, int nsteps, int mode, bool fused, int block,
                                  int ppt, int S, const long long *off, long long total,
                                  const RaggedBwd &a_in, const float *basis, int d,
                                  float *dtheta, float *sse, void *ws, unsigned long long *ties,
                                  unsigned *err, cudaStream_t s) {
    int *tile_off;
    RaggedBwd a = a_in;
    ragged_carve(t, S, ws, &tile_off, &a.partials, &a.sse_partials, &a.lane_slots);
    if (S == 0) return cudaSuccess;
    k_ragged_plan<<<1, 1024, 0, s>>>(S, off, total, 32 * ppt, tile_off, err);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const bool small = t.nC <= 256;
#define CPAB_RA(M, CT)                                                                        \
    return fused ? launch_ra_t<M, CT, true>(t, nsteps, block, ppt, S, off, tile_off, a, basis, \
                                            d, dtheta, sse, ties, err, s)                     \
                 : launch_ra_t<M, CT, false>(t, nsteps, block, ppt, S, off, tile_off, a,      \
                                             basis, d, dtheta, sse, ties, err, s);
    if (mode == 0) {
        if (small) { CPAB_RA(0, uint8_t) }
        CPAB_RA(0, uint16_t)
    }
    if (mode == 2) {
        if (small) { CPAB_RA(2, uint8_t) }
        CPAB_RA(2, uint16_t)
    }
    if (small) { CPAB_RA(1, uint8_t) }
    CPAB_RA(1, uint16_t)
#undef CPAB_RA
}

}  // namespace cpab
