// Forward integration of points through the CPA field (transform_grid).
//
// Same scheme as the reference kernels (libcpab/core/cpab_ops.cu:268-388): for
// nsteps steps, look up the cell of p and apply that cell's step map.  Design
// on sm_103a:
//   * one CTA per (theta, tile of blockDim*PPT points); the theta's cell table
//     is staged in shared memory once by a TMA bulk copy (the reference
//     re-reads T_c from global memory at every step);
//   * each thread integrates PPT independent points interleaved, so the
//     dependent lookup -> load -> affine chain of one trajectory overlaps with
//     the others';
//   * certified FP32 cell lookup (cpab_common.cuh) instead of the reference's
//     FP64 fmod/divide at every step;
//   * compensated update p <- p + E [p;1] with E = T - I (or the reference's
//     p <- T [p;1] when handed the reference's T tables);
//   * structure-of-arrays point I/O, coalesced along the point index.
#include <atomic>
#include <map>
#include <mutex>

#include "cpab_launch.h"

namespace cpab {

template <int N, bool COMP, int PPT>
__global__ void __launch_bounds__(256)
    k_integrate(Tess t, int nsteps, const float *__restrict__ points, int broadcast, long long nP,
                const float *__restrict__ table, int tiles, float *__restrict__ out,
                int *__restrict__ trace, unsigned long long *ties, unsigned *err) {
    constexpr int P = N * (N + 1);
    extern __shared__ float4 smem4[];
    __shared__ uint64_t bar;
    float *tab = reinterpret_cast<float *>(smem4);
    const int th = blockIdx.y;
    const int tile = blockIdx.x;
    const int tab_floats = t.nC * P;
    if (!stage_table(tab, table + (long long)th * tab_floats, tab_floats, &bar, err)) return;

    const float *src = points + (broadcast ? (long long)th * N * nP : 0ll);
    float p[PPT][N];
    long long idx[PPT];
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
        idx[j] = ((long long)tile * PPT + j) * blockDim.x + threadIdx.x;
        const bool v = idx[j] < nP;
#pragma unroll
        for (int r = 0; r < N; ++r) p[j][r] = v ? __ldg(src + r * nP + idx[j]) : 0.5f;
    }
    for (int s = 0; s < nsteps; ++s) {
#pragma unroll
        for (int j = 0; j < PPT; ++j) {
            const int c = find_cell<N>(p[j], t, ties);
            if (trace && idx[j] < nP) trace[((long long)th * nP + idx[j]) * nsteps + s] = c;
            float M[P], y[N];
            load_cell<N>(tab, c, M);
            affine_apply<N>(M, p[j], y);
#pragma unroll
            for (int r = 0; r < N; ++r) p[j][r] = COMP ? p[j][r] + y[r] : y[r];
        }
    }
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
        if (idx[j] < nP) {
#pragma unroll
            for (int r = 0; r < N; ++r) out[((long long)th * N + r) * nP + idx[j]] = p[j][r];
        }
    }
}

template <int N, bool COMP, int PPT>
static cudaError_t launch_integrate_t(const Tess &t, int nsteps, const float *points,
                                      int broadcast, long long nP, const float *table,
                                      int n_theta, float *out, int *trace,
                                      unsigned long long *ties, unsigned *err, cudaStream_t s,
                                      int block) {
    const long long per = (long long)block * PPT;
    const int tiles = (int)((nP + per - 1) / per);
    if ((long long)tiles * n_theta == 0) return cudaSuccess;
    if (n_theta > 65535) return cudaErrorInvalidConfiguration;   // theta on grid y
    const dim3 grid((unsigned)tiles, (unsigned)n_theta);
    const size_t smem = (size_t)t.nC * N * (N + 1) * sizeof(float);
    auto kern = k_integrate<N, COMP, PPT>;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
    }
    kern<<<grid, block, smem, s>>>(t, nsteps, points, broadcast, nP, table, tiles, out,
                                             trace, ties, err);
    return cudaGetLastError();
}

cudaError_t launch_integrate(const Tess &t, int nsteps, const float *points, int broadcast,
                             long long nP, const float *table, bool compensated, int n_theta,
                             float *out, int *trace, unsigned long long *ties, unsigned *err,
                             cudaStream_t s, const LaunchShape *force) {
    // Default: 256 threads, two points per thread once there is enough work
    // to fill the GPU twice; or the autotuned / forced shape.
    LaunchShape sh;
    if (force) {
        sh = *force;
    } else if (!tuned_get(kTuneIntegrate, tune_key(t, nsteps, compensated ? 1 : 0, nP, n_theta,
                                                   broadcast), &sh)) {
        sh.block = 256;
        sh.ppt = (long long)n_theta * nP >= (long long)num_sms() * 2048 * 2 ? 2 : 1;
    }
    if (sh.block < 32 || sh.block > 256 || sh.block % 32 || (sh.ppt != 1 && sh.ppt != 2))
        return cudaErrorInvalidConfiguration;
    const bool two = sh.ppt == 2;
    const int block = sh.block;
#define CPAB_INTEGRATE(N)                                                                          \
    if (compensated)                                                                               \
        return two ? launch_integrate_t<N, true, 2>(t, nsteps, points, broadcast, nP, table,       \
                                                    n_theta, out, trace, ties, err, s, block)      \
                   : launch_integrate_t<N, true, 1>(t, nsteps, points, broadcast, nP, table,       \
                                                    n_theta, out, trace, ties, err, s, block);     \
    return two ? launch_integrate_t<N, false, 2>(t, nsteps, points, broadcast, nP, table,          \
                                                 n_theta, out, trace, ties, err, s, block)         \
               : launch_integrate_t<N, false, 1>(t, nsteps, points, broadcast, nP, table,          \
                                                 n_theta, out, trace, ties, err, s, block);
    switch (t.ndim) {
        case 1: { CPAB_INTEGRATE(1) }
        case 2: { CPAB_INTEGRATE(2) }
        default: { CPAB_INTEGRATE(3) }
    }
#undef CPAB_INTEGRATE
}

template <int N>
__global__ void k_findcellidx(Tess t, const float *__restrict__ points, long long nP,
                              int *__restrict__ out, unsigned long long *ties) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nP) return;
    float p[N];
#pragma unroll
    for (int r = 0; r < N; ++r) p[r] = points[r * nP + i];
    out[i] = find_cell<N>(p, t, ties);
}

cudaError_t launch_findcellidx(const Tess &t, const float *points, long long nP, int *out,
                               unsigned long long *ties, cudaStream_t s) {
    if (nP == 0) return cudaSuccess;
    const int block = 256;
    const unsigned grid = (unsigned)((nP + block - 1) / block);
    switch (t.ndim) {
        case 1: k_findcellidx<1><<<grid, block, 0, s>>>(t, points, nP, out, ties); break;
        case 2: k_findcellidx<2><<<grid, block, 0, s>>>(t, points, nP, out, ties); break;
        default: k_findcellidx<3><<<grid, block, 0, s>>>(t, points, nP, out, ties); break;
    }
    return cudaGetLastError();
}

// ---------------------------- tuned launch shapes ----------------------------
namespace {
std::mutex g_shape_mu;
std::map<std::pair<int, std::array<long long, 10>>, LaunchShape> g_shapes;
}  // namespace

TuneKey tune_key(const Tess &t, int nsteps, int mode, long long a, long long b, long long c) {
    return TuneKey{t.ndim, t.nc[0], t.nc[1], t.nc[2], (long long)nsteps * 4 + mode, a, b, c};
}

static std::array<long long, 10> full_key(const TuneKey &k) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        dev = 0;
    }
    std::array<long long, 10> f{};
    f[0] = dev;
    for (int i = 0; i < 8; ++i) f[i + 1] = k[i];
    return f;
}

bool tuned_get(int kind, const TuneKey &key, LaunchShape *shape) {
    const auto k = std::make_pair(kind, full_key(key));
    std::lock_guard<std::mutex> lock(g_shape_mu);
    auto it = g_shapes.find(k);
    if (it == g_shapes.end()) return false;
    *shape = it->second;
    return true;
}

void tuned_set(int kind, const TuneKey &key, const LaunchShape &shape) {
    const auto k = std::make_pair(kind, full_key(key));
    std::lock_guard<std::mutex> lock(g_shape_mu);
    if (g_shapes.size() > 4096) g_shapes.clear();
    g_shapes[k] = shape;
}

void tuned_clear() {
    std::lock_guard<std::mutex> lock(g_shape_mu);
    g_shapes.clear();
}

// SM count of the current device, looked up once per device (relaxed atomics:
// concurrent first calls store the same value).
int num_sms() {
    constexpr int kDevices = 64;
    static std::atomic<int> cached[kDevices];
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        dev = 0;
    }
    if (dev < 0 || dev >= kDevices) dev = 0;
    int v = cached[dev].load(std::memory_order_relaxed);
    if (v == 0) {
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            cudaGetLastError();
            n = 0;
        }
        v = n > 0 ? n : 152;
        cached[dev].store(v, std::memory_order_relaxed);
    }
    return v;
}

}  // namespace cpab
