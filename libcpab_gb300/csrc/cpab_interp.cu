// Linear / bilinear / trilinear sampling with clamp-to-edge, and its backward.
//
// Semantics follow libcpab/pytorch/interpolation.py:18-172 exactly:
//   x = grid_x * (W-1);  x0 = clamp(floor(x), 0, W-1);  x1 = clamp(floor(x)+1, 0, W-1)
//   xd = x - x0 (x0 after clamping); lerp first along x, then y, then z.
// Layouts are the reference's: data [nb, C, W(, H(, D))], grid [nb, ndim, nP]
// with the meshgrid's x fastest (k = ix + W_out*(iy + H_out*iz)), and output
// [nb, C, W_out(, H_out(, D_out))].  The reference builds ~30 launches of
// int64 index tensors and gathers (plus a host-built batch index that is
// copied to the device on every call); here one thread handles one output
// point for all channels.
//
// Memory order: the grid is meshgrid-ordered (x fastest) while data and
// output have the last axis fastest.  In 2D/3D a block therefore takes a
// 32 x 32 tile of (x, last axis) points (at one y in 3D), reads the tile's
// grid coordinates coalesced along x into shared memory, and then works in
// output order (last axis across the lanes): the output stores are
// contiguous and neighbouring lanes gather neighbouring data elements.  The
// backward writes d(grid) back through the same tile.  1D needs no tiling.
//
// Backward: d(data) is a scatter-add (float atomics into a zeroed buffer, like
// the reference's autograd index_put accumulation); d(grid) follows the
// gradient of the lerp weights, as autograd does through xd, yd, zd.
#include <cuda.h>
#include <cudaTypedefs.h>

#include "cpab_interp.cuh"

namespace cpab {

constexpr unsigned kMaxGridY = 65535;

// 1D: grid order is output order.
template <int N>
__global__ void __launch_bounds__(256)
    k_interpolate(Geo g, const float *__restrict__ data, int C, const float *__restrict__ grid,
                  float *__restrict__ out, int nb) {
    static_assert(N == 1, "2D and 3D use k_interpolate_tiled");
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= g.nP) return;
    const int oo = k;
    for (int b = blockIdx.y; b < nb; b += gridDim.y) {
        float p[N];
#pragma unroll
        for (int j = 0; j < N; ++j) p[j] = __ldg(grid + ((long long)b * N + j) * g.nP + k);
        const Corner<N> cr = corners<N>(p, g);
        for (int c = 0; c < C; ++c) {
            const long long plane = (long long)b * C + c;
            out[plane * g.nP + oo] = lerp_corners<N>(data + plane * g.nD, cr);
        }
    }
}

template <int N>
__global__ void __launch_bounds__(256)
    k_interpolate_backward(Geo g, const float *__restrict__ data, int C,
                           const float *__restrict__ grid, const float *__restrict__ gout,
                           float *__restrict__ ddata, float *__restrict__ dgrid, int nb) {
    static_assert(N == 1, "2D and 3D use k_interpolate_backward_tiled");
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= g.nP) return;
    const int oo = k;
    for (int b = blockIdx.y; b < nb; b += gridDim.y) {
        float p[N];
#pragma unroll
        for (int j = 0; j < N; ++j) p[j] = __ldg(grid + ((long long)b * N + j) * g.nP + k);
        const Corner<N> cr = corners<N>(p, g);
        float gf[N];
#pragma unroll
        for (int j = 0; j < N; ++j) gf[j] = 0.f;
        for (int c = 0; c < C; ++c) {
            const long long plane = (long long)b * C + c;
            const float w = __ldg(gout + plane * g.nP + oo);
            lerp_grads<N>(data + plane * g.nD, cr, w, ddata ? ddata + plane * g.nD : nullptr, gf);
        }
        if (dgrid) {
#pragma unroll
            for (int j = 0; j < N; ++j)
                dgrid[((long long)b * N + j) * g.nP + k] = gf[j] * g.sizem1[j];
        }
    }
}

// --------------------------- tiled 2D / 3D kernels ---------------------------
constexpr int kTile = 32, kRows = 8;   // 32 x 32 tile, 256 threads

// Tile t of an image: a = x index (grid-fast), z = last-axis index
// (output-fast), mid = y index in 3D (0 in 2D).
struct TileGeo {
    int ta, tz;   // tiles along x and along the last axis
};

template <int N>
__device__ __forceinline__ void tile_coords(const Geo &g, const TileGeo &tg, int t, int &a0,
                                            int &z0, int &mid) {
    const int per = tg.ta * tg.tz;
    mid = (N == 3) ? t / per : 0;
    const int r = t - mid * per;
    a0 = (r % tg.ta) * kTile;
    z0 = (r / tg.ta) * kTile;
}

// meshgrid index of (x = a, y = mid, last = z) and output offset
template <int N>
__device__ __forceinline__ int grid_index(const Geo &g, int a, int mid, int z) {
    if constexpr (N == 2) return a + g.outsize[0] * z;
    else return a + g.outsize[0] * (mid + g.outsize[1] * z);
}
template <int N>
__device__ __forceinline__ int out_index(const Geo &g, int a, int mid, int z) {
    if constexpr (N == 2) return a * g.outsize[1] + z;
    else return (a * g.outsize[1] + mid) * g.outsize[2] + z;
}

// Stage the tile's grid coordinates: sp[j][z_local][a_local].
template <int N>
__device__ __forceinline__ void load_grid_tile(const Geo &g, const float *gb, int a0, int z0,
                                               int mid, float (*sp)[kTile][kTile + 1]) {
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int A = g.outsize[0], Z = g.outsize[N - 1];
#pragma unroll
    for (int r = 0; r < kTile / kRows; ++r) {
        const int zl = ty + kRows * r, a = a0 + tx, z = z0 + zl;
        if (a < A && z < Z) {
            const int k = grid_index<N>(g, a, mid, z);
#pragma unroll
            for (int j = 0; j < N; ++j) sp[j][zl][tx] = __ldg(gb + (long long)j * g.nP + k);
        }
    }
}

// Asynchronous 4-byte copy global -> shared (cp.async, L1-allocating); with
// bytes = 0 nothing is read and the word is zero-filled.
__device__ __forceinline__ void cp_async4(float *dst, const float *src, unsigned bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(smem_u32(dst)), "l"(src),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
    asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// Forward.  A block takes the same tile of images_per_block<N>() images in
// turn and fetches the next image's grid tile while it samples the current
// one: in 2D into registers (loaded before the current image's gathers and
// stored to shared memory after them), in 3D with cp.async into the other
// half of a double-buffered shared tile (no registers held: 42 instead of 60
// registers per thread, 6 blocks per SM instead of 4; 8 x 128^3 volumes 0.129
// -> 0.118 ms; in 2D the register version is faster, 0.32 against 0.36 ms at
// 1024 x 3 x 224^2).  With the channel count known at compile time (CC = C,
// 1..4) a thread issues the corner loads of all channels before the first
// lerp: the gathers are latency-bound, and the extra loads in flight took the
// 1024 x 3 x 224^2 case from 3.7 to 4.5 TB/s.  CC = 0: any C, channel by
// channel.
template <int N>
__host__ __device__ constexpr int images_per_block() { return N == 3 ? 4 : 2; }

template <int N, int CC>
__global__ void __launch_bounds__(256)
    k_interpolate_tiled(Geo g, TileGeo tg, const float *__restrict__ data, int C,
                        const float *__restrict__ grid, float *__restrict__ out, int nb) {
    constexpr bool kAsync = N == 3;
    constexpr int RR = kTile / kRows;
    __shared__ float sp[kAsync ? 2 : 1][N][kTile][kTile + 1];
    int a0, z0, mid;
    tile_coords<N>(g, tg, blockIdx.x, a0, z0, mid);
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int A = g.outsize[0], Z = g.outsize[N - 1];
    float nxt[kAsync ? 1 : RR][N];   // 2D: the next image's grid tile
    // the grid tile of image b, as load_grid_tile would stage it (points
    // outside the image: zeros): 3D into buffer hb by cp.async, 2D into nxt
    auto fetch = [&](int b, int hb) {
        const float *gb = grid + (long long)b * N * g.nP;
#pragma unroll
        for (int r = 0; r < RR; ++r) {
            const int zl = ty + kRows * r, a = a0 + tx, z = z0 + zl;
            const bool in = a < A && z < Z;
            const int k = in ? grid_index<N>(g, a, mid, z) : 0;
#pragma unroll
            for (int j = 0; j < N; ++j) {
                if constexpr (kAsync)
                    cp_async4(&sp[hb][j][zl][tx], gb + (long long)j * g.nP + k, in ? 4u : 0u);
                else
                    nxt[r][j] = in ? __ldg(gb + (long long)j * g.nP + k) : 0.f;
            }
        }
        if constexpr (kAsync) cp_async_commit();
    };
    int b = blockIdx.y, h = 0;
    if (b < nb) fetch(b, 0);
    for (; b < nb; b += gridDim.y) {
        if constexpr (kAsync) {
            cp_async_wait_all();   // this thread's copies of image b have landed
            __syncthreads();       // everyone's; and the other buffer is no longer read
            if (b + (int)gridDim.y < nb) fetch(b + gridDim.y, h ^ 1);
        } else {
            __syncthreads();
#pragma unroll
            for (int r = 0; r < RR; ++r)
#pragma unroll
                for (int j = 0; j < N; ++j) sp[0][j][ty + kRows * r][tx] = nxt[r][j];
            __syncthreads();
            if (b + (int)gridDim.y < nb) fetch(b + gridDim.y, 0);
        }
#pragma unroll 1
        for (int r = 0; r < RR; ++r) {
            const int al = ty + kRows * r, a = a0 + al, z = z0 + tx;
            if (a >= A || z >= Z) continue;
            float p[N];
#pragma unroll
            for (int j = 0; j < N; ++j) p[j] = sp[h][j][tx][al];
            const Corner<N> cr = corners<N>(p, g);
            const int o = out_index<N>(g, a, mid, z);
            if constexpr (CC > 0) {
                float v[CC][1 << N];
#pragma unroll
                for (int c = 0; c < CC; ++c) {
                    const float *D = data + ((long long)b * CC + c) * g.nD;
#pragma unroll
                    for (int m = 0; m < (1 << N); ++m) v[c][m] = __ldg(D + cr.off[m]);
                }
#pragma unroll
                for (int c = 0; c < CC; ++c)
                    out[((long long)b * CC + c) * g.nP + o] = lerp_values<N>(v[c], cr.f);
            } else {
                for (int c = 0; c < C; ++c) {
                    const long long plane = (long long)b * C + c;
                    out[plane * g.nP + o] = lerp_corners<N>(data + plane * g.nD, cr);
                }
            }
        }
        if constexpr (kAsync) h ^= 1;
    }
}

// 2D / 3D forward with the grid tile staged by the tensor memory accelerator.
// One cp.async.bulk.tensor per image copies the tile's box of the grid (2D:
// 32 x, 32 y, 2 components; 3D: 32 x, 1 y, 32 z, 3 components) into shared
// memory with the 128-byte swizzle (the 128-byte row of x values of row
// R = 32 j + z_local has its 16-byte chunks permuted by chunk ^ (R & 7)),
// double-buffered on two mbarriers, so the staging costs no per-point
// instructions; points outside the image read the zero fill.  Lane z_local
// then reads the four x values of its chunk (x_local = 4 warp + u) with one
// 16-byte load per component, conflict-free under the swizzle, and samples TP
// points at a time with all their corner loads issued before the first lerp.
// Corners are addressed from one base pointer per point (CornerStep).  The
// output is stored directly: the lanes of a warp write 32 consecutive z.
// Identical results to k_interpolate_tiled, fewer instructions: on 8 x 128^3
// volumes 0.095 against 0.125 ms (110 instead of 183 instructions per point);
// on 3 x 224^2 images 0.032 against 0.037 ms at 64 images, 0.311 against
// 0.323 ms at 1024.  Blocks per SM are capped so that the shared-memory
// carve-out leaves most of L1 to the gathers (3D at 4 blocks: 77 % sector
// hits; at 6 or 8 the hit rate and the speed drop).
template <int N>
__host__ __device__ constexpr int tma_box() { return N * kTile * kTile; }   // floats per grid tile
template <int N>
__host__ __device__ constexpr int tma_smem() { return 1024 + 2 * tma_box<N>() * 4 + 2 * 8; }

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int c0, int c1,
                                            int c2, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *map, int c0, int c1,
                                            int c2, int c3, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3),
        "r"(smem_u32(bar))
        : "memory");
}

// The grid tile of image b into buf (completion on bar).
template <int N>
__device__ __forceinline__ void tma_grid_tile(float *buf, const CUtensorMap *map, int a0, int mid,
                                              int z0, int b, uint64_t *bar) {
    mbar_arrive_expect_tx(bar, tma_box<N>() * 4);
    if constexpr (N == 2) tma_load_3d(buf, map, a0, z0, 2 * b, bar);
    else tma_load_4d(buf, map, a0, mid, z0, 3 * b, bar);
}

// Points whose corner loads are issued together, and blocks per SM.  3D: the
// gathered values of one group stay within 64 registers per thread for one
// or two channels; three channels take one point at a time and up to 80
// registers (four would spill: they use k_interpolate_tiled<3, 4>).  2D: one
// point at a time, 6 blocks per SM (40 registers), 5 for four channels.
template <int N, int CC>
__host__ __device__ constexpr int tma_points_per_group() { return N == 3 && CC == 1 ? 4 : 1; }
template <int N, int CC>
__host__ __device__ constexpr int tma_blocks_per_sm() {
    return N == 2 ? (CC <= 3 ? 6 : 5) : CC <= 2 ? 4 : 3;
}

template <int N, int CC, bool FB>
__global__ void __launch_bounds__(256, tma_blocks_per_sm<N, CC>())
    k_interpolate_tma(const __grid_constant__ CUtensorMap gmap, Geo g, TileGeo tg,
                      const float *__restrict__ data, float *__restrict__ out, int nb,
                      unsigned *err) {
    constexpr int TP = tma_points_per_group<N, CC>(), BOX = tma_box<N>();
    extern __shared__ unsigned char smem_raw[];
    // the swizzle pattern follows address bits 7-9: 1024-byte aligned buffers
    float *gbuf = reinterpret_cast<float *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t *bar = reinterpret_cast<uint64_t *>(gbuf + 2 * BOX);
    int a0, z0, mid;
    tile_coords<N>(g, tg, blockIdx.x, a0, z0, mid);
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int A = g.outsize[0], Z = g.outsize[N - 1];
    const bool leader = threadIdx.x == 0;
    if (leader) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
    }
    __syncthreads();
    int b = blockIdx.y;
    if (leader && b < nb) tma_grid_tile<N>(gbuf, &gmap, a0, mid, z0, b, &bar[0]);
    const int chunk = ((ty ^ (tx & 7)) << 4);   // byte offset of this lane's x chunk in its row
    for (int k = 0; b < nb; b += gridDim.y, ++k) {
        const int hb = k & 1;
        const unsigned parity = (k >> 1) & 1;
        const bool got = mbar_wait_bounded(&bar[hb], parity);
        // every thread is done with the other buffer (image k - 1) past this barrier
        if (__syncthreads_or(!got)) {
            if (leader) raise_error(err, kErrTmaTimeout);
            mbar_wait_bounded(&bar[hb], parity);   // a second bounded wait for the copy in flight
            break;
        }
        if (leader && b + (int)gridDim.y < nb)
            tma_grid_tile<N>(gbuf + (hb ^ 1) * BOX, &gmap, a0, mid, z0, b + gridDim.y,
                             &bar[hb ^ 1]);
        const unsigned char *gt = reinterpret_cast<const unsigned char *>(gbuf + hb * BOX);
        float pp[4][N];
#pragma unroll
        for (int j = 0; j < N; ++j) {
            const float4 q = *reinterpret_cast<const float4 *>(gt + (kTile * j + tx) * 128 + chunk);
            pp[0][j] = q.x;
            pp[1][j] = q.y;
            pp[2][j] = q.z;
            pp[3][j] = q.w;
        }
        const float *Db = data + (long long)b * CC * g.nD;
        float *Ob = out + (long long)b * CC * g.nP;
        const int z = z0 + tx;
#pragma unroll
        for (int u0 = 0; u0 < 4; u0 += TP) {
            float v[TP][CC][1 << N];
            float f[TP][N];
#pragma unroll
            for (int w = 0; w < TP; ++w) {
                const CornerStep<N> cr = corner_steps<N, FB>(pp[u0 + w], g);
#pragma unroll
                for (int c = 0; c < CC; ++c) {
                    const float *P = Db + (long long)c * g.nD + cr.base;
#pragma unroll
                    for (int m = 0; m < (1 << N); ++m) v[w][c][m] = __ldg(P + cr.delta(m));
                }
#pragma unroll
                for (int j = 0; j < N; ++j) f[w][j] = cr.f[j];
            }
#pragma unroll
            for (int w = 0; w < TP; ++w) {
                const int a = a0 + 4 * ty + u0 + w;
                if (a < A && z < Z) {
                    const int o = out_index<N>(g, a, mid, z);
#pragma unroll
                    for (int c = 0; c < CC; ++c)
                        Ob[(long long)c * g.nP + o] = lerp_values<N>(v[w][c], f[w]);
                }
            }
        }
    }
}

template <int N>
__global__ void __launch_bounds__(256)
    k_interpolate_backward_tiled(Geo g, TileGeo tg, const float *__restrict__ data, int C,
                                 const float *__restrict__ grid, const float *__restrict__ gout,
                                 float *__restrict__ ddata, float *__restrict__ dgrid, int nb) {
    __shared__ float sp[N][kTile][kTile + 1];
    int a0, z0, mid;
    tile_coords<N>(g, tg, blockIdx.x, a0, z0, mid);
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int A = g.outsize[0], Z = g.outsize[N - 1];
    for (int b = blockIdx.y; b < nb; b += gridDim.y) {
        __syncthreads();
        load_grid_tile<N>(g, grid + (long long)b * N * g.nP, a0, z0, mid, sp);
        __syncthreads();
        float gfs[kTile / kRows][N];
#pragma unroll
        for (int r = 0; r < kTile / kRows; ++r) {
            const int al = ty + kRows * r, a = a0 + al, z = z0 + tx;
#pragma unroll
            for (int j = 0; j < N; ++j) gfs[r][j] = 0.f;
            if (a >= A || z >= Z) continue;
            float p[N];
#pragma unroll
            for (int j = 0; j < N; ++j) p[j] = sp[j][tx][al];
            const Corner<N> cr = corners<N>(p, g);
            const int o = out_index<N>(g, a, mid, z);
            for (int c = 0; c < C; ++c) {
                const long long plane = (long long)b * C + c;
                const float w = __ldg(gout + plane * g.nP + o);
                lerp_grads<N>(data + plane * g.nD, cr, w, ddata ? ddata + plane * g.nD : nullptr,
                              gfs[r]);
            }
        }
        if (!dgrid) continue;
        __syncthreads();
#pragma unroll
        for (int r = 0; r < kTile / kRows; ++r) {
            const int al = ty + kRows * r;
#pragma unroll
            for (int j = 0; j < N; ++j) sp[j][tx][al] = gfs[r][j] * g.sizem1[j];
        }
        __syncthreads();
        float *db = dgrid + (long long)b * N * g.nP;
#pragma unroll
        for (int r = 0; r < kTile / kRows; ++r) {
            const int zl = ty + kRows * r, a = a0 + tx, z = z0 + zl;
            if (a < A && z < Z) {
                const int k = grid_index<N>(g, a, mid, z);
#pragma unroll
                for (int j = 0; j < N; ++j) db[(long long)j * g.nP + k] = sp[j][zl][tx];
            }
        }
    }
}

static TileGeo make_tiles(int ndim, const Geo &g, unsigned *blocks) {
    TileGeo tg;
    tg.ta = (g.outsize[0] + kTile - 1) / kTile;
    tg.tz = (g.outsize[ndim - 1] + kTile - 1) / kTile;
    *blocks = (unsigned)tg.ta * tg.tz * (ndim == 3 ? (unsigned)g.outsize[1] : 1u);
    return tg;
}

// cuTensorMapEncodeTiled through the CUDA runtime's entry-point query (no link
// against libcuda); null where the installed CUDA driver does not provide it.
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000,
                                             cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            f = nullptr;
        }
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    }();
    return fn;
}

// The grid [nb, N, (D_out,) H_out, W_out] (x fastest) as an (N + 1)-D tensor
// map with the box of k_interpolate_tma.  False where the tensor memory
// accelerator cannot address it: a grid not 16-byte aligned or a row stride
// (W_out floats) not a multiple of 16 bytes.
static bool encode_grid_map(CUtensorMap *map, int ndim, const float *grid, const int *outsize,
                            int nb) {
    const PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc || (reinterpret_cast<uintptr_t>(grid) & 15u) || (outsize[0] & 3)) return false;
    cuuint64_t dims[4], strides[3];
    cuuint32_t box[4];
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    cuuint64_t stride = 4;
    for (int j = 0; j < ndim; ++j) {
        dims[j] = (cuuint64_t)outsize[j];
        stride *= dims[j];
        strides[j] = stride;   // bytes from one index of axis j + 1 to the next
        box[j] = (ndim == 3 && j == 1) ? 1u : (cuuint32_t)kTile;
    }
    dims[ndim] = (cuuint64_t)ndim * nb;   // (image, component) planes
    box[ndim] = (cuuint32_t)ndim;
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, ndim + 1, const_cast<float *>(grid), dims,
               strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
               CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int N, int CC>
static cudaError_t launch_tma(const CUtensorMap &map, const Geo &g, const TileGeo &tg,
                              dim3 tgrid, const float *data, float *out, int nb, unsigned *err,
                              cudaStream_t s) {
    if (g.nD < (1 << 23))
        k_interpolate_tma<N, CC, true>
            <<<tgrid, 256, tma_smem<N>(), s>>>(map, g, tg, data, out, nb, err);
    else
        k_interpolate_tma<N, CC, false>
            <<<tgrid, 256, tma_smem<N>(), s>>>(map, g, tg, data, out, nb, err);
    return cudaGetLastError();
}

cudaError_t launch_interpolate(int ndim, const float *data, int nb, int C, const int *size,
                               const float *grid, const int *outsize, float *out,
                               unsigned *err, cudaStream_t s) {
    const Geo g = make_geo(ndim, size, outsize);
    if ((long long)nb * g.nP == 0) return cudaSuccess;
    const int block = 256;
    const dim3 gridn((unsigned)((g.nP + block - 1) / block),
                     (unsigned)(nb < (int)kMaxGridY ? nb : kMaxGridY));
    if (ndim == 1) {
        k_interpolate<1><<<gridn, block, 0, s>>>(g, data, C, grid, out, nb);
        return cudaGetLastError();
    }
    unsigned blocks = 0;
    const TileGeo tg = make_tiles(ndim, g, &blocks);
    const int ipb = ndim == 3 ? images_per_block<3>() : images_per_block<2>();
    const dim3 tgrid(blocks, (gridn.y + ipb - 1) / ipb);
    CUtensorMap map;
    if (C <= (ndim == 3 ? 3 : 4) && encode_grid_map(&map, ndim, grid, outsize, nb)) {
        if (ndim == 2) {
            switch (C) {
                case 1: return launch_tma<2, 1>(map, g, tg, tgrid, data, out, nb, err, s);
                case 2: return launch_tma<2, 2>(map, g, tg, tgrid, data, out, nb, err, s);
                case 3: return launch_tma<2, 3>(map, g, tg, tgrid, data, out, nb, err, s);
                default: return launch_tma<2, 4>(map, g, tg, tgrid, data, out, nb, err, s);
            }
        }
        switch (C) {
            case 1: return launch_tma<3, 1>(map, g, tg, tgrid, data, out, nb, err, s);
            case 2: return launch_tma<3, 2>(map, g, tg, tgrid, data, out, nb, err, s);
            default: return launch_tma<3, 3>(map, g, tg, tgrid, data, out, nb, err, s);
        }
    }
#define CPAB_IT(NN, CC) k_interpolate_tiled<NN, CC><<<tgrid, block, 0, s>>>(g, tg, data, C, grid, out, nb)
    if (ndim == 2) {
        switch (C) {
            case 1: CPAB_IT(2, 1); break;
            case 2: CPAB_IT(2, 2); break;
            case 3: CPAB_IT(2, 3); break;
            case 4: CPAB_IT(2, 4); break;
            default: CPAB_IT(2, 0); break;
        }
    } else {
        switch (C) {
            case 1: CPAB_IT(3, 1); break;
            case 2: CPAB_IT(3, 2); break;
            case 3: CPAB_IT(3, 3); break;
            case 4: CPAB_IT(3, 4); break;
            default: CPAB_IT(3, 0); break;
        }
    }
#undef CPAB_IT
    return cudaGetLastError();
}

cudaError_t launch_interpolate_backward(int ndim, const float *data, int nb, int C,
                                        const int *size, const float *grid, const int *outsize,
                                        const float *gout, float *ddata, float *dgrid,
                                        cudaStream_t s) {
    const Geo g = make_geo(ndim, size, outsize);
    if ((long long)nb * g.nP == 0) return cudaSuccess;
    const int block = 256;
    const dim3 gridn((unsigned)((g.nP + block - 1) / block),
                     (unsigned)(nb < (int)kMaxGridY ? nb : kMaxGridY));
    if (ndim == 1) {
        k_interpolate_backward<1><<<gridn, block, 0, s>>>(g, data, C, grid, gout, ddata, dgrid, nb);
        return cudaGetLastError();
    }
    unsigned blocks = 0;
    const TileGeo tg = make_tiles(ndim, g, &blocks);
    const dim3 tgrid(blocks, gridn.y);
    if (ndim == 2)
        k_interpolate_backward_tiled<2><<<tgrid, block, 0, s>>>(g, tg, data, C, grid, gout, ddata,
                                                               dgrid, nb);
    else
        k_interpolate_backward_tiled<3><<<tgrid, block, 0, s>>>(g, tg, data, C, grid, gout, ddata,
                                                               dgrid, nb);
    return cudaGetLastError();
}

}  // namespace cpab
