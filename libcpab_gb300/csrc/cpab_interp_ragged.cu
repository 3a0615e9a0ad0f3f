// Ragged interpolation: S images of mixed sizes sampled in one launch.
//
// The reference's interpolator takes one data size and one outsize per call
// (libcpab/pytorch/interpolation.py:39-40, 104-106), so a batch of images of
// different sizes is a loop of transform_data calls (libcpab/cpab.py:304-331).
// Here image s has its own size and outsize, and all images are sampled by
// one launch with the reference's arithmetic (the helpers of
// cpab_interp.cuh, shared with cpab_interp.cu and the fused kernels, so every
// image's output is bit-identical to cpab_interpolate on that image alone).
//
// Layout (one int64 plan row of kImagePlanFields per image, built on the host
// by cpab_ragged_images_plan and read by the kernels from device memory):
//   data  packed [C, size_s] blocks, image s at C * data_off[s];
//   grid  [ndim, total], image s in the columns pts_off[s] ..
//         pts_off[s] + prod(outsize_s), meshgrid order (x fastest);
//   out   packed [C, outsize_s] blocks, image s at C * pts_off[s].
//
// Work unit: one 256-thread block per tile.  1D: 256 consecutive points.
// 2D / 3D: 8 x-rows x 32 last-axis columns (at one y in 3D).  The 32 lanes
// of a warp take consecutive last-axis points, so output stores are
// contiguous and neighbouring lanes gather neighbouring data elements; the 8
// warps of a block read 8 consecutive x of the meshgrid-ordered grid at each
// column, i.e. whole 32-byte sectors between them (through L1).
//
// A block finds its image by binary search over the tile prefix and checks
// the plan rows it uses (positive extents below 2^22, per-image element
// counts below 2^31, offset deltas equal to the extents' products, end
// offsets within the buffers' sizes) before it touches memory; a block whose
// rows fail the check raises CPAB_DEV_BAD_OFFSETS and does nothing.
#include "cpab_interp.cuh"

namespace cpab {

namespace {

constexpr int kImgRows = 8, kImgCols = 32, kImgBlock = 256;

struct ImageTile {
    Geo g;             // size, sizem1, nP, nD (outsize used for the extents)
    long long dbase;   // first data point of the image (times C = element offset)
    long long pbase;   // first grid column / output point of the image
    int a, mid, z;     // this thread's point (x index, y index in 3D, last-axis index)
    bool live;         // the point exists (inside the image's extents)
};

// Locate tile t, check the plan rows, and place this thread's point.
// Returns false (after flagging) when the plan rows are inconsistent.
template <int N>
__device__ __forceinline__ bool image_tile(const long long *__restrict__ plan, int S,
                                           long long data_points, long long total, long long t,
                                           ImageTile &it, unsigned *err) {
    constexpr int F = kImagePlanFields;
    const long long *last = plan + (long long)S * F;
    if (t == 0 && threadIdx.x == 0 &&
        (plan[0] != 0 || plan[1] != 0 || last[1] != total || last[2] != (long long)gridDim.x))
        raise_error(err, kErrBadOffsets);   // the launch would not cover every point
    if (!(plan[2] <= t && t < last[2])) {
        raise_error(err, kErrBadOffsets);
        return false;
    }
    int lo = 0, hi = S;   // plan[lo].tile <= t < plan[hi].tile
    while (hi - lo > 1) {
        const int m = (lo + hi) >> 1;
        if (plan[(long long)m * F + 2] <= t) lo = m;
        else hi = m;
    }
    const long long *r0 = plan + (long long)lo * F, *r1 = r0 + F;
    long long nP = 1, nD = 1;
    bool ok = r0[0] >= 0 && r0[1] >= 0;
    int size[3] = {1, 1, 1}, outsize[3] = {1, 1, 1};
#pragma unroll
    for (int j = 0; j < N; ++j) {
        const long long sj = r0[3 + j], oj = r0[6 + j];
        ok = ok && sj >= 1 && sj < (1 << 22) && oj >= 1 && oj < (1 << 22);
        if (!ok) break;
        size[j] = (int)sj;
        outsize[j] = (int)oj;
        nD *= sj;
        nP *= oj;
        ok = nD < (1ll << 31) && nP < (1ll << 31);
    }
    ok = ok && r1[0] - r0[0] == nD && r1[1] - r0[1] == nP &&
         r1[2] - r0[2] == image_tile_count(N, outsize) && r1[0] <= data_points &&
         r1[1] <= total;
    if (!ok) {
        raise_error(err, kErrBadOffsets);
        return false;
    }
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        it.g.size[j] = size[j];
        it.g.outsize[j] = outsize[j];
        it.g.sizem1[j] = (float)(size[j] - 1);
    }
    it.g.nP = (int)nP;
    it.g.nD = (int)nD;
    it.dbase = r0[0];
    it.pbase = r0[1];
    const int lt = (int)(t - r0[2]);   // tile within the image, < 2^31 (tiles <= points)
    if constexpr (N == 1) {
        it.a = lt * kImgBlock + (int)threadIdx.x;
        it.mid = 0;
        it.z = 0;
        it.live = it.a < outsize[0];
    } else {
        const int ta = (outsize[0] + kImgRows - 1) / kImgRows;
        const int tz = (outsize[N - 1] + kImgCols - 1) / kImgCols;
        const int per = ta * tz;
        it.mid = (N == 3) ? lt / per : 0;
        const int r = lt - it.mid * per;
        it.a = (r % ta) * kImgRows + (int)(threadIdx.x >> 5);
        it.z = (r / ta) * kImgCols + (int)(threadIdx.x & 31);
        it.live = it.a < outsize[0] && it.z < outsize[N - 1];
    }
    return true;
}

// meshgrid index (x fastest) and output index (last axis fastest)
template <int N>
__device__ __forceinline__ int img_grid_index(const ImageTile &it) {
    if constexpr (N == 1) return it.a;
    else if constexpr (N == 2) return it.a + it.g.outsize[0] * it.z;
    else return it.a + it.g.outsize[0] * (it.mid + it.g.outsize[1] * it.z);
}
template <int N>
__device__ __forceinline__ int img_out_index(const ImageTile &it) {
    if constexpr (N == 1) return it.a;
    else if constexpr (N == 2) return it.a * it.g.outsize[1] + it.z;
    else return (it.a * it.g.outsize[1] + it.mid) * it.g.outsize[2] + it.z;
}

template <int N>
__global__ void __launch_bounds__(kImgBlock)
    k_interpolate_ragged(const long long *__restrict__ plan, int S, long long data_points,
                         const float *__restrict__ data, int C, long long total,
                         const float *__restrict__ grid, float *__restrict__ out,
                         unsigned *err) {
    ImageTile it;
    if (!image_tile<N>(plan, S, data_points, total, blockIdx.x, it, err) || !it.live) return;
    const long long col = it.pbase + img_grid_index<N>(it);
    float p[N];
#pragma unroll
    for (int j = 0; j < N; ++j) p[j] = __ldg(grid + (long long)j * total + col);
    const Corner<N> cr = corners<N>(p, it.g);
    const float *D = data + it.dbase * C;
    float *O = out + it.pbase * C + img_out_index<N>(it);
    for (int c = 0; c < C; ++c)
        O[(long long)c * it.g.nP] = lerp_corners<N>(D + (long long)c * it.g.nD, cr);
}

template <int N>
__global__ void __launch_bounds__(kImgBlock)
    k_interpolate_ragged_backward(const long long *__restrict__ plan, int S,
                                  long long data_points, const float *__restrict__ data, int C,
                                  long long total, const float *__restrict__ grid,
                                  const float *__restrict__ gout, float *__restrict__ ddata,
                                  float *__restrict__ dgrid, unsigned *err) {
    ImageTile it;
    if (!image_tile<N>(plan, S, data_points, total, blockIdx.x, it, err) || !it.live) return;
    const long long col = it.pbase + img_grid_index<N>(it);
    float p[N];
#pragma unroll
    for (int j = 0; j < N; ++j) p[j] = __ldg(grid + (long long)j * total + col);
    const Corner<N> cr = corners<N>(p, it.g);
    const float *D = data + it.dbase * C;
    float *DD = ddata ? ddata + it.dbase * C : nullptr;
    const float *G = gout + it.pbase * C + img_out_index<N>(it);
    float gf[N];
#pragma unroll
    for (int j = 0; j < N; ++j) gf[j] = 0.f;
    for (int c = 0; c < C; ++c) {
        const long long plane = (long long)c * it.g.nD;
        lerp_grads<N>(D + plane, cr, __ldg(G + (long long)c * it.g.nP), DD ? DD + plane : nullptr,
                      gf);
    }
    if (dgrid) {
#pragma unroll
        for (int j = 0; j < N; ++j) dgrid[(long long)j * total + col] = gf[j] * it.g.sizem1[j];
    }
}

}  // namespace

cudaError_t launch_interpolate_ragged(int ndim, int S, const long long *plan,
                                      long long data_points, const float *data, int C,
                                      long long total, long long tiles, const float *grid,
                                      float *out, unsigned *err, cudaStream_t s) {
    if (tiles <= 0) return cudaSuccess;
    const dim3 gridn((unsigned)tiles);
    switch (ndim) {
    case 1:
        k_interpolate_ragged<1><<<gridn, kImgBlock, 0, s>>>(plan, S, data_points, data, C, total,
                                                            grid, out, err);
        break;
    case 2:
        k_interpolate_ragged<2><<<gridn, kImgBlock, 0, s>>>(plan, S, data_points, data, C, total,
                                                            grid, out, err);
        break;
    default:
        k_interpolate_ragged<3><<<gridn, kImgBlock, 0, s>>>(plan, S, data_points, data, C, total,
                                                            grid, out, err);
    }
    return cudaGetLastError();
}

cudaError_t launch_interpolate_ragged_backward(int ndim, int S, const long long *plan,
                                               long long data_points, const float *data, int C,
                                               long long total, long long tiles,
                                               const float *grid, const float *gout,
                                               float *ddata, float *dgrid, unsigned *err,
                                               cudaStream_t s) {
    if (tiles <= 0) return cudaSuccess;
    const dim3 gridn((unsigned)tiles);
    switch (ndim) {
    case 1:
        k_interpolate_ragged_backward<1><<<gridn, kImgBlock, 0, s>>>(
            plan, S, data_points, data, C, total, grid, gout, ddata, dgrid, err);
        break;
    case 2:
        k_interpolate_ragged_backward<2><<<gridn, kImgBlock, 0, s>>>(
            plan, S, data_points, data, C, total, grid, gout, ddata, dgrid, err);
        break;
    default:
        k_interpolate_ragged_backward<3><<<gridn, kImgBlock, 0, s>>>(
            plan, S, data_points, data, C, total, grid, gout, ddata, dgrid, err);
    }
    return cudaGetLastError();
}

}  // namespace cpab
