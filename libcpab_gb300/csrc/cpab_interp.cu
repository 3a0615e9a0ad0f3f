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
// point for all channels.  Grid: x over points of an image, y over images.
//
// Backward: d(data) is a scatter-add (float atomics into a zeroed buffer, like
// the reference's autograd index_put accumulation); d(grid) follows the
// gradient of the lerp weights, as autograd does through xd, yd, zd.
#include "cpab_interp.cuh"

namespace cpab {

constexpr unsigned kMaxGridY = 65535;

template <int N>
__global__ void __launch_bounds__(256)
    k_interpolate(Geo g, const float *__restrict__ data, int C, const float *__restrict__ grid,
                  float *__restrict__ out, int nb) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= g.nP) return;
    const int oo = out_offset<N>(k, g);
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
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= g.nP) return;
    const int oo = out_offset<N>(k, g);
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

cudaError_t launch_interpolate(int ndim, const float *data, int nb, int C, const int *size,
                               const float *grid, const int *outsize, float *out,
                               cudaStream_t s) {
    const Geo g = make_geo(ndim, size, outsize);
    if ((long long)nb * g.nP == 0) return cudaSuccess;
    const int block = 256;
    const dim3 gridn((unsigned)((g.nP + block - 1) / block),
                     (unsigned)(nb < (int)kMaxGridY ? nb : kMaxGridY));
    switch (ndim) {
        case 1: k_interpolate<1><<<gridn, block, 0, s>>>(g, data, C, grid, out, nb); break;
        case 2: k_interpolate<2><<<gridn, block, 0, s>>>(g, data, C, grid, out, nb); break;
        default: k_interpolate<3><<<gridn, block, 0, s>>>(g, data, C, grid, out, nb); break;
    }
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
    switch (ndim) {
        case 1: k_interpolate_backward<1><<<gridn, block, 0, s>>>(g, data, C, grid, gout, ddata, dgrid, nb); break;
        case 2: k_interpolate_backward<2><<<gridn, block, 0, s>>>(g, data, C, grid, gout, ddata, dgrid, nb); break;
        default: k_interpolate_backward<3><<<gridn, block, 0, s>>>(g, data, C, grid, gout, ddata, dgrid, nb); break;
    }
    return cudaGetLastError();
}

}  // namespace cpab
