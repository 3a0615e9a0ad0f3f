// Fused composition of transformations: transform_data through T_K o ... o T_1.
//
// The reference's CpabSequential.transform_data (libcpab/sequential.py:
// 109-128) builds the meshgrid, calls transform_grid once per transformation
// (each a separate launch, with the grid in global memory in between) and
// interpolates the final grid.  Here one kernel takes every grid point
// through all stages in registers (each stage with its own tessellation,
// table and step count; compensated update and exact lookup as in
// k_transform_data) and samples the data at the end.  The stages' tables of
// the block's image are staged in shared memory one after another.
#include "cpab_interp.cuh"

namespace cpab {

template <int N, int PPT>
__global__ void __launch_bounds__(256)
    k_sequential_transform_data(SeqStages sq, Geo g, const float *__restrict__ lin, int C,
                                const float *__restrict__ data, float *__restrict__ out,
                                float *__restrict__ grid_out, unsigned long long *ties,
                                unsigned *err) {
    constexpr int P = N * (N + 1);
    constexpr int KS = kMaxPre + 1;
    extern __shared__ float4 smem4[];
    float *tab = reinterpret_cast<float *>(smem4);
    const int b = blockIdx.y, tile = blockIdx.x;
    int off[KS];
    int o = 0;
#pragma unroll
    for (int k = 0; k < KS; ++k) {
        off[k] = o;
        if (k < sq.K) {
            const int G = sq.t[k].nC * P;
            const float *src = sq.E[k] + (long long)b * G;
            for (int i = threadIdx.x; i < G; i += blockDim.x) tab[o + i] = __ldg(src + i);
            o += (G + 3) & ~3;
        }
    }
    __syncthreads();
    float p[PPT][N];
    int oi[PPT];
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
        oi[j] = (tile * PPT + j) * (int)blockDim.x + (int)threadIdx.x;
        if (oi[j] < g.nP) {
            unsigned idx[N];
            unsigned r = (unsigned)oi[j];
#pragma unroll
            for (int a = N - 1; a >= 0; --a) {
                const unsigned q = fast_div(r, g.dout[a]);
                idx[a] = r - q * g.outsize[a];
                r = q;
            }
            int lo = 0;
#pragma unroll
            for (int a = 0; a < N; ++a) {
                p[j][a] = __ldg(lin + lo + idx[a]);
                lo += g.outsize[a];
            }
        } else {
#pragma unroll
            for (int a = 0; a < N; ++a) p[j][a] = 0.5f;
        }
    }
#pragma unroll
    for (int k = 0; k < KS; ++k) {
        if (k >= sq.K) break;
        const Tess &t = sq.t[k];
        const float *tk = tab + off[k];
        for (int s = 0; s < sq.nsteps[k]; ++s) {
#pragma unroll
            for (int j = 0; j < PPT; ++j) {
                int c = find_cell<N>(p[j], t, ties);
                float M[P], y[N];
                load_cell<N>(tk, c, M);
                affine_apply<N>(M, p[j], y);
#pragma unroll
                for (int r = 0; r < N; ++r) p[j][r] += y[r];
            }
        }
    }
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
        if (oi[j] >= g.nP) continue;
        const Corner<N> cr = corners<N>(p[j], g);
        for (int c = 0; c < C; ++c)
            out[((long long)b * C + c) * g.nP + oi[j]] =
                lerp_corners<N>(data + ((long long)b * C + c) * g.nD, cr);
        if (grid_out) {
#pragma unroll
            for (int r = 0; r < N; ++r) grid_out[((long long)b * N + r) * g.nP + oi[j]] = p[j][r];
        }
    }
}

cudaError_t launch_sequential_transform_data(const SeqStages &sq, const float *lin,
                                             const int *outsize, int nb, const float *data,
                                             int C, const int *size, float *out,
                                             float *grid_out, unsigned long long *ties,
                                             unsigned *err, cudaStream_t s) {
    const int ndim = sq.t[0].ndim;
    const Geo g = make_geo(ndim, size, outsize);
    if ((long long)nb * g.nP == 0) return cudaSuccess;
    if (nb > 65535) return cudaErrorInvalidConfiguration;   // images on grid y
    const int block = 256;
    const bool two = (long long)nb * g.nP >= (long long)num_sms() * 2048 * 2;
    const int ppt = two ? 2 : 1;
    const long long per = (long long)block * ppt;
    const int tiles = (int)((g.nP + per - 1) / per);
    const dim3 grid((unsigned)tiles, (unsigned)nb);
    size_t floats = 0;
    for (int k = 0; k < sq.K; ++k) floats += (size_t)((sq.t[k].nC * ndim * (ndim + 1) + 3) & ~3);
    const size_t smem = floats * sizeof(float);
#define CPAB_SQ(N, PP)                                                                        \
    {                                                                                         \
        auto kern = k_sequential_transform_data<N, PP>;                                       \
        if (smem > 48 * 1024) {                                                               \
            cudaError_t e = cudaFuncSetAttribute(                                             \
                kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);                \
            if (e != cudaSuccess) return e;                                                   \
        }                                                                                     \
        kern<<<grid, block, smem, s>>>(sq, g, lin, C, data, out, grid_out, ties, err);        \
        return cudaGetLastError();                                                            \
    }
    switch (ndim) {
        case 1: if (two) CPAB_SQ(1, 2) else CPAB_SQ(1, 1)
        case 2: if (two) CPAB_SQ(2, 2) else CPAB_SQ(2, 1)
        default: if (two) CPAB_SQ(3, 2) else CPAB_SQ(3, 1)
    }
#undef CPAB_SQ
}

}  // namespace cpab
