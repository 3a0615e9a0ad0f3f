// Device helpers for linear / bilinear / trilinear sampling, shared by
// cpab_interp.cu and the fused transform_data kernels (cpab_fused.cu).
// Semantics: libcpab/pytorch/interpolation.py:18-172 (see cpab_interp.cu).
#pragma once
#include "cpab_launch.h"

namespace cpab {

struct Geo {
    int size[3];      // data extent per axis (W, H, D)
    int outsize[3];   // output extent per axis
    long long nP;     // prod(outsize)
    long long nD;     // prod(size)
};

template <int N>
struct Corner {
    long long off[1 << N];   // element offsets of the 2^N corners, corner bit j = axis j high
    float f[N];              // lerp weights xd, yd, zd
};

template <int N>
__device__ __forceinline__ Corner<N> corners(const float (&p)[N], const Geo &g) {
    Corner<N> cr;
    long long i0[N], i1[N];
#pragma unroll
    for (int j = 0; j < N; ++j) {
        const float x = p[j] * (float)(g.size[j] - 1);
        const float fl = floorf(x);
        // floor() then int64 conversion as torch does; clamp into the data.
        long long a = (fl != fl) ? 0ll : (long long)fl;
        long long b = a + 1;
        a = a < 0 ? 0 : (a > g.size[j] - 1 ? g.size[j] - 1 : a);
        b = b < 0 ? 0 : (b > g.size[j] - 1 ? g.size[j] - 1 : b);
        i0[j] = a;
        i1[j] = b;
        cr.f[j] = x - (float)a;
    }
#pragma unroll
    for (int m = 0; m < (1 << N); ++m) {
        long long o = 0;
#pragma unroll
        for (int j = 0; j < N; ++j) o = o * g.size[j] + (((m >> j) & 1) ? i1[j] : i0[j]);
        cr.off[m] = o;
    }
    return cr;
}

// Lerp in the reference's order: along x first, then y, then z.
template <int N>
__device__ __forceinline__ float lerp_corners(const float *D, const Corner<N> &cr) {
    float v[1 << N];
#pragma unroll
    for (int m = 0; m < (1 << N); ++m) v[m] = __ldg(D + cr.off[m]);
#pragma unroll
    for (int j = 0; j < N; ++j) {
        const float w1 = cr.f[j], w0 = 1.f - cr.f[j];
#pragma unroll
        for (int m = 0; m < (1 << (N - 1 - j)); ++m)
            v[m] = __fadd_rn(__fmul_rn(v[2 * m], w0), __fmul_rn(v[2 * m + 1], w1));
        // after pass j, v[m] holds the lerp over axes 0..j for corner bits above j
    }
    return v[0];
}

// Offsets in corner order for lerp_corners: pass j pairs entries (2m, 2m+1),
// so corner index bits must be ordered with axis 0 as the lowest bit after
// each pass.  corners() builds index m with bit j = axis j; pass 0 pairs m
// with m^1 (axis 0), leaving entries indexed by the remaining bits (axis 1 as
// bit 0), and so on.

// Output element offset of point k within one (b, c) plane: [W_out(, H_out(, D_out))]
// with the last axis fastest, while k has axis 0 fastest.
template <int N>
__device__ __forceinline__ long long out_offset(long long k, const Geo &g) {
    if constexpr (N == 1) return k;
    else if constexpr (N == 2) {
        const long long ix = k % g.outsize[0], iy = k / g.outsize[0];
        return ix * g.outsize[1] + iy;
    } else {
        const long long ix = k % g.outsize[0];
        const long long r = k / g.outsize[0];
        const long long iy = r % g.outsize[1], iz = r / g.outsize[1];
        return (ix * g.outsize[1] + iy) * g.outsize[2] + iz;
    }
}

// d(lerp)/d(f_j) and the per-corner weights, for the backward passes.
template <int N>
__device__ __forceinline__ void lerp_grads(const float *D, const Corner<N> &cr, float w,
                                           float *ddata_plane, float (&gf)[N]) {
    float v[1 << N];
#pragma unroll
    for (int m = 0; m < (1 << N); ++m) v[m] = __ldg(D + cr.off[m]);
#pragma unroll
    for (int m = 0; m < (1 << N); ++m) {
        // chain order of autograd: last lerp (highest axis) first
        float wt = w;
#pragma unroll
        for (int j = N - 1; j >= 0; --j) wt *= ((m >> j) & 1) ? cr.f[j] : (1.f - cr.f[j]);
        if (ddata_plane) atomicAdd(ddata_plane + cr.off[m], wt);
    }
#pragma unroll
    for (int j = 0; j < N; ++j) {
        // d/df_j: difference along axis j, weighted by the other axes' lerp weights
        float s = 0.f;
#pragma unroll
        for (int m = 0; m < (1 << N); ++m) {
            if ((m >> j) & 1) continue;
            float wt = 1.f;
#pragma unroll
            for (int q = 0; q < N; ++q)
                if (q != j) wt *= ((m >> q) & 1) ? cr.f[q] : (1.f - cr.f[q]);
            s = fmaf(wt, v[m | (1 << j)] - v[m], s);
        }
        gf[j] += w * s;
    }
}

inline Geo make_geo(int ndim, const int *size, const int *outsize) {
    Geo g;
    g.nP = 1;
    g.nD = 1;
    for (int j = 0; j < 3; ++j) {
        g.size[j] = j < ndim ? size[j] : 1;
        g.outsize[j] = j < ndim ? outsize[j] : 1;
    }
    for (int j = 0; j < ndim; ++j) {
        g.nP *= outsize[j];
        g.nD *= size[j];
    }
    return g;
}

}  // namespace cpab
