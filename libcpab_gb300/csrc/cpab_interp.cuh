// Device helpers for linear / bilinear / trilinear sampling, shared by
// cpab_interp.cu and the fused transform_data kernels (cpab_fused.cu).
// Semantics: libcpab/pytorch/interpolation.py:18-172 (see cpab_interp.cu).
#pragma once
#include "cpab_launch.h"

namespace cpab {

// Per-image extents.  Per-image element counts are below 2^31 (checked by the
// C ABI), so in-image indices are 32-bit: 64-bit integer division and
// float->int64 conversion run on GB300's narrow FP64 pipe.
struct Geo {
    int size[3];       // data extent per axis (W, H, D)
    int outsize[3];    // output extent per axis
    float sizem1[3];   // size - 1, as float (coordinate scale)
    int nP;            // prod(outsize)
    int nD;            // prod(size)
    FastDiv dout[3];   // division by outsize[j]
};

template <int N>
struct Corner {
    int off[1 << N];   // element offsets of the 2^N corners, corner bit j = axis j high
    float f[N];        // lerp weights xd, yd, zd
};

// x = p*(size-1); x0 = clamp(floor(x)), x1 = clamp(floor(x)+1); xd = x - x0.
// Floor and clamp are done in float (NaN -> 0, huge -> edge, as a saturating
// conversion does) and the small integers are read from the float bits.
template <int N>
__device__ __forceinline__ void corner_indices(const float (&p)[N], const Geo &g, int (&i0)[N],
                                               int (&i1)[N], float (&f)[N]) {
#pragma unroll
    for (int j = 0; j < N; ++j) {
        const float x = p[j] * g.sizem1[j];
        const float k = round_small(x);
        const float fl = (k > x) ? k - 1.f : k;
        const float a = fminf(fmaxf(fl, 0.f), g.sizem1[j]);
        const float b = fminf(fmaxf(fl + 1.f, 0.f), g.sizem1[j]);
        i0[j] = small_float_to_int(a);
        i1[j] = small_float_to_int(b);
        f[j] = x - a;
    }
}

template <int N>
__device__ __forceinline__ Corner<N> corners(const float (&p)[N], const Geo &g) {
    Corner<N> cr;
    int i0[N], i1[N];
    corner_indices<N>(p, g, i0, i1, cr.f);
#pragma unroll
    for (int m = 0; m < (1 << N); ++m) {
        int o = 0;
#pragma unroll
        for (int j = 0; j < N; ++j) o = o * g.size[j] + (((m >> j) & 1) ? i1[j] : i0[j]);
        cr.off[m] = o;
    }
    return cr;
}

// Lerp in the reference's order: along x first, then y, then z.
// v[m]: corner values, corner bit j = axis j high.
template <int N>
__device__ __forceinline__ float lerp_values(float (&v)[1 << N], const float (&f)[N]) {
#pragma unroll
    for (int j = 0; j < N; ++j) {
        const float w1 = f[j], w0 = 1.f - f[j];
#pragma unroll
        for (int m = 0; m < (1 << (N - 1 - j)); ++m)
            v[m] = __fadd_rn(__fmul_rn(v[2 * m], w0), __fmul_rn(v[2 * m + 1], w1));
        // after pass j, v[m] holds the lerp over axes 0..j for corner bits above j
    }
    return v[0];
}

template <int N>
__device__ __forceinline__ float lerp_corners(const float *D, const Corner<N> &cr) {
    float v[1 << N];
#pragma unroll
    for (int m = 0; m < (1 << N); ++m) v[m] = __ldg(D + cr.off[m]);
    return lerp_values<N>(v, cr.f);
}

// The same corners as one base offset plus one step per axis: corner m is at
// base + the steps of the axes whose bit is set in m.  A gather then forms one
// 64-bit address per point (P = D + base) and reaches the other corners by
// 32-bit steps from it.  The step is the axis stride when x1 = x0 + 1 (floor
// in [0, size - 2]) and 0 where both clamp to the same edge; floorf agrees with
// corner_indices' float floor on every input (NaN included: the clamps map it
// to 0).  FB: the base is accumulated in float, exact while the image has
// fewer than 2^23 elements (every partial sum is an integer below 2^23).
template <int N>
struct CornerStep {
    int base;
    int step[N];
    float f[N];
    __device__ __forceinline__ int delta(int m) const {
        int o = 0;
#pragma unroll
        for (int j = 0; j < N; ++j)
            if ((m >> j) & 1) o += step[j];
        return o;
    }
};

template <int N, bool FB>
__device__ __forceinline__ CornerStep<N> corner_steps(const float (&p)[N], const Geo &g) {
    CornerStep<N> cr;
    float a[N];
    bool up[N];
#pragma unroll
    for (int j = 0; j < N; ++j) {
        const float x = __fmul_rn(p[j], g.sizem1[j]);
        const float fl = floorf(x);
        a[j] = fminf(fmaxf(fl, 0.f), g.sizem1[j]);
        cr.f[j] = __fsub_rn(x, a[j]);
        up[j] = fl >= 0.f && fl < g.sizem1[j];
    }
    int st[N];   // element strides, last axis fastest
    st[N - 1] = 1;
#pragma unroll
    for (int j = N - 2; j >= 0; --j) st[j] = st[j + 1] * g.size[j + 1];
    if constexpr (FB) {
        float bf = a[N - 1];
#pragma unroll
        for (int j = N - 2; j >= 0; --j) bf = __fmaf_rn(a[j], (float)st[j], bf);
        cr.base = float_bits(__fadd_rn(bf, 8388608.f)) - 0x4B000000;   // + 2^23: integer bits
    } else {
        int o = 0;
#pragma unroll
        for (int j = 0; j < N; ++j) o += small_float_to_int(a[j]) * st[j];
        cr.base = o;
    }
#pragma unroll
    for (int j = 0; j < N; ++j) cr.step[j] = up[j] ? st[j] : 0;
    return cr;
}

// Offsets in corner order for lerp_corners: pass j pairs entries (2m, 2m+1),
// so corner index bits must be ordered with axis 0 as the lowest bit after
// each pass.  corners() builds index m with bit j = axis j; pass 0 pairs m
// with m^1 (axis 0), leaving entries indexed by the remaining bits (axis 1 as
// bit 0), and so on.

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
        g.sizem1[j] = (float)(g.size[j] - 1);
        g.dout[j] = make_fastdiv((unsigned)g.outsize[j]);
    }
    for (int j = 0; j < ndim; ++j) {
        g.nP *= outsize[j];
        g.nD *= size[j];
    }
    return g;
}

// Per-image element counts must stay below 2^31 and extents below 2^22
// (exact float coordinates); checked by the C ABI before make_geo.
inline bool geo_fits(int ndim, const int *size, const int *outsize) {
    long long nP = 1, nD = 1;
    for (int j = 0; j < ndim; ++j) {
        if (size[j] >= (1 << 22) || outsize[j] >= (1 << 22)) return false;
        nP *= outsize[j];
        nD *= size[j];
    }
    return nP < (1ll << 31) && nD < (1ll << 31);
}

}  // namespace cpab
