// Exact-flow integration: an opt-in scheme with no counterpart in the
// reference, whose integrator is the fixed-step scheme of cpab_integrate.cu
// (libcpab/core/cpab_ops.cu:268-388).  Here a point follows the true flow of
// the continuous piecewise-affine field for time 1: inside a cell the flow is
// p(t) = p + E(t) [p;1] with E(t) = expm(t [A;0]) - I, and the point changes
// cell where its trajectory meets a face.  It differs from the reference's
// 50-step result by up to ~1e-3 on strongly expanding fields and is checked
// against its own FP64 oracle.
//
//   * 1D: closed form.  With v(x) = a x + b, the time to reach the boundary
//     xb in the direction of motion is log(v(xb)/v(x))/a, evaluated as
//     (d/v) log1p(z)/z with d = xb - x, z = a d / v (stable as a -> 0); the
//     flow for time t is x + v t expm1(a t)/(a t).  A point stops at a fixed
//     point (v changes sign before the boundary).  When the hit time lands
//     within 1e-6 of the remaining time, the comparison is redone in FP64.
//   * 2D / 3D: certified sub-steps.  With d the distance from p to the
//     nearest face line/plane of its cell (the domain boundary is not a face:
//     edge cells extend past it), the speed within distance d + e of p is at
//     most |v(p)| + ||A_lin|| (d + e), so a step of time (d + e) / that bound
//     stays in the cell or passes a face by at most e = 1e-5 (where the two
//     cells' fields differ by O(e)).  Each step uses the exact in-cell flow
//     E(dt); the cell is looked up with the reference's rules before each
//     step.  Steps shrink geometrically towards a face, so a crossing costs
//     ~10-20 steps; a trajectory that needs more than kExactMaxIter steps
//     raises kErrIterLimit and returns its position at that point.
#include "cpab_expm.cuh"

namespace cpab {

constexpr int kExactMaxIter = 4096;
constexpr float kOvershoot = 1e-5f;

__device__ __forceinline__ float phi1f(float y) {   // expm1(y) / y
    return (fabsf(y) < 1e-30f) ? 1.f : expm1f(y) / y;
}
__device__ __forceinline__ float log1p_ratio(float z) {   // log1p(z) / z
    return (fabsf(z) < 1e-30f) ? 1.f : log1pf(z) / z;
}

// 1D closed-form flow for time 1 (table A: [nC][2] = {a, b}).
__device__ float exact_flow_1d(float x, const float *tab, const Tess &t, unsigned *err,
                               unsigned long long *iters) {
    const int nc = t.nc[0];
    float tr = 1.f;
    int c = cell_1d(x, t);
    int it = 0;
    for (; it <= nc + 1 && tr > 0.f; ++it) {
        const float a = tab[2 * c], b = tab[2 * c + 1];
        const float v = fmaf(a, x, b);
        if (v == 0.f || !(fabsf(x) < 1e30f)) break;
        const bool right = v > 0.f;
        const bool has_face = right ? (c < nc - 1) : (c > 0);
        float tb = INFINITY, xb = 0.f;
        if (has_face) {
            xb = (float)(right ? c + 1 : c) * t.inc[0];
            const float vb = fmaf(a, xb, b);
            if ((vb > 0.f) == right && vb != 0.f) {
                const float d = xb - x;
                tb = (d / v) * log1p_ratio(a * d / v);
            }
        }
        bool cross = tb < tr;
        if (fabsf(tb - tr) <= 1e-6f) {   // decide the near-tie in FP64
            const double d = (double)xb - (double)x, vd = fma((double)a, (double)x, (double)b);
            const double z = (double)a * d / vd;
            const double tbd = (fabs(z) < 1e-300) ? d / vd : (d / vd) * (log1p(z) / z);
            cross = tbd < (double)tr;
        }
        if (!cross) {
            x = fmaf(v * tr, phi1f(a * tr), x);
            tr = 0.f;
            break;
        }
        x = xb;
        tr -= tb;
        c += right ? 1 : -1;
    }
    if (iters) atomicAdd(iters, (unsigned long long)it);
    return x;
}

// Conservative distance (domain units) from p to the face lines of its
// cell's square/cube and to the sub-cell diagonals/planes; the domain
// boundary is excluded (edge cells extend past it).
template <int N>
__device__ __forceinline__ float face_distance(const float (&p)[N], const Tess &t) {
    float sub[N];
    float d = INFINITY;
    float imin = t.inc[0];
#pragma unroll
    for (int j = 0; j < N; ++j) {
        float fi, r;
        split_exact(p[j], t.inc[j], t.rinc[j], fi, r);
        const float ci = fminf(fmaxf(fi, 0.f), t.ncf[j] - 1.f);
        const float x = fmaf(r, t.rinc[j], fi - ci);
        sub[j] = x;
        if (ci > 0.f) d = fminf(d, fabsf(x) * t.inc[j]);
        if (ci < t.ncf[j] - 1.f) d = fminf(d, fabsf(1.f - x) * t.inc[j]);
        imin = fminf(imin, t.inc[j]);
    }
    if constexpr (N == 2) {
        const float s = imin * 0.70710678f;
        d = fminf(d, fabsf(sub[0] - sub[1]) * s);
        d = fminf(d, fabsf((sub[0] + sub[1]) - 1.f) * s);
    } else if constexpr (N == 3) {
        // the tetrahedron planes of both parities: z - x - y, x + y + z - 2,
        // y - x - z, x - y - z and their images under x <-> y, y -> 1 - x
        const float s = imin * 0.57735027f;
        const float x = sub[0], y = sub[1], z = sub[2];
        const float xf = y, yf = 1.f - x;
        d = fminf(d, fabsf((z - x) - y) * s);
        d = fminf(d, fabsf(((x + y) + z) - 2.f) * s);
        d = fminf(d, fabsf((y - x) - z) * s);
        d = fminf(d, fabsf((x - y) - z) * s);
        d = fminf(d, fabsf((z - xf) - yf) * s);
        d = fminf(d, fabsf(((xf + yf) + z) - 2.f) * s);
        d = fminf(d, fabsf((yf - xf) - z) * s);
        d = fminf(d, fabsf((xf - yf) - z) * s);
    }
    // rounding of the sub-cell coordinates (< 2^-22 of a cell)
    return fmaxf(d - 4e-7f * imin, 0.f);
}

template <int N>
__device__ void exact_flow_nd(float (&p)[N], const float *tab, const Tess &t,
                              unsigned long long *ties, unsigned *err,
                              unsigned long long *iters) {
    constexpr int P = N * (N + 1);
    float tr = 1.f;
    int it = 0;
    for (; it < kExactMaxIter && tr > 0.f; ++it) {
        const int c = find_cell<N>(p, t, ties);
        float M[P];
        load_cell<N>(tab, c, M);
        float v[N], speed2 = 0.f, anorm2 = 0.f;
        affine_apply<N>(M, p, v);
#pragma unroll
        for (int r = 0; r < N; ++r) {
            speed2 = fmaf(v[r], v[r], speed2);
#pragma unroll
            for (int k = 0; k < N; ++k) anorm2 = fmaf(M[r * (N + 1) + k], M[r * (N + 1) + k], anorm2);
        }
        const float reach = face_distance<N>(p, t) + kOvershoot;
        const float bound = sqrtf(speed2) + sqrtf(anorm2) * reach;
        if (!(bound > 0.f)) break;                   // at rest (or non-finite)
        const float dt = fminf(tr, reach / bound);
        float Ml[N][N], vt[N], El[N][N], Et[N];
#pragma unroll
        for (int r = 0; r < N; ++r) {
#pragma unroll
            for (int k = 0; k < N; ++k) Ml[r][k] = dt * M[r * (N + 1) + k];
            vt[r] = dt * M[r * (N + 1) + N];
        }
        expm1_affine<N>(Ml, vt, El, Et);
        float q[N];
#pragma unroll
        for (int r = 0; r < N; ++r) {
            float acc = Et[r];
#pragma unroll
            for (int k = 0; k < N; ++k) acc = fmaf(El[r][k], p[k], acc);
            q[r] = p[r] + acc;
        }
#pragma unroll
        for (int r = 0; r < N; ++r) p[r] = q[r];
        tr -= dt;
    }
    if (it >= kExactMaxIter) raise_error(err, kErrIterLimit);
    if (iters) atomicAdd(iters, (unsigned long long)it);
}

template <int N>
__global__ void __launch_bounds__(256)
    k_integrate_exact(Tess t, const float *__restrict__ points, int broadcast, long long nP,
                      const float *__restrict__ A, int tiles, float *__restrict__ out,
                      unsigned long long *ties, unsigned *err, unsigned long long *iters) {
    constexpr int P = N * (N + 1);
    extern __shared__ float4 smem4[];
    __shared__ uint64_t bar;
    float *tab = reinterpret_cast<float *>(smem4);
    const int th = blockIdx.y;
    const int G = t.nC * P;
    if (!stage_table(tab, A + (long long)th * G, G, &bar, err)) return;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nP) return;
    const float *src = points + (broadcast ? (long long)th * N * nP : 0ll);
    float p[N];
#pragma unroll
    for (int r = 0; r < N; ++r) p[r] = __ldg(src + r * nP + idx);
    if constexpr (N == 1) p[0] = exact_flow_1d(p[0], tab, t, err, iters);
    else exact_flow_nd<N>(p, tab, t, ties, err, iters);
#pragma unroll
    for (int r = 0; r < N; ++r) out[((long long)th * N + r) * nP + idx] = p[r];
}

cudaError_t launch_integrate_exact(const Tess &t, const float *points, int broadcast,
                                   long long nP, const float *A, int n_theta, float *out,
                                   unsigned long long *ties, unsigned *err,
                                   unsigned long long *iters, cudaStream_t s) {
    const int block = 256;
    const long long tiles = (nP + block - 1) / block;
    if (tiles * n_theta == 0) return cudaSuccess;
    if (n_theta > 65535 || tiles > 0x7fffffffll) return cudaErrorInvalidConfiguration;
    const dim3 grid((unsigned)tiles, (unsigned)n_theta);
    const size_t smem = (size_t)t.nC * t.ndim * (t.ndim + 1) * sizeof(float);
#define CPAB_EX(N)                                                                            \
    {                                                                                         \
        auto kern = k_integrate_exact<N>;                                                     \
        if (smem > 48 * 1024) {                                                               \
            cudaError_t e = cudaFuncSetAttribute(                                             \
                kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);                \
            if (e != cudaSuccess) return e;                                                   \
        }                                                                                     \
        kern<<<grid, block, smem, s>>>(t, points, broadcast, nP, A, (int)tiles, out, ties, err, \
                                       iters);                                                \
        return cudaGetLastError();                                                            \
    }
    switch (t.ndim) {
        case 1: CPAB_EX(1)
        case 2: CPAB_EX(2)
        default: CPAB_EX(3)
    }
#undef CPAB_EX
}

}  // namespace cpab
