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
#include "cpab_adjoint.cuh"
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

// ------------------------------ exact-flow adjoint ---------------------------
// Reverse-mode derivative of the exact flow for time 1, by integrating the
// flow backwards from the forward result.  The field is continuous across
// faces, so the flow's derivative is the product of the in-cell flows'
// derivatives with no term for the crossing times (the velocity jump that
// such a term multiplies is zero); any partition of the time into in-cell
// sub-steps gives the same derivative if each sub-step stays in one cell.  The
// sweep therefore re-derives its own sub-steps:
// from the end point p (time remaining tr), with the certified rule of the
// forward (the same bound for the field reversed), it takes dt in the cell c
// of p and steps back, p_prev = expm(-dt X_c) p~ (X_c = [A_c; 0]).  For that
// sub-step, read forwards as q' = T q with T = expm(dt X_c):
//     lambda_prev = T_lin^T lambda,
//     dL/dA_c += dt [L_exp(dt X_c^T, [lambda p~_prev^T; 0])]_{top rows}
// (the adjoint Frechet derivative of expm, as in the exact mode of the
// fixed-step adjoint).  A sub-step that passed a face (by at most 1e-5, as in
// the forward) is corrected to first order in the time it spent on the far
// side, so the overshoot costs the derivative only at second order.
// dL/dA_c accumulates per lane while the lane stays in
// a cell and is flushed into the warp's cell table with warp_flush (fixed
// summation order: dtheta is reproducible).  The loop runs until every lane
// of the warp has used up its time, so all lanes reach every flush.
template <int N>
__global__ void __launch_bounds__(128)
    k_adjoint_exact(Tess t, const float *__restrict__ out, long long nP,
                    const float *__restrict__ A, int parts, int tiles,
                    const float *__restrict__ gout, float *__restrict__ dpoints,
                    float *__restrict__ partials, unsigned long long *ties, unsigned *err) {
    constexpr int P = N * (N + 1);
    extern __shared__ float4 smem4[];
    __shared__ uint64_t bar;
    const int B = blockDim.x, W = B / 32, tid = threadIdx.x;
    const int th = blockIdx.y, part = blockIdx.x;
    const int G = t.nC * P, Gr = round4(G);
    float *tab = reinterpret_cast<float *>(smem4);
    float *gw = tab + Gr;
    if (!stage_table(tab, A + (long long)th * G, G, &bar, err)) return;
    for (int i = tid; i < W * Gr; i += B) gw[i] = 0.f;
    __syncthreads();
    float *warp_tab = gw + (size_t)(tid >> 5) * Gr;
    for (int tile = part; tile < tiles; tile += parts) {
        const long long idx = (long long)tile * B + tid;
        const bool live = idx < nP;
        float p[N], lam[N], acc[P];
#pragma unroll
        for (int r = 0; r < N; ++r) {
            p[r] = live ? __ldg(out + ((long long)th * N + r) * nP + idx) : 0.5f;
            lam[r] = live ? __ldg(gout + ((long long)th * N + r) * nP + idx) : 0.f;
        }
#pragma unroll
        for (int i = 0; i < P; ++i) acc[i] = 0.f;
        int gcell = -1, it = 0;
        float tr = live ? 1.f : 0.f;
        // cell of p (looked up once per sub-step: the cell of a sub-step's
        // start is the next sub-step's cell)
        int cc = live ? find_cell<N>(p, t, ties) : 0;
        // correction owed to the cell the point enters next (see below)
        float pend[P];
#pragma unroll
        for (int i = 0; i < P; ++i) pend[i] = 0.f;
        while (__any_sync(0xffffffffu, tr > 0.f)) {
            const bool act = tr > 0.f;
            float M[P];
            float dt = 0.f;
            if (act) {
                load_cell<N>(tab, cc, M);
                float v[N], speed2 = 0.f, anorm2 = 0.f;
                affine_apply<N>(M, p, v);
#pragma unroll
                for (int r = 0; r < N; ++r) {
                    speed2 = fmaf(v[r], v[r], speed2);
#pragma unroll
                    for (int k = 0; k < N; ++k)
                        anorm2 = fmaf(M[r * (N + 1) + k], M[r * (N + 1) + k], anorm2);
                }
                const float reach = face_distance<N>(p, t) + kOvershoot;
                const float bound = sqrtf(speed2) + sqrtf(anorm2) * reach;
                // a cell whose field vanishes at p and has no linear part is
                // at rest everywhere: the remaining time in one sub-step
                dt = (bound > 0.f) ? fminf(tr, reach / bound) : tr;
                if (!(dt > 0.f)) dt = tr;   // non-finite input: stop below
            }
            const bool change = act && cc != gcell;
            warp_flush<P>(change && gcell >= 0, gcell, acc, warp_tab);
            if (change) {
                gcell = cc;
#pragma unroll
                for (int i = 0; i < P; ++i) {
                    acc[i] = pend[i];
                    pend[i] = 0.f;
                }
            }
            if (act) {
                // the sub-step's start: q = p + (expm(-dt X) - I) p~
                float Ml[N][N], vt[N], El[N][N], Et[N];
#pragma unroll
                for (int r = 0; r < N; ++r) {
#pragma unroll
                    for (int k = 0; k < N; ++k) Ml[r][k] = -dt * M[r * (N + 1) + k];
                    vt[r] = -dt * M[r * (N + 1) + N];
                }
                expm1_affine<N>(Ml, vt, El, Et);
                float q[N + 1];
#pragma unroll
                for (int r = 0; r < N; ++r) {
                    float a = Et[r];
#pragma unroll
                    for (int k = 0; k < N; ++k) a = fmaf(El[r][k], p[k], a);
                    q[r] = p[r] + a;
                }
                q[N] = 1.f;
                // Y = dt X^T; direction [lambda q^T; 0]
                float Y[N + 1][N + 1], Wd[N + 1][N + 1], L[N + 1][N + 1], R[N + 1][N + 1];
#pragma unroll
                for (int i = 0; i <= N; ++i)
#pragma unroll
                    for (int j = 0; j <= N; ++j) {
                        Y[j][i] = (i < N) ? dt * M[i * (N + 1) + j] : 0.f;
                        Wd[i][j] = (i < N) ? lam[i] * q[j] : 0.f;
                    }
                frechet_expm<N + 1>(Y, Wd, L, R);
#pragma unroll
                for (int i = 0; i < N; ++i)
#pragma unroll
                    for (int j = 0; j <= N; ++j)
                        acc[i * (N + 1) + j] = fmaf(dt, L[i][j], acc[i * (N + 1) + j]);
                // R = T^T: lambda_prev[k] = sum_r T[r][k] lambda[r]
                float nl[N];
#pragma unroll
                for (int k = 0; k < N; ++k) {
                    float a = 0.f;
#pragma unroll
                    for (int r = 0; r < N; ++r) a = fmaf(R[k][r], lam[r], a);
                    nl[k] = a;
                }
                float qp[N];
#pragma unroll
                for (int r = 0; r < N; ++r) qp[r] = q[r];
                const int cn = find_cell<N>(qp, t, ties);
                if (cn != cc) {
                    // The sub-step began in cell cn and crossed into cc, but
                    // was taken with cc's field throughout.  The fields agree
                    // on the face, so g(x) = (A_cc - A_cn) [x;1] vanishes
                    // there and is linear: the time spent in cn is
                    // tau = dt |g(q)| / (|g(q)| + |g(p)|) to first order.
                    // Correct to first order in tau: the cotangent gets
                    // tau (A_cn - A_cc)_lin^T lambda, and tau lambda q~^T
                    // moves from cc's gradient to cn's (owed until the lane
                    // enters cn, at its next sub-step).
                    float Mn[P];
                    load_cell<N>(tab, cn, Mn);
                    float gq = 0.f, gp = 0.f;
#pragma unroll
                    for (int r = 0; r < N; ++r) {
                        float a = M[r * (N + 1) + N] - Mn[r * (N + 1) + N];
                        float b = a;
#pragma unroll
                        for (int k = 0; k < N; ++k) {
                            const float dm = M[r * (N + 1) + k] - Mn[r * (N + 1) + k];
                            a = fmaf(dm, q[k], a);
                            b = fmaf(dm, p[k], b);
                        }
                        gq = fmaf(a, a, gq);
                        gp = fmaf(b, b, gp);
                    }
                    gq = sqrtf(gq);
                    gp = sqrtf(gp);
                    const float tau = (gq + gp > 0.f) ? dt * (gq / (gq + gp)) : 0.f;
                    float cl[N];
#pragma unroll
                    for (int k = 0; k < N; ++k) {
                        float a = 0.f;
#pragma unroll
                        for (int r = 0; r < N; ++r)
                            a = fmaf(Mn[r * (N + 1) + k] - M[r * (N + 1) + k], nl[r], a);
                        cl[k] = fmaf(tau, a, nl[k]);
                    }
#pragma unroll
                    for (int i = 0; i < N; ++i)
#pragma unroll
                        for (int j = 0; j <= N; ++j) {
                            const float w = tau * nl[i] * q[j];
                            acc[i * (N + 1) + j] -= w;
                            pend[i * (N + 1) + j] = w;
                        }
#pragma unroll
                    for (int k = 0; k < N; ++k) nl[k] = cl[k];
                }
                const bool finite = isfinite(q[0]) && (N < 2 || isfinite(q[N - 1]));
#pragma unroll
                for (int r = 0; r < N; ++r) {
                    p[r] = q[r];
                    lam[r] = nl[r];
                }
                cc = cn;
                tr = (dt >= tr) ? 0.f : tr - dt;
                if (++it >= kExactMaxIter || !finite) {
                    if (finite) raise_error(err, kErrIterLimit);
                    tr = 0.f;
                }
            }
        }
        // what is left: the current cell's sum, then a correction owed to the
        // cell of the start point (its last sub-step began across a face)
        warp_flush<P>(gcell >= 0, gcell, acc, warp_tab);
        bool owed = false;
#pragma unroll
        for (int i = 0; i < P; ++i) owed |= pend[i] != 0.f;
        warp_flush<P>(owed, cc, pend, warp_tab);
        if (dpoints && live) {
#pragma unroll
            for (int r = 0; r < N; ++r) dpoints[((long long)th * N + r) * nP + idx] = lam[r];
        }
    }
    __syncthreads();
    for (int i = tid; i < G; i += B) {
        float s = 0.f;
        for (int w = 0; w < W; ++w) s += gw[(size_t)w * Gr + i];
        partials[((long long)th * parts + part) * G + i] = s;
    }
}

// Block size of the exact-flow adjoint: the largest of 128/64/32 threads
// whose per-warp tables and cell table fit in shared memory (0: none).
static int exact_adjoint_block(const Tess &t, size_t *smem) {
    int dev = 0, max_optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (max_optin <= 0) max_optin = 48 * 1024;
    const size_t Gr = (size_t)round4(t.nC * t.ndim * (t.ndim + 1));
    for (int b = 128; b >= 32; b /= 2) {
        const size_t sm = (1 + (size_t)b / 32) * Gr * sizeof(float);
        if (sm <= (size_t)max_optin) {
            *smem = sm;
            return b;
        }
    }
    return 0;
}

bool plan_adjoint_exact(const Tess &t, long long nP, int n_theta, AdjointPlan *plan) {
    size_t smem = 0;
    const int block = exact_adjoint_block(t, &smem);
    if (!block || nP <= 0 || n_theta <= 0) return false;
    const long long tiles = (nP + block - 1) / block;
    if (tiles > 0x7fffffffll) return false;
    const long long target = 2ll * num_sms() * (1024 / block);
    long long parts = (target + n_theta - 1) / n_theta;
    if (parts > tiles) parts = tiles;
    if (parts < 1) parts = 1;
    plan->block = block;
    plan->tiles = (int)tiles;
    plan->parts = (int)parts;
    plan->smem = smem;
    plan->partial_floats = (size_t)n_theta * parts * t.nC * t.ndim * (t.ndim + 1);
    plan->gw_floats = 0;
    return true;
}

cudaError_t launch_adjoint_exact(const Tess &t, const AdjointPlan &plan, const float *out,
                                 long long nP, const float *A, int n_theta, const float *gout,
                                 float *dpoints, float *partials, unsigned long long *ties,
                                 unsigned *err, cudaStream_t s) {
    if (n_theta == 0 || nP == 0) return cudaSuccess;
    if (n_theta > 65535) return cudaErrorInvalidConfiguration;
    const dim3 grid((unsigned)plan.parts, (unsigned)n_theta);
#define CPAB_AEX(N)                                                                           \
    {                                                                                         \
        auto kern = k_adjoint_exact<N>;                                                       \
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                             (int)plan.smem);                                 \
        if (e != cudaSuccess) return e;                                                       \
        kern<<<grid, plan.block, plan.smem, s>>>(t, out, nP, A, plan.parts, plan.tiles, gout, \
                                                 dpoints, partials, ties, err);               \
        return cudaGetLastError();                                                            \
    }
    switch (t.ndim) {
        case 1: CPAB_AEX(1)
        case 2: CPAB_AEX(2)
        default: CPAB_AEX(3)
    }
#undef CPAB_AEX
}

}  // namespace cpab
