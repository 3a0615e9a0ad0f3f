// Compensated exponential of an affine generator, shared by the cell-table
// kernel (cpab_tables.cu) and the exact-flow integrator (cpab_exact.cu).
//
// With X = [[M, v],[0, 0]] one has expm(X) - I = [[M phi(M), phi(M) v],[0, 0]]
// where phi(M) = sum_k M^k/(k+1)!.  phi is evaluated by Taylor series on
// M/2^s (||M/2^s||_1 <= 1/2, degree 10, truncation < 1e-11) and scaled back
// with the identity phi(2Y) = phi(Y) (I + Y phi(Y) / 2), which never forms
// I + (small) and so keeps the increment to full FP32 relative precision.
#pragma once
#include "cpab_launch.h"

namespace cpab {

template <int N>
__device__ __forceinline__ void matmul_nn(const float (&a)[N][N], const float (&b)[N][N],
                                          float (&c)[N][N]) {
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
        for (int j = 0; j < N; ++j) {
            float acc = 0.f;
#pragma unroll
            for (int k = 0; k < N; ++k) acc = fmaf(a[i][k], b[k][j], acc);
            c[i][j] = acc;
        }
}

// E = expm([[M, v],[0,0]]) - I restricted to the top N rows, for M = dt*A_lin,
// v = dt*A_trans.  Outputs E_lin (N x N) and E_t (N).
template <int N>
__device__ __forceinline__ void expm1_affine(const float (&M)[N][N], const float (&v)[N],
                                             float (&El)[N][N], float (&Et)[N]) {
    float norm = 0.f;
#pragma unroll
    for (int j = 0; j < N; ++j) {
        float s = 0.f;
#pragma unroll
        for (int i = 0; i < N; ++i) s += fabsf(M[i][j]);
        norm = fmaxf(norm, s);
    }
    // sq = ceil(log2(norm / 0.5)) from the exponent bits (no conversions):
    // norm = m 2^e with m in [0.5, 1) needs e squarings if m == 0.5, else e + 1
    int sq = 0;
    if (norm > 0.5f) {
        const int bits = __float_as_int(norm);
        const int e = ((bits >> 23) & 0xff) - 126;
        sq = min(64, ((bits & 0x7fffff) == 0) ? e : e + 1);
    }
    const float scale = __int_as_float((127 - sq) << 23);
    float Y[N][N];
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
        for (int j = 0; j < N; ++j) Y[i][j] = M[i][j] * scale;
    // Horner: phi(Y) = I + Y/2 (I + Y/3 (I + ... (I + Y/11)))
    float P[N][N];
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
        for (int j = 0; j < N; ++j) P[i][j] = (i == j) ? 1.f : 0.f;
#pragma unroll
    for (int k = 11; k >= 2; --k) {
        float YP[N][N];
        matmul_nn<N>(Y, P, YP);
        const float r = 1.f / (float)k;   // a constant once the loop is unrolled
#pragma unroll
        for (int i = 0; i < N; ++i)
#pragma unroll
            for (int j = 0; j < N; ++j) P[i][j] = fmaf(YP[i][j], r, (i == j) ? 1.f : 0.f);
    }
    // phi(2Y) = phi(Y) (I + Y phi(Y)/2), repeated sq times.
    for (int s = 0; s < sq; ++s) {
        float YP[N][N], W[N][N], Pn[N][N];
        matmul_nn<N>(Y, P, YP);
#pragma unroll
        for (int i = 0; i < N; ++i)
#pragma unroll
            for (int j = 0; j < N; ++j) W[i][j] = fmaf(YP[i][j], 0.5f, (i == j) ? 1.f : 0.f);
        matmul_nn<N>(P, W, Pn);
#pragma unroll
        for (int i = 0; i < N; ++i)
#pragma unroll
            for (int j = 0; j < N; ++j) {
                P[i][j] = Pn[i][j];
                Y[i][j] *= 2.f;
            }
    }
    matmul_nn<N>(M, P, El);
#pragma unroll
    for (int i = 0; i < N; ++i) {
        float acc = 0.f;
#pragma unroll
        for (int k = 0; k < N; ++k) acc = fmaf(P[i][k], v[k], acc);
        Et[i] = acc;
    }
}

}  // namespace cpab
