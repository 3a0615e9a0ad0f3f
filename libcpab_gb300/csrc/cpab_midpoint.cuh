// The reference's midpoint rule, step for step in its own arithmetic: the
// trajectory whose sensitivity the reference-mode gradient is (used by the
// adjoint kernels; compiled for the host by tests/midpoint_check.cu).
#pragma once
#include <cmath>

namespace cpab {

struct Steps {
    float h, hh, hh2;   // 1/N, 1/(2N), 1/(2N^2)
    // the double step sizes of the reference's midpoint rule, h = 1/N and
    // h/2, each split into two floats (hi + lo) for the emulated double
    // updates of ref_mid_step
    float h_hi, h_lo, hm_hi, hm_lo;
};

inline Steps make_steps(int nsteps) {
    Steps st;
    st.h = (float)(1.0 / nsteps);
    st.hh = (float)(0.5 / nsteps);
    st.hh2 = (float)(0.5 / ((double)nsteps * nsteps));
    const double h = 1.0 / nsteps;
    st.h_hi = (float)h;
    st.h_lo = (float)(h - (double)st.h_hi);
    st.hm_hi = 0.5f * st.h_hi;     // h/2 splits exactly into the halves of h's parts
    st.hm_lo = 0.5f * st.h_lo;
    return st;
}

// Single IEEE operations, never contracted into FMAs (on the host the
// harness is built with -ffp-contract=off).
__host__ __device__ __forceinline__ float op_mul(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
__host__ __device__ __forceinline__ float op_add(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
__host__ __device__ __forceinline__ float op_sub(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
__host__ __device__ __forceinline__ float op_fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
    return __fmaf_rn(a, b, c);
#else
    return std::fma(a, b, c);
#endif
}

// The reference evaluates A [p;1] in float with every product and sum
// rounded on its own, left to right (libcpab/core/cpab_ops.cpp:192-206, built
// for x86-64 without FMA contraction): ((A0 p0 + A1 p1) + A2).
template <int N>
__host__ __device__ __forceinline__ void affine_ref(const float *M, const float (&x)[N],
                                                    float (&y)[N]) {
#pragma unroll
    for (int r = 0; r < N; ++r) {
        float acc = op_mul(M[r * (N + 1)], x[0]);
#pragma unroll
        for (int c = 1; c < N; ++c) acc = op_add(acc, op_mul(M[r * (N + 1) + c], x[c]));
        y[r] = op_add(acc, M[r * (N + 1) + N]);
    }
}

// (float)(p + H * v) with the product and the sum taken in double, as the
// reference's `p + h * v / 2.0` and `p += v * h` with a double h
// (libcpab/core/cpab_ops.cpp:310, :365).  H = hi + lo (two floats); hi * v is
// split exactly by an FMA, p + hi*v by TwoSum (Knuth), and the remaining
// terms are added before the single rounding to float.  The float-float sum
// is within ~2^-47 (|p| + |H v|) of p + H v, so the result is the float the
// double evaluation rounds to, except where p + H v lies that close to the
// midpoint between two floats (tests/test_midpoint_host.py counts them: on
// the order of 1e-7 of the updates).
__host__ __device__ __forceinline__ float add_mul_f64(float p, float v, float hi, float lo) {
    const float t = op_mul(hi, v);
    const float te = op_fma(hi, v, -t);
    const float s = op_add(p, t);
    const float bp = op_sub(s, p);
    const float e = op_add(op_sub(p, op_sub(s, bp)), op_sub(t, bp));
    return op_add(s, op_add(op_fma(lo, v, te), e));
}

// One step of the reference's midpoint rule in its own operation order
// (libcpab/core/cpab_ops.cpp:306-365; cpab_ops.cu:528-581) with the cell's
// A (N x (N+1), row-major):
//   v = A [p;1];  pMid = p + h v / 2;  vMid = A [pMid;1];  p' = p + h vMid.
// The trajectory (and so its cell sequence) is the reference's, bit for bit
// up to the rare double-rounding cases of add_mul_f64.
template <int N>
__host__ __device__ __forceinline__ void ref_mid_step(const float (&A)[N * (N + 1)],
                                                      const Steps &st, float (&p)[N]) {
    float v[N], pm[N];
    affine_ref<N>(A, p, v);
#pragma unroll
    for (int r = 0; r < N; ++r) pm[r] = add_mul_f64(p[r], v[r], st.hm_hi, st.hm_lo);
    affine_ref<N>(A, pm, v);
#pragma unroll
    for (int r = 0; r < N; ++r) p[r] = add_mul_f64(p[r], v[r], st.h_hi, st.h_lo);
}

}  // namespace cpab
