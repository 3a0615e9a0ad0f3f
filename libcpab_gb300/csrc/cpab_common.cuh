// Shared device code for the CPAB integration kernels (sm_103a).
//
// Cell lookup
// -----------
// The reference decides the cell of a point in double precision
// (libcpab/core/cpab_ops.cu:21-227 for CUDA, libcpab/core/cpab_ops.cpp:26-184
// for the CPU).  GB300 has a low FP64 rate, so lookups here run in FP32:
//   * the cell index along each axis (floor(p/inc)) and the remainder
//     p - i*inc are computed exactly with two FMAs (split_exact);
//   * the sub-cell tests (triangle diagonals, tetrahedron planes; in 2D also
//     the out-of-domain rules, which are the same tests on the edge square)
//     use FP32 values with a proven error bound; when a test lands within its
//     margin of zero, the lookup is redone with an FP64 replica of the
//     reference's arithmetic.
// The result is bit-identical to the reference lookup for every float input.
// The FP64 branch is taken only for genuine near-ties (a point within ~2e-6 of
// a diagonal or plane, including 3D points pushed onto a domain corner) and
// non-finite input; it is counted when a counter is supplied.
//
// Tables
// ------
// Per-theta cell tables use the reference's dense layout
// [n_theta, nC, ndim, ndim+1] (row-major affine maps), for A (velocity),
// T = expm(dt*A) (step map) and E = T - I (step increment).  One theta's
// table is staged into shared memory with a TMA bulk copy
// (cp.async.bulk + mbarrier) when it is 16-byte aligned and a multiple of 16
// bytes, else with plain loads.  Every mbarrier wait is bounded; on timeout
// the kernel raises a bit in the device error word and stops.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

namespace cpab {

constexpr int kMaxDim = 3;

// Bits of the device error word (read back by cpab_device_status()).
enum : unsigned {
    kErrTmaTimeout = 1u << 0,   // a bulk copy into shared memory did not complete
    kErrBadCell = 1u << 1,      // reserved: every lookup returns a cell in [0, nC)
    kErrBadOffsets = 1u << 3,   // a ragged series had invalid offsets (skipped)
    kErrIterLimit = 1u << 4,    // an exact-flow trajectory hit its step limit
};

// Host-computed description of one tessellation.  The float constants are
// computed exactly as the reference computes them (float inc = 1.0/nc, float
// products nc*inc) so the FP64 replica below reproduces its comparisons.
struct Tess {
    int ndim;
    int nc[3];
    int nC;
    float inc[3];     // (float)(1.0 / nc)
    float rinc[3];    // (float)(1.0 / inc)  (approximate reciprocal, fast path only)
    float wlim[3];    // (float)nc * inc     (float product)
    float clamp3[3];  // 3D clamp limits (float)(nc*inc - 1e-8), z uses inc_x
    int band[3];      // 1 if (float)(nc*inc) > nc*inc: floats in [nc*inc, wlim) exist
    int band_any;     // band[0] | band[1] | band[2]
    int tier2;        // 2D second-tier tie decisions apply (square cells, see cell_2d_tier2)
    int pow2;         // every nc[j] (j < ndim, ndim >= 2) is a power of two: p / inc == p * nc
    float ncf[3];     // nc as float
};

// The lookup functions are host+device so that a host harness can check the
// FP32 path against the FP64 replica on adversarial inputs.  Single IEEE
// operations that must not be contracted into an FMA use these wrappers.
#define CPAB_HD __host__ __device__
#if defined(__CUDA_ARCH__)
#define CPAB_MUL_RN(a, b) __fmul_rn((a), (b))
#define CPAB_ADD_RN(a, b) __fadd_rn((a), (b))
#define CPAB_SUB_RN(a, b) __fsub_rn((a), (b))
#else
#define CPAB_MUL_RN(a, b) ((a) * (b))
#define CPAB_ADD_RN(a, b) ((a) + (b))
#define CPAB_SUB_RN(a, b) ((a) - (b))
#endif

// Fill the tessellation constants exactly as the reference computes them
// (libcpab/core/cpab_ops.cpp:40-45, 108-110, 139-141).  nc must hold ndim
// positive counts; returns the number of cells.
inline int tess_init(int ndim, const int *nc, Tess *t) {
    *t = Tess();
    t->ndim = ndim;
    long long cells = 1;
    for (int j = 0; j < 3; ++j) {
        const int n = j < ndim ? nc[j] : 1;
        t->nc[j] = n;
        t->inc[j] = (float)(1.0 / n);
        t->rinc[j] = (float)(1.0 / (double)t->inc[j]);
        t->wlim[j] = (float)n * t->inc[j];
        t->band[j] = (double)t->wlim[j] > (double)n * (double)t->inc[j];
        t->band_any |= t->band[j];
        t->ncf[j] = (float)n;
        cells *= n;
    }
    t->nC = (int)(cells * (ndim == 1 ? 1 : ndim == 2 ? 4 : 5));
    // cell_2d_tier2 needs one divisor for both axes and no float strictly
    // between wlim - 1e-9 (the reference's clamp) and wlim
    t->tier2 = ndim == 2 && t->inc[0] == t->inc[1];
    for (int j = 0; j < 2; ++j)
        t->tier2 &= (double)nextafterf(t->wlim[j], 0.f) <= (double)t->wlim[j] - 0.000000001;
    t->pow2 = ndim >= 2;
    for (int j = 0; j < ndim; ++j) t->pow2 &= (t->nc[j] & (t->nc[j] - 1)) == 0;
    if (ndim == 3) {
        t->clamp3[0] = (float)((double)((float)nc[0] * t->inc[0]) - 1e-8);
        t->clamp3[1] = (float)((double)((float)nc[1] * t->inc[1]) - 1e-8);
        t->clamp3[2] = (float)((double)((float)nc[2] * t->inc[0]) - 1e-8);  // inc_x, as the reference
    }
    return t->nC;
}

CPAB_HD inline int mymin_ref(int a, double b) { return !(b < a) ? a : (int)round(b); }

// Rounding and float->int without conversion instructions (on GB300 these
// issue to the narrow FP64 pipe and throttled the lookup): adding 1.5*2^23
// rounds |x| < 2^22 to the nearest integer and leaves it in the low
// mantissa bits.
constexpr float kRoundMagic = 12582912.0f;      // 1.5 * 2^23
constexpr int kRoundMagicBits = 0x4B400000;     // bit pattern of kRoundMagic

CPAB_HD inline int float_bits(float x) {
#if defined(__CUDA_ARCH__)
    return __float_as_int(x);
#else
    int i;
    memcpy(&i, &x, sizeof(i));
    return i;
#endif
}

// Nearest integer (ties to even) of |x| < 2^22.
CPAB_HD inline float round_small(float x) {
    return CPAB_SUB_RN(CPAB_ADD_RN(x, kRoundMagic), kRoundMagic);
}

// int value of an integral float with |x| < 2^22.
CPAB_HD inline int small_float_to_int(float x) {
    return float_bits(CPAB_ADD_RN(x, kRoundMagic)) - kRoundMagicBits;
}

// Division of 32-bit unsigned numerators by a fixed divisor d >= 1 with one
// multiply-high (Granlund & Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994): m = floor(2^32 (2^l - d) / d) + 1 with
// l = ceil(log2 d); q = (hi + ((n - hi) >> 1)) >> (l - 1), hi = mulhi(n, m).
// Exact for every 32-bit n; avoids the int<->float conversions of the
// generic division sequence.
struct FastDiv {
    unsigned d, m;
    int s;   // l - 1, or -1 for d == 1
};

inline FastDiv make_fastdiv(unsigned d) {
    FastDiv f;
    f.d = d;
    int l = 0;
    while ((1ull << l) < d) ++l;
    f.m = (unsigned)(((1ull << 32) * ((1ull << l) - d)) / d + 1);
    f.s = l - 1;
    return f;
}

CPAB_HD inline unsigned fast_div(unsigned n, const FastDiv &f) {
    if (f.s < 0) return n;
#if defined(__CUDA_ARCH__)
    const unsigned hi = __umulhi(n, f.m);
#else
    const unsigned hi = (unsigned)(((unsigned long long)n * f.m) >> 32);
#endif
    return (hi + ((n - hi) >> 1)) >> f.s;
}

// ------------------------------- 1D ---------------------------------------
// floor(p * nc) with the float product, clamped to [0, nc-1]
// (cpab_ops.cu:14-19).  Non-finite and huge products saturate like CUDA's
// float->int conversion: +inf and large values give nc-1, -inf and NaN give 0.
CPAB_HD inline int cell_1d(float p, const Tess &t) {
    const float q = CPAB_MUL_RN(p, t.ncf[0]);
    const float k = round_small(q);
    float f = (k > q) ? k - 1.f : k;                    // floor, exact for |q| < 2^22
    f = fminf(fmaxf(f, 0.f), t.ncf[0] - 1.f);          // NaN -> 0
    return small_float_to_int(f);
}

// ------------------------------- 2D ---------------------------------------
// FP64 replica of the reference's 2D lookup (cpab_ops.cpp:33-104).
static CPAB_HD __noinline__ int cell_2d_exact(float fpx, float fpy, const Tess &t) {
    const int nx = t.nc[0], ny = t.nc[1];
    const double px = fpx, py = fpy;
    const double ix = t.inc[0], iy = t.inc[1];
    const double wx = t.wlim[0], wy = t.wlim[1];
    double cx = (0.0 < px) ? px : 0.0;
    double cy = (0.0 < py) ? py : 0.0;
    const double mx = wx - 0.000000001, my = wy - 0.000000001;
    if (cx > mx) cx = mx;
    if (cy > my) cy = my;
    const double rx = fmod(cx, ix), ry = fmod(cy, iy);
    const double fx = rx / ix, fy = ry / iy;
    int c = 4 * (mymin_ref(nx - 1, (cx - rx) / ix) + mymin_ref(ny - 1, (cy - ry) / iy) * nx);
    if (px <= 0) {
        if (py <= 0 && py / iy < px / ix) return c;
        if (py >= wy && py / iy - ny > -px / ix) return c + 2;
        return c + 3;
    }
    if (px >= wx) {
        if (py <= 0 && -py / iy > px / ix - nx) return c;
        if (py >= wy && py / iy - ny > px / ix - nx) return c + 2;
        return c + 1;
    }
    if (py <= 0) return c;
    if (py >= wy) return c + 2;
    if (fx < fy) return (1 - fx < fy) ? c + 2 : c + 3;
    return (1 - fx < fy) ? c + 1 : c;
}

// Exact floor(p / inc), as a float, and the remainder p - fi*inc, in FP32.
// k = rint(p * rinc) is within 1/2 of the true quotient; the sign of
// fma(-k, inc, p) (one rounding of the exact p - k*inc, which keeps its sign)
// decides between k and k-1.  For p >= 0 the remainder lies in [0, inc) on
// inc's ulp grid, so the second fma returns it exactly: these are the
// reference's fmod/divide results (cpab_ops.cpp:47-54) without FP64.
CPAB_HD inline void split_exact(float p, float inc, float rinc, float &fi, float &rem) {
    const float k = round_small(p * rinc);
    fi = (fmaf(-k, inc, p) >= 0.f) ? k : k - 1.f;
    rem = fmaf(-fi, inc, p);
}

// |p * rinc| below this keeps every integer in split_exact exact.
constexpr float kSplitLimit = 2097152.0f;   // 2^21

// cell_2d_fast's code for "a triangle decision is within its margin".
constexpr int kTie2 = -2;

// Margin of the FP32 sub-cell tests.  A sub-cell coordinate rem*rinc differs
// from the reference's double rem/inc by at most 2^-22; a two-term test then
// carries an error below (1+|x|+|y|) 2^-21 and a three-term test below
// 2^-20.  Decisions closer than these margins go to the FP64 replica.
constexpr float kMargin2 = 1.9073486328125e-06f;   // 2^-19
constexpr float kMargin3 = 3.814697265625e-06f;    // 2^-18

// FP32 2D lookup with the reference's semantics for every finite point;
// returns kTie2 when a triangle decision is within its error margin (the
// second tier may decide it) and -1 in the other deferred cases.
//
// Outside the domain the reference applies its left/right/above/below rules
// (cpab_ops.cpp:57-90).  Each of them is the in-square triangle test applied
// to the edge square with unclamped sub-cell coordinates, e.g. left of and
// above the domain it takes triangle 0 iff py/iy < px/ix, i.e. y < x, which
// is what the test below gives there.  So one formula serves all points: the
// square is the clamped exact split, the coordinates are measured from it,
// and only exact ties (margin) differ.  NaN/Inf fail the margin test.
CPAB_HD inline int cell_2d_fast(float px, float py, const Tess &t) {
    float fi, ri, fj, rj;
    split_exact(px, t.inc[0], t.rinc[0], fi, ri);
    split_exact(py, t.inc[1], t.rinc[1], fj, rj);
    // far away, huge or non-finite coordinates: FP64 replica
    if (!(fabsf(px * t.rinc[0]) < kSplitLimit) || !(fabsf(py * t.rinc[1]) < kSplitLimit))
        return -1;
    const float ci = fminf(fmaxf(fi, 0.f), t.ncf[0] - 1.f);
    const float cj = fminf(fmaxf(fj, 0.f), t.ncf[1] - 1.f);
    // In-domain points past nc*inc (possible only when the float product
    // nc*inc rounds above it: band_any, fixed per tessellation) get the fmod
    // remainder, not the continuous one.
    if (t.band_any &&
        ((t.band[0] && fi > ci && px < t.wlim[0]) || (t.band[1] && fj > cj && py < t.wlim[1])))
        return -1;
    const float x = fmaf(ri, t.rinc[0], fi - ci);
    const float y = fmaf(rj, t.rinc[1], fj - cj);
    const float dxy = x - y, sxy = (x + y) - 1.f;
    const float m = kMargin2 * ((1.f + fabsf(x)) + fabsf(y));
    if (!(fabsf(dxy) > m) || !(fabsf(sxy) > m)) return kTie2;
    // triangle: 0 (dxy >= 0, sxy <= 0), 1 (dxy >= 0, sxy > 0), 2 (dxy < 0,
    // sxy > 0), 3 (dxy < 0, sxy <= 0) = (sxy > 0) xor (dxy < 0 ? 3 : 0)
    const int tri = (sxy > 0.f ? 1 : 0) ^ (dxy < 0.f ? 3 : 0);
    return small_float_to_int(4.f * fmaf(cj, t.ncf[0], ci)) + tri;
}

// Second tier for triangle decisions inside the FP32 margin, for square
// cells (inc_x == inc_y, Tess::tier2).  Trajectories that sit on a tie for
// many steps (zero-boundary domain corners are fixed points up to ~1e-17
// drift) would otherwise take the FP64 replica at every step.  It follows the
// reference's branch order (cpab_ops.cpp:57-98) and decides each comparison
// exactly where that is provable, else returns -1 (FP64 replica):
//  * fx < fy, i.e. rx/ix < ry/iy, and py/iy < px/ix: with one divisor the
//    correctly rounded double quotients of two distinct floats keep their
//    order (relative gap >= 2^-24 >> 2^-53), so the float comparison decides;
//  * 1 - fx < fy: the reference's double evaluation is within 3*2^-53 of
//    1 - (rx + ry)/ix; T = (ix - rx) - ry in double is within 2^-52 ix of its
//    exact value, so |T| > 2^-48 ix decides the test by the sign of T;
//  * the out-of-domain rules outside in x and y (cpab_ops.cpp:59-82), e.g.
//    py/iy - ny > -px/ix: multiplied by ix = iy they compare
//    D = px + py - ny*iy (or py - px - (ny - nx) ix, px + py - nx ix) with 0.
//    Each side of the reference's comparison carries at most two roundings
//    (2^-52 relative); D evaluated in double carries at most 2^-52 of
//    |px| + |py| + (nx + ny) ix, so |D| above 2^-48 of that decides by its
//    sign.  Identical evaluations (px == py, nx == ny) compare equal.
//  * with power-of-two cell counts (Tess::pow2) division by inc is
//    multiplication by nc, exact in double, so a comparison that the bounds
//    above leave open is evaluated with the reference's own operations.
// rx and ry are split_exact's float remainders, equal to the reference's
// fmod for 0 < p < wlim (and p <= wlim - 1e-9 there, by Tess::tier2).  Called
// only after cell_2d_fast returned kTie2, i.e. past the band and range checks,
// so the clamped split is the reference's square.
static CPAB_HD __noinline__ int cell_2d_tier2(float px, float py, const Tess &t) {
    float fi, ri, fj, rj;
    split_exact(px, t.inc[0], t.rinc[0], fi, ri);
    split_exact(py, t.inc[1], t.rinc[1], fj, rj);
    const float ci = fminf(fmaxf(fi, 0.f), t.ncf[0] - 1.f);
    const float cj = fminf(fmaxf(fj, 0.f), t.ncf[1] - 1.f);
    const int c = small_float_to_int(4.f * fmaf(cj, t.ncf[0], ci));
    const double kEps = 3.552713678800501e-15;   // 2^-48
    const double nix = (double)t.nc[0] * (double)t.inc[0], niy = (double)t.nc[1] * (double)t.inc[1];
    const double scale = (fabs((double)px) + fabs((double)py)) + (nix + niy);
    int tri;
    if (px <= 0.f) {
        if (py <= 0.f) {
            tri = (py < px) ? 0 : 3;
        } else if (py >= t.wlim[1]) {                 // py/iy - ny > -px/ix ?
            const double D = ((double)px + (double)py) - niy;
            if (fabs(D) > kEps * scale) tri = D > 0.0 ? 2 : 3;
            else if (t.pow2) tri = ((double)py * t.nc[1] - t.nc[1] > -((double)px * t.nc[0])) ? 2 : 3;
            else return -1;
        } else {
            tri = 3;
        }
    } else if (px >= t.wlim[0]) {
        if (py <= 0.f) {                              // -py/iy > px/ix - nx ?
            const double D = ((double)px + (double)py) - nix;
            if (fabs(D) > kEps * scale) tri = D < 0.0 ? 0 : 1;
            else if (t.pow2) tri = (-((double)py * t.nc[1]) > (double)px * t.nc[0] - t.nc[0]) ? 0 : 1;
            else return -1;
        } else if (py >= t.wlim[1]) {                 // py/iy - ny > px/ix - nx ?
            if (px == py && t.nc[0] == t.nc[1]) {
                tri = 1;
            } else {
                const double D = ((double)py - (double)px) -
                                 ((double)t.nc[1] - (double)t.nc[0]) * (double)t.inc[0];
                if (fabs(D) > kEps * scale) tri = D > 0.0 ? 2 : 1;
                else if (t.pow2)
                    tri = ((double)py * t.nc[1] - t.nc[1] > (double)px * t.nc[0] - t.nc[0]) ? 2 : 1;
                else return -1;
            }
        } else {
            tri = 1;
        }
    } else if (py <= 0.f) {
        tri = 0;
    } else if (py >= t.wlim[1]) {
        tri = 2;
    } else {
        const double T = ((double)t.inc[0] - (double)ri) - (double)rj;
        bool s;                                                                   // 1 - fx < fy
        if (fabs(T) > kEps * (double)t.inc[0]) s = T < 0.0;
        else if (t.pow2) s = 1.0 - (double)ri * t.nc[0] < (double)rj * t.nc[1];
        else return -1;
        tri = (ri < rj) ? (s ? 2 : 3) : (s ? 1 : 0);
    }
    return c + tri;
}

// FP32 decision of both tiers (-1: the FP64 replica must decide).
CPAB_HD inline int cell_2d_fp32(float px, float py, const Tess &t) {
    const int c = cell_2d_fast(px, py, t);
    if (c >= 0 || c != kTie2 || !t.tier2) return c >= 0 ? c : -1;
    return cell_2d_tier2(px, py, t);
}

__device__ __forceinline__ int cell_2d(float px, float py, const Tess &t,
                                       unsigned long long *ties) {
    int c = cell_2d_fast(px, py, t);
    if (c >= 0) return c;
    if (c == kTie2 && t.tier2) {
        c = cell_2d_tier2(px, py, t);
        if (c >= 0) return c;
    }
    if (ties) atomicAdd(ties, 1ull);
    return cell_2d_exact(px, py, t);
}

// ------------------------------- 3D ---------------------------------------
// FP64 replica of the reference's 3D lookup (cpab_ops.cpp:106-184), including
// the push-inside rule that tests only x and y, and the z clamp that uses
// inc_x.
static CPAB_HD __noinline__ int cell_3d_exact(float p0, float p1, float p2, const Tess &t) {
    const int nx = t.nc[0], ny = t.nc[1], nz = t.nc[2];
    const float ix = t.inc[0], iy = t.inc[1], iz = t.inc[2];
    float q0 = p0, q1 = p1, q2 = p2;
    if (q0 < 0.0 || q0 > 1.0 || q1 < 0.0 || q1 > 1.0) {
        const float h = 0.5f;
        q0 = CPAB_SUB_RN(q0, h); q1 = CPAB_SUB_RN(q1, h); q2 = CPAB_SUB_RN(q2, h);
        const float a0 = fabsf(q0), a1 = fabsf(q1), a2 = fabsf(q2);
        const float s0 = (a0 < a1 && a0 < a2) ? CPAB_MUL_RN(h, ix) : 0.0f;
        const float s1 = (a1 < a0 && a0 < a2) ? CPAB_MUL_RN(h, iy) : 0.0f;
        const float s2 = (a2 < a0 && a0 < a1) ? CPAB_MUL_RN(h, iz) : 0.0f;
        if (a0 > h) q0 = copysignf(CPAB_SUB_RN(h, s0), q0);
        if (a1 > h) q1 = copysignf(CPAB_SUB_RN(h, s1), q1);
        if (a2 > h) q2 = copysignf(CPAB_SUB_RN(h, s2), q2);
        q0 = CPAB_ADD_RN(q0, h); q1 = CPAB_ADD_RN(q1, h); q2 = CPAB_ADD_RN(q2, h);
    }
    const float zero = 0.0f;
    float c0 = (zero < q0) ? q0 : zero; if (q0 != q0) c0 = zero;
    float c1 = (zero < q1) ? q1 : zero; if (q1 != q1) c1 = zero;
    float c2 = (zero < q2) ? q2 : zero; if (q2 != q2) c2 = zero;
    if (t.clamp3[0] < c0) c0 = t.clamp3[0];
    if (t.clamp3[1] < c1) c1 = t.clamp3[1];
    if (t.clamp3[2] < c2) c2 = t.clamp3[2];
    const double r0 = fmod((double)c0, (double)ix);
    const double r1 = fmod((double)c1, (double)iy);
    const double r2 = fmod((double)c2, (double)iz);
    const int i = mymin_ref(nx - 1, ((double)c0 - r0) / (double)ix);
    const int j = mymin_ref(ny - 1, ((double)c1 - r1) / (double)iy);
    const int k = mymin_ref(nz - 1, ((double)c2 - r2) / (double)iz);
    int c = 5 * (i + j * nx + k * nx * ny);
    double x = r0 / (double)ix, y = r1 / (double)iy, z = r2 / (double)iz;
    bool flip;
    if (k % 2 == 0) flip = (i % 2 == 0 && j % 2 == 1) || (i % 2 == 1 && j % 2 == 0);
    else flip = (i % 2 == 0 && j % 2 == 0) || (i % 2 == 1 && j % 2 == 1);
    if (flip) { const double tmp = x; x = y; y = 1 - tmp; }
    if (-x - y + z >= 0) return c + 1;
    if (x + y + z - 2 >= 0) return c + 2;
    if (-x + y - z >= 0) return c + 3;
    if (x - y - z >= 0) return c + 4;
    return c;
}

CPAB_HD inline int cell_3d_fast(float p0, float p1, float p2, const Tess &t) {
    // The reference's push-inside rule (x or y outside [0,1]) is float
    // arithmetic: it is applied here with the same operations, and leaves
    // every coordinate in [0,1].  The reference then clamps each coordinate to
    // [0, clamp3] (in float) and splits it, which split_exact does exactly.
    // Only the tetrahedron plane tests need a margin.
    if (!(fabsf(p0) <= 1e30f) || !(fabsf(p1) <= 1e30f) || !(fabsf(p2) <= 1e30f)) return -1;
    if (!(p0 >= 0.f && p0 <= 1.f && p1 >= 0.f && p1 <= 1.f)) {
        const float h = 0.5f;
        p0 = CPAB_SUB_RN(p0, h); p1 = CPAB_SUB_RN(p1, h); p2 = CPAB_SUB_RN(p2, h);
        const float a0 = fabsf(p0), a1 = fabsf(p1), a2 = fabsf(p2);
        const float s0 = (a0 < a1 && a0 < a2) ? CPAB_MUL_RN(h, t.inc[0]) : 0.0f;
        const float s1 = (a1 < a0 && a0 < a2) ? CPAB_MUL_RN(h, t.inc[1]) : 0.0f;
        const float s2 = (a2 < a0 && a0 < a1) ? CPAB_MUL_RN(h, t.inc[2]) : 0.0f;
        if (a0 > h) p0 = copysignf(CPAB_SUB_RN(h, s0), p0);
        if (a1 > h) p1 = copysignf(CPAB_SUB_RN(h, s1), p1);
        if (a2 > h) p2 = copysignf(CPAB_SUB_RN(h, s2), p2);
        p0 = CPAB_ADD_RN(p0, h); p1 = CPAB_ADD_RN(p1, h); p2 = CPAB_ADD_RN(p2, h);
    }
    {
        const float c0 = (p0 < t.clamp3[0]) ? p0 : t.clamp3[0];
        const float c1 = (p1 < t.clamp3[1]) ? p1 : t.clamp3[1];
        float c2 = (0.f < p2) ? p2 : 0.f;
        c2 = (c2 < t.clamp3[2]) ? c2 : t.clamp3[2];
        float f0, f1, f2, r0, r1, r2;
        split_exact(c0, t.inc[0], t.rinc[0], f0, r0);
        split_exact(c1, t.inc[1], t.rinc[1], f1, r1);
        split_exact(c2, t.inc[2], t.rinc[2], f2, r2);
        // mymin: the index is capped at nc-1, the remainder is not
        const int i = small_float_to_int(fminf(f0, t.ncf[0] - 1.f));
        const int j = small_float_to_int(fminf(f1, t.ncf[1] - 1.f));
        const int k = small_float_to_int(fminf(f2, t.ncf[2] - 1.f));
        float x = r0 * t.rinc[0], y = r1 * t.rinc[1];
        const float z = r2 * t.rinc[2];
        const bool flip = ((i ^ j ^ k) & 1) != 0;   // the reference's parity rule
        if (flip) { const float tmp = x; x = y; y = 1.f - tmp; }
        const int c = 5 * (i + j * t.nc[0] + k * t.nc[0] * t.nc[1]);
        const float t1 = (z - x) - y;
        if (fabsf(t1) > kMargin3) {
            if (t1 > 0.f) return c + 1;
            const float t2 = ((x + y) + z) - 2.f;
            if (fabsf(t2) > kMargin3) {
                if (t2 > 0.f) return c + 2;
                const float t3 = (y - x) - z;
                if (fabsf(t3) > kMargin3) {
                    if (t3 > 0.f) return c + 3;
                    const float t4 = (x - y) - z;
                    if (fabsf(t4) > kMargin3) return (t4 > 0.f) ? c + 4 : c;
                }
            }
        }
    }
    return -1;
}

// Second tier for 3D with power-of-two cell counts (Tess::pow2): inc is then
// 2^-k, so the reference's sub-cell coordinates r/inc (cpab_ops.cpp:150-155)
// equal r * nc exactly in double, and its tetrahedron tests
// (cpab_ops.cpp:165-177) are evaluated with the same double operations in the
// same order.  With cell_3d_fast's push, clamp and exact split (all float
// operations of the reference) this reproduces the reference's decision for
// every finite point without fmod or division.  Ties on the tetrahedron
// planes are common on regular grids (3 % of a 128^3 meshgrid at [4,4,4]).
static CPAB_HD __noinline__ int cell_3d_tier2(float p0, float p1, float p2, const Tess &t) {
    if (!t.pow2) return -1;
    if (!(fabsf(p0) <= 1e30f) || !(fabsf(p1) <= 1e30f) || !(fabsf(p2) <= 1e30f)) return -1;
    if (!(p0 >= 0.f && p0 <= 1.f && p1 >= 0.f && p1 <= 1.f)) {
        const float h = 0.5f;
        p0 = CPAB_SUB_RN(p0, h); p1 = CPAB_SUB_RN(p1, h); p2 = CPAB_SUB_RN(p2, h);
        const float a0 = fabsf(p0), a1 = fabsf(p1), a2 = fabsf(p2);
        const float s0 = (a0 < a1 && a0 < a2) ? CPAB_MUL_RN(h, t.inc[0]) : 0.0f;
        const float s1 = (a1 < a0 && a0 < a2) ? CPAB_MUL_RN(h, t.inc[1]) : 0.0f;
        const float s2 = (a2 < a0 && a0 < a1) ? CPAB_MUL_RN(h, t.inc[2]) : 0.0f;
        if (a0 > h) p0 = copysignf(CPAB_SUB_RN(h, s0), p0);
        if (a1 > h) p1 = copysignf(CPAB_SUB_RN(h, s1), p1);
        if (a2 > h) p2 = copysignf(CPAB_SUB_RN(h, s2), p2);
        p0 = CPAB_ADD_RN(p0, h); p1 = CPAB_ADD_RN(p1, h); p2 = CPAB_ADD_RN(p2, h);
    }
    const float c0 = (p0 < t.clamp3[0]) ? p0 : t.clamp3[0];
    const float c1 = (p1 < t.clamp3[1]) ? p1 : t.clamp3[1];
    float c2 = (0.f < p2) ? p2 : 0.f;
    c2 = (c2 < t.clamp3[2]) ? c2 : t.clamp3[2];
    float f0, f1, f2, r0, r1, r2;
    split_exact(c0, t.inc[0], t.rinc[0], f0, r0);
    split_exact(c1, t.inc[1], t.rinc[1], f1, r1);
    split_exact(c2, t.inc[2], t.rinc[2], f2, r2);
    const int i = small_float_to_int(fminf(f0, t.ncf[0] - 1.f));
    const int j = small_float_to_int(fminf(f1, t.ncf[1] - 1.f));
    const int k = small_float_to_int(fminf(f2, t.ncf[2] - 1.f));
    double x = (double)r0 * (double)t.nc[0], y = (double)r1 * (double)t.nc[1];
    const double z = (double)r2 * (double)t.nc[2];
    if (((i ^ j ^ k) & 1) != 0) {
        const double tmp = x;
        x = y;
        y = 1 - tmp;
    }
    const int c = 5 * (i + j * t.nc[0] + k * t.nc[0] * t.nc[1]);
    if (-x - y + z >= 0) return c + 1;
    if (x + y + z - 2 >= 0) return c + 2;
    if (-x + y - z >= 0) return c + 3;
    if (x - y - z >= 0) return c + 4;
    return c;
}

// FP32-side decision of both 3D tiers (-1: the FP64 replica must decide).
CPAB_HD inline int cell_3d_fp32(float p0, float p1, float p2, const Tess &t) {
    const int c = cell_3d_fast(p0, p1, p2, t);
    return c >= 0 ? c : cell_3d_tier2(p0, p1, p2, t);
}

__device__ __forceinline__ int cell_3d(float p0, float p1, float p2, const Tess &t,
                                       unsigned long long *ties) {
    int c = cell_3d_fast(p0, p1, p2, t);
    if (c >= 0) return c;
    c = cell_3d_tier2(p0, p1, p2, t);
    if (c >= 0) return c;
    if (ties) atomicAdd(ties, 1ull);
    return cell_3d_exact(p0, p1, p2, t);
}

// The cell of p with the reference's rules.  Every path returns an index in
// [0, nC) for every input, NaN and infinities included: the FP32 paths clamp
// the square (or interval) indices to [0, nc-1] and add a sub-cell index in
// [0, 4) or [0, 5); the FP64 replicas clamp like the reference (NaN and
// negative coordinates to 0, large ones to nc-1).  The kernels therefore
// index their shared-memory tables with it unchecked.
template <int N>
__device__ __forceinline__ int find_cell(const float (&p)[N], const Tess &t,
                                         unsigned long long *ties) {
    if constexpr (N == 1) return cell_1d(p[0], t);
    else if constexpr (N == 2) return cell_2d(p[0], p[1], t, ties);
    else return cell_3d(p[0], p[1], p[2], t, ties);
}

// --------------------------- device error word ------------------------------
__device__ __forceinline__ void raise_error(unsigned *err, unsigned bits) {
    if (err) atomicOr(err, bits);
}

// --------------------------- TMA bulk staging -------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes,
                                         uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait: each try_wait suspends for a hardware time slice, so the
// limit corresponds to well over a second before giving up.
constexpr unsigned kWaitLimit = 1u << 22;

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, unsigned parity) {
    for (unsigned it = 0; it < kWaitLimit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Copy `floats` floats from global src to shared dst.  Collective over the
// CTA; must be called by all threads.  Returns false (after raising
// kErrTmaTimeout) if the bulk copy did not complete in time; the caller must
// then return without touching dst.
__device__ __forceinline__ bool stage_table(float *dst, const float *src, int floats,
                                            uint64_t *bar, unsigned *err) {
    const unsigned bytes = (unsigned)floats * 4u;
    const bool use_tma = ((reinterpret_cast<uintptr_t>(src) & 15u) == 0) && ((bytes & 15u) == 0) &&
                         bytes > 0;
    if (!use_tma) {
        for (int i = threadIdx.x; i < floats; i += blockDim.x) dst[i] = __ldg(src + i);
        __syncthreads();
        return true;
    }
    if (threadIdx.x == 0) mbar_init(bar, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_arrive_expect_tx(bar, bytes);
        constexpr unsigned kChunk = 16384;
        for (unsigned off = 0; off < bytes; off += kChunk) {
            const unsigned n = (bytes - off < kChunk) ? (bytes - off) : kChunk;
            bulk_g2s(reinterpret_cast<char *>(dst) + off, reinterpret_cast<const char *>(src) + off,
                     n, bar);
        }
    }
    bool ok = mbar_wait_bounded(bar, 0);
    if (!ok) {
        raise_error(err, kErrTmaTimeout);
        mbar_wait_bounded(bar, 0);   // give copies in flight a second bounded chance
    }
    ok = __syncthreads_and(ok);
    return ok;
}

// ---------------------------- affine helpers ---------------------------------
// y = M[:, :N] x + M[:, N] for one cell map (row-major N x (N+1)).
template <int N>
__device__ __forceinline__ void affine_apply(const float *M, const float (&x)[N], float (&y)[N]) {
#pragma unroll
    for (int r = 0; r < N; ++r) {
        float acc = M[r * (N + 1) + N];
#pragma unroll
        for (int c = 0; c < N; ++c) acc = fmaf(M[r * (N + 1) + c], x[c], acc);
        y[r] = acc;
    }
}

// Load one cell's N x (N+1) map from shared memory into registers.
template <int N>
__device__ __forceinline__ void load_cell(const float *tab, int c, float (&M)[N * (N + 1)]) {
    const float *src = tab + c * (N * (N + 1));
    if constexpr (N == 1) {
        const float2 v = *reinterpret_cast<const float2 *>(src);
        M[0] = v.x; M[1] = v.y;
    } else if constexpr (N == 2) {
        const float2 a = reinterpret_cast<const float2 *>(src)[0];
        const float2 b = reinterpret_cast<const float2 *>(src)[1];
        const float2 d = reinterpret_cast<const float2 *>(src)[2];
        M[0] = a.x; M[1] = a.y; M[2] = b.x; M[3] = b.y; M[4] = d.x; M[5] = d.y;
    } else {
        const float4 a = reinterpret_cast<const float4 *>(src)[0];
        const float4 b = reinterpret_cast<const float4 *>(src)[1];
        const float4 d = reinterpret_cast<const float4 *>(src)[2];
        M[0] = a.x; M[1] = a.y; M[2] = a.z; M[3] = a.w;
        M[4] = b.x; M[5] = b.y; M[6] = b.z; M[7] = b.w;
        M[8] = d.x; M[9] = d.y; M[10] = d.z; M[11] = d.w;
    }
}

}  // namespace cpab
