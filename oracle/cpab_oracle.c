/*
 * CPU oracle for the CPAB integration path.  TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, in plain C, the reference's CPU implementation of the
 * hot path so that tests can check the CUDA kernels against it and bench.py
 * can time it as the CPU baseline.  Nothing in the libcpab_gb300 package links
 * or calls it.
 *
 * Restated from SkafteNicki/libcpab:
 *   libcpab/core/cpab_ops.cpp:22-24    mymin
 *   libcpab/core/cpab_ops.cpp:26-31    findcellidx_1D
 *   libcpab/core/cpab_ops.cpp:33-104   findcellidx_2D (double-precision lookup,
 *                                      out-of-domain rules)
 *   libcpab/core/cpab_ops.cpp:106-184  findcellidx_3D (push-inside rule that
 *                                      ignores z, z clamp with nz*inc_x)
 *   libcpab/core/cpab_ops.cpp:224-260  cpab_forward_op  (p <- T_c [p;1])
 *   libcpab/core/cpab_ops.cpp:262-372  cpab_backward_op (midpoint-rule forward
 *                                      sensitivity), here contracted with the
 *                                      incoming cotangent as in
 *                                      libcpab/pytorch/transformer.py:201
 *   libcpab/pytorch/interpolation.py:18-172  linear/bilinear/trilinear sampling
 *                                      with clamp-to-edge, and its autograd
 *                                      backward (scatter-add into d(data),
 *                                      gradient through xd/yd/zd)
 *
 * Build with -ffp-contract=off: the reference is compiled for x86-64 without
 * FMA, so contracting a*b+c would change roundings (GCC contracts by default
 * on aarch64).  Loops over (theta, point) are split across OpenMP threads;
 * each (theta, point) is computed exactly as the single-threaded reference
 * does, so the thread count never changes a result.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int ref_round_min(int a, double b) { return !(b < a) ? a : (int)round(b); }

int oracle_cell_1d(const float *p, int nx) {
    int idx = (int)floorf(p[0] * (float)nx);
    if (idx > nx - 1) idx = nx - 1;
    if (idx < 0) idx = 0;
    return idx;
}

int oracle_cell_2d(const float *p, int nx, int ny) {
    const double px = p[0], py = p[1];
    const float ix = (float)(1.0 / nx), iy = (float)(1.0 / ny);
    const float wx = (float)nx * ix, wy = (float)ny * iy;   /* float products */
    double cx = px > 0.0 ? px : 0.0;
    double cy = py > 0.0 ? py : 0.0;
    if (cx > wx - 0.000000001) cx = wx - 0.000000001;
    if (cy > wy - 0.000000001) cy = wy - 0.000000001;
    const double rx = fmod(cx, (double)ix), ry = fmod(cy, (double)iy);
    const double fx = rx / ix, fy = ry / iy;
    int c = 4 * (ref_round_min(nx - 1, (cx - rx) / ix) +
                 ref_round_min(ny - 1, (cy - ry) / iy) * nx);
    if (px <= 0) {                                     /* left of domain */
        if (py <= 0 && py / iy < px / ix) return c;
        if (py >= ny * iy && py / iy - ny > -px / ix) return c + 2;
        return c + 3;
    }
    if (px >= nx * ix) {                               /* right of domain */
        if (py <= 0 && -py / iy > px / ix - nx) return c;
        if (py >= ny * iy && py / iy - ny > px / ix - nx) return c + 2;
        return c + 1;
    }
    if (py <= 0) return c;                             /* above */
    if (py >= ny * iy) return c + 2;                   /* below */
    if (fx < fy) return (1 - fx < fy) ? c + 2 : c + 3;
    return (1 - fx < fy) ? c + 1 : c;
}

int oracle_cell_3d(const float *p, int nx, int ny, int nz) {
    const float ix = (float)(1.0 / nx), iy = (float)(1.0 / ny), iz = (float)(1.0 / nz);
    float q0 = p[0], q1 = p[1], q2 = p[2];
    if (q0 < 0.0 || q0 > 1.0 || q1 < 0.0 || q1 > 1.0) {   /* z is not tested */
        const float h = 0.5f;
        q0 -= h; q1 -= h; q2 -= h;
        const float a0 = fabsf(q0), a1 = fabsf(q1), a2 = fabsf(q2);
        const float s0 = (a0 < a1 && a0 < a2) ? h * ix : 0.0f;
        const float s1 = (a1 < a0 && a0 < a2) ? h * iy : 0.0f;
        const float s2 = (a2 < a0 && a0 < a1) ? h * iz : 0.0f;
        if (a0 > h) q0 = copysignf(h - s0, q0);
        if (a1 > h) q1 = copysignf(h - s1, q1);
        if (a2 > h) q2 = copysignf(h - s2, q2);
        q0 += h; q1 += h; q2 += h;
    }
    const float zero = 0.0f;
    const float m0 = (float)((float)nx * ix - 1e-8);
    const float m1 = (float)((float)ny * iy - 1e-8);
    const float m2 = (float)((float)nz * ix - 1e-8);     /* inc_x, as in the reference */
    float c0 = q0 > zero ? q0 : zero; if (m0 < c0) c0 = m0;
    float c1 = q1 > zero ? q1 : zero; if (m1 < c1) c1 = m1;
    float c2 = q2 > zero ? q2 : zero; if (m2 < c2) c2 = m2;
    const double r0 = fmodf(c0, ix), r1 = fmodf(c1, iy), r2 = fmodf(c2, iz);
    const int i = ref_round_min(nx - 1, ((double)c0 - r0) / ix);
    const int j = ref_round_min(ny - 1, ((double)c1 - r1) / iy);
    const int k = ref_round_min(nz - 1, ((double)c2 - r2) / iz);
    int c = 5 * (i + j * nx + k * nx * ny);
    double x = r0 / ix, y = r1 / iy, z = r2 / iz;
    int flip;
    if (k % 2 == 0) flip = (i % 2 == 0 && j % 2 == 1) || (i % 2 == 1 && j % 2 == 0);
    else flip = (i % 2 == 0 && j % 2 == 0) || (i % 2 == 1 && j % 2 == 1);
    if (flip) { double t = x; x = y; y = 1 - t; }
    if (-x - y + z >= 0) return c + 1;
    if (x + y + z - 2 >= 0) return c + 2;
    if (-x + y - z >= 0) return c + 3;
    if (x - y - z >= 0) return c + 4;
    return c;
}

int oracle_cell(int ndim, const float *p, const int *nc) {
    if (ndim == 1) return oracle_cell_1d(p, nc[0]);
    if (ndim == 2) return oracle_cell_2d(p, nc[0], nc[1]);
    return oracle_cell_3d(p, nc[0], nc[1], nc[2]);
}

static int cells_of(int ndim, const int *nc) {
    if (ndim == 1) return nc[0];
    if (ndim == 2) return 4 * nc[0] * nc[1];
    return 5 * nc[0] * nc[1] * nc[2];
}

/* x = M [b;1] with M an ndim x (ndim+1) row-major block. */
static void affine(int n, float *x, const float *M, const float *b) {
    for (int r = 0; r < n; r++) {
        float acc = M[r * (n + 1)] * b[0];
        for (int c = 1; c < n; c++) acc = acc + M[r * (n + 1) + c] * b[c];
        x[r] = acc + M[r * (n + 1) + n];
    }
}

static void linear(int n, float *x, const float *M, const float *b) {
    for (int r = 0; r < n; r++) {
        float acc = M[r * (n + 1)] * b[0];
        for (int c = 1; c < n; c++) acc = acc + M[r * (n + 1) + c] * b[c];
        x[r] = acc;
    }
}

int oracle_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* Cell index of every point: p is [ndim, nP] (SoA). */
void oracle_findcellidx(int ndim, const int *nc, const float *points, long nP, int *out) {
    #pragma omp parallel for schedule(static)
    for (long i = 0; i < nP; i++) {
        float p[3];
        for (int j = 0; j < ndim; j++) p[j] = points[j * nP + i];
        out[i] = oracle_cell(ndim, p, nc);
    }
}

/*
 * Forward integration with the per-cell step maps T (reference layout
 * [n_theta, nC, ndim, ndim+1]).  points are [ndim, nP] (broadcast=0) or
 * [n_theta, ndim, nP] (broadcast=1); out is [n_theta, ndim, nP].
 * cells (optional, may be NULL) receives the cell used at each step,
 * [n_theta, nP, nsteps].
 */
void oracle_forward(int ndim, const int *nc, int nsteps, const float *points, int broadcast,
                    long nP, const float *trels, int n_theta, float *out, int *cells) {
    const int nC = cells_of(ndim, nc);
    const int ppc = ndim * (ndim + 1);
    #pragma omp parallel for collapse(2) schedule(static)
    for (int t = 0; t < n_theta; t++) {
        for (long i = 0; i < nP; i++) {
            float p[3], q[3];
            const float *src = points + (broadcast ? (long)t * nP * ndim : 0);
            for (int j = 0; j < ndim; j++) p[j] = src[i + j * nP];
            for (int s = 0; s < nsteps; s++) {
                const int c = oracle_cell(ndim, p, nc);
                if (cells) cells[((long)t * nP + i) * nsteps + s] = c;
                affine(ndim, q, trels + ((long)t * nC + c) * ppc, p);
                for (int j = 0; j < ndim; j++) p[j] = q[j];
            }
            for (int j = 0; j < ndim; j++) out[(long)t * ndim * nP + i + j * nP] = p[j];
        }
    }
}

/*
 * Reference analytic gradient: for every (theta, point, k) integrate the
 * midpoint-rule sensitivity q_k of the midpoint trajectory (h in double,
 * positions and q in float), then dtheta[t,k] = sum_{j,i} grad[t,j,i]*q_k.
 * As is [n_theta, nC, ndim, ndim+1]; Bs is [d, nC, ndim, ndim+1].
 * dtheta is [n_theta, d].  The sum over points is accumulated in double.
 */
void oracle_backward(int ndim, const int *nc, int nsteps, const float *points, int broadcast,
                     long nP, const float *As, int n_theta, const float *Bs, int d,
                     const float *grad, double *dtheta) {
    const int nC = cells_of(ndim, nc);
    const int ppc = ndim * (ndim + 1);
    const double h = 1.0 / nsteps;
    #pragma omp parallel for collapse(2) schedule(dynamic, 1)
    for (int t = 0; t < n_theta; t++) {
        for (int k = 0; k < d; k++) {
            double acc = 0.0;
            for (long i = 0; i < nP; i++) {
                float p[3], v[3], pm[3], vm[3], q[3] = {0, 0, 0}, qm[3];
                float bt[3], aq[3], u[3], um[3];
                const float *src = points + (broadcast ? (long)t * nP * ndim : 0);
                for (int j = 0; j < ndim; j++) p[j] = src[i + j * nP];
                for (int s = 0; s < nsteps; s++) {
                    const int c = oracle_cell(ndim, p, nc);
                    const float *A = As + ((long)t * nC + c) * ppc;
                    const float *B = Bs + ((long)k * nC + c) * ppc;
                    affine(ndim, v, A, p);
                    for (int j = 0; j < ndim; j++) pm[j] = (float)(p[j] + h * v[j] / 2.0);
                    affine(ndim, vm, A, pm);
                    affine(ndim, bt, B, p);
                    linear(ndim, aq, A, q);
                    for (int j = 0; j < ndim; j++) u[j] = bt[j] + aq[j];
                    for (int j = 0; j < ndim; j++) qm[j] = (float)(q[j] + h * u[j] / 2.0);
                    affine(ndim, bt, B, pm);
                    linear(ndim, aq, A, qm);
                    for (int j = 0; j < ndim; j++) um[j] = bt[j] + aq[j];
                    for (int j = 0; j < ndim; j++) q[j] = (float)(q[j] + um[j] * h);
                    for (int j = 0; j < ndim; j++) p[j] = (float)(p[j] + vm[j] * h);
                }
                for (int j = 0; j < ndim; j++)
                    acc += (double)grad[(long)t * ndim * nP + i + j * nP] * (double)q[j];
            }
            dtheta[(long)t * d + k] = acc;
        }
    }
}

/*
 * The midpoint trajectory that cpab_backward_op differentiates
 * (libcpab/core/cpab_ops.cpp:300-366: v = A[p;1], pMid = p + h v / 2 with h a
 * double, vMid = A[pMid;1], p += vMid * h) for the points [ndim, nP] of one
 * theta with cell table As [nC, ndim, ndim+1].  out [ndim, nP] receives the
 * end points, cells [nP, nsteps] the cell of every step.
 */
void oracle_midpoint_trajectory(int ndim, const int *nc, int nsteps, const float *points,
                                long nP, const float *As, float *out, int *cells) {
    const int ppc = ndim * (ndim + 1);
    const double h = 1.0 / nsteps;
    #pragma omp parallel for schedule(static)
    for (long i = 0; i < nP; i++) {
        float p[3], v[3], pm[3], vm[3];
        for (int j = 0; j < ndim; j++) p[j] = points[i + j * nP];
        for (int s = 0; s < nsteps; s++) {
            const int c = oracle_cell(ndim, p, nc);
            cells[i * nsteps + s] = c;
            const float *A = As + (long)c * ppc;
            affine(ndim, v, A, p);
            for (int j = 0; j < ndim; j++) pm[j] = (float)(p[j] + h * v[j] / 2.0);
            affine(ndim, vm, A, pm);
            for (int j = 0; j < ndim; j++) p[j] = (float)(p[j] + vm[j] * h);
        }
        for (int j = 0; j < ndim; j++) out[i + j * nP] = p[j];
    }
}

/* ---------------- interpolation (libcpab/pytorch/interpolation.py) ---------------- */

static long clampl(long v, long lo, long hi) { return v < lo ? lo : (v > hi ? hi : v); }

/*
 * Forward sampling.  data is [nb, C, W(, H(, D))] (pytorch layout), grid is
 * [nb, ndim, nP] with nP = prod(outsize) and the meshgrid's x fastest.  out is
 * [nb, C, out_w(, out_h(, out_d))], i.e. for point index
 * k = ix + out_w*(iy + out_h*iz) the element out[b, c, ix, iy, iz].
 */
void oracle_interpolate(int ndim, const float *data, int nb, int C, const int *size,
                        const float *grid, const int *outsize, float *out) {
    long nP = 1, nD = 1;
    for (int j = 0; j < ndim; j++) { nP *= outsize[j]; nD *= size[j]; }
    #pragma omp parallel for collapse(2) schedule(static)
    for (int b = 0; b < nb; b++) {
        for (long k = 0; k < nP; k++) {
            float f[3]; long i0[3], i1[3];
            long rem = k, o[3] = {0, 0, 0};
            for (int j = 0; j < ndim; j++) { o[j] = rem % outsize[j]; rem /= outsize[j]; }
            for (int j = 0; j < ndim; j++) {
                const float x = grid[((long)b * ndim + j) * nP + k] * (float)(size[j] - 1);
                const long x0 = (long)floorf(x);
                i0[j] = clampl(x0, 0, size[j] - 1);
                i1[j] = clampl(x0 + 1, 0, size[j] - 1);
                f[j] = x - (float)i0[j];
            }
            long ooff = 0;   /* out index over (ix, iy, iz) with iz fastest */
            for (int j = 0; j < ndim; j++) ooff = ooff * outsize[j] + o[j];
            for (int c = 0; c < C; c++) {
                const float *D = data + ((long)b * C + c) * nD;
                float v;
                if (ndim == 1) {
                    v = D[i0[0]] * (1 - f[0]) + D[i1[0]] * f[0];
                } else if (ndim == 2) {
                    const long H = size[1];
                    const float c00 = D[i0[0] * H + i0[1]], c01 = D[i0[0] * H + i1[1]];
                    const float c10 = D[i1[0] * H + i0[1]], c11 = D[i1[0] * H + i1[1]];
                    const float a0 = c00 * (1 - f[0]) + c10 * f[0];
                    const float a1 = c01 * (1 - f[0]) + c11 * f[0];
                    v = a0 * (1 - f[1]) + a1 * f[1];
                } else {
                    const long H = size[1], Dd = size[2];
#define AT(a, b2, c2) D[((a) * H + (b2)) * Dd + (c2)]
                    const float c000 = AT(i0[0], i0[1], i0[2]), c001 = AT(i0[0], i0[1], i1[2]);
                    const float c010 = AT(i0[0], i1[1], i0[2]), c011 = AT(i0[0], i1[1], i1[2]);
                    const float c100 = AT(i1[0], i0[1], i0[2]), c101 = AT(i1[0], i0[1], i1[2]);
                    const float c110 = AT(i1[0], i1[1], i0[2]), c111 = AT(i1[0], i1[1], i1[2]);
#undef AT
                    const float a00 = c000 * (1 - f[0]) + c100 * f[0];
                    const float a01 = c001 * (1 - f[0]) + c101 * f[0];
                    const float a10 = c010 * (1 - f[0]) + c110 * f[0];
                    const float a11 = c011 * (1 - f[0]) + c111 * f[0];
                    const float a0 = a00 * (1 - f[1]) + a10 * f[1];
                    const float a1 = a01 * (1 - f[1]) + a11 * f[1];
                    v = a0 * (1 - f[2]) + a1 * f[2];
                }
                out[((long)b * C + c) * nP + ooff] = v;
            }
        }
    }
}

/*
 * Backward of oracle_interpolate for cotangent gout (layout of out).
 * ddata (layout of data) is accumulated in double and must be zeroed by the
 * caller; dgrid (layout of grid) is overwritten.  Accumulation is serial
 * over batches' points inside each batch so the result does not depend on
 * the thread count (one thread per batch image).
 */
void oracle_interpolate_backward(int ndim, const float *data, int nb, int C, const int *size,
                                 const float *grid, const int *outsize, const float *gout,
                                 double *ddata, float *dgrid) {
    long nP = 1, nD = 1;
    for (int j = 0; j < ndim; j++) { nP *= outsize[j]; nD *= size[j]; }
    #pragma omp parallel for schedule(static)
    for (int b = 0; b < nb; b++) {
        for (long k = 0; k < nP; k++) {
            float f[3]; long i0[3], i1[3];
            long rem = k, o[3] = {0, 0, 0};
            for (int j = 0; j < ndim; j++) { o[j] = rem % outsize[j]; rem /= outsize[j]; }
            for (int j = 0; j < ndim; j++) {
                const float x = grid[((long)b * ndim + j) * nP + k] * (float)(size[j] - 1);
                const long x0 = (long)floorf(x);
                i0[j] = clampl(x0, 0, size[j] - 1);
                i1[j] = clampl(x0 + 1, 0, size[j] - 1);
                f[j] = x - (float)i0[j];
            }
            long ooff = 0;
            for (int j = 0; j < ndim; j++) ooff = ooff * outsize[j] + o[j];
            double g[3] = {0, 0, 0};
            for (int c = 0; c < C; c++) {
                const float *D = data + ((long)b * C + c) * nD;
                double *G = ddata + ((long)b * C + c) * nD;
                const double w = gout[((long)b * C + c) * nP + ooff];
                if (ndim == 1) {
                    G[i0[0]] += w * (1 - f[0]);
                    G[i1[0]] += w * f[0];
                    g[0] += w * ((double)D[i1[0]] - D[i0[0]]);
                } else if (ndim == 2) {
                    const long H = size[1];
                    const double fx = f[0], fy = f[1];
                    const double c00 = D[i0[0] * H + i0[1]], c01 = D[i0[0] * H + i1[1]];
                    const double c10 = D[i1[0] * H + i0[1]], c11 = D[i1[0] * H + i1[1]];
                    G[i0[0] * H + i0[1]] += w * (1 - fx) * (1 - fy);
                    G[i1[0] * H + i0[1]] += w * fx * (1 - fy);
                    G[i0[0] * H + i1[1]] += w * (1 - fx) * fy;
                    G[i1[0] * H + i1[1]] += w * fx * fy;
                    g[0] += w * ((c10 - c00) * (1 - fy) + (c11 - c01) * fy);
                    g[1] += w * ((c01 * (1 - fx) + c11 * fx) - (c00 * (1 - fx) + c10 * fx));
                } else {
                    const long H = size[1], Dd = size[2];
                    const double fx = f[0], fy = f[1], fz = f[2];
                    double cv[2][2][2];
                    for (int a = 0; a < 2; a++)
                        for (int bb = 0; bb < 2; bb++)
                            for (int cc = 0; cc < 2; cc++) {
                                const long ia = a ? i1[0] : i0[0], ib = bb ? i1[1] : i0[1],
                                           ic = cc ? i1[2] : i0[2];
                                const long off = (ia * H + ib) * Dd + ic;
                                cv[a][bb][cc] = D[off];
                                G[off] += w * (a ? fx : 1 - fx) * (bb ? fy : 1 - fy) *
                                          (cc ? fz : 1 - fz);
                            }
                    /* d/dfx, d/dfy, d/dfz of the trilinear form */
                    double gx = 0, gy = 0, gz = 0;
                    for (int bb = 0; bb < 2; bb++)
                        for (int cc = 0; cc < 2; cc++)
                            gx += (cv[1][bb][cc] - cv[0][bb][cc]) * (bb ? fy : 1 - fy) *
                                  (cc ? fz : 1 - fz);
                    for (int a = 0; a < 2; a++)
                        for (int cc = 0; cc < 2; cc++)
                            gy += (cv[a][1][cc] - cv[a][0][cc]) * (a ? fx : 1 - fx) *
                                  (cc ? fz : 1 - fz);
                    for (int a = 0; a < 2; a++)
                        for (int bb = 0; bb < 2; bb++)
                            gz += (cv[a][bb][1] - cv[a][bb][0]) * (a ? fx : 1 - fx) *
                                  (bb ? fy : 1 - fy);
                    g[0] += w * gx; g[1] += w * gy; g[2] += w * gz;
                }
            }
            for (int j = 0; j < ndim; j++)
                dgrid[((long)b * ndim + j) * nP + k] = (float)(g[j] * (double)(size[j] - 1));
        }
    }
}
