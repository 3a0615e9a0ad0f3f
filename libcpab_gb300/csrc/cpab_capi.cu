// extern "C" entry points declared in include/cpab_gb300.h: argument
// validation, tessellation constants, error reporting, and dispatch to the
// kernel launchers.
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <vector>

#include "../../include/cpab_gb300.h"
#include "cpab_interp.cuh"
#include "cpab_launch.h"

using namespace cpab;

namespace {

thread_local char g_err[512] = "";

int fail(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

bool grad_mode_ok(int mode) {
    return mode == CPAB_GRAD_REFERENCE || mode == CPAB_GRAD_EXACT ||
           mode == CPAB_GRAD_REFERENCE_MAP;
}

int cuda_fail(cudaError_t e, const char *what) {
    return fail(CPAB_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

// Device error word, one per device (file-scope __device__ variable; its
// device address is looked up once per device).
// The per-device address caches are filled by whichever host thread calls
// first; relaxed atomics make the concurrent fills (all of the same value)
// well defined.
__device__ unsigned g_device_error;
constexpr int kMaxDevices = 64;
std::atomic<unsigned *> g_err_ptr[kMaxDevices];

unsigned *device_error_word() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();   // leave no error behind for the next launch check
        return nullptr;
    }
    if (dev < 0 || dev >= kMaxDevices) return nullptr;
    unsigned *w = g_err_ptr[dev].load(std::memory_order_relaxed);
    if (!w) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_device_error) != cudaSuccess || !p) {
            cudaGetLastError();
            return nullptr;
        }
        w = static_cast<unsigned *>(p);
        g_err_ptr[dev].store(w, std::memory_order_relaxed);
    }
    return w;
}

// Validate a tessellation and fill its constants (tess_init).
int make_tess(int ndim, const int *nc, Tess *t) {
    if (ndim < 1 || ndim > 3) return fail(CPAB_ERR_ARGUMENT, "ndim must be 1, 2 or 3 (got %d)", ndim);
    if (!nc) return fail(CPAB_ERR_ARGUMENT, "nc is NULL");
    long long ncells = 1;
    for (int j = 0; j < ndim; ++j) {
        if (nc[j] < 1 || nc[j] > 4096)
            return fail(CPAB_ERR_ARGUMENT, "nc[%d] = %d out of range [1, 4096]", j, nc[j]);
        ncells *= nc[j];
    }
    ncells *= (ndim == 1 ? 1 : ndim == 2 ? 4 : 5);
    if (ncells > 65535) return fail(CPAB_ERR_UNSUPPORTED, "too many cells (%lld > 65535)", ncells);
    tess_init(ndim, nc, t);
    return CPAB_OK;
}

int check_steps(int nsteps) {
    if (nsteps < 1 || nsteps > 100000)
        return fail(CPAB_ERR_ARGUMENT, "nsteps must be in [1, 100000] (got %d)", nsteps);
    return CPAB_OK;
}

cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

int check_sizes(int ndim, const int *v, const char *name) {
    if (!v) return fail(CPAB_ERR_ARGUMENT, "%s is NULL", name);
    for (int j = 0; j < ndim; ++j)
        if (v[j] < 1) return fail(CPAB_ERR_ARGUMENT, "%s[%d] = %d must be positive", name, j, v[j]);
    return CPAB_OK;
}

// Image geometry: positive extents, per-image sizes within the kernels'
// 32-bit indexing, and at most 65535 images (one grid row each, as the
// reference's launches put the batch on the grid's y dimension).
int check_geo(int ndim, const int *size, const int *outsize, int nb) {
    int rc;
    if ((rc = check_sizes(ndim, size, "size")) || (rc = check_sizes(ndim, outsize, "outsize")))
        return rc;
    if (!geo_fits(ndim, size, outsize))
        return fail(CPAB_ERR_UNSUPPORTED, "image too large (per-image elements must be < 2^31)");
    if (nb > 65535) return fail(CPAB_ERR_UNSUPPORTED, "at most 65535 images per call (got %d)", nb);
    return CPAB_OK;
}

int check_theta_count(int n_theta) {
    if (n_theta > 65535)
        return fail(CPAB_ERR_UNSUPPORTED, "at most 65535 transformations per call (got %d)", n_theta);
    return CPAB_OK;
}

}  // namespace

extern "C" {

const char *cpab_last_error(void) { return g_err; }

int cpab_version(void) { return 10000; }

int cpab_num_cells(int ndim, const int *nc) {
    Tess t;
    if (make_tess(ndim, nc, &t) != CPAB_OK) return -1;
    return t.nC;
}

int cpab_cell_tables(int ndim, const int *nc, int nsteps, const float *theta, int n_theta,
                     int d, const float *basis, float *A, float *T, float *E, void *stream) {
    g_err[0] = 0;
    Tess t;
    int rc = make_tess(ndim, nc, &t);
    if (rc) return rc;
    if ((rc = check_steps(nsteps))) return rc;
    if (n_theta < 0 || d < 0) return fail(CPAB_ERR_ARGUMENT, "need n_theta >= 0 and d >= 0");
    if (n_theta > 0 && d > 0 && (!theta || !basis))
        return fail(CPAB_ERR_ARGUMENT, "theta or basis is NULL");
    cudaError_t e = launch_cell_tables(t, nsteps, theta, n_theta, d, basis, A, T, E, as_stream(stream));
    return e == cudaSuccess ? CPAB_OK : cuda_fail(e, "cell tables launch");
}

static int integrate_common(int ndim, const int *nc, int nsteps, const float *points,
                            int broadcast, long long nP, const float *table, bool comp,
                            int n_theta, float *out, int *trace, unsigned long long *ties,
                            void *stream, const LaunchShape *force = nullptr) {
    g_err[0] = 0;
    Tess t;
    int rc = make_tess(ndim, nc, &t);
    if (rc) return rc;
    if ((rc = check_steps(nsteps))) return rc;
    if (nP < 0 || n_theta < 0) return fail(CPAB_ERR_ARGUMENT, "negative size");
    if ((rc = check_theta_count(n_theta))) return rc;
    if (nP == 0 || n_theta == 0) return CPAB_OK;
    if (!points || !table || !out) return fail(CPAB_ERR_ARGUMENT, "points, table or out is NULL");
    unsigned *err = device_error_word();
    cudaError_t e = launch_integrate(t, nsteps, points, broadcast ? 1 : 0, nP, table, comp, n_theta,
                                     out, trace, ties, err, as_stream(stream), force);
    return e == cudaSuccess ? CPAB_OK : cuda_fail(e, "integrate launch");
}

int cpab_forward(int ndim, const int *nc, int nsteps, const float *points, int broadcast,
                 long long nP, const float *trels, int n_theta, float *out, void *stream) {
    return integrate_common(ndim, nc, nsteps, points, broadcast, nP, trels, false, n_theta, out,
                            nullptr, nullptr, stream);
}

int cpab_integrate(int ndim, const int *nc, int nsteps, const float *points, int broadcast,
                   long long nP, const float *E, int n_theta, float *out,
                   unsigned long long *ties, void *stream) {
    return integrate_common(ndim, nc, nsteps, points, broadcast, nP, E, true, n_theta, out,
                            nullptr, ties, stream);
}

int cpab_integrate_exact(int ndim, const int *nc, const float *points, int broadcast,
                         long long nP, const float *A, int n_theta, float *out,
                         unsigned long long *ties, unsigned long long *steps, void *stream) {
    g_err[0] = 0;
    Tess t;
    int rc = make_tess(ndim, nc, &t);
    if (rc) return rc;
    if (nP < 0 || n_theta < 0) return fail(CPAB_ERR_ARGUMENT, "negative size");
    if ((rc = check_theta_count(n_theta))) return rc;
    if (nP == 0 || n_theta == 0) return CPAB_OK;
    if (!points || !A || !out) return fail(CPAB_ERR_ARGUMENT, "points, A or out is NULL");
    cudaError_t e = launch_integrate_exact(t, points, broadcast ? 1 : 0, nP, A, n_theta, out, ties,
                                           device_error_word(), steps, as_stream(stream));
    return e == cudaSuccess ? CPAB_OK : cuda_fail(e, "exact-flow launch");
}

size_t cpab_backward_exact_workspace(int ndim, const int *nc, long long nP, int n_theta) {
    g_err[0] = 0;
    Tess t;
    if (make_tess(ndim, nc, &t)) return 0;
    if (nP <= 0 || n_theta <= 0) return 0;
    AdjointPlan plan;
    if (!plan_adjoint_exact(t, nP, n_theta, &plan)) {
        fail(CPAB_ERR_UNSUPPORTED, "tessellation too large for the exact-flow adjoint");
        return 0;
    }
    return plan.partial_floats * sizeof(float);
}

int cpab_backward_exact(int ndim, const int *nc, const float *out, long long nP, const float *A,
                        int n_theta, const float *basis, int d, const float *grad_out,
                        float *dtheta, float *dpoints, void *workspace, size_t workspace_bytes,
                        unsigned long long *ties, void *stream) {
    g_err[0] = 0;
    Tess t;
    int rc = make_tess(ndim, nc, &t);
    if (rc) return rc;
    if (nP < 0 || n_theta < 0 || d < 0) return fail(CPAB_ERR_ARGUMENT, "invalid sizes");
    if ((rc = check_theta_count(n_theta))) return rc;
    if (n_theta == 0 || (d == 0 && !dpoints)) return CPAB_OK;
    if (!A || (d > 0 && (!dtheta || !basis)))
        return fail(CPAB_ERR_ARGUMENT, "dtheta, basis or A is NULL");
    cudaStream_t s = as_stream(stream);
    if (nP == 0) {
        if (d == 0) return CPAB_OK;
        cudaError_t e = cudaMemsetAsync(dtheta, 0, (size_t)n_theta * d * sizeof(float), s);
        return e == cudaSuccess ? CPAB_OK : cuda_fail(e, "memset");
    }
    if (!out || !grad_out) return fail(CPAB_ERR_ARGUMENT, "out or grad_out is NULL");
    AdjointPlan plan;
    if (!plan_adjoint_exact(t, nP, n_theta, &plan))
        return fail(CPAB_ERR_UNSUPPORTED, "tessellation too large for the exact-flow adjoint");
    const size_t need = plan.partial_floats * sizeof(float);
    if (!workspace || workspace_bytes < need)
        return fail(CPAB_ERR_WORKSPACE, "workspace of %zu bytes needed (got %zu)", need,
                    workspace ? workspace_bytes : (size_t)0);
    float *partials = static_cast<float *>(workspace);
    cudaError_t e = launch_adjoint_exact(t, plan, out, nP, A, n_theta, grad_out, dpoints,
                                         partials, ties, device_error_word(), s);
    if (e != cudaSuccess) return cuda_fail(e, "exact-flow adjoint launch");
    if (d == 0) return CPAB_OK;
    e = launch_finalize(t, 1, kFinalizeDirect, partials, plan.parts, A, basis, d, n_theta,
                        dtheta, s);
    return e == cudaSuccess ? CPAB_OK : cuda_fail(e, "finalize launch");
}

int cpab_integrate_trace(int ndim, const int *nc, int nsteps, const float *points, int broadcast,
                         long long nP, const float *E, int n_theta, float *out, int *cells,
                         void *stream) {
    if (!cells) return fail(CPAB_ERR_ARGUMENT, "cells is NULL");
    return integrate_common(ndim, nc, nsteps, points, broadcast, nP, E, true, n_theta, out, cells,
                            nullptr, stream);
}

size_t cpab_backward_workspace(int ndim, const int *nc, int nsteps, long long nP, int n_theta) {
    g_err[0] = 0;
    Tess t;
    if (make_tess(ndim, nc, &t) || check_steps(nsteps)) return 0;
    if (nP <= 0 || n_theta <= 0) return 0;
    AdjointPlan plan;
    if (!plan_adjoint(t, nsteps, nP, n_theta, &plan)) {
        fail(CPAB_ERR_UNSUPPORTED, "tessellation/nsteps too large for the adjoint kernel");
        return 0;
    }
    return plan.ws_floats() * sizeof(float);
}

}  // extern "C"

static int backward_impl(int ndim, const int *nc, int nsteps, int mode, const float *points,
                         int broadcast, long long nP, const float *A, const float *E,
                         int n_theta, const float *basis, int d, const float *grad_out,
                         float *dtheta, float *dpoints, void *workspace,
                         size_t workspace_bytes, unsigned long long *ties, void *stream,
                         const LaunchShape *force) {
    g_err[0] = 0;
    Tess t;
    int rc = make_tess(ndim, nc, &t);
    if (rc) return rc;
    if ((rc = check_steps(nsteps))) return rc;
    if (!grad_mode_ok(mode))
        return fail(CPAB_ERR_ARGUMENT, "unknown gradient mode %d", mode);
    if (nP < 0 || n_theta < 0 || d < 0) return fail(CPAB_ERR_ARGUMENT, "invalid sizes");
    if ((rc = check_theta_count(n_theta))) return rc;
    if (n_theta == 0 || (d == 0 && !dpoints)) return CPAB_OK;   // nothing to compute
    if (!A || (d > 0 && (!dtheta || !basis)))
        return fail(CPAB_ERR_ARGUMENT, "dtheta, basis or A is NULL");
    if (mode == CPAB_GRAD_EXACT && !E) return fail(CPAB_ERR_ARGUMENT, "exact mode needs E");
    cudaStream_t s = as_stream(stream);
    if (nP == 0) {
        if (d == 0) return CPAB_OK;
        cudaError_t e = cudaMemsetAsync(dtheta, 0, (size_t)n_theta * d * sizeof(float), s);
        return e == cudaSuccess ? CPAB_OK : cuda_fail(e, "memset");
    }
    if (!points || !grad_out) return fail(CPAB_ERR_ARGUMENT, "points or grad_out is NULL");
    AdjointPlan plan;
    if (!plan_adjoint(t, nsteps, nP, n_theta, &plan, true, force))
        return fail(CPAB_ERR_UNSUPPORTED, "tessellation/nsteps too large for the adjoint kernel");
    const size_t need = plan.ws_floats() * sizeof(float);
    if (!workspace || workspace_bytes < need)
        return fail(CPAB_ERR_WORKSPACE, "workspace of %zu bytes needed (got %zu)", need,
                    workspace ? workspace_bytes : (size_t)0);
    float *partials = static_cast<float *>(workspace);
    unsigned *err = device_error_word();
    cudaError_t e = launch_adjoint(t, nsteps, mode, plan, points, broadcast ? 1 : 0, nP,
                                   mode == CPAB_GRAD_EXACT ? E : A, n_theta, grad_out, dpoints,
                                   partials, ties, err, s);
    if (e != cudaSuccess) return cuda_fail(e, "adjoint launch");
    if (d == 0) return CPAB_OK;
    e = launch_finalize(t, nsteps, mode, partials, plan.parts, A, basis, d, n_theta, dtheta, s);
    return e == cudaSuccess ? CPAB_OK : cuda_fail(e, "finalize launch");
}

extern "C" {

int cpab_backward(int ndim, const int *nc, int nsteps, int mode, const float *points,
                  int broadcast, long long nP, const float *A, const float *E, int n_theta,
                  const float *basis, int d, const float *grad_out, float *dtheta,
                  float *dpoints, void *workspace, size_t workspace_bytes,
                  unsigned long long *ties, void *stream) {
    return backward_impl(ndim, nc, nsteps, mode, points, broadcast, nP, A, E, n_theta, basis, d,
                         grad_out, dtheta, dpoints, workspace, workspace_bytes, ties, stream,
                         nullptr);
}

int cpab_interpolate(int ndim, const float *data, int nb, int C, const int *size,
                     const float *grid, const int *outsize, float *out, void *stream) {
    g_err[0] = 0;
    if (ndim < 1 || ndim > 3) return fail(CPAB_ERR_ARGUMENT, "ndim must be 1, 2 or 3");
    int rc;
    if ((rc = check_geo(ndim, size, outsize, nb)))
        return rc;
    if (nb < 0 || C < 1) return fail(CPAB_ERR_ARGUMENT, "invalid nb or C");
    if (nb == 0) return CPAB_OK;
    if (!data || !grid || !out) return fail(CPAB_ERR_ARGUMENT, "data, grid or out is NULL");
    cudaError_t e = launch_interpolate(ndim, data, nb, C, size, grid, outsize, out,
                                       device_error_word(), as_stream(stream));
    return e == cudaSuccess ? CPAB_OK : cuda_fail(e, "interpolate launch");
}

int cpab_interpolate_backward(int ndim, const float *data, int nb, int C, const int *size,
                              const float *grid, const int *outsize, const float *grad_out,
                              float *ddata, float *dgrid, void *stream) {
    g_err[0] = 0;
    if (ndim < 1 || ndim > 3) return fail(CPAB_ERR_ARGUMENT, "ndim must be 1, 2 or 3");
    int rc;
    if ((rc = check_geo(ndim, size, outsize, nb)))
        return rc;
    if (nb < 0 || C < 1) return fail(CPAB_ERR_ARGUMENT, "invalid nb or C");
    if (nb == 0) return CPAB_OK;
    if (!data || !grid || !grad_out) return fail(CPAB_ERR_ARGUMENT, "data, grid or grad_out is NULL");
    cudaStream_t s = as_stream(stream);
    if (ddata) {
        size_t n = (size_t)nb * C;
        for (int j = 0; j < ndim; ++j) n *= (size_t)size[j];
        cudaError_t e = cudaMemsetAsync(ddata, 0, n * sizeof(float), s);
        if (e != cudaSuccess) return cuda_fail(e, "memset");
    }
    cudaError_t e = launch_interpolate_backward(ndim, data, nb, C, size, grid, outsize, grad_out,
                                                ddata, dgrid, s);
    return e == cudaSuccess ? CPAB_OK : cuda_fail(e, "interpolate backward launch");
}

}  // extern "C"

static int td_forward(int ndim, const int *nc, int nsteps, const float *lin, const int *outsize,
                      const float *E, int nb, const float *data, int C, const int *size,
                      float *out, float *grid_out, unsigned long long *ties, void *stream,
                      const LaunchShape *force) {
    g_err[0] = 0;
    Tess t;
    int rc = make_tess(ndim, nc, &t);
    if (rc) return rc;
    if ((rc = check_steps(nsteps))) return rc;
    if ((rc = check_geo(ndim, size, outsize, nb)))
        return rc;
    if (nb < 0 || C < 1) return fail(CPAB_ERR_ARGUMENT, "invalid nb or C");
    if (nb == 0) return CPAB_OK;
    if (!lin || !E || !data || !out) return fail(CPAB_ERR_ARGUMENT, "lin, E, data or out is NULL");
    cudaError_t e = launch_transform_data(t, nsteps, lin, outsize, E, nb, data, C, size, out,
                                          grid_out, ties, device_error_word(), as_stream(stream),
                                          force);
    return e == cudaSuccess ? CPAB_OK : cuda_fail(e, "transform_data launch");
}

extern "C" {

int cpab_transform_data(int ndim, const int *nc, int nsteps, const float *lin,
                        const int *outsize, const float *E, int nb, const float *data, int C,
                        const int *size, float *out, float *grid_out,
                        unsigned long long *ties, void *stream) {
    return td_forward(ndim, nc, nsteps, lin, outsize, E, nb, data, C, size, out, grid_out, ties,
                      stream, nullptr);
}

int cpab_transform_grid_image(int ndim, const int *nc, int nsteps, const float *lin,
                              const int *outsize, const float *E, int nb, float *grid_out,
                              unsigned long long *ties, void *stream) {
    g_err[0] = 0;
    Tess t;
    int rc = make_tess(ndim, nc, &t);
    if (rc) return rc;
    if ((rc = check_steps(nsteps))) return rc;
    if ((rc = check_geo(ndim, outsize, outsize, nb))) return rc;
    if (nb < 0) return fail(CPAB_ERR_ARGUMENT, "invalid nb");
    if (nb == 0) return CPAB_OK;
    if (!lin || !E || !grid_out) return fail(CPAB_ERR_ARGUMENT, "lin, E or grid_out is NULL");
    cudaError_t e = launch_transform_data(t, nsteps, lin, outsize, E, nb, nullptr, 0, outsize,
                                          nullptr, grid_out, ties, device_error_word(),
                                          as_stream(stream));
    return e == cudaSuccess ? CPAB_OK : cuda_fail(e, "transform_grid_image launch");
}

int cpab_sample_grid(int ndim, const float *data, int nb, int C, const int *size,
                     const float *grid, const int *outsize, float *out, void *stream) {
    g_err[0] = 0;
    if (ndim < 1 || ndim > 3) return fail(CPAB_ERR_ARGUMENT, "ndim must be 1, 2 or 3");
    int rc;
    if ((rc = check_geo(ndim, size, outsize, nb))) return rc;
    if (nb < 0 || C < 1) return fail(CPAB_ERR_ARGUMENT, "invalid nb or C");
    if (nb == 0) return CPAB_OK;
    if (!data || !grid || !out) return fail(CPAB_ERR_ARGUMENT, "data, grid or out is NULL");
    cudaError_t e = launch_sample_grid(ndim, grid, nb, data, C, size, outsize, out,
                                       as_stream(stream));
    return e == cudaSuccess ? CPAB_OK : cuda_fail(e, "sample_grid launch");
}

// ------------------------- ragged images (mixed sizes) -----------------------
static_assert(CPAB_IMAGE_PLAN_FIELDS == kImagePlanFields, "plan row width");

int cpab_ragged_images_plan(int ndim, int S, const int *sizes, const int *outsizes,
                            long long *plan, long long *totals) {
    g_err[0] = 0;
    if (ndim < 1 || ndim > 3) return fail(CPAB_ERR_ARGUMENT, "ndim must be 1, 2 or 3");
    if (S < 0) return fail(CPAB_ERR_ARGUMENT, "need S >= 0");
    if (!plan || !totals || (S > 0 && !sizes))
        return fail(CPAB_ERR_ARGUMENT, "sizes, plan or totals is NULL");
    constexpr int F = kImagePlanFields;
    long long data_points = 0, total = 0, tiles = 0;
    for (int s = 0; s < S; ++s) {
        const int *sz = sizes + (long long)s * ndim;
        const int *osz = outsizes ? outsizes + (long long)s * ndim : sz;
        int rc = check_geo(ndim, sz, osz, 1);
        if (rc) {
            char why[sizeof g_err];
            snprintf(why, sizeof why, "%s", g_err);
            return fail(rc, "image %d: %s", s, why);
        }
        long long *row = plan + (long long)s * F;
        row[0] = data_points;
        row[1] = total;
        row[2] = tiles;
        long long nD = 1, nP = 1;
        for (int j = 0; j < 3; ++j) {
            row[3 + j] = j < ndim ? sz[j] : 1;
            row[6 + j] = j < ndim ? osz[j] : 1;
            nD *= row[3 + j];
            nP *= row[6 + j];
        }
        row[9] = 0;
        data_points += nD;
        total += nP;
        tiles += image_tile_count(ndim, osz);
        if (total >= (1ll << 31) || data_points >= (1ll << 40))
            return fail(CPAB_ERR_UNSUPPORTED,
                        "ragged images: at most 2^31 - 1 output points and 2^40 data points");
    }
    long long *last = plan + (long long)S * F;
    for (int f = 0; f < F; ++f) last[f] = 0;
    last[0] = data_points;
    last[1] = total;
    last[2] = tiles;
    totals[0] = data_points;
    totals[1] = total;
    totals[2] = tiles;
    return CPAB_OK;
}

static int check_ragged_images(int ndim, int S, int C, const long long *plan,
                               long long data_points, long long total, long long tiles) {
    if (ndim < 1 || ndim > 3) return fail(CPAB_ERR_ARGUMENT, "ndim must be 1, 2 or 3");
    if (S < 0 || C < 1 || data_points < 0 || total < 0 || tiles < 0)
        return fail(CPAB_ERR_ARGUMENT, "need S >= 0, C >= 1 and non-negative totals");
    if (total >= (1ll << 31) || tiles > total)
        return fail(CPAB_ERR_UNSUPPORTED, "ragged images: total below 2^31 and tiles <= total");
    if ((double)data_points * C >= 0x1p60 || (double)total * C >= 0x1p60)
        return fail(CPAB_ERR_UNSUPPORTED, "ragged images: C * points must stay below 2^60");
    if (tiles > 0 && (S == 0 || !plan)) return fail(CPAB_ERR_ARGUMENT, "plan is NULL");
    return CPAB_OK;
}

int cpab_interpolate_ragged(int ndim, int S, int C, const long long *plan,
                            long long data_points, long long total, long long tiles,
                            const float *data, const float *grid, float *out, void *stream) {
    g_err[0] = 0;
    int rc = check_ragged_images(ndim, S, C, plan, data_points, total, tiles);
    if (rc) return rc;
    if (tiles == 0) return CPAB_OK;
    if (!data || !grid || !out) return fail(CPAB_ERR_ARGUMENT, "data, grid or out is NULL");
    unsigned *err = device_error_word();
    if (!err) return fail(CPAB_ERR_CUDA, "device error word unavailable");
    cudaError_t e = launch_interpolate_ragged(ndim, S, plan, data_points, data, C, total, tiles,
                                              grid, out, err, as_stream(stream));
    return e == cudaSuccess ? CPAB_OK : cuda_fail(e, "ragged interpolate launch");
}

int cpab_interpolate_ragged_backward(int ndim, int S, int C, const long long *plan,
                                     long long data_points, long long total, long long tiles,
                                     const float *data, const float *grid,
                                     const float *grad_out, float *ddata, float *dgrid,
                                     void *stream) {
    g_err[0] = 0;
    int rc = check_ragged_images(ndim, S, C, plan, data_points, total, tiles);
    if (rc) return rc;
    cudaStream_t s = as_stream(stream);
    if (ddata && data_points > 0) {
        cudaError_t e = cudaMemsetAsync(ddata, 0, (size_t)data_points * C * sizeof(float), s);
        if (e != cudaSuccess) return cuda_fail(e, "memset");
    }
    if (tiles == 0) return CPAB_OK;
    if (!data || !grid || !grad_out)
        return fail(CPAB_ERR_ARGUMENT, "data, grid or grad_out is NULL");
    unsigned *err = device_error_word();
    if (!err) return fail(CPAB_ERR_CUDA, "device error word unavailable");
    cudaError_t e = launch_interpolate_ragged_backward(ndim, S, plan, data_points, data, C, total,
                                                       tiles, grid, grad_out, ddata, dgrid, err,
                                                       s);
    return e == cudaSuccess ? CPAB_OK : cuda_fail(e, "ragged interpolate backward launch");
}

size_t cpab_transform_data_backward_workspace(int ndim, const int *nc, int nsteps, int mode,
                                              const int *outsize, int nb) {
    g_err[0] = 0;
    Tess t;
    if (make_tess(ndim, nc, &t) || check_steps(nsteps) || check_sizes(ndim, outsize, "outsize"))
        return 0;
    if (nb <= 0 || (!grad_mode_ok(mode))) return 0;
    long long nP = 1;
    for (int j = 0; j < ndim; ++j) nP *= outsize[j];
    AdjointPlan plan;
    if (!plan_transform_data_backward(t, nsteps, mode, nP, nb, &plan)) {
        fail(CPAB_ERR_UNSUPPORTED, "tessellation/nsteps too large for the adjoint kernel");
        return 0;
    }
    return plan.ws_floats() * sizeof(float);
}

}  // extern "C"

// transform_data backward of the last transformation of a composition whose
// earlier stages (pre, may be NULL) move the grid first.
static int td_backward(int ndim, const int *nc, int nsteps, int mode, const float *lin,
                       const int *outsize, const float *A, const float *E,
                       const float *grid_saved, int nb, const float *data, int C,
                       const int *size, const float *basis, int d, const float *grad_out,
                       float *ddata, float *dtheta, void *workspace, size_t workspace_bytes,
                       unsigned long long *ties, void *stream, const PreStages *pre,
                       const LaunchShape *force = nullptr) {
    g_err[0] = 0;
    Tess t;
    int rc = make_tess(ndim, nc, &t);
    if (rc) return rc;
    if ((rc = check_steps(nsteps))) return rc;
    if ((rc = check_geo(ndim, size, outsize, nb)))
        return rc;
    if (!grad_mode_ok(mode))
        return fail(CPAB_ERR_ARGUMENT, "unknown gradient mode %d", mode);
    if (nb < 0 || C < 1 || d < 0) return fail(CPAB_ERR_ARGUMENT, "invalid nb, C or d");
    if (nb == 0) return CPAB_OK;
    if (!lin || !A || !data || !grad_out || (d > 0 && (!basis || !dtheta)))
        return fail(CPAB_ERR_ARGUMENT, "lin, A, data, basis, grad_out or dtheta is NULL");
    if (mode == CPAB_GRAD_EXACT && !E) return fail(CPAB_ERR_ARGUMENT, "exact mode needs E");
    if (mode != CPAB_GRAD_EXACT && !grid_saved)
        return fail(CPAB_ERR_ARGUMENT, "reference mode needs grid_saved");
    long long nP = 1;
    for (int j = 0; j < ndim; ++j) nP *= outsize[j];
    AdjointPlan plan;
    if (!plan_transform_data_backward(t, nsteps, mode, nP, nb, &plan, force))
        return fail(CPAB_ERR_UNSUPPORTED, "tessellation/nsteps too large for the adjoint kernel");
    const size_t need = plan.ws_floats() * sizeof(float);
    if (!workspace || workspace_bytes < need)
        return fail(CPAB_ERR_WORKSPACE, "workspace of %zu bytes needed (got %zu)", need,
                    workspace ? workspace_bytes : (size_t)0);
    cudaStream_t s = as_stream(stream);
    if (ddata) {
        size_t n = (size_t)nb * C;
        for (int j = 0; j < ndim; ++j) n *= (size_t)size[j];
        cudaError_t e = cudaMemsetAsync(ddata, 0, n * sizeof(float), s);
        if (e != cudaSuccess) return cuda_fail(e, "memset");
    }
    float *partials = static_cast<float *>(workspace);
    cudaError_t e = launch_transform_data_backward(
        t, nsteps, mode, plan, lin, outsize, mode == CPAB_GRAD_EXACT ? E : A, grid_saved, nb, data,
        C, size, grad_out, ddata, partials, ties, device_error_word(), s, pre);
    if (e != cudaSuccess) return cuda_fail(e, "transform_data backward launch");
    if (d == 0) return CPAB_OK;
    e = launch_finalize(t, nsteps, mode, partials, plan.parts, A, basis, d, nb, dtheta, s);
    return e == cudaSuccess ? CPAB_OK : cuda_fail(e, "finalize launch");
}

// Stages 0..K-1 of a composition (nc: K*ndim ints, nsteps: K ints, E: K
// device pointers).
static int make_stages(int ndim, int K, const int *nc, const int *nsteps,
                       const float *const *E, SeqStages *sq) {
    if (K < 1 || K > kMaxPre + 1)
        return fail(CPAB_ERR_ARGUMENT, "a composition has 1 to %d transformations (got %d)",
                    kMaxPre + 1, K);
    if (!nc || !nsteps || !E) return fail(CPAB_ERR_ARGUMENT, "nc, nsteps or E is NULL");
    sq->K = K;
    for (int k = 0; k < K; ++k) {
        int rc = make_tess(ndim, nc + k * ndim, &sq->t[k]);
        if (rc) return rc;
        if ((rc = check_steps(nsteps[k]))) return rc;
        if (!E[k]) return fail(CPAB_ERR_ARGUMENT, "E[%d] is NULL", k);
        sq->nsteps[k] = nsteps[k];
        sq->E[k] = E[k];
    }
    return CPAB_OK;
}

extern "C" {

int cpab_transform_data_backward(int ndim, const int *nc, int nsteps, int mode,
                                 const float *lin, const int *outsize, const float *A,
                                 const float *E, const float *grid_saved, int nb,
                                 const float *data, int C, const int *size, const float *basis,
                                 int d, const float *grad_out, float *ddata, float *dtheta,
                                 void *workspace, size_t workspace_bytes,
                                 unsigned long long *ties, void *stream) {
    return td_backward(ndim, nc, nsteps, mode, lin, outsize, A, E, grid_saved, nb, data, C, size,
                       basis, d, grad_out, ddata, dtheta, workspace, workspace_bytes, ties,
                       stream, nullptr);
}

int cpab_sequential_transform_data(int ndim, int K, const int *nc, const int *nsteps,
                                   const float *lin, const int *outsize, const float *const *E,
                                   int nb, const float *data, int C, const int *size, float *out,
                                   float *grid_out, unsigned long long *ties, void *stream) {
    g_err[0] = 0;
    if (ndim < 1 || ndim > 3) return fail(CPAB_ERR_ARGUMENT, "ndim must be 1, 2 or 3");
    SeqStages sq;
    int rc = make_stages(ndim, K, nc, nsteps, E, &sq);
    if (rc) return rc;
    if ((rc = check_geo(ndim, size, outsize, nb))) return rc;
    if (nb < 0 || C < 1) return fail(CPAB_ERR_ARGUMENT, "invalid nb or C");
    if (nb == 0) return CPAB_OK;
    if (!lin || !data || !out) return fail(CPAB_ERR_ARGUMENT, "lin, data or out is NULL");
    cudaError_t e = launch_sequential_transform_data(sq, lin, outsize, nb, data, C, size, out,
                                                     grid_out, ties, device_error_word(),
                                                     as_stream(stream));
    return e == cudaSuccess ? CPAB_OK : cuda_fail(e, "sequential transform_data launch");
}

int cpab_sequential_transform_data_backward(int ndim, int K, const int *nc, const int *nsteps,
                                            int mode, const float *lin, const int *outsize,
                                            const float *const *E, const float *A_last,
                                            const float *grid_saved, int nb, const float *data,
                                            int C, const int *size, const float *basis_last,
                                            int d_last, const float *grad_out, float *ddata,
                                            float *dtheta_last, void *workspace,
                                            size_t workspace_bytes, unsigned long long *ties,
                                            void *stream) {
    g_err[0] = 0;
    if (ndim < 1 || ndim > 3) return fail(CPAB_ERR_ARGUMENT, "ndim must be 1, 2 or 3");
    SeqStages sq;
    int rc = make_stages(ndim, K, nc, nsteps, E, &sq);
    if (rc) return rc;
    PreStages pre;
    pre.K = K - 1;
    for (int k = 0; k < K - 1; ++k) {
        pre.t[k] = sq.t[k];
        pre.nsteps[k] = sq.nsteps[k];
        pre.E[k] = sq.E[k];
    }
    return td_backward(ndim, nc + (K - 1) * ndim, nsteps[K - 1], mode, lin, outsize, A_last,
                       E[K - 1], grid_saved, nb, data, C, size, basis_last, d_last, grad_out,
                       ddata, dtheta_last, workspace, workspace_bytes, ties, stream, &pre);
}

int cpab_findcellidx(int ndim, const int *nc, const float *points, long long nP, int *out,
                     unsigned long long *ties, void *stream) {
    g_err[0] = 0;
    Tess t;
    int rc = make_tess(ndim, nc, &t);
    if (rc) return rc;
    if (nP < 0) return fail(CPAB_ERR_ARGUMENT, "negative nP");
    if (nP == 0) return CPAB_OK;
    if (!points || !out) return fail(CPAB_ERR_ARGUMENT, "points or out is NULL");
    cudaError_t e = launch_findcellidx(t, points, nP, out, ties, as_stream(stream));
    return e == cudaSuccess ? CPAB_OK : cuda_fail(e, "findcellidx launch");
}

int cpab_device_status(unsigned *flags, int clear) {
    g_err[0] = 0;
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_fail(e, "device synchronize");
    unsigned *p = device_error_word();
    unsigned v = 0;
    if (p) {
        e = cudaMemcpy(&v, p, sizeof(v), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(e, "read device error word");
        if (clear) {
            e = cudaMemset(p, 0, sizeof(unsigned));
            if (e != cudaSuccess) return cuda_fail(e, "clear device error word");
        }
    }
    if (flags) *flags = v;
    return CPAB_OK;
}

}  // extern "C"

// ------------------------- ragged batched 1D series -------------------------
namespace {

// Kinds of ragged kernels with their own launch shape (autotuner key).
constexpr int kRaggedForward = 0, kRaggedAdjoint = 1;

// Launch shape: the autotuned one for this problem if cpab_ragged1d_tune ran
// on it, else the defaults (forward: 256 threads, 2 points per lane;
// adjoint: the largest block whose shared memory fits, 1 pass per tile).
bool ragged_shape(int kind, int mode, const Tess &t, int nsteps, int S, long long total,
                  int *block, int *ppt) {
    if (ragged_get_tuned(kind, mode, t, nsteps, S, total, block, ppt)) return true;
    if (kind == kRaggedForward) {
        *block = 256;
        *ppt = 2;
        return true;
    }
    *ppt = 1;
    const int cands[3] = {256, 128, 64};
    for (int i = 0; i < 3; ++i)
        if (ragged_adjoint_smem_for(t, nsteps, mode, cands[i])) {
            *block = cands[i];
            return true;
        }
    return false;
}

int check_ragged(int nc, int nsteps, int S, long long total, const long long *offsets, Tess *t) {
    int rc = make_tess(1, &nc, t);
    if (rc) return rc;
    if ((rc = check_steps(nsteps))) return rc;
    if (S < 0 || total < 0) return fail(CPAB_ERR_ARGUMENT, "need S >= 0 and total >= 0");
    // warp tiles are counted in 32-bit integers (at most 128 points per tile)
    if (total + (long long)S * 128 >= (1ll << 31))
        return fail(CPAB_ERR_UNSUPPORTED, "total + 128 * S must be below 2^31");
    if (S > 0 && !offsets) return fail(CPAB_ERR_ARGUMENT, "offsets is NULL");
    return CPAB_OK;
}

int check_ragged_ws(const Tess &t, int S, void *workspace, size_t workspace_bytes) {
    const size_t need = ragged_workspace_bytes(t, S);
    if (!workspace || workspace_bytes < need)
        return fail(CPAB_ERR_WORKSPACE, "workspace of %zu bytes needed (got %zu)", need,
                    workspace ? workspace_bytes : (size_t)0);
    return CPAB_OK;
}

int ragged_adjoint_run(const Tess &t, int nsteps, int mode, bool fused, int block, int ppt,
                       int S, const long long *offsets, long long total, RaggedBwd a,
                       const float *basis, int d, float *dtheta, float *sse, void *ws,
                       unsigned long long *ties, cudaStream_t s) {
    if (a.dvalues && total > 0) {
        cudaError_t e = cudaMemsetAsync(a.dvalues, 0, (size_t)total * sizeof(float), s);
        if (e != cudaSuccess) return cuda_fail(e, "memset");
    }
    cudaError_t e = launch_ragged_adjoint(t, nsteps, mode, fused, block, ppt, S, offsets, total,
                                          a, basis, d, d > 0 ? dtheta : nullptr, sse, ws, ties,
                                          device_error_word(), s);
    return e == cudaSuccess ? CPAB_OK : cuda_fail(e, "ragged adjoint launch");
}

}  // namespace

extern "C" {

size_t cpab_ragged1d_workspace(int nc, int nsteps, int S) {
    g_err[0] = 0;
    Tess t;
    if (make_tess(1, &nc, &t) || check_steps(nsteps)) return 0;
    if (S < 0) {
        fail(CPAB_ERR_ARGUMENT, "need S >= 0");
        return 0;
    }
    return ragged_workspace_bytes(t, S);
}

int cpab_ragged1d_forward(int nc, int nsteps, const float *E, int S, const long long *offsets,
                          long long total, const float *values, float *out, void *workspace,
                          size_t workspace_bytes, unsigned long long *ties, void *stream) {
    g_err[0] = 0;
    Tess t;
    int rc = check_ragged(nc, nsteps, S, total, offsets, &t);
    if (rc) return rc;
    if (S == 0 || total == 0) return CPAB_OK;
    if (!E || !values || !out) return fail(CPAB_ERR_ARGUMENT, "E, values or out is NULL");
    if ((rc = check_ragged_ws(t, S, workspace, workspace_bytes))) return rc;
    int block, ppt;
    ragged_shape(kRaggedForward, 0, t, nsteps, S, total, &block, &ppt);
    cudaError_t e = launch_ragged_forward(t, nsteps, block, ppt, S, offsets, total, E, values, out,
                                          workspace, ties, device_error_word(), as_stream(stream));
    return e == cudaSuccess ? CPAB_OK : cuda_fail(e, "ragged forward launch");
}

int cpab_ragged1d_backward(int nc, int nsteps, int mode, const float *A, const float *E, int S,
                           const long long *offsets, long long total, const float *basis, int d,
                           const float *values, const float *grad_out, float *dtheta,
                           float *dvalues, void *workspace, size_t workspace_bytes,
                           unsigned long long *ties, void *stream) {
    g_err[0] = 0;
    Tess t;
    int rc = check_ragged(nc, nsteps, S, total, offsets, &t);
    if (rc) return rc;
    if (!grad_mode_ok(mode))
        return fail(CPAB_ERR_ARGUMENT, "unknown gradient mode %d", mode);
    if (d < 0) return fail(CPAB_ERR_ARGUMENT, "negative d");
    if (S == 0) return CPAB_OK;
    if (!A || !E || (total > 0 && (!values || !grad_out)) || (d > 0 && (!basis || !dtheta)))
        return fail(CPAB_ERR_ARGUMENT, "A, E, values, grad_out, basis or dtheta is NULL");
    if ((rc = check_ragged_ws(t, S, workspace, workspace_bytes))) return rc;
    int block, ppt;
    if (!ragged_shape(kRaggedAdjoint, mode, t, nsteps, S, total, &block, &ppt))
        return fail(CPAB_ERR_UNSUPPORTED, "tessellation/nsteps too large for the adjoint kernel");
    RaggedBwd a = {};
    a.A = A;
    a.E = E;
    a.values = values;
    a.gout = grad_out;
    a.dvalues = dvalues;
    return ragged_adjoint_run(t, nsteps, mode, false, block, ppt, S, offsets, total, a, basis, d,
                              dtheta, nullptr, workspace, ties, as_stream(stream));
}

int cpab_ragged1d_mse(int nc, int nsteps, int mode, const float *A, const float *E, int S,
                      const long long *offsets, long long total, const float *basis, int d,
                      const float *values, const float *target, float loss_scale, float *out,
                      float *sse, float *dtheta, float *dvalues, void *workspace,
                      size_t workspace_bytes, unsigned long long *ties, void *stream) {
    g_err[0] = 0;
    Tess t;
    int rc = check_ragged(nc, nsteps, S, total, offsets, &t);
    if (rc) return rc;
    if (!grad_mode_ok(mode))
        return fail(CPAB_ERR_ARGUMENT, "unknown gradient mode %d", mode);
    if (d < 0) return fail(CPAB_ERR_ARGUMENT, "negative d");
    if (S == 0) return CPAB_OK;
    if (!A || !E || !sse || (total > 0 && (!values || !target)) || (d > 0 && (!basis || !dtheta)))
        return fail(CPAB_ERR_ARGUMENT, "A, E, values, target, sse, basis or dtheta is NULL");
    if ((rc = check_ragged_ws(t, S, workspace, workspace_bytes))) return rc;
    int block, ppt;
    if (!ragged_shape(kRaggedAdjoint, mode, t, nsteps, S, total, &block, &ppt))
        return fail(CPAB_ERR_UNSUPPORTED, "tessellation/nsteps too large for the adjoint kernel");
    RaggedBwd a = {};
    a.A = A;
    a.E = E;
    a.values = values;
    a.target = target;
    a.loss_scale = loss_scale;
    a.out = out;
    a.dvalues = dvalues;
    return ragged_adjoint_run(t, nsteps, mode, true, block, ppt, S, offsets, total, a, basis, d,
                              dtheta, sse, workspace, ties, as_stream(stream));
}

int cpab_ragged1d_tune(int kind, int nc, int nsteps, int mode, const float *A, const float *E,
                       int S, const long long *offsets, long long total, const float *basis,
                       int d, const float *values, const float *target, float loss_scale,
                       float *out, float *sse, float *dtheta, float *dvalues, void *workspace,
                       size_t workspace_bytes, const int *force, int *shape, float *best_ms,
                       void *stream) {
    g_err[0] = 0;
    Tess t;
    int rc = check_ragged(nc, nsteps, S, total, offsets, &t);
    if (rc) return rc;
    if (kind != kRaggedForward && kind != kRaggedAdjoint)
        return fail(CPAB_ERR_ARGUMENT, "kind must be 0 (forward) or 1 (adjoint)");
    if (!grad_mode_ok(mode))
        return fail(CPAB_ERR_ARGUMENT, "unknown gradient mode %d", mode);
    if (S == 0 || total == 0) return fail(CPAB_ERR_ARGUMENT, "nothing to tune (no points)");
    if (!E || !values || !out || (kind == kRaggedAdjoint &&
                                  (!A || !target || !sse || (d > 0 && (!basis || !dtheta)))))
        return fail(CPAB_ERR_ARGUMENT, "a required pointer is NULL");
    if ((rc = check_ragged_ws(t, S, workspace, workspace_bytes))) return rc;
    cudaStream_t s = as_stream(stream);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) == cudaSuccess && cap != cudaStreamCaptureStatusNone)
        return fail(CPAB_ERR_ARGUMENT, "cpab_ragged1d_tune times launches; call it outside capture");
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        return cuda_fail(cudaGetLastError(), "event create");
    RaggedBwd a = {};
    a.A = A;
    a.E = E;
    a.values = values;
    a.target = target;
    a.loss_scale = loss_scale;
    a.out = out;
    a.dvalues = dvalues;
    unsigned *err = device_error_word();
    auto run = [&](int block, int ppt) -> int {
        if (kind == kRaggedForward) {
            cudaError_t e = launch_ragged_forward(t, nsteps, block, ppt, S, offsets, total, E,
                                                  values, out, workspace, nullptr, err, s);
            return e == cudaSuccess ? CPAB_OK : cuda_fail(e, "ragged forward launch");
        }
        return ragged_adjoint_run(t, nsteps, mode, true, block, ppt, S, offsets, total, a, basis,
                                  d, dtheta, sse, workspace, nullptr, s);
    };
    const int blocks[3] = {64, 128, 256};
    const int ppts[3] = {1, 2, 4};
    const int n_ppt = 3;
    float best = 3.0e38f;
    int bb = 0, bp = 0;
    if (force) {   // one shape, validated, kept without timing
        bool ok_b = false, ok_p = false;
        for (int bi = 0; bi < 3; ++bi) ok_b |= force[0] == blocks[bi];
        for (int pi = 0; pi < n_ppt; ++pi) ok_p |= force[1] == ppts[pi];
        if (!ok_b || !ok_p ||
            (kind == kRaggedAdjoint && !ragged_adjoint_smem_for(t, nsteps, mode, force[0]))) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return fail(CPAB_ERR_ARGUMENT, "launch shape {%d, %d} is not one of the candidates "
                        "that fit", force[0], force[1]);
        }
        bb = force[0];
        bp = force[1];
        best = 0.f;
    }
    for (int bi = 0; bi < 3 && rc == CPAB_OK && !force; ++bi) {
        if (kind == kRaggedAdjoint && !ragged_adjoint_smem_for(t, nsteps, mode, blocks[bi]))
            continue;
        for (int pi = 0; pi < n_ppt && rc == CPAB_OK; ++pi) {
            if ((rc = run(blocks[bi], ppts[pi]))) break;   // warm-up
            float ms = 3.0e38f;
            for (int rep = 0; rep < 3 && rc == CPAB_OK; ++rep) {
                cudaEventRecord(e0, s);
                rc = run(blocks[bi], ppts[pi]);
                cudaEventRecord(e1, s);
                cudaError_t e = cudaEventSynchronize(e1);
                if (e != cudaSuccess) rc = cuda_fail(e, "tuning run");
                float m = 0.f;
                cudaEventElapsedTime(&m, e0, e1);
                if (m < ms) ms = m;
            }
            if (rc == CPAB_OK && ms < best) {
                best = ms;
                bb = blocks[bi];
                bp = ppts[pi];
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if (!bb) return fail(CPAB_ERR_UNSUPPORTED, "no launch shape fits this tessellation");
    ragged_set_tuned(kind, mode, t, nsteps, S, total, bb, bp);
    if (shape) {
        shape[0] = bb;
        shape[1] = bp;
    }
    if (best_ms) *best_ms = best;
    return run(bb, bp);   // leave the outputs of the chosen shape
}

// ---------------------------- ragged point sets ------------------------------
size_t cpab_ragged_points_workspace(int ndim, const int *nc, int S) {
    g_err[0] = 0;
    Tess t;
    if (make_tess(ndim, nc, &t)) return 0;
    if (S < 0) {
        fail(CPAB_ERR_ARGUMENT, "need S >= 0");
        return 0;
    }
    return ragged_points_workspace_bytes(t, S);
}

static int check_ragged_points(int ndim, const int *nc, int nsteps, int S, long long total,
                               const long long *offsets, void *workspace,
                               size_t workspace_bytes, Tess *t) {
    int rc = make_tess(ndim, nc, t);
    if (rc) return rc;
    if ((rc = check_steps(nsteps))) return rc;
    if (S < 0 || total < 0) return fail(CPAB_ERR_ARGUMENT, "need S >= 0 and total >= 0");
    if (total + (long long)S * 128 >= (1ll << 31))
        return fail(CPAB_ERR_UNSUPPORTED, "total + 128 * S must be below 2^31");
    if (S == 0) return CPAB_OK;
    if (!offsets) return fail(CPAB_ERR_ARGUMENT, "offsets is NULL");
    const size_t need = ragged_points_workspace_bytes(*t, S);
    if (!workspace || workspace_bytes < need)
        return fail(CPAB_ERR_WORKSPACE, "workspace of %zu bytes needed (got %zu)", need,
                    workspace ? workspace_bytes : (size_t)0);
    return CPAB_OK;
}

static int points_forward_impl(int ndim, const int *nc, int nsteps, const float *E, int S,
                               const long long *offsets, long long total, const float *points,
                               float *out, void *workspace, size_t workspace_bytes,
                               unsigned long long *ties, void *stream, const LaunchShape *force) {
    g_err[0] = 0;
    Tess t;
    int rc = check_ragged_points(ndim, nc, nsteps, S, total, offsets, workspace,
                                 workspace_bytes, &t);
    if (rc) return rc;
    if (S == 0 || total == 0) return CPAB_OK;
    if (!E || !points || !out) return fail(CPAB_ERR_ARGUMENT, "E, points or out is NULL");
    cudaError_t e = launch_ragged_points_forward(t, nsteps, S, offsets, total, E, points, out,
                                                 workspace, ties, device_error_word(),
                                                 as_stream(stream), force);
    return e == cudaSuccess ? CPAB_OK : cuda_fail(e, "ragged points forward launch");
}

static int points_backward_impl(int ndim, const int *nc, int nsteps, int mode, const float *A,
                                const float *E, int S, const long long *offsets,
                                long long total, const float *basis, int d,
                                const float *points, const float *grad_out, float *dtheta,
                                float *dpoints, void *workspace, size_t workspace_bytes,
                                unsigned long long *ties, void *stream,
                                const LaunchShape *force) {
    g_err[0] = 0;
    Tess t;
    int rc = check_ragged_points(ndim, nc, nsteps, S, total, offsets, workspace,
                                 workspace_bytes, &t);
    if (rc) return rc;
    if (!grad_mode_ok(mode))
        return fail(CPAB_ERR_ARGUMENT, "unknown gradient mode %d", mode);
    if (d < 0) return fail(CPAB_ERR_ARGUMENT, "negative d");
    if (S == 0) return CPAB_OK;
    if (!A || (mode == CPAB_GRAD_EXACT && !E) || (total > 0 && (!points || !grad_out)) ||
        (d > 0 && (!basis || !dtheta)))
        return fail(CPAB_ERR_ARGUMENT, "A, E, points, grad_out, basis or dtheta is NULL");
    cudaStream_t s = as_stream(stream);
    if (dpoints && total > 0) {
        cudaError_t e = cudaMemsetAsync(dpoints, 0, (size_t)total * ndim * sizeof(float), s);
        if (e != cudaSuccess) return cuda_fail(e, "memset");
    }
    cudaError_t e = launch_ragged_points_backward(t, nsteps, mode, S, offsets, total, A, E,
                                                  points, grad_out, dpoints, basis, d,
                                                  d > 0 ? dtheta : nullptr, workspace, ties,
                                                  device_error_word(), s, force);
    if (e == cudaErrorInvalidConfiguration)
        return fail(CPAB_ERR_UNSUPPORTED, "tessellation/nsteps too large for the adjoint kernel");
    return e == cudaSuccess ? CPAB_OK : cuda_fail(e, "ragged points adjoint launch");
}

int cpab_ragged_points_forward(int ndim, const int *nc, int nsteps, const float *E, int S,
                               const long long *offsets, long long total, const float *points,
                               float *out, void *workspace, size_t workspace_bytes,
                               unsigned long long *ties, void *stream) {
    return points_forward_impl(ndim, nc, nsteps, E, S, offsets, total, points, out, workspace,
                               workspace_bytes, ties, stream, nullptr);
}

int cpab_ragged_points_backward(int ndim, const int *nc, int nsteps, int mode, const float *A,
                                const float *E, int S, const long long *offsets,
                                long long total, const float *basis, int d,
                                const float *points, const float *grad_out, float *dtheta,
                                float *dpoints, void *workspace, size_t workspace_bytes,
                                unsigned long long *ties, void *stream) {
    return points_backward_impl(ndim, nc, nsteps, mode, A, E, S, offsets, total, basis, d, points,
                                grad_out, dtheta, dpoints, workspace, workspace_bytes, ties,
                                stream, nullptr);
}

}  // extern "C"

// --------------------------------------------------------------------------
// cpab_backward without a caller-provided workspace.
//
// Some callers cannot allocate device memory at the point where they need a
// gradient: a host runtime that owns all device memory through its own pool
// and hands out only the tensors of the computation, or code running where
// allocation is not permitted.  They cannot call cudaMalloc (or have torch do
// it) to obtain the scratch that cpab_backward needs.  This variant keeps
// that scratch -- the per-CTA partial cell gradients -- in a fixed array in
// the library's device memory instead.
//
// * The array holds kNoAllocScratchFloats floats (8 MiB).  Every GPU that
//   loads this library reserves it until the process exits.
// * A problem needs n_theta * nC * ndim * (ndim + 1) floats per CTA slice;
//   the variant uses as many CTAs per theta as fit (at most as many as
//   cpab_backward would) and rejects problems where a single slice per theta
//   does not fit.
// * The array's device address is looked up with cudaGetSymbolAddress on the
//   first call on each device (with that device current).  Make that first
//   call before capturing the stream into a CUDA graph.
// * The adjoint kernel writes every scratch element it later reads, so no
//   clearing is needed, and the array keeps the last call's values.  All
//   calls share the one array: calls that can overlap on the GPU (different
//   streams, or other host threads) race and must be serialised by the
//   caller.
// * Nothing here calls cudaMalloc, cudaFree or an allocating library routine.
// --------------------------------------------------------------------------
namespace {

constexpr size_t kNoAllocScratchFloats = size_t(1) << 21;
__device__ __align__(256) float g_noalloc_scratch[kNoAllocScratchFloats];
std::atomic<float *> g_noalloc_ptr[kMaxDevices];

float *noalloc_scratch(int *rc) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *rc = cuda_fail(e, "cudaGetDevice");
        return nullptr;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        *rc = fail(CPAB_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
        return nullptr;
    }
    float *ptr = g_noalloc_ptr[dev].load(std::memory_order_relaxed);
    if (!ptr) {
        e = cudaGetSymbolAddress((void **)&ptr, g_noalloc_scratch);
        if (e != cudaSuccess) {
            cudaGetLastError();   // the failure is reported here, not by the next launch
            *rc = cuda_fail(e, "cudaGetSymbolAddress of the no-alloc scratch");
            return nullptr;
        }
        if (!ptr) {
            *rc = fail(CPAB_ERR_CUDA, "cudaGetSymbolAddress of the no-alloc scratch gave no "
                                      "address");
            return nullptr;
        }
        g_noalloc_ptr[dev].store(ptr, std::memory_order_relaxed);
    }
    *rc = CPAB_OK;
    return ptr;
}

}  // namespace

extern "C" {

int cpab_backward_noalloc(int ndim, const int *nc, int nsteps, int mode, const float *points,
                          int broadcast, long long nP, const float *A, const float *E,
                          int n_theta, const float *basis, int d, const float *grad_out,
                          float *dtheta, float *dpoints, unsigned long long *ties,
                          void *stream) {
    g_err[0] = 0;
    Tess t;
    int rc = make_tess(ndim, nc, &t);
    if (rc) return rc;
    if ((rc = check_steps(nsteps))) return rc;
    if (!grad_mode_ok(mode))
        return fail(CPAB_ERR_ARGUMENT, "unknown gradient mode %d", mode);
    if (nP < 0 || n_theta < 0 || d < 0) return fail(CPAB_ERR_ARGUMENT, "invalid sizes");
    if ((rc = check_theta_count(n_theta))) return rc;
    if (n_theta == 0 || (d == 0 && !dpoints)) return CPAB_OK;
    if (!A || (d > 0 && (!dtheta || !basis)))
        return fail(CPAB_ERR_ARGUMENT, "dtheta, basis or A is NULL");
    if (mode == CPAB_GRAD_EXACT && !E) return fail(CPAB_ERR_ARGUMENT, "exact mode needs E");
    cudaStream_t s = as_stream(stream);
    if (nP == 0) {
        if (d == 0) return CPAB_OK;
        cudaError_t e = cudaMemsetAsync(dtheta, 0, (size_t)n_theta * d * sizeof(float), s);
        return e == cudaSuccess ? CPAB_OK : cuda_fail(e, "memset");
    }
    if (!points || !grad_out) return fail(CPAB_ERR_ARGUMENT, "points or grad_out is NULL");
    const size_t slice = (size_t)n_theta * t.nC * ndim * (ndim + 1);
    if (slice > kNoAllocScratchFloats)
        return fail(CPAB_ERR_WORKSPACE,
                    "no-alloc scratch holds %zu floats; this problem needs at least %zu "
                    "(n_theta * nC * ndim * (ndim+1)); use cpab_backward with a workspace",
                    kNoAllocScratchFloats, slice);
    AdjointPlan plan;   // per-warp tables in shared memory: the scratch holds the partials only
    if (!plan_adjoint(t, nsteps, nP, n_theta, &plan, false))
        return fail(CPAB_ERR_UNSUPPORTED, "tessellation/nsteps too large for the adjoint kernel");
    const long long fit = (long long)(kNoAllocScratchFloats / slice);
    if (plan.parts > fit) plan.parts = (int)fit;
    plan.partial_floats = slice * plan.parts;
    float *partials = noalloc_scratch(&rc);
    if (!partials) return rc;
    unsigned *err = device_error_word();
    cudaError_t e = launch_adjoint(t, nsteps, mode, plan, points, broadcast ? 1 : 0, nP,
                                   mode == CPAB_GRAD_EXACT ? E : A, n_theta, grad_out, dpoints,
                                   partials, ties, err, s);
    if (e != cudaSuccess) return cuda_fail(e, "adjoint launch");
    if (d == 0) return CPAB_OK;
    e = launch_finalize(t, nsteps, mode, partials, plan.parts, A, basis, d, n_theta, dtheta, s);
    return e == cudaSuccess ? CPAB_OK : cuda_fail(e, "finalize launch");
}

}  // extern "C"

// -------------------------------- autotuner ----------------------------------
// Each tuner times the launch shapes of one kernel family on the caller's own
// arguments (one warm-up launch, then the best of three timed with CUDA events
// on the caller's stream), keeps the fastest for later calls on the same
// problem (device, tessellation, nsteps, mode, sizes) and finishes with a run
// of the chosen shape, so its outputs are those of a plain call.  A shape
// changes only how work is spread over threads and CTAs: every point follows
// the same arithmetic, so outputs per point are identical and sums over
// points (dtheta, d(data)) change only in their float summation order.
namespace {

constexpr int kSkip = -1000;   // the candidate does not apply to this problem

int refuse_capture(cudaStream_t s, const char *who) {
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) {
        cudaGetLastError();
        return fail(CPAB_ERR_CUDA, "%s: cannot query the stream's capture state", who);
    }
    if (cap != cudaStreamCaptureStatusNone)
        return fail(CPAB_ERR_ARGUMENT, "%s times launches; call it outside stream capture", who);
    return CPAB_OK;
}

// Device scratch of one tuning call (freed on return).
struct Scratch {
    void *p = nullptr;
    size_t bytes = 0;
    ~Scratch() {
        if (p) cudaFree(p);
    }
    int reserve(size_t b) {
        if (b <= bytes) return CPAB_OK;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&p, b);
        if (e != cudaSuccess) return cuda_fail(e, "tuning workspace");
        bytes = b;
        return CPAB_OK;
    }
};

void put_shape(const LaunchShape &sh, int *shape) {
    if (!shape) return;
    shape[0] = sh.block;
    shape[1] = sh.ppt;
    shape[2] = sh.parts;
    shape[3] = sh.staging;
}

LaunchShape get_shape(const int *v) {
    LaunchShape sh;
    sh.block = v[0];
    sh.ppt = v[1];
    sh.parts = v[2];
    sh.staging = v[3];
    return sh;
}

// Forward kernels: 32..256 threads (multiple of 32), ppt in {1, 2} (or
// {1, 2, 4} for the ragged point sets).
int check_forward_shape(const LaunchShape &sh, int max_ppt) {
    const bool ppt_ok = sh.ppt == 1 || sh.ppt == 2 || (max_ppt >= 4 && sh.ppt == 4);
    if (sh.block < 32 || sh.block > 256 || sh.block % 32 || !ppt_ok)
        return fail(CPAB_ERR_ARGUMENT, "launch shape {%d, %d}: threads must be a multiple of 32 in "
                    "[32, 256] and points per thread 1, 2%s", sh.block, sh.ppt,
                    max_ppt >= 4 ? " or 4" : "");
    return CPAB_OK;
}

// Adjoint kernels: 64, 128 or 256 threads; parts >= 1; staging 0 (shared) or
// 1 (global, 2D/3D only).
int check_adjoint_shape(const LaunchShape &sh, int ndim) {
    if ((sh.block != 64 && sh.block != 128 && sh.block != 256) || sh.parts < 1 ||
        sh.staging < 0 || sh.staging > 1 || (ndim == 1 && sh.staging == 1))
        return fail(CPAB_ERR_ARGUMENT, "launch shape {%d, parts %d, staging %d}: threads 64, 128 "
                    "or 256, parts >= 1, staging 0 or 1 (1 only in 2D/3D)", sh.block, sh.parts,
                    sh.staging);
    return CPAB_OK;
}

std::vector<LaunchShape> forward_candidates(int max_ppt) {
    std::vector<LaunchShape> c;
    for (int b : {64, 128, 256})
        for (int p = 1; p <= max_ppt; p *= 2) {
            LaunchShape sh;
            sh.block = b;
            sh.ppt = p;
            c.push_back(sh);
        }
    return c;
}

// Adjoint candidates: every (threads, staging) that the planner accepts, each
// with the planner's CTA count per theta/image and with half and twice that.
// plan(shape, &plan) resolves a shape with parts = 0 to the planner's.
template <typename P>
std::vector<LaunchShape> adjoint_candidates(int ndim, P plan, size_t *ws_max) {
    std::vector<LaunchShape> c;
    *ws_max = 0;
    for (int g = 0; g < (ndim >= 2 ? 2 : 1); ++g)
        for (int b : {64, 128, 256}) {
            LaunchShape sh;
            sh.block = b;
            sh.staging = g;
            AdjointPlan pl;
            if (!plan(sh, &pl) || pl.block != b || (pl.gw_floats != 0) != (g == 1)) continue;
            const int base = pl.parts;
            for (int m = 0; m < 3; ++m) {
                const int parts = m == 0 ? base : m == 1 ? (base + 1) / 2 : base * 2;
                if (m > 0 && (parts == base || parts > pl.tiles)) continue;
                LaunchShape v = sh;
                v.parts = parts;
                AdjointPlan pv;
                if (!plan(v, &pv)) continue;
                v.parts = pv.parts;
                bool dup = false;
                for (const LaunchShape &o : c)
                    dup |= o.block == v.block && o.staging == v.staging && o.parts == v.parts;
                if (dup) continue;
                c.push_back(v);
                *ws_max = std::max(*ws_max, pv.ws_floats() * sizeof(float));
            }
        }
    return c;
}

// Times run(shape) over the candidates; *best and *best_ms receive the
// fastest.  run returns CPAB_OK, kSkip or an error code (which ends tuning).
template <typename F>
int time_candidates(const std::vector<LaunchShape> &cands, cudaStream_t s, F run,
                    LaunchShape *best, float *best_ms) {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        cudaError_t e = cudaGetLastError();
        if (e0) cudaEventDestroy(e0);
        return cuda_fail(e, "event create");
    }
    int rc = CPAB_OK;
    float bt = 3.0e38f;
    bool found = false;
    for (const LaunchShape &c : cands) {
        rc = run(c);   // warm-up
        if (rc == kSkip) {
            rc = CPAB_OK;
            continue;
        }
        if (rc) break;
        float ms = 3.0e38f;
        for (int rep = 0; rep < 3 && rc == CPAB_OK; ++rep) {
            cudaEventRecord(e0, s);
            rc = run(c);
            cudaEventRecord(e1, s);
            cudaError_t e = cudaEventSynchronize(e1);
            if (e != cudaSuccess) rc = cuda_fail(e, "tuning run");
            float m = 0.f;
            if (rc == CPAB_OK && cudaEventElapsedTime(&m, e0, e1) == cudaSuccess && m < ms) ms = m;
        }
        if (rc) break;
        if (ms < bt) {
            bt = ms;
            *best = c;
            found = true;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if (!found) return fail(CPAB_ERR_UNSUPPORTED, "no launch shape fits this problem");
    if (best_ms) *best_ms = bt;
    return CPAB_OK;
}

// Tune (or, with force, pin) one kernel family: candidates are timed unless
// force names the one shape to keep; the kept shape is stored under (kind,
// key) and run once more to leave its outputs.
template <typename F>
int tune_family(int kind, const TuneKey &key, std::vector<LaunchShape> cands,
                const LaunchShape *force, cudaStream_t s, F run, int *shape, float *best_ms) {
    LaunchShape best;
    int rc;
    if (force) {
        best = *force;
        if (best_ms) *best_ms = 0.f;
    } else if ((rc = time_candidates(cands, s, run, &best, best_ms))) {
        return rc;
    }
    rc = run(best);
    if (rc == kSkip) return fail(CPAB_ERR_UNSUPPORTED, "the launch shape does not fit this problem");
    if (rc) return rc;
    // the run reads the tuner's own workspace, freed when the caller returns
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "tuning run");
    tuned_set(kind, key, best);
    put_shape(best, shape);
    return CPAB_OK;
}

}  // namespace

extern "C" {

int cpab_integrate_tune(int ndim, const int *nc, int nsteps, const float *points, int broadcast,
                        long long nP, const float *E, int n_theta, float *out, const int *force,
                        int *shape, float *best_ms, void *stream) {
    g_err[0] = 0;
    Tess t;
    int rc = make_tess(ndim, nc, &t);
    if (rc) return rc;
    if ((rc = check_steps(nsteps))) return rc;
    if (nP <= 0 || n_theta <= 0) return fail(CPAB_ERR_ARGUMENT, "nothing to tune (no points)");
    if ((rc = check_theta_count(n_theta))) return rc;
    if (!points || !E || !out) return fail(CPAB_ERR_ARGUMENT, "points, E or out is NULL");
    cudaStream_t s = as_stream(stream);
    if ((rc = refuse_capture(s, "cpab_integrate_tune"))) return rc;
    LaunchShape fs;
    if (force && (rc = check_forward_shape(fs = get_shape(force), 2))) return rc;
    auto run = [&](const LaunchShape &sh) {
        return integrate_common(ndim, nc, nsteps, points, broadcast, nP, E, true, n_theta, out,
                                nullptr, nullptr, stream, &sh);
    };
    return tune_family(kTuneIntegrate, tune_key(t, nsteps, 1, nP, n_theta, broadcast ? 1 : 0),
                       forward_candidates(2), force ? &fs : nullptr, s, run, shape, best_ms);
}

int cpab_backward_tune(int ndim, const int *nc, int nsteps, int mode, const float *points,
                       int broadcast, long long nP, const float *A, const float *E, int n_theta,
                       const float *basis, int d, const float *grad_out, float *dtheta,
                       float *dpoints, const int *force, int *shape, float *best_ms,
                       void *stream) {
    g_err[0] = 0;
    Tess t;
    int rc = make_tess(ndim, nc, &t);
    if (rc) return rc;
    if ((rc = check_steps(nsteps))) return rc;
    if (!grad_mode_ok(mode)) return fail(CPAB_ERR_ARGUMENT, "unknown gradient mode %d", mode);
    if (nP <= 0 || n_theta <= 0 || d < 0 || (d == 0 && !dpoints))
        return fail(CPAB_ERR_ARGUMENT, "nothing to tune (no points or no outputs)");
    if ((rc = check_theta_count(n_theta))) return rc;
    cudaStream_t s = as_stream(stream);
    if ((rc = refuse_capture(s, "cpab_backward_tune"))) return rc;
    LaunchShape fs;
    if (force && (rc = check_adjoint_shape(fs = get_shape(force), ndim))) return rc;
    auto plan = [&](const LaunchShape &sh, AdjointPlan *pl) {
        return plan_adjoint(t, nsteps, nP, n_theta, pl, true, &sh);
    };
    size_t ws_max = 0;
    std::vector<LaunchShape> cands = adjoint_candidates(ndim, plan, &ws_max);
    if (force) {
        AdjointPlan pl;
        if (!plan(fs, &pl))
            return fail(CPAB_ERR_UNSUPPORTED, "the launch shape does not fit this problem");
        ws_max = pl.ws_floats() * sizeof(float);
    }
    Scratch ws;
    if ((rc = ws.reserve(ws_max))) return rc;
    auto run = [&](const LaunchShape &sh) {
        return backward_impl(ndim, nc, nsteps, mode, points, broadcast, nP, A, E, n_theta, basis,
                             d, grad_out, dtheta, dpoints, ws.p, ws.bytes, nullptr, stream, &sh);
    };
    return tune_family(kTuneAdjoint, tune_key(t, nsteps, 0, nP, n_theta, 0), cands,
                       force ? &fs : nullptr, s, run, shape, best_ms);
}

int cpab_transform_data_tune(int ndim, const int *nc, int nsteps, const float *lin,
                             const int *outsize, const float *E, int nb, const float *data, int C,
                             const int *size, float *out, float *grid_out, const int *force,
                             int *shape, float *best_ms, void *stream) {
    g_err[0] = 0;
    Tess t;
    int rc = make_tess(ndim, nc, &t);
    if (rc) return rc;
    if ((rc = check_steps(nsteps))) return rc;
    if ((rc = check_geo(ndim, size, outsize, nb))) return rc;
    if (nb <= 0 || C < 1) return fail(CPAB_ERR_ARGUMENT, "nothing to tune (nb < 1 or C < 1)");
    cudaStream_t s = as_stream(stream);
    if ((rc = refuse_capture(s, "cpab_transform_data_tune"))) return rc;
    LaunchShape fs;
    if (force && (rc = check_forward_shape(fs = get_shape(force), 2))) return rc;
    long long nP = 1;
    for (int j = 0; j < ndim; ++j) nP *= outsize[j];
    auto run = [&](const LaunchShape &sh) {
        return td_forward(ndim, nc, nsteps, lin, outsize, E, nb, data, C, size, out, grid_out,
                          nullptr, stream, &sh);
    };
    return tune_family(kTuneFusedForward, tune_key(t, nsteps, 0, nP, nb, C),
                       forward_candidates(2), force ? &fs : nullptr, s, run, shape, best_ms);
}

int cpab_transform_data_backward_tune(int ndim, const int *nc, int nsteps, int mode,
                                      const float *lin, const int *outsize, const float *A,
                                      const float *E, const float *grid_saved, int nb,
                                      const float *data, int C, const int *size,
                                      const float *basis, int d, const float *grad_out,
                                      float *ddata, float *dtheta, const int *force, int *shape,
                                      float *best_ms, void *stream) {
    g_err[0] = 0;
    Tess t;
    int rc = make_tess(ndim, nc, &t);
    if (rc) return rc;
    if ((rc = check_steps(nsteps))) return rc;
    if ((rc = check_geo(ndim, size, outsize, nb))) return rc;
    if (!grad_mode_ok(mode)) return fail(CPAB_ERR_ARGUMENT, "unknown gradient mode %d", mode);
    if (nb <= 0 || C < 1 || d < 0) return fail(CPAB_ERR_ARGUMENT, "nothing to tune (nb < 1)");
    cudaStream_t s = as_stream(stream);
    if ((rc = refuse_capture(s, "cpab_transform_data_backward_tune"))) return rc;
    LaunchShape fs;
    if (force && (rc = check_adjoint_shape(fs = get_shape(force), ndim))) return rc;
    long long nP = 1;
    for (int j = 0; j < ndim; ++j) nP *= outsize[j];
    auto plan = [&](const LaunchShape &sh, AdjointPlan *pl) {
        return plan_transform_data_backward(t, nsteps, mode, nP, nb, pl, &sh);
    };
    size_t ws_max = 0;
    std::vector<LaunchShape> cands = adjoint_candidates(ndim, plan, &ws_max);
    if (force) {
        AdjointPlan pl;
        if (!plan(fs, &pl))
            return fail(CPAB_ERR_UNSUPPORTED, "the launch shape does not fit this problem");
        ws_max = pl.ws_floats() * sizeof(float);
    }
    Scratch ws;
    if ((rc = ws.reserve(ws_max))) return rc;
    auto run = [&](const LaunchShape &sh) {
        return td_backward(ndim, nc, nsteps, mode, lin, outsize, A, E, grid_saved, nb, data, C,
                           size, basis, d, grad_out, ddata, dtheta, ws.p, ws.bytes, nullptr,
                           stream, nullptr, &sh);
    };
    return tune_family(kTuneFusedBackward, tune_key(t, nsteps, mode, nP, nb, 0), cands,
                       force ? &fs : nullptr, s, run, shape, best_ms);
}

int cpab_ragged_points_tune(int kind, int ndim, const int *nc, int nsteps, int mode,
                            const float *A, const float *E, int S, const long long *offsets,
                            long long total, const float *basis, int d, const float *points,
                            const float *grad_out, float *out, float *dtheta, float *dpoints,
                            const int *force, int *shape, float *best_ms, void *stream) {
    g_err[0] = 0;
    Tess t;
    int rc = make_tess(ndim, nc, &t);
    if (rc) return rc;
    if (kind != 0 && kind != 1)
        return fail(CPAB_ERR_ARGUMENT, "kind must be 0 (forward) or 1 (backward)");
    if (!grad_mode_ok(mode)) return fail(CPAB_ERR_ARGUMENT, "unknown gradient mode %d", mode);
    if (S <= 0 || total <= 0) return fail(CPAB_ERR_ARGUMENT, "nothing to tune (no points)");
    cudaStream_t s = as_stream(stream);
    if ((rc = refuse_capture(s, "cpab_ragged_points_tune"))) return rc;
    LaunchShape fs;
    if (force) {
        fs = get_shape(force);
        if (kind == 0 && (rc = check_forward_shape(fs, 4))) return rc;
        if (kind == 1 && fs.block != 64 && fs.block != 128 && fs.block != 256)
            return fail(CPAB_ERR_ARGUMENT, "backward launch shape: threads 64, 128 or 256");
    }
    Scratch ws;
    if ((rc = ws.reserve(ragged_points_workspace_bytes(t, S)))) return rc;
    if (kind == 0) {
        auto run = [&](const LaunchShape &sh) {
            return points_forward_impl(ndim, nc, nsteps, E, S, offsets, total, points, out, ws.p,
                                       ws.bytes, nullptr, stream, &sh);
        };
        return tune_family(kTunePointsForward, tune_key(t, nsteps, 0, S, total, 0),
                           forward_candidates(4), force ? &fs : nullptr, s, run, shape, best_ms);
    }
    std::vector<LaunchShape> cands;
    for (int b : {64, 128, 256}) {
        LaunchShape sh;
        sh.block = b;
        cands.push_back(sh);
    }
    auto run = [&](const LaunchShape &sh) {
        int r = points_backward_impl(ndim, nc, nsteps, mode, A, E, S, offsets, total, basis, d,
                                     points, grad_out, dtheta, dpoints, ws.p, ws.bytes, nullptr,
                                     stream, &sh);
        // a block whose shared memory does not fit is skipped (the launcher
        // reports it as an unsupported configuration before any launch)
        return r == CPAB_ERR_UNSUPPORTED ? kSkip : r;
    };
    return tune_family(kTunePointsBackward, tune_key(t, nsteps, mode, S, total, 0), cands,
                       force ? &fs : nullptr, s, run, shape, best_ms);
}

void cpab_tune_reset(void) { tuned_clear(); }

}  // extern "C"
