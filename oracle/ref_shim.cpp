// C-linkage wrappers around the reference's own CPU ops (TEST INFRASTRUCTURE).
//
// oracle/build.py compiles this file together with the reference's
// libcpab/core/cpab_ops.cpp, taken from where it lies in the read-only
// reference checkout, into oracle/_ref/libcpab_ref.so.  The wrappers only
// forward arguments; every number they return is computed by the reference.
// The library exists only where the reference checkout exists.
#include "cpab_ops.h"

extern "C" {
int ref_findcellidx(int ndim, const float* p, const int* nc) {
    return findcellidx(ndim, p, nc);
}
void ref_forward(float* newpoints, const float* points, const float* trels,
                 const int* nstepsolver, const int* nc, int ndim, int nP,
                 int batch_size, int broadcast) {
    cpab_forward_op(newpoints, points, trels, nstepsolver, nc, ndim, nP, batch_size,
                    broadcast);
}
void ref_backward(float* grad, const float* points, const float* As, const float* Bs,
                  const int* nstepsolver, const int* nc, int n_theta, int d, int ndim,
                  int nP, int nC, int broadcast) {
    cpab_backward_op(grad, points, As, Bs, nstepsolver, nc, n_theta, d, ndim, nP, nC,
                     broadcast);
}
}
