// Host harness for the reference-mode trajectory of the adjoint kernels
// (libcpab_gb300/csrc/cpab_midpoint.cuh; compiled by tests/test_midpoint_host.py
// with nvcc and -ffp-contract=off; runs on the CPU).
//
// usage: midpoint_check ops  <in.bin> <out.bin>
//   in:  float hi, float lo, int64 n, float p[n], float v[n]
//   out: float add_mul_f64(p, v, hi, lo)[n]
// usage: midpoint_check traj <in.bin> <out.bin>
//   in:  int32 ndim, int32 nc[3], int32 nsteps, int64 nP, float A[nC][ndim][ndim+1],
//        float points[ndim][nP]
//   out: float end[ndim][nP], int32 cells[nP][nsteps]
// The trajectory steps with ref_mid_step and looks cells up with the FP64
// replica of the reference's lookup (the kernels' FP32 tiers answer the same,
// tests/test_lookup_host.py).
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../libcpab_gb300/csrc/cpab_common.cuh"
#include "../libcpab_gb300/csrc/cpab_midpoint.cuh"

template <int N>
static void run_traj(const cpab::Tess &t, int nsteps, int64_t nP, const std::vector<float> &A,
                     const std::vector<float> &pts, std::vector<float> &end,
                     std::vector<int32_t> &cells) {
    const cpab::Steps st = cpab::make_steps(nsteps);
    constexpr int P = N * (N + 1);
    for (int64_t i = 0; i < nP; ++i) {
        float p[N];
        for (int r = 0; r < N; ++r) p[r] = pts[r * nP + i];
        for (int s = 0; s < nsteps; ++s) {
            int c;
            if (N == 1) c = cpab::cell_1d(p[0], t);
            else if (N == 2) c = cpab::cell_2d_exact(p[0], p[N > 1 ? 1 : 0], t);
            else c = cpab::cell_3d_exact(p[0], p[N > 1 ? 1 : 0], p[N > 2 ? 2 : 0], t);
            cells[i * nsteps + s] = c;
            float M[P];
            for (int k = 0; k < P; ++k) M[k] = A[(size_t)c * P + k];
            cpab::ref_mid_step<N>(M, st, p);
        }
        for (int r = 0; r < N; ++r) end[r * nP + i] = p[r];
    }
}

int main(int argc, char **argv) {
    if (argc != 4) return 2;
    FILE *f = fopen(argv[2], "rb");
    if (!f) return 3;
    if (!strcmp(argv[1], "ops")) {
        float hl[2];
        int64_t n = 0;
        if (fread(hl, 4, 2, f) != 2 || fread(&n, 8, 1, f) != 1) return 4;
        std::vector<float> p(n), v(n), r(n);
        if (fread(p.data(), 4, n, f) != (size_t)n || fread(v.data(), 4, n, f) != (size_t)n)
            return 5;
        fclose(f);
        for (int64_t i = 0; i < n; ++i) r[i] = cpab::add_mul_f64(p[i], v[i], hl[0], hl[1]);
        FILE *o = fopen(argv[3], "wb");
        if (!o) return 6;
        fwrite(r.data(), 4, n, o);
        fclose(o);
        return 0;
    }
    int32_t hdr[5];
    int64_t nP = 0;
    if (fread(hdr, 4, 5, f) != 5 || fread(&nP, 8, 1, f) != 1) return 4;
    const int ndim = hdr[0], nsteps = hdr[4];
    cpab::Tess t;
    cpab::tess_init(ndim, hdr + 1, &t);
    std::vector<float> A((size_t)t.nC * ndim * (ndim + 1)), pts((size_t)ndim * nP);
    if (fread(A.data(), 4, A.size(), f) != A.size() ||
        fread(pts.data(), 4, pts.size(), f) != pts.size())
        return 5;
    fclose(f);
    std::vector<float> end((size_t)ndim * nP);
    std::vector<int32_t> cells((size_t)nP * nsteps);
    if (ndim == 1) run_traj<1>(t, nsteps, nP, A, pts, end, cells);
    else if (ndim == 2) run_traj<2>(t, nsteps, nP, A, pts, end, cells);
    else run_traj<3>(t, nsteps, nP, A, pts, end, cells);
    FILE *o = fopen(argv[3], "wb");
    if (!o) return 6;
    fwrite(end.data(), 4, end.size(), o);
    fwrite(cells.data(), 4, cells.size(), o);
    fclose(o);
    return 0;
}
