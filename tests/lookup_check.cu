// Host harness for the cell lookup of libcpab_gb300/csrc/cpab_common.cuh
// (compiled by tests/test_lookup_host.py with nvcc; runs on the CPU).
//
// usage: lookup_check <in.bin> <out.bin>
//   in:  int32 ndim, int32 nc[3], int64 n, float32 points[ndim][n]
//   out: int32 fast[n] (-1 where the FP32 tiers defer), int32 exact[n]
#include <cstdio>
#include <cstdint>
#include <vector>

#include "../libcpab_gb300/csrc/cpab_common.cuh"

int main(int argc, char **argv) {
    if (argc != 3) return 2;
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 3;
    int32_t hdr[4];
    int64_t n = 0;
    if (fread(hdr, 4, 4, f) != 4 || fread(&n, 8, 1, f) != 1) return 4;
    const int ndim = hdr[0];
    std::vector<float> p((size_t)ndim * n);
    if (fread(p.data(), 4, p.size(), f) != p.size()) return 5;
    fclose(f);
    cpab::Tess t;
    cpab::tess_init(ndim, hdr + 1, &t);
    std::vector<int32_t> fast(n), exact(n);
    for (int64_t i = 0; i < n; ++i) {
        const float x = p[i], y = ndim > 1 ? p[n + i] : 0.f, z = ndim > 2 ? p[2 * n + i] : 0.f;
        if (ndim == 1) {
            fast[i] = exact[i] = cpab::cell_1d(x, t);
        } else if (ndim == 2) {
            fast[i] = cpab::cell_2d_fp32(x, y, t);
            exact[i] = cpab::cell_2d_exact(x, y, t);
        } else {
            fast[i] = cpab::cell_3d_fp32(x, y, z, t);
            exact[i] = cpab::cell_3d_exact(x, y, z, t);
        }
    }
    FILE *o = fopen(argv[2], "wb");
    if (!o) return 6;
    fwrite(fast.data(), 4, n, o);
    fwrite(exact.data(), 4, n, o);
    fclose(o);
    return 0;
}
