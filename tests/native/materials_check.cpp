// Host run of the element kernel's constitutive updates (edelweissfe_gb300/csrc/materials.h,
// the same source that the device compiles) on a batch of points read from a file, so that a
// Python test can compare them with the oracle.
//
// Input (binary, native endianness): int32 nPts, int32 material (0 linear elastic, 1 J2),
// double props[8], then per point sig[6], kappa, de[6].
// Output: per point ok (1 or 0), sig[6], kappa, lt, mt, c1, n[6] (17 doubles).
// Build: g++ -O2 -std=c++17 -ffp-contract=off materials_check.cpp
#include <cstdint>
#include <cstdio>
#include <vector>

#include "../../edelweissfe_gb300/csrc/materials.h"

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: materials_check <input> <output>\n");
        return 2;
    }
    std::FILE* in = std::fopen(argv[1], "rb");
    if (!in) return 2;
    int32_t nPts = 0, mat = 0;
    double props[8];
    if (std::fread(&nPts, 4, 1, in) != 1 || std::fread(&mat, 4, 1, in) != 1 || std::fread(props, 8, 8, in) != 8)
        return 2;
    std::vector<double> pts((size_t)nPts * 13);
    if (std::fread(pts.data(), 8, pts.size(), in) != pts.size()) return 2;
    std::fclose(in);
    std::vector<double> out((size_t)nPts * 17, 0.0);
    for (int32_t p = 0; p < nPts; ++p) {
        const double* x = &pts[(size_t)p * 13];
        double sig[6], de[6], kappa = x[6];
        for (int i = 0; i < 6; ++i) {
            sig[i] = x[i];
            de[i] = x[7 + i];
        }
        ef::MatOut o{};
        bool ok = true;
        if (mat == 1)
            ok = ef::mat_von_mises(props, sig, &kappa, de, o);
        else
            ef::mat_linear_elastic(props, sig, de, o);
        double* y = &out[(size_t)p * 17];
        y[0] = ok ? 1.0 : 0.0;
        for (int i = 0; i < 6; ++i) y[1 + i] = sig[i];
        y[7] = kappa;
        y[8] = o.lt;
        y[9] = o.mt;
        y[10] = o.c1;
        for (int i = 0; i < 6; ++i) y[11 + i] = o.c1 != 0.0 ? o.n[i] : 0.0;
    }
    std::FILE* f = std::fopen(argv[2], "wb");
    if (!f) return 2;
    std::fwrite(out.data(), 8, out.size(), f);
    std::fclose(f);
    return 0;
}
