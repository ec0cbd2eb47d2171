// Host check of the smoothed-aggregation index maps (edelweissfe_gb300/csrc/amg_sa_pattern.h):
// the prolongator, A P and P^T A P formed through the maps as segmented sums (the loops the
// device kernels run) against dense products on a small structured pattern with random blocks,
// a Dirichlet mask and an arbitrary aggregation.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <random>
#include <vector>

#include "../../edelweissfe_gb300/csrc/amg_sa_pattern.h"

static const int BF = 3, BC = 6;

// tentative prolongation block of a finer node with offset d from its aggregate centroid
static void pblock(const double* d, double P[BF][BC]) {
    for (int i = 0; i < BF; ++i)
        for (int j = 0; j < BC; ++j) P[i][j] = 0.0;
    P[0][0] = P[1][1] = P[2][2] = 1.0;
    P[1][3] = -d[2];
    P[2][3] = d[1];
    P[0][4] = d[2];
    P[2][4] = -d[0];
    P[0][5] = -d[1];
    P[1][5] = d[0];
}

int main() {
    const int gx = 6, gy = 5, gz = 4, nF = gx * gy * gz, n = BF * nF;
    std::mt19937_64 g(11);
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    auto id = [&](int i, int j, int k) { return (i * gy + j) * gz + k; };
    // 27-point block pattern
    std::vector<int32_t> rowPtr(nF + 1, 0), colIdx;
    for (int i = 0; i < gx; ++i)
        for (int j = 0; j < gy; ++j)
            for (int k = 0; k < gz; ++k) {
                for (int a = -1; a <= 1; ++a)
                    for (int b = -1; b <= 1; ++b)
                        for (int c = -1; c <= 1; ++c) {
                            const int ii = i + a, jj = j + b, kk = k + c;
                            if (ii < 0 || jj < 0 || kk < 0 || ii >= gx || jj >= gy || kk >= gz) continue;
                            colIdx.push_back(id(ii, jj, kk));
                        }
                rowPtr[id(i, j, k) + 1] = (int32_t)colIdx.size();
            }
    const int nnz = (int)colIdx.size();
    // symmetric random blocks with a dominant diagonal; dense copy
    std::vector<double> A((size_t)n * n, 0.0), vals((size_t)nnz * 9);
    for (int m = 0; m < nF; ++m)
        for (int k = rowPtr[m]; k < rowPtr[m + 1]; ++k) {
            const int c = colIdx[k];
            if (c < m) continue;
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    double v = u(g);
                    if (c == m) v = a == b ? 30.0 : 0.5 * (v + 0.0);
                    A[(size_t)(3 * m + a) * n + 3 * c + b] = v;
                    A[(size_t)(3 * c + b) * n + 3 * m + a] = v;
                }
        }
    for (int m = 0; m < nF; ++m)
        for (int k = rowPtr[m]; k < rowPtr[m + 1]; ++k)
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) vals[(size_t)k * 9 + 3 * a + b] = A[(size_t)(3 * m + a) * n + 3 * colIdx[k] + b];
    // mask: first x-plane clamped, a few single DOFs
    std::vector<uint8_t> mask(n, 0);
    for (int j = 0; j < gy; ++j)
        for (int k = 0; k < gz; ++k)
            for (int a = 0; a < 3; ++a) mask[3 * id(0, j, k) + a] = 1;
    mask[3 * id(3, 2, 1) + 1] = 1;
    // aggregation: 2x2x2 boxes
    std::vector<int32_t> agg(nF);
    const int ax = (gx + 1) / 2, ay = (gy + 1) / 2, az = (gz + 1) / 2, nC = ax * ay * az;
    for (int i = 0; i < gx; ++i)
        for (int j = 0; j < gy; ++j)
            for (int k = 0; k < gz; ++k) agg[id(i, j, k)] = ((i / 2) * ay + j / 2) * az + k / 2;
    std::vector<double> offs(3 * nF);
    for (auto& o : offs) o = 0.3 * u(g);
    // masked operator A' and block-Jacobi inverse (identity on masked rows/columns)
    std::vector<double> Am = A;
    for (int r = 0; r < n; ++r)
        for (int c = 0; c < n; ++c)
            if (mask[r] || mask[c]) Am[(size_t)r * n + c] = 0.0;
    std::vector<double> Dinv((size_t)nF * 9);
    for (int m = 0; m < nF; ++m) {
        double D[3][3];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                D[a][b] = Am[(size_t)(3 * m + a) * n + 3 * m + b];
                if (mask[3 * m + a] || mask[3 * m + b]) D[a][b] = a == b ? 1.0 : 0.0;
            }
        const double det = D[0][0] * (D[1][1] * D[2][2] - D[1][2] * D[2][1]) -
                           D[0][1] * (D[1][0] * D[2][2] - D[1][2] * D[2][0]) +
                           D[0][2] * (D[1][0] * D[2][1] - D[1][1] * D[2][0]);
        double I[3][3] = {{(D[1][1] * D[2][2] - D[1][2] * D[2][1]), -(D[0][1] * D[2][2] - D[0][2] * D[2][1]),
                           (D[0][1] * D[1][2] - D[0][2] * D[1][1])},
                          {-(D[1][0] * D[2][2] - D[1][2] * D[2][0]), (D[0][0] * D[2][2] - D[0][2] * D[2][0]),
                           -(D[0][0] * D[1][2] - D[0][2] * D[1][0])},
                          {(D[1][0] * D[2][1] - D[1][1] * D[2][0]), -(D[0][0] * D[2][1] - D[0][1] * D[2][0]),
                           (D[0][0] * D[1][1] - D[0][1] * D[1][0])}};
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) Dinv[(size_t)m * 9 + 3 * a + b] = I[a][b] / det;
    }
    const double w = 0.37;
    // ---- dense reference ----
    const int nc = BC * nC;
    std::vector<double> Pt((size_t)n * nc, 0.0);
    for (int m = 0; m < nF; ++m) {
        double P[BF][BC];
        pblock(&offs[3 * m], P);
        for (int a = 0; a < BF; ++a)
            for (int j = 0; j < BC; ++j) Pt[(size_t)(3 * m + a) * nc + BC * agg[m] + j] = P[a][j];
    }
    std::vector<double> AP0((size_t)n * nc, 0.0), Ps((size_t)n * nc, 0.0);
    for (int r = 0; r < n; ++r)
        for (int c = 0; c < n; ++c) {
            const double a = Am[(size_t)r * n + c];
            if (a == 0.0) continue;
            for (int j = 0; j < nc; ++j) AP0[(size_t)r * nc + j] += a * Pt[(size_t)c * nc + j];
        }
    for (int m = 0; m < nF; ++m)
        for (int a = 0; a < 3; ++a) {
            const int r = 3 * m + a;
            for (int j = 0; j < nc; ++j) {
                double s = 0.0;
                for (int b = 0; b < 3; ++b) s += Dinv[(size_t)m * 9 + 3 * a + b] * AP0[(size_t)(3 * m + b) * nc + j];
                Ps[(size_t)r * nc + j] = mask[r] ? 0.0 : Pt[(size_t)r * nc + j] - w * s;
            }
        }
    std::vector<double> APd((size_t)n * nc, 0.0), Acd((size_t)nc * nc, 0.0);
    for (int r = 0; r < n; ++r)
        for (int c = 0; c < n; ++c) {
            const double a = Am[(size_t)r * n + c];
            if (a == 0.0) continue;
            for (int j = 0; j < nc; ++j) APd[(size_t)r * nc + j] += a * Ps[(size_t)c * nc + j];
        }
    for (int r = 0; r < n; ++r)
        for (int i = 0; i < nc; ++i) {
            const double p = Ps[(size_t)r * nc + i];
            if (p == 0.0) continue;
            for (int j = 0; j < nc; ++j) Acd[(size_t)i * nc + j] += p * APd[(size_t)r * nc + j];
        }
    // ---- through the maps ----
    ef::SAPattern S;
    ef::build_sa_pattern(nF, rowPtr.data(), colIdx.data(), agg.data(), nC, S);
    const size_t nP = S.pCol.size(), nAP = S.apCol.size(), nCc = S.cCol.size();
    auto Ablk = [&](int k, int a, int b) {
        const int m = -1;
        (void)m;
        return vals[(size_t)k * 9 + 3 * a + b];
    };
    std::vector<double> Pv(nP * BF * BC), APv(nAP * BF * BC), Acv(nCc * BC * BC);
    for (size_t b = 0; b < nP; ++b) {
        const int m = S.pRow[b], J = S.pCol[b];
        double acc[BF][BC] = {};
        for (int64_t t = S.pSeg[b]; t < S.pSeg[b + 1]; ++t) {
            const int k = S.pSrc[t], c = colIdx[k];
            double P[BF][BC];
            pblock(&offs[3 * c], P);
            for (int a = 0; a < BF; ++a)
                for (int j = 0; j < BC; ++j)
                    for (int q = 0; q < BF; ++q) {
                        const double av = (mask[3 * m + a] || mask[3 * c + q]) ? 0.0 : Ablk(k, a, q);
                        acc[a][j] += av * P[q][j];
                    }
        }
        double Pm[BF][BC];
        pblock(&offs[3 * m], Pm);
        for (int a = 0; a < BF; ++a)
            for (int j = 0; j < BC; ++j) {
                double s = 0.0;
                for (int q = 0; q < BF; ++q) s += Dinv[(size_t)m * 9 + 3 * a + q] * acc[q][j];
                const double v = (J == agg[m] ? Pm[a][j] : 0.0) - w * s;
                Pv[b * BF * BC + a * BC + j] = mask[3 * m + a] ? 0.0 : v;
            }
    }
    for (size_t ab = 0; ab < nAP; ++ab) {
        double acc[BF][BC] = {};
        for (int64_t t = S.apSeg[ab]; t < S.apSeg[ab + 1]; ++t) {
            const int k = S.apK[t], pb = S.apP[t];
            int m = 0;
            while (!(S.apRowPtr[m] <= (int)ab && (int)ab < S.apRowPtr[m + 1])) ++m;
            const int c = colIdx[k];
            for (int a = 0; a < BF; ++a)
                for (int j = 0; j < BC; ++j)
                    for (int q = 0; q < BF; ++q) {
                        const double av = (mask[3 * m + a] || mask[3 * c + q]) ? 0.0 : Ablk(k, a, q);
                        acc[a][j] += av * Pv[(size_t)pb * BF * BC + q * BC + j];
                    }
        }
        for (int a = 0; a < BF; ++a)
            for (int j = 0; j < BC; ++j) APv[ab * BF * BC + a * BC + j] = acc[a][j];
    }
    for (size_t cb = 0; cb < nCc; ++cb) {
        double acc[BC][BC] = {};
        for (int64_t t = S.cSeg[cb]; t < S.cSeg[cb + 1]; ++t) {
            const int pb = S.cP[t], ab = S.cAP[t];
            for (int i = 0; i < BC; ++i)
                for (int j = 0; j < BC; ++j)
                    for (int q = 0; q < BF; ++q)
                        acc[i][j] += Pv[(size_t)pb * BF * BC + q * BC + i] * APv[(size_t)ab * BF * BC + q * BC + j];
        }
        for (int i = 0; i < BC; ++i)
            for (int j = 0; j < BC; ++j) Acv[cb * BC * BC + i * BC + j] = acc[i][j];
    }
    // ---- compare ----
    double eP = 0, eAP = 0, eC = 0, sP = 0, sAP = 0, sC = 0;
    std::vector<uint8_t> seenP((size_t)n * nc, 0), seenAP((size_t)n * nc, 0), seenC((size_t)nc * nc, 0);
    for (int m = 0; m < nF; ++m)
        for (int b = S.pRowPtr[m]; b < S.pRowPtr[m + 1]; ++b)
            for (int a = 0; a < BF; ++a)
                for (int j = 0; j < BC; ++j) {
                    const size_t di = (size_t)(3 * m + a) * nc + BC * S.pCol[b] + j;
                    eP = std::fmax(eP, std::fabs(Pv[(size_t)b * BF * BC + a * BC + j] - Ps[di]));
                    seenP[di] = 1;
                }
    for (int m = 0; m < nF; ++m)
        for (int b = S.apRowPtr[m]; b < S.apRowPtr[m + 1]; ++b)
            for (int a = 0; a < BF; ++a)
                for (int j = 0; j < BC; ++j) {
                    const size_t di = (size_t)(3 * m + a) * nc + BC * S.apCol[b] + j;
                    eAP = std::fmax(eAP, std::fabs(APv[(size_t)b * BF * BC + a * BC + j] - APd[di]));
                    seenAP[di] = 1;
                }
    for (int I = 0; I < nC; ++I)
        for (int b = S.cRowPtr[I]; b < S.cRowPtr[I + 1]; ++b)
            for (int i = 0; i < BC; ++i)
                for (int j = 0; j < BC; ++j) {
                    const size_t di = (size_t)(BC * I + i) * nc + BC * S.cCol[b] + j;
                    eC = std::fmax(eC, std::fabs(Acv[(size_t)b * BC * BC + i * BC + j] - Acd[di]));
                    seenC[di] = 1;
                }
    // dense entries outside the patterns must be zero
    for (size_t i = 0; i < Ps.size(); ++i) {
        if (!seenP[i]) sP = std::fmax(sP, std::fabs(Ps[i]));
        if (!seenAP[i]) sAP = std::fmax(sAP, std::fabs(APd[i]));
    }
    for (size_t i = 0; i < Acd.size(); ++i)
        if (!seenC[i]) sC = std::fmax(sC, std::fabs(Acd[i]));
    double scale = 0;
    for (double v : Acd) scale = std::fmax(scale, std::fabs(v));
    std::printf("P %zu blocks, AP %zu, coarse %zu; max diff P %.2e AP %.2e Ac %.2e (scale %.2e); outside "
                "patterns %.2e %.2e %.2e\n",
                nP, nAP, nCc, eP, eAP, eC, scale, sP, sAP, sC);
    const bool ok = eP < 1e-12 && eAP < 1e-11 && eC < 1e-10 * scale && sP == 0.0 && sAP == 0.0 && sC == 0.0;
    std::printf("%s\n", ok ? "failures 0" : "failures 1");
    return ok ? 0 : 1;
}
