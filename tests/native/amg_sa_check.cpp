// Host check of the smoothed-aggregation setup and transfer operators: the index maps of
// edelweissfe_gb300/csrc/amg_sa_pattern.h and the per-thread bodies that the device kernels run
// (edelweissfe_gb300/csrc/amg_sa_body.h, compiled here for the host) are run over every index of
// small block systems and compared with dense FP64 products:
//   P = P_t - w D^-1 A P_t (zero on masked rows), AP = A P, A_c = P^T A P (dead coarse DOFs
//   identity), the restriction P^T t (dead coarse DOFs zero) and the prolongation x += alpha P xc
//   (masked rows untouched),
// for the 3-DOF finer level (a Dirichlet mask) and the 6-DOF coarser levels (a dead-DOF mask),
// with and without a mask.  The dense products must also vanish outside the patterns.
// Build: g++ -O2 -std=c++17 -ffp-contract=off amg_sa_check.cpp
#include <cmath>
#include <cstdint>
#include <algorithm>
#include <cstdio>
#include <random>
#include <utility>
#include <vector>

#include "../../edelweissfe_gb300/csrc/amg_sa_body.h"
#include "../../edelweissfe_gb300/csrc/amg_sa_pattern.h"

using ef::BC;

// inverse of a dense BF x BF matrix by Gauss-Jordan with partial pivoting (FP64)
template <int BF>
static void invert(double A[BF][BF], double R[BF][BF]) {
    double M[BF][2 * BF];
    for (int i = 0; i < BF; ++i)
        for (int j = 0; j < 2 * BF; ++j) M[i][j] = j < BF ? A[i][j] : (j - BF == i ? 1.0 : 0.0);
    for (int c = 0; c < BF; ++c) {
        int p = c;
        for (int r = c + 1; r < BF; ++r)
            if (std::fabs(M[r][c]) > std::fabs(M[p][c])) p = r;
        for (int j = 0; j < 2 * BF; ++j) std::swap(M[c][j], M[p][j]);
        const double d = M[c][c];
        for (int j = 0; j < 2 * BF; ++j) M[c][j] /= d;
        for (int r = 0; r < BF; ++r) {
            if (r == c) continue;
            const double f = M[r][c];
            for (int j = 0; j < 2 * BF; ++j) M[r][j] -= f * M[c][j];
        }
    }
    for (int i = 0; i < BF; ++i)
        for (int j = 0; j < BF; ++j) R[i][j] = M[i][BF + j];
}

static double max_abs(const std::vector<double>& v) {
    double s = 0;
    for (double x : v) s = std::fmax(s, std::fabs(x));
    return s;
}

// dense row-major product O = L R (rows x inner) (inner x cols)
static std::vector<double> matmul(const std::vector<double>& L, const std::vector<double>& R, int rows, int inner,
                                  int cols) {
    std::vector<double> O((size_t)rows * cols, 0.0);
    for (int r = 0; r < rows; ++r)
        for (int q = 0; q < inner; ++q) {
            const double l = L[(size_t)r * inner + q];
            if (l == 0.0) continue;
            for (int c = 0; c < cols; ++c) O[(size_t)r * cols + c] += l * R[(size_t)q * cols + c];
        }
    return O;
}

// one level transition on a gx x gy x gz grid of BF-DOF nodes (27-point block pattern, random
// symmetric blocks with a dominant diagonal, 2 x 2 x 2 aggregates); returns the number of failures
template <int BF>
static int check_level(const char* name, int gx, int gy, int gz, uint64_t seed, bool useMask) {
    const int nF = gx * gy * gz, n = BF * nF;
    std::mt19937_64 g(seed);
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    auto id = [&](int i, int j, int k) { return (i * gy + j) * gz + k; };
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
    // symmetric operator, rounded to the FP32 values that the device holds
    std::vector<double> A((size_t)n * n, 0.0);
    for (int m = 0; m < nF; ++m)
        for (int k = rowPtr[m]; k < rowPtr[m + 1]; ++k) {
            const int c = colIdx[k];
            if (c < m) continue;
            for (int a = 0; a < BF; ++a)
                for (int b = 0; b < BF; ++b) {
                    if (c == m && b < a) continue;
                    double v = u(g);
                    v = (double)(float)(c == m ? (a == b ? 10.0 * BF : 0.5 * v) : v);
                    A[(size_t)(BF * m + a) * n + BF * c + b] = v;
                    A[(size_t)(BF * c + b) * n + BF * m + a] = v;
                }
        }
    std::vector<float> vals((size_t)nnz * BF * BF);  // row-major BF x BF per block
    for (int m = 0; m < nF; ++m)
        for (int k = rowPtr[m]; k < rowPtr[m + 1]; ++k)
            for (int a = 0; a < BF; ++a)
                for (int b = 0; b < BF; ++b)
                    vals[(size_t)k * BF * BF + BF * a + b] = (float)A[(size_t)(BF * m + a) * n + BF * colIdx[k] + b];
    // finer mask: BF = 3 a clamped x-plane and one single DOF (Dirichlet); BF = 6 the rotations of
    // the first x-plane and one whole node (dead coarse DOFs of the level above)
    std::vector<uint8_t> mask(n, 0);
    if (useMask) {
        for (int j = 0; j < gy; ++j)
            for (int k = 0; k < gz; ++k)
                for (int a = BF == 3 ? 0 : 3; a < BF; ++a) mask[BF * id(0, j, k) + a] = 1;
        if (BF == 3)
            mask[BF * id(gx / 2, gy / 2, 1) + 1] = 1;
        else
            for (int a = 0; a < BF; ++a) mask[BF * id(gx - 1, 0, 0) + a] = 1;
    }
    // aggregation: 2 x 2 x 2 boxes
    const int ay = (gy + 1) / 2, az = (gz + 1) / 2, nC = ((gx + 1) / 2) * ay * az;
    std::vector<int32_t> agg(nF);
    for (int i = 0; i < gx; ++i)
        for (int j = 0; j < gy; ++j)
            for (int k = 0; k < gz; ++k) agg[id(i, j, k)] = ((i / 2) * ay + j / 2) * az + k / 2;
    std::vector<float> offs(3 * nF);
    for (auto& o : offs) o = (float)(0.3 * u(g));
    // dead coarse DOFs: the rotations of aggregate 1 and translation 0 of the last aggregate
    const int nc = BC * nC;
    std::vector<uint8_t> dead(nc, 0);
    for (int j = 3; j < BC; ++j) dead[BC * 1 + j] = 1;
    dead[BC * (nC - 1)] = 1;
    // masked operator and block-Jacobi inverse (identity on masked rows/columns), FP32 as on the device
    std::vector<double> Am = A;
    for (int r = 0; r < n; ++r)
        for (int c = 0; c < n; ++c)
            if (mask[r] || mask[c]) Am[(size_t)r * n + c] = 0.0;
    std::vector<float> binv((size_t)nF * BF * BF);
    for (int m = 0; m < nF; ++m) {
        double D[BF][BF], R[BF][BF];
        for (int a = 0; a < BF; ++a)
            for (int b = 0; b < BF; ++b) {
                D[a][b] = Am[(size_t)(BF * m + a) * n + BF * m + b];
                if (mask[BF * m + a] || mask[BF * m + b]) D[a][b] = a == b ? 1.0 : 0.0;
            }
        invert<BF>(D, R);
        for (int a = 0; a < BF; ++a)
            for (int b = 0; b < BF; ++b) binv[(size_t)m * BF * BF + BF * a + b] = (float)R[a][b];
    }
    const float w = 0.37f, alpha = 1.25f;
    // ---- dense FP64 reference ----
    std::vector<double> Pt((size_t)n * nc, 0.0);
    for (int m = 0; m < nF; ++m) {
        float P[BF][BC];
        ef::pblock<BF>(&offs[3 * m], P);
        for (int a = 0; a < BF; ++a)
            for (int j = 0; j < BC; ++j) Pt[(size_t)(BF * m + a) * nc + BC * agg[m] + j] = P[a][j];
    }
    const std::vector<double> AP0 = matmul(Am, Pt, n, n, nc);
    std::vector<double> Ps((size_t)n * nc, 0.0);
    for (int m = 0; m < nF; ++m)
        for (int a = 0; a < BF; ++a) {
            const int r = BF * m + a;
            for (int j = 0; j < nc; ++j) {
                double s = 0.0;
                for (int b = 0; b < BF; ++b)
                    s += (double)binv[(size_t)m * BF * BF + BF * a + b] * AP0[(size_t)(BF * m + b) * nc + j];
                Ps[(size_t)r * nc + j] = mask[r] ? 0.0 : Pt[(size_t)r * nc + j] - (double)w * s;
            }
        }
    const std::vector<double> APd = matmul(Am, Ps, n, n, nc);
    std::vector<double> PsT((size_t)nc * n);
    for (int r = 0; r < n; ++r)
        for (int c = 0; c < nc; ++c) PsT[(size_t)c * n + r] = Ps[(size_t)r * nc + c];
    std::vector<double> Acd = matmul(PsT, APd, nc, n, nc);
    for (int i = 0; i < nc; ++i)
        for (int j = 0; j < nc; ++j)
            if (dead[i] || dead[j]) Acd[(size_t)i * nc + j] = i == j ? 1.0 : 0.0;
    std::vector<double> t(n), xc(nc), x0(n);
    std::vector<float> tf(n), xcf(nc), xf(n);
    for (int i = 0; i < n; ++i) tf[i] = (float)u(g), t[i] = tf[i];
    for (int i = 0; i < nc; ++i) xcf[i] = (float)u(g), xc[i] = xcf[i];
    for (int i = 0; i < n; ++i) xf[i] = (float)u(g), x0[i] = xf[i];
    std::vector<double> rcd = matmul(PsT, t, nc, n, 1);
    for (int i = 0; i < nc; ++i)
        if (dead[i]) rcd[i] = 0.0;
    const std::vector<double> pxd = matmul(Ps, xc, n, nc, 1);
    std::vector<double> xd(n);
    for (int i = 0; i < n; ++i) xd[i] = mask[i] ? x0[i] : x0[i] + (double)alpha * pxd[i];
    // ---- through the maps and the device bodies ----
    ef::SAPattern S;
    ef::build_sa_pattern(nF, rowPtr.data(), colIdx.data(), agg.data(), nC, S);
    const int64_t nP = (int64_t)S.pCol.size(), nAP = (int64_t)S.apCol.size(), nCb = (int64_t)S.cCol.size();
    std::vector<int32_t> apRow(nAP), cRob(nCb);
    for (int m = 0; m < nF; ++m)
        for (int32_t a = S.apRowPtr[m]; a < S.apRowPtr[m + 1]; ++a) apRow[a] = m;
    for (int I = 0; I < nC; ++I)
        for (int32_t b = S.cRowPtr[I]; b < S.cRowPtr[I + 1]; ++b) cRob[b] = I;
    const uint8_t* fm = useMask ? mask.data() : nullptr;
    std::vector<float> Pv(nP * BF * BC), APv(nAP * BF * BC), Acv(nCb * BC * BC), rc(nc);
    for (int64_t b = 0; b < nP; ++b)
        ef::sa_prolongator_block<BF>(b, S.pRow.data(), S.pCol.data(), S.pSeg.data(), S.pSrc.data(), colIdx.data(),
                                     vals.data(), fm, offs.data(), agg.data(), binv.data(), w, Pv.data());
    for (int64_t a = 0; a < nAP; ++a)
        ef::sa_ap_block<BF>(a, apRow.data(), S.apSeg.data(), S.apK.data(), S.apP.data(), colIdx.data(), vals.data(), fm,
                            Pv.data(), APv.data());
    // AP by pairs (the row-group kernel): each pair's product, then the sums of each AP block's pairs
    std::vector<float> APv2(nAP * BF * BC, 0.f);
    for (int m = 0; m < nF; ++m)
        for (int32_t a = S.apRowPtr[m]; a < S.apRowPtr[m + 1]; ++a)
            for (int64_t t = S.apSeg[a]; t < S.apSeg[a + 1]; ++t) {
                float cpair[BF * BC];
                ef::sa_ap_pair<BF>(t, m, S.apK.data(), S.apP.data(), colIdx.data(), vals.data(), fm, Pv.data(), cpair);
                for (int p = 0; p < BF * BC; ++p) APv2[(size_t)a * BF * BC + p] += cpair[p];
            }
    for (int64_t c = 0; c < nCb; ++c)
        ef::sa_galerkin_block<BF>(c, S.cSeg.data(), S.cP.data(), S.cAP.data(), Pv.data(), APv.data(), cRob.data(),
                                  S.cCol.data(), dead.data(), Acv.data());
    for (int I = 0; I < nC; ++I) {
        double sum[BC] = {};
        for (int lane = 0; lane < 32; ++lane) {
            float a[BC];
            ef::sa_restrict_partial<BF>(I, lane, 32, S.tPtr.data(), S.tIdx.data(), S.pRow.data(), Pv.data(), tf.data(),
                                        a);
            for (int j = 0; j < BC; ++j) sum[j] += a[j];
        }
        for (int j = 0; j < BC; ++j) rc[BC * I + j] = dead[BC * I + j] ? 0.f : (float)sum[j];
    }
    for (int m = 0; m < nF; ++m)
        ef::sa_prolong_row<BF>(m, S.pRowPtr.data(), S.pCol.data(), Pv.data(), xcf.data(), fm, xf.data(), alpha);
    // the two-stage forms: block products, then per coarse node / per finer row sums
    std::vector<float> cb((size_t)nP * BC), rc2(nc), xf2(x0.begin(), x0.end());
    for (int64_t b = 0; b < nP; ++b) ef::sa_restrict_contrib<BF>(b, S.pRow.data(), Pv.data(), tf.data(), cb.data());
    for (int I = 0; I < nC; ++I) {
        double sum[BC] = {};
        for (int lane = 0; lane < 32; ++lane) {
            float a[BC];
            ef::sa_restrict_sum_partial(I, lane, 32, S.tPtr.data(), S.tIdx.data(), cb.data(), a);
            for (int j = 0; j < BC; ++j) sum[j] += a[j];
        }
        for (int j = 0; j < BC; ++j) rc2[BC * I + j] = dead[BC * I + j] ? 0.f : (float)sum[j];
    }
    for (int64_t b = 0; b < nP; ++b) ef::sa_prolong_contrib<BF>(b, S.pCol.data(), Pv.data(), xcf.data(), cb.data());
    for (int m = 0; m < nF; ++m) ef::sa_prolong_apply<BF>(m, S.pRowPtr.data(), cb.data(), fm, xf2.data(), alpha);
    // the one-pass forms: the restriction from the transpose-order copy of P over 128 threads per
    // coarse node, the prolongation in groups of 64 consecutive finer rows, as the kernels run them
    std::vector<float> PT((size_t)nP * BF * BC), rc3(nc), xf3(x0.begin(), x0.end());
    std::vector<int32_t> rowT(nP);
    for (int64_t k = 0; k < nP; ++k) {
        rowT[k] = S.pRow[S.tIdx[k]];
        ef::sa_block_copy<BF>(k, S.tIdx.data(), Pv.data(), PT.data());
    }
    for (int I = 0; I < nC; ++I) {
        double sum[BC] = {};
        for (int lane = 0; lane < 128; ++lane) {
            float a[BC];
            ef::sa_restrict_onepass_partial<BF>(I, lane, 128, S.tPtr.data(), rowT.data(), PT.data(), tf.data(), a);
            for (int j = 0; j < BC; ++j) sum[j] += a[j];
        }
        for (int j = 0; j < BC; ++j) rc3[BC * I + j] = dead[BC * I + j] ? 0.f : (float)sum[j];
    }
    for (int r0 = 0; r0 < nF; r0 += 64) {
        const int r1 = std::min(r0 + 64, nF);
        const int64_t b0 = S.pRowPtr[r0], b1 = S.pRowPtr[r1];
        std::vector<float> q((size_t)(b1 - b0) * BF);
        for (int64_t b = b0; b < b1; ++b)
            ef::sa_prolong_onepass_block<BF>(b, S.pCol.data(), Pv.data(), xcf.data(), &q[(size_t)(b - b0) * BF]);
        for (int m = r0; m < r1; ++m)
            ef::sa_prolong_onepass_row<BF>(m, b0, S.pRowPtr.data(), q.data(), fm, xf3.data(), alpha);
    }
    // ---- compare (FP32 arithmetic against FP64: relative to each product's largest entry) ----
    double eP = 0, eAP = 0, eC = 0, eR = 0, eX = 0, oP = 0, oAP = 0, oC = 0;
    std::vector<uint8_t> seenP((size_t)n * nc, 0), seenAP((size_t)n * nc, 0), seenC((size_t)nc * nc, 0);
    for (int m = 0; m < nF; ++m) {
        for (int b = S.pRowPtr[m]; b < S.pRowPtr[m + 1]; ++b)
            for (int a = 0; a < BF; ++a)
                for (int j = 0; j < BC; ++j) {
                    const size_t di = (size_t)(BF * m + a) * nc + BC * S.pCol[b] + j;
                    eP = std::fmax(eP, std::fabs(Pv[(size_t)b * BF * BC + a * BC + j] - Ps[di]));
                    seenP[di] = 1;
                }
        for (int b = S.apRowPtr[m]; b < S.apRowPtr[m + 1]; ++b)
            for (int a = 0; a < BF; ++a)
                for (int j = 0; j < BC; ++j) {
                    const size_t di = (size_t)(BF * m + a) * nc + BC * S.apCol[b] + j;
                    eAP = std::fmax(eAP, std::fabs(APv[(size_t)b * BF * BC + a * BC + j] - APd[di]));
                    seenAP[di] = 1;
                }
    }
    for (int I = 0; I < nC; ++I)
        for (int b = S.cRowPtr[I]; b < S.cRowPtr[I + 1]; ++b)
            for (int i = 0; i < BC; ++i)
                for (int j = 0; j < BC; ++j) {
                    const size_t di = (size_t)(BC * I + i) * nc + BC * S.cCol[b] + j;
                    eC = std::fmax(eC, std::fabs(Acv[(size_t)b * BC * BC + i * BC + j] - Acd[di]));
                    seenC[di] = 1;
                }
    for (size_t i = 0; i < Ps.size(); ++i) {
        if (!seenP[i]) oP = std::fmax(oP, std::fabs(Ps[i]));
        if (!seenAP[i]) oAP = std::fmax(oAP, std::fabs(APd[i]));
    }
    for (size_t i = 0; i < Acd.size(); ++i)
        if (!seenC[i]) oC = std::fmax(oC, std::fabs(Acd[i]));
    // fused post-smoothing blocks C = alpha (P - omega D^-1 A P) in the pattern of AP
    double eCp = 0, sCp = 0;
    {
        const float om = 0.7f, al = 0.9f;
        std::vector<int32_t> apToP(nAP, -1);
        for (int m = 0; m < nF; ++m)
            for (int32_t a = S.apRowPtr[m]; a < S.apRowPtr[m + 1]; ++a)
                apToP[a] = (int32_t)ef::sa_find(S.pCol, S.pRowPtr[m], S.pRowPtr[m + 1], S.apCol[a]);
        for (int m = 0; m < nF; ++m)
            for (int32_t a = S.apRowPtr[m]; a < S.apRowPtr[m + 1]; ++a) {
                float C[BF * BC];
                ef::sa_post_block<BF>(a, apRow.data(), apToP.data(), Pv.data(), APv.data(), binv.data(), om, al, C);
                for (int i = 0; i < BF; ++i)
                    for (int j = 0; j < BC; ++j) {
                        const size_t col = BC * (size_t)S.apCol[a] + j;
                        double z = 0.0;
                        for (int q = 0; q < BF; ++q)
                            z += (double)binv[(size_t)m * BF * BF + BF * i + q] * APd[(size_t)(BF * m + q) * nc + col];
                        const double cd = al * (Ps[(size_t)(BF * m + i) * nc + col] - om * z);
                        eCp = std::fmax(eCp, std::fabs(C[i * BC + j] - cd));
                        sCp = std::fmax(sCp, std::fabs(cd));
                    }
            }
    }
    double eR2 = 0, eX2 = 0, eR3 = 0, eX3 = 0, eAP2 = 0;
    for (int m = 0; m < nF; ++m)
        for (int b = S.apRowPtr[m]; b < S.apRowPtr[m + 1]; ++b)
            for (int a = 0; a < BF; ++a)
                for (int j = 0; j < BC; ++j) {
                    const size_t di = (size_t)(BF * m + a) * nc + BC * S.apCol[b] + j;
                    eAP2 = std::fmax(eAP2, std::fabs(APv2[(size_t)b * BF * BC + a * BC + j] - APd[di]));
                }
    for (int i = 0; i < nc; ++i) eR = std::fmax(eR, std::fabs(rc[i] - rcd[i]));
    for (int i = 0; i < n; ++i) eX = std::fmax(eX, std::fabs(xf[i] - xd[i]));
    for (int i = 0; i < nc; ++i) eR2 = std::fmax(eR2, std::fabs(rc2[i] - rcd[i]));
    for (int i = 0; i < n; ++i) eX2 = std::fmax(eX2, std::fabs(xf2[i] - xd[i]));
    for (int i = 0; i < nc; ++i) eR3 = std::fmax(eR3, std::fabs(rc3[i] - rcd[i]));
    for (int i = 0; i < n; ++i) eX3 = std::fmax(eX3, std::fabs(xf3[i] - xd[i]));
    const double sP = max_abs(Ps), sAP = max_abs(APd), sC = max_abs(Acd), sR = max_abs(rcd), sX = max_abs(xd);
    const double tol = 2e-6;
    int fails = 0;
    fails += !(eP <= tol * sP) + !(eAP <= tol * sAP) + !(eC <= tol * sC) + !(eR <= tol * sR) + !(eX <= tol * sX);
    fails += !(eR2 <= tol * sR) + !(eX2 <= tol * sX);
    fails += !(eR3 <= tol * sR) + !(eX3 <= tol * sX) + !(eAP2 <= tol * sAP) + !(eCp <= tol * sCp);
    fails += (oP != 0.0) + (oAP != 0.0) + (oC != 0.0);
    // masked finer rows: P exactly zero
    for (int m = 0; m < nF; ++m)
        for (int a = 0; a < BF; ++a) {
            if (!mask[BF * m + a]) continue;
            for (int b = S.pRowPtr[m]; b < S.pRowPtr[m + 1]; ++b)
                for (int j = 0; j < BC; ++j) fails += Pv[(size_t)b * BF * BC + a * BC + j] != 0.f;
        }
    std::printf("%s: P %lld blocks, AP %lld, coarse %lld; rel diff P %.1e AP %.1e (pairs %.1e) Ac %.1e restrict %.1e "
                "prolong %.1e (two-stage %.1e %.1e, one-pass %.1e %.1e); post C %.1e; outside patterns %.1e %.1e "
                "%.1e; failures %d\n",
                name, (long long)nP, (long long)nAP, (long long)nCb, eP / sP, eAP / sAP, eAP2 / sAP, eC / sC, eR / sR,
                eX / sX, eR2 / sR, eX2 / sX, eR3 / sR, eX3 / sX, eCp / sCp, oP, oAP, oC, fails);
    return fails;
}

int main() {
    int fails = 0;
    fails += check_level<3>("3-DOF level, Dirichlet mask", 6, 5, 4, 11, true);
    fails += check_level<3>("3-DOF level, no mask", 5, 4, 4, 12, false);
    fails += check_level<6>("6-DOF level, dead-DOF mask", 5, 4, 3, 13, true);
    fails += check_level<6>("6-DOF level, no mask", 4, 4, 3, 14, false);
    std::printf("failures %d\n", fails);
    return fails == 0 ? 0 : 1;
}
