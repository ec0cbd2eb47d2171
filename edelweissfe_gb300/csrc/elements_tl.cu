// Batched total-Lagrange hyperelastic element kernels (C3D8TL / C3D20TL families, NeoHookeWa).
//
// Reference semantics (EdelweissFE):
//   elements/displacementtlelement/element.py:346-427        computeYourself (hyperelastic branch)
//   elements/displacementtlelement/_elementcomputationmatrices.py:70-106 (F), :247-281 (nablaN),
//                                                             :284-306 (makeH2D)
//   materials/neohooke/neohookepencegouformulationa.py:107-141 computeKirchhoff
//
// Per Gauss point, with g0_a = dN_a/dX (geometry cache), F = I + sum_a U_a (x) g0_a, J = det F,
// lb = (K - 2mu/3)(J^2 - J) - mu, mb = (K - 2mu/3)(2J^2 - J), tau = mu F F^T + lb I:
//   g_a   = F^-T g0_a                                      (NAi of the reference)
//   Pe_a -= w detJ tau g_a                                 (= nablaN^T inv(F) tau)
//   K_ab += w detJ [mu (g0_a . g0_b) I + mb g_a (x) g_b - lb g_b (x) g_a]
// The stiffness is the reference's einsum over dtau/dF = mu(d_ik F_jl + F_il d_jk) + mb d_ij F^-1_lk
// minus the tau term, contracted in closed form: mu F g0_b (x) g_a - (tau g_b) (x) g_a reduces to
// -lb g_b (x) g_a because tau g_b = mu F g0_b + lb g_b.  The block K_ba equals K_ab^T, so only
// the node pairs a <= b are formed, as for the small-strain elements.
// State per Gauss point: [tau (11,22,33,12,23,13), Green-Lagrange E (11,22,33,2E12,2E23,2E13),
// strain-energy density W] (utils/voigtnotation.py doVoigtStress / doVoigtStrain).

#include <math.h>

#include "ef_common.cuh"

namespace ef {

constexpr int kTLBlock = 128;

__device__ __forceinline__ int tl_pair_a(int p, int nn) {
    int a = 0;
    int start = 0;
    while (start + (nn - a) <= p) {
        start += nn - a;
        ++a;
    }
    return a;
}

template <int NN, int NQ, typename KT>
struct TLShared {
    static constexpr int TPE = (NQ <= 8) ? 8 : 32;
    static constexpr int EPB = kTLBlock / TPE;
    double u[EPB][NN][3];
    double g0[EPB][NQ][NN][3];
    double g[EPB][NQ][NN][3];
    double tw[EPB][NQ][6];  // tau * w detJ (11,22,33,12,23,13)
    KT sc[EPB][NQ][3];      // mu w detJ, mb w detJ, lb w detJ
};

// F^-1 and det F of a 3x3 matrix
__device__ __forceinline__ double inv3(const double (*F)[3], double (*Fi)[3]) {
    const double c00 = F[1][1] * F[2][2] - F[1][2] * F[2][1];
    const double c01 = F[1][2] * F[2][0] - F[1][0] * F[2][2];
    const double c02 = F[1][0] * F[2][1] - F[1][1] * F[2][0];
    const double det = F[0][0] * c00 + F[0][1] * c01 + F[0][2] * c02;
    const double id = 1.0 / det;
    Fi[0][0] = c00 * id;
    Fi[1][0] = c01 * id;
    Fi[2][0] = c02 * id;
    Fi[0][1] = (F[0][2] * F[2][1] - F[0][1] * F[2][2]) * id;
    Fi[1][1] = (F[0][0] * F[2][2] - F[0][2] * F[2][0]) * id;
    Fi[2][1] = (F[0][1] * F[2][0] - F[0][0] * F[2][1]) * id;
    Fi[0][2] = (F[0][1] * F[1][2] - F[0][2] * F[1][1]) * id;
    Fi[1][2] = (F[0][2] * F[1][0] - F[0][0] * F[1][2]) * id;
    Fi[2][2] = (F[0][0] * F[1][1] - F[0][1] * F[1][0]) * id;
    return det;
}

template <int NN, int NQ, typename KT, bool VIJ>
__global__ void __launch_bounds__(kTLBlock) tl_kernel(int nEl, const int32_t* __restrict__ nodeDof,
                                                      const double* __restrict__ geo, const double* __restrict__ U,
                                                      double* __restrict__ stateOut, PropsArg props,
                                                      const double* __restrict__ propsTable,
                                                      const int32_t* __restrict__ elemRow,
                                                      KT* __restrict__ Kout, double* __restrict__ Pe,
                                                      double* __restrict__ tang, int* __restrict__ flags) {
    constexpr int TPE = (NQ <= 8) ? 8 : 32;
    constexpr int EPB = kTLBlock / TPE;
    constexpr int NP = NN * (NN + 1) / 2;
    constexpr int ND = 3 * NN;
    constexpr int NG = 3 * NN + 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TLShared<NN, NQ, KT>& sh = *reinterpret_cast<TLShared<NN, NQ, KT>*>(smem_raw);
    const int tid = threadIdx.x;
    const int le = tid / TPE;
    const int lane = tid % TPE;
    const int e = blockIdx.x * EPB + le;
    const bool valid = e < nEl;
    if (valid) {
        for (int a = lane; a < NN; a += TPE) {
            const int d = nodeDof[(int64_t)e * NN + a];
            sh.u[le][a][0] = U[d + 0];
            sh.u[le][a][1] = U[d + 1];
            sh.u[le][a][2] = U[d + 2];
        }
    }
    __syncthreads();

    // ---- Gauss-point phase: F, material, spatial gradients ------------------------------------
    if (valid && lane < NQ) {
        const int q = lane;
        const double* gq = geo + ((int64_t)e * NQ + q) * NG;
        double H[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (int a = 0; a < NN; ++a) {
            double ga[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                ga[c] = gq[3 * a + c];
                sh.g0[le][q][a][c] = ga[c];
            }
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) H[i][j] += sh.u[le][a][i] * ga[j];
        }
        const double wdet = gq[3 * NN];
        double F[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) F[i][j] = H[i][j] + (i == j ? 1.0 : 0.0);
        double Fi[3][3];
        const double J = inv3(F, Fi);
        const double* pv = propsTable ? propsTable + 8 * (int64_t)elemRow[e] : props.v;
        const double mu = pv[0], Kb = pv[1];
        const double kk = Kb - 2.0 / 3.0 * mu;
        const double lb = kk * (J * J - J) - mu;
        const double mb = kk * (2.0 * J * J - J);
        double b[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) b[i][j] = F[i][0] * F[j][0] + F[i][1] * F[j][1] + F[i][2] * F[j][2];
        double tau[6] = {mu * b[0][0] + lb, mu * b[1][1] + lb, mu * b[2][2] + lb,
                         mu * b[0][1],      mu * b[1][2],      mu * b[0][2]};
        // Green-Lagrange strain E = (H + H^T + H^T H) / 2
        double E[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
                E[i][j] = 0.5 * (H[i][j] + H[j][i] + H[0][i] * H[0][j] + H[1][i] * H[1][j] + H[2][i] * H[2][j]);
        const double I1 = b[0][0] + b[1][1] + b[2][2];
        const double W = mu / 2.0 * (I1 - 3.0) + (Kb / 2.0 - mu / 3.0) * (J - 1.0) * (J - 1.0) - mu * log(J);
        const int64_t nQPtot = (int64_t)nEl * NQ;
        const int64_t qi = (int64_t)e * NQ + q;
        const double sv[6] = {E[0][0], E[1][1], E[2][2], 2.0 * E[0][1], 2.0 * E[1][2], 2.0 * E[0][2]};
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            stateOut[i * nQPtot + qi] = tau[i];
            stateOut[(6 + i) * nQPtot + qi] = sv[i];
            if (!(tau[i] == tau[i])) atomicOr(flags, EF_FLAG_NAN);
        }
        stateOut[12 * nQPtot + qi] = W;
#pragma unroll
        for (int i = 0; i < 6; ++i) sh.tw[le][q][i] = tau[i] * wdet;
        sh.sc[le][q][0] = (KT)(mu * wdet);
        sh.sc[le][q][1] = (KT)(mb * wdet);
        sh.sc[le][q][2] = (KT)(lb * wdet);
        for (int a = 0; a < NN; ++a) {
            const double* g0 = sh.g0[le][q][a];
#pragma unroll
            for (int i = 0; i < 3; ++i) sh.g[le][q][a][i] = Fi[0][i] * g0[0] + Fi[1][i] * g0[1] + Fi[2][i] * g0[2];
        }
        if (tang) {
            // FP64 tangent data of this Gauss point for the matrix-free refinement residual
            tang[0 * nQPtot + qi] = mu * wdet;
            tang[1 * nQPtot + qi] = mb * wdet;
            tang[2 * nQPtot + qi] = lb * wdet;
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) tang[(3 + 3 * i + j) * nQPtot + qi] = Fi[i][j];
        }
    }
    __syncthreads();
    if (!valid) return;

    // ---- residual: Pe_a = -sum_q (tau w detJ) g_a (FP64) ---------------------------------------
    for (int a = lane; a < NN; a += TPE) {
        double f0 = 0, f1 = 0, f2 = 0;
        for (int q = 0; q < NQ; ++q) {
            const double* t = sh.tw[le][q];
            const double gx = sh.g[le][q][a][0], gy = sh.g[le][q][a][1], gz = sh.g[le][q][a][2];
            f0 += t[0] * gx + t[3] * gy + t[5] * gz;
            f1 += t[3] * gx + t[1] * gy + t[4] * gz;
            f2 += t[5] * gx + t[4] * gy + t[2] * gz;
        }
        double* pe = Pe + (int64_t)e * ND + 3 * a;
        pe[0] = -f0;
        pe[1] = -f1;
        pe[2] = -f2;
    }

    // ---- stiffness blocks a <= b ---------------------------------------------------------------
    for (int p = lane; p < NP; p += TPE) {
        const int a = tl_pair_a(p, NN);
        const int b = a + (p - (a * NN - a * (a - 1) / 2));
        KT k[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (int q = 0; q < NQ; ++q) {
            const KT mw = sh.sc[le][q][0], mbw = sh.sc[le][q][1], lbw = sh.sc[le][q][2];
            const double* g0a = sh.g0[le][q][a];
            const double* g0b = sh.g0[le][q][b];
            const KT d0 = (KT)(g0a[0] * g0b[0] + g0a[1] * g0b[1] + g0a[2] * g0b[2]);
            const KT ga[3] = {(KT)sh.g[le][q][a][0], (KT)sh.g[le][q][a][1], (KT)sh.g[le][q][a][2]};
            const KT gb[3] = {(KT)sh.g[le][q][b][0], (KT)sh.g[le][q][b][1], (KT)sh.g[le][q][b][2]};
            const KT s = mw * d0;
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) k[i][j] += mbw * ga[i] * gb[j] - lbw * gb[i] * ga[j];
#pragma unroll
            for (int i = 0; i < 3; ++i) k[i][i] += s;
        }
        if (VIJ) {
            KT* ke = Kout + (int64_t)e * ND * ND;
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    ke[(3 * a + i) * ND + 3 * b + j] = k[i][j];
                    if (a != b) ke[(3 * b + j) * ND + 3 * a + i] = k[i][j];
                }
        } else {
            KT* kb = Kout + ((int64_t)e * NP + p) * 9;
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) kb[i * 3 + j] = k[i][j];
        }
    }
}

// y_e = K_e x_e from the stored FP64 Gauss-point data (mu w, mb w, lb w, F^-1), matrix-free:
//   y_a = sum_q mu w Hx g0_a + mb w tr(F^-1 Hx) g_a - lb w F^-T Hx^T g_a,  Hx = sum_b x_b (x) g0_b
template <int NN, int NQ>
struct TLApplyShared {
    static constexpr int TPE = (NQ <= 8) ? 8 : 32;
    static constexpr int EPB = kTLBlock / TPE;
    double xv[EPB][NN][3];
    double A[EPB][NQ][9];   // per Gauss point: mu w Hx
    double Bm[EPB][NQ][9];  // per Gauss point: mb w tr(F^-1 Hx) F^-T - lb w F^-T Hx^T F^-T
};

template <int NN, int NQ>
__global__ void __launch_bounds__(kTLBlock) tl_apply_kernel(int nEl, const int32_t* __restrict__ nodeDof,
                                                            const double* __restrict__ geo,
                                                            const double* __restrict__ x,
                                                            const double* __restrict__ tang,
                                                            double* __restrict__ ye) {
    constexpr int TPE = (NQ <= 8) ? 8 : 32;
    constexpr int EPB = kTLBlock / TPE;
    constexpr int ND = 3 * NN;
    constexpr int NG = 3 * NN + 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TLApplyShared<NN, NQ>& sh = *reinterpret_cast<TLApplyShared<NN, NQ>*>(smem_raw);
    const int tid = threadIdx.x;
    const int le = tid / TPE;
    const int lane = tid % TPE;
    const int e = blockIdx.x * EPB + le;
    const bool valid = e < nEl;
    if (valid) {
        for (int a = lane; a < NN; a += TPE) {
            const int d = nodeDof[(int64_t)e * NN + a];
            sh.xv[le][a][0] = x[d + 0];
            sh.xv[le][a][1] = x[d + 1];
            sh.xv[le][a][2] = x[d + 2];
        }
    }
    __syncthreads();
    if (valid && lane < NQ) {
        const int q = lane;
        const double* gq = geo + ((int64_t)e * NQ + q) * NG;
        double Hx[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (int b = 0; b < NN; ++b)
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) Hx[i][j] += sh.xv[le][b][i] * gq[3 * b + j];
        const int64_t nQPtot = (int64_t)nEl * NQ;
        const int64_t qi = (int64_t)e * NQ + q;
        const double mw = tang[qi], mbw = tang[nQPtot + qi], lbw = tang[2 * nQPtot + qi];
        double Fi[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) Fi[i][j] = tang[(3 + 3 * i + j) * nQPtot + qi];
        double tr = 0.0;  // tr(F^-1 Hx)
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) tr += Fi[i][j] * Hx[j][i];
        // y_a = A g0_a + Bm g0_a with A = mu w Hx and, since g_a = F^-T g0_a,
        // Bm = (mb w tr) F^-T - lb w F^-T Hx^T F^-T
        double M[3][3];  // Hx^T F^-T
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) M[i][j] = Hx[0][i] * Fi[j][0] + Hx[1][i] * Fi[j][1] + Hx[2][i] * Fi[j][2];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                sh.A[le][q][3 * i + j] = mw * Hx[i][j];
                const double fm = Fi[0][i] * M[0][j] + Fi[1][i] * M[1][j] + Fi[2][i] * M[2][j];
                sh.Bm[le][q][3 * i + j] = mbw * tr * Fi[j][i] - lbw * fm;
            }
    }
    __syncthreads();
    if (!valid) return;
    for (int a = lane; a < NN; a += TPE) {
        double y0 = 0, y1 = 0, y2 = 0;
        for (int q = 0; q < NQ; ++q) {
            const double* gq = geo + ((int64_t)e * NQ + q) * NG + 3 * a;
            const double g0 = gq[0], g1 = gq[1], g2 = gq[2];
            const double* A = sh.A[le][q];
            const double* Bm = sh.Bm[le][q];
            y0 += (A[0] + Bm[0]) * g0 + (A[1] + Bm[1]) * g1 + (A[2] + Bm[2]) * g2;
            y1 += (A[3] + Bm[3]) * g0 + (A[4] + Bm[4]) * g1 + (A[5] + Bm[5]) * g2;
            y2 += (A[6] + Bm[6]) * g0 + (A[7] + Bm[7]) * g1 + (A[8] + Bm[8]) * g2;
        }
        double* o = ye + (int64_t)e * ND + 3 * a;
        o[0] = y0;
        o[1] = y1;
        o[2] = y2;
    }
}

template <int NN, int NQ, typename KT>
static ef_status launch_tl(const Group& g, const double* U, void* K, int vij, double* Pe, double* tang, int* flags,
                           cudaStream_t s) {
    constexpr int EPB = TLShared<NN, NQ, KT>::EPB;
    const int grid = (g.nEl + EPB - 1) / EPB;
    if (grid == 0) return EF_OK;
    PropsArg pa;
    for (int i = 0; i < 8; ++i) pa.v[i] = g.props[i];
    pa.cutback = g.cutback;
    double* sOut = g.state[1 - g.cur];
    const size_t smem = sizeof(TLShared<NN, NQ, KT>);
    if (vij) {
        auto k = tl_kernel<NN, NQ, KT, true>;
        EF_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k<<<grid, kTLBlock, smem, ef::counted(s)>>>(g.nEl, g.nodeDof, g.geo, U, sOut, pa, g.propsTable, g.elemRow,
                                                    (KT*)K, Pe, tang, flags);
    } else {
        auto k = tl_kernel<NN, NQ, KT, false>;
        EF_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k<<<grid, kTLBlock, smem, ef::counted(s)>>>(g.nEl, g.nodeDof, g.geo, U, sOut, pa, g.propsTable, g.elemRow,
                                                    (KT*)K, Pe, tang, flags);
    }
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

template <int NN, int NQ>
static ef_status launch_tl_apply(const Group& g, const double* x, const double* tang, double* ye, cudaStream_t s) {
    constexpr int EPB = TLApplyShared<NN, NQ>::EPB;
    const int grid = (g.nEl + EPB - 1) / EPB;
    if (grid == 0) return EF_OK;
    const size_t smem = sizeof(TLApplyShared<NN, NQ>);
    auto k = tl_apply_kernel<NN, NQ>;
    EF_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k<<<grid, kTLBlock, smem, ef::counted(s)>>>(g.nEl, g.nodeDof, g.geo, x, tang, ye);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

}  // namespace ef

using namespace ef;

#define EF_TL_TYPES(M) M(8, 8) M(8, 1) M(8, 27) M(20, 27) M(20, 8)

// Number of FP64 values per Gauss point that the total-Lagrange kernels keep for the
// matrix-free refinement residual.
int ef_tl_tangent_size() { return 12; }

ef_status ef_launch_total_lagrange(const Group& g, const double* U, void* Kout, int kDouble, int kLayoutVIJ,
                                   double* Pe, double* tang, int* flags, cudaStream_t s) {
    if (g.mat != MAT_NEOHOOKE_WA) {
        ef_set_error("total-Lagrange elements: material not available");
        return EF_ERR_ARG;
    }
#define EF_TL(NN_, NQ_)                                                                                \
    if (g.nNodes == NN_ && g.nQP == NQ_)                                                               \
        return kDouble ? launch_tl<NN_, NQ_, double>(g, U, Kout, kLayoutVIJ, Pe, tang, flags, s)       \
                       : launch_tl<NN_, NQ_, float>(g, U, Kout, kLayoutVIJ, Pe, tang, flags, s);
    EF_TL_TYPES(EF_TL)
#undef EF_TL
    ef_set_error("unsupported element type for the total-Lagrange kernel");
    return EF_ERR_ARG;
}

ef_status ef_launch_total_lagrange_apply(const Group& g, const double* x, const double* tang, double* ye,
                                         cudaStream_t s) {
#define EF_TA(NN_, NQ_) \
    if (g.nNodes == NN_ && g.nQP == NQ_) return launch_tl_apply<NN_, NQ_>(g, x, tang, ye, s);
    EF_TL_TYPES(EF_TA)
#undef EF_TA
    ef_set_error("unsupported element type for the total-Lagrange tangent apply");
    return EF_ERR_ARG;
}
