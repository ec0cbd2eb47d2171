// Batched small-strain displacement element kernels (C3D8 / C3D20 families).
//
// One kernel launch evaluates every element of a group: shape-function
// gradients, strain increment, the constitutive update per Gauss point
// (linear elastic or J2 radial return in FP64), the element residual Pe in
// FP64 and the element stiffness Ke (FP32 or FP64) as 3x3 node-pair blocks.
//
// Reference semantics (EdelweissFE):
//   elements/displacementelement/element.py:290-346   computeYourself
//   elements/displacementelement/_elementcomputationmatrices.py:306-366,679-817 (hex8)
//   elements/displacementelement/_elementcomputationmatrices.py:369-495,820+   (hex20)
//   materials/linearelastic/linearelastic.py:95-125,185-210
//   materials/vonmises/vonmises.py:35-56,105-124,186-254
//
// Thread mapping: TPE threads per element (8 for <= 8 Gauss points, 32
// otherwise); thread `lane` of an element owns Gauss point `lane` for the
// constitutive phase, node `lane` for the residual phase and node pairs
// lane, lane+TPE, ... for the stiffness phase.  Per-element scratch lives in
// shared memory; the state is structure-of-arrays [var][element*nQP + qp] so
// that the constitutive phase reads and writes it coalesced.

#include <math.h>

#include "dfloat_bits.h"
#include "ef_common.cuh"
#include "materials.h"

namespace ef {

constexpr int kBlock = 128;

template <int NN>
struct PairTab {
    static constexpr int NP = NN * (NN + 1) / 2;
};

__device__ __forceinline__ int pair_a(int p, int nn) {
    // inverse of p(a,b) = a*nn - a*(a-1)/2 + (b-a), a <= b
    int a = 0;
    int start = 0;
    while (start + (nn - a) <= p) {
        start += nn - a;
        ++a;
    }
    return a;
}

// Double-float arithmetic (Dekker 1971; Knuth's TwoSum): a value is an unevaluated pair of
// FP32 numbers hi + lo with |lo| <= ulp(hi) / 2, about 48 significant bits.  The element kernel
// forms its strain and residual contractions this way on the FP32 pipe, because the FP64 pipe
// of this GPU (2 lanes per SM and cycle) bounds the kernel.  The rounded operations are written
// with the _rn intrinsics so that the compiler cannot contract them into FMAs.
struct DF {
    float hi, lo;
};

__host__ __device__ __forceinline__ float2 df_split(double d) {
    const float hi = (float)d;
    return make_float2(hi, (float)(d - (double)hi));
}

__device__ __forceinline__ double df_value(const DF& a) { return (double)a.hi + (double)a.lo; }

// the same conversions by integer operations on the bit patterns (dfloat_bits.h), which keep them
// off the FP64 pipe; hi is truncated instead of rounded (the pair still holds 47 bits)
__device__ __forceinline__ float2 df_split_i(double d) {
    uint32_t h, l;
    split_bits((uint64_t)__double_as_longlong(d), &h, &l);
    return make_float2(__uint_as_float(h), __uint_as_float(l));
}
__device__ __forceinline__ double widen_i(float f) { return __longlong_as_double((long long)widen_bits(__float_as_uint(f))); }
__device__ __forceinline__ double df_value_i(const DF& a) { return widen_i(a.hi) + widen_i(a.lo); }
__device__ __forceinline__ float2 df_split_sel(double d, int intConv) { return intConv ? df_split_i(d) : df_split(d); }
__device__ __forceinline__ double df_value_sel(const DF& a, int intConv) {
    return intConv ? df_value_i(a) : df_value(a);
}
// NaN test: a floating-point compare (FP64 pipe), or with intConv the exponent-all-ones,
// nonzero-fraction test on the bit pattern (integer pipe)
__device__ __forceinline__ bool is_nan_sel(double x, int intConv) {
    if (intConv) return ((unsigned long long)__double_as_longlong(x) << 1) > (0x7FF0000000000000ull << 1);
    return !(x == x);
}

// acc += a * b for a = (ah, al), b = (bh, bl): the product ah bh exactly (its rounding error from
// an FMA), the cross terms ah bl + al bh in FP32 (relative 2^-24 of the product), al bl dropped
// (2^-48); the sum with acc.hi by TwoSum, every error term into acc.lo
__device__ __forceinline__ void df_fma(DF& acc, float2 a, float2 b) {
    const float p = __fmul_rn(a.x, b.x);
    const float pe = __fmaf_rn(a.x, b.x, -p);
    const float x = __fmaf_rn(a.x, b.y, __fmul_rn(a.y, b.x));
    const float s = __fadd_rn(acc.hi, p);
    const float bv = __fsub_rn(s, acc.hi);
    const float err = __fadd_rn(__fsub_rn(acc.hi, __fsub_rn(s, bv)), __fsub_rn(p, bv));
    acc.hi = s;
    acc.lo = __fadd_rn(acc.lo, __fadd_rn(err, __fadd_rn(pe, x)));
}

// Gauss-point geometry in FP64: J = dN/dS x (reference formulation, including the C3D20
// row-2 Jacobian term), det J and g_a = dN_a/dx = inv(J) dN_a/dS.
template <int NN>
__device__ __forceinline__ double qp_geometry(const ElemTables* __restrict__ T, int q, const double (*xr)[3],
                                              double (*g)[3]) {
    double J[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            double s = 0;
#pragma unroll
            for (int a = 0; a < NN; ++a) s += T->dNdS_d[q][r][a] * xr[a][c];
            J[r][c] = s;
        }
    if (NN == 20 && T->quirk) {
        // reference _J3D20 (_elementcomputationmatrices.py:481-495) row-2 term a5*zeta instead of a5*xi
        const double f = T->quirkFac[q];
#pragma unroll
        for (int c = 0; c < 3; ++c) J[2][c] += f * 0.25 * (-xr[9][c] + xr[11][c] + xr[13][c] - xr[15][c]);
    }
    const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
    const double id = 1.0 / det;
    double iJ[3][3];
    iJ[0][0] = c00 * id;
    iJ[1][0] = c01 * id;
    iJ[2][0] = c02 * id;
    iJ[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
    iJ[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
    iJ[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
    iJ[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
    iJ[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
    iJ[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
    for (int a = 0; a < NN; ++a)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            g[a][c] = iJ[c][0] * T->dNdS_d[q][0][a] + iJ[c][1] * T->dNdS_d[q][1][a] + iJ[c][2] * T->dNdS_d[q][2][a];
    return det;
}

// Geometry cache, computed once per element group (initializeElement, element.py:194-205):
// geo[(e*NQ + q) * (3*NN + 1) + 3a + c] = dN_a/dx_c, last entry = w_q det J.
template <int NN, int NQ>
__global__ void geometry_kernel(const ElemTables* __restrict__ T, int nEl, const int32_t* __restrict__ nodeDof,
                                const double* __restrict__ X, double* __restrict__ geo, float2* __restrict__ geoS,
                                int* __restrict__ flags) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)nEl * NQ) return;
    const int64_t e = t / NQ;
    const int q = (int)(t % NQ);
    double xr[NN][3];
    const int d0 = nodeDof[e * NN];
    for (int a = 0; a < NN; ++a) {
        const int d = nodeDof[e * NN + a];
#pragma unroll
        for (int c = 0; c < 3; ++c) xr[a][c] = X[d + c] - X[d0 + c];
    }
    double g[NN][3];
    const double det = qp_geometry<NN>(T, q, xr, g);
    if (!(det > 0.0)) atomicOr(flags, EF_FLAG_BADDET);
    double* o = geo + t * (3 * NN + 1);
    for (int a = 0; a < NN; ++a)
#pragma unroll
        for (int c = 0; c < 3; ++c) o[3 * a + c] = g[a][c];
    o[3 * NN] = T->w[q] * det;
    if (geoS) {
        float2* os = geoS + t * (3 * NN + 1);
        for (int k = 0; k <= 3 * NN; ++k) os[k] = df_split(o[k]);
    }
}

// a split value in the stiffness precision: hi for FP32, hi + lo for FP64
template <typename KT>
__device__ __forceinline__ KT gk_value(float2 v);
template <>
__device__ __forceinline__ float gk_value<float>(float2 v) {
    return v.x;
}
template <>
__device__ __forceinline__ double gk_value<double>(float2 v) {
    return (double)v.x + (double)v.y;
}

template <int NN, int NQ, typename KT>
struct SSShared {
    static constexpr int TPE = (NQ <= 8) ? 8 : 32;
    static constexpr int EPB = kBlock / TPE;
    // per-element rows padded by one entry, so that the elements of a warp fall on different banks
    float2 du[EPB][NN * 3 + 1];       // dU split into FP32 pairs, [3a + i]
    float2 g[EPB][NQ * NN * 3 + 1];   // dN/dx split into FP32 pairs, [(q NN + a) 3 + c] (the FP32 stiffness reads hi)
    float2 sw[EPB][NQ * 6 + 1];       // sigma w detJ split into FP32 pairs, [6q + i]
    KT tn[EPB][NQ][9];                // lt*w, mt*w, c1*w, n[6]
};

// Element loop of one group: strain increment, constitutive update, Pe (FP64) and Ke blocks (KT).
template <int NN, int NQ, typename KT, int MAT, bool VIJ>
__global__ void __launch_bounds__(kBlock, 5) small_strain_kernel(
    int nEl, const int32_t* __restrict__ nodeDof, const float2* __restrict__ geoS, const double* __restrict__ dU,
    const double* __restrict__ stateIn, double* __restrict__ stateOut, PropsArg props,
    const double* __restrict__ propsTable, const int32_t* __restrict__ elemRow, KT* __restrict__ Kout,
    double* __restrict__ Pe, double* __restrict__ tang, int* __restrict__ flags, int intConv) {
    constexpr int TPE = (NQ <= 8) ? 8 : 32;
    constexpr int EPB = kBlock / TPE;
    constexpr int NP = PairTab<NN>::NP;
    constexpr int ND = 3 * NN;
    constexpr int NG = 3 * NN + 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SSShared<NN, NQ, KT>& sh = *reinterpret_cast<SSShared<NN, NQ, KT>*>(smem_raw);
    const int tid = threadIdx.x;
    const int le = tid / TPE;
    const int lane = tid % TPE;
    const int e = blockIdx.x * EPB + le;
    const bool valid = e < nEl;

    if (valid) {
        for (int a = lane; a < NN; a += TPE) {
            const int d = nodeDof[(int64_t)e * NN + a];
            sh.du[le][3 * a + 0] = df_split_sel(dU[d + 0], intConv);
            sh.du[le][3 * a + 1] = df_split_sel(dU[d + 1], intConv);
            sh.du[le][3 * a + 2] = df_split_sel(dU[d + 2], intConv);
        }
    }
    __syncthreads();

    // ---- Gauss-point phase ---------------------------------------------------
    if (valid && lane < NQ) {
        const int q = lane;
        const float2* gq = geoS + ((int64_t)e * NQ + q) * NG;
        // displacement-increment gradient H = sum_a dU_a (x) g_a in double-float arithmetic
        DF H[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) H[i][j] = DF{0.f, 0.f};
#pragma unroll 4
        for (int a = 0; a < NN; ++a) {
            float2 ga[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                ga[c] = gq[3 * a + c];
                sh.g[le][(q * NN + a) * 3 + c] = ga[c];
            }
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const float2 u = sh.du[le][3 * a + i];
#pragma unroll
                for (int j = 0; j < 3; ++j) df_fma(H[i][j], u, ga[j]);
            }
        }
        const float2 wq = gq[3 * NN];
        const double wdet = df_value_sel(DF{wq.x, wq.y}, intConv);
        const double de[6] = {df_value_sel(H[0][0], intConv), df_value_sel(H[1][1], intConv),
                              df_value_sel(H[2][2], intConv),
                              df_value_sel(H[0][1], intConv) + df_value_sel(H[1][0], intConv),
                              df_value_sel(H[0][2], intConv) + df_value_sel(H[2][0], intConv),
                              df_value_sel(H[1][2], intConv) + df_value_sel(H[2][1], intConv)};
        const int64_t nQPtot = (int64_t)nEl * NQ;
        const int64_t qi = (int64_t)e * NQ + q;
        double sig[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) sig[i] = stateIn[i * nQPtot + qi];
        MatOut mo;
        const double* pv = propsTable ? propsTable + 8 * (int64_t)elemRow[e] : props.v;
        if (MAT == MAT_VON_MISES) {
            double kap = stateIn[12 * nQPtot + qi];
            if (!mat_von_mises(pv, sig, &kap, de, mo)) {
                atomicOr(flags, EF_FLAG_RETURNMAP);
                atomicMin(flags + 1, __float_as_int(props.cutback));
            }
            stateOut[12 * nQPtot + qi] = kap;
            if (is_nan_sel(kap, intConv)) atomicOr(flags, EF_FLAG_NAN);
        } else {
            mat_linear_elastic(pv, sig, de, mo);
        }
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            stateOut[i * nQPtot + qi] = sig[i];
            stateOut[(6 + i) * nQPtot + qi] = stateIn[(6 + i) * nQPtot + qi] + de[i];
            if (is_nan_sel(sig[i], intConv)) atomicOr(flags, EF_FLAG_NAN);
        }
#pragma unroll
        for (int i = 0; i < 6; ++i) sh.sw[le][6 * q + i] = df_split_sel(sig[i] * wdet, intConv);
        if (tang) {
            // FP64 tangent of this Gauss point for the exact (matrix-free) refinement residual
            tang[0 * nQPtot + qi] = mo.lt * wdet;
            tang[1 * nQPtot + qi] = mo.mt * wdet;
            tang[2 * nQPtot + qi] = mo.c1 * wdet;
#pragma unroll
            for (int i = 0; i < 6; ++i) tang[(3 + i) * nQPtot + qi] = mo.c1 != 0.0 ? mo.n[i] : 0.0;
        }
        sh.tn[le][q][0] = (KT)(mo.lt * wdet);
        sh.tn[le][q][1] = (KT)(mo.mt * wdet);
        sh.tn[le][q][2] = (KT)(mo.c1 * wdet);
        if (mo.c1 != 0.0) {
#pragma unroll
            for (int i = 0; i < 6; ++i) sh.tn[le][q][3 + i] = (KT)mo.n[i];
        }
    }
    __syncthreads();
    if (!valid) return;

    // ---- residual: Pe_a = -sum_q (sigma w detJ) . g_qa  (double-float accumulation) ----
    for (int a = lane; a < NN; a += TPE) {
        DF f0{0.f, 0.f}, f1{0.f, 0.f}, f2{0.f, 0.f};
#pragma unroll 2
        for (int q = 0; q < NQ; ++q) {
            const float2* s = &sh.sw[le][6 * q];
            const float2* gg = &sh.g[le][(q * NN + a) * 3];
            const float2 gx = gg[0], gy = gg[1], gz = gg[2];
            df_fma(f0, s[0], gx);
            df_fma(f0, s[3], gy);
            df_fma(f0, s[4], gz);
            df_fma(f1, s[3], gx);
            df_fma(f1, s[1], gy);
            df_fma(f1, s[5], gz);
            df_fma(f2, s[4], gx);
            df_fma(f2, s[5], gy);
            df_fma(f2, s[2], gz);
        }
        double* pe = Pe + (int64_t)e * ND + 3 * a;
        pe[0] = -df_value_sel(f0, intConv);
        pe[1] = -df_value_sel(f1, intConv);
        pe[2] = -df_value_sel(f2, intConv);
    }

    // ---- stiffness: K_ab = sum_q lt ga(x)gb + mt (gb(x)ga + ga.gb I) - c1 va(x)vb ----
    for (int p = lane; p < NP; p += TPE) {
        const int a = pair_a(p, NN);
        const int b = a + (p - (a * NN - a * (a - 1) / 2));
        KT k[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (int q = 0; q < NQ; ++q) {
            const KT* tn = sh.tn[le][q];
            const float2* gA = &sh.g[le][(q * NN + a) * 3];
            const float2* gB = &sh.g[le][(q * NN + b) * 3];
            const KT ga0 = gk_value<KT>(gA[0]), ga1 = gk_value<KT>(gA[1]), ga2 = gk_value<KT>(gA[2]);
            const KT gb0 = gk_value<KT>(gB[0]), gb1 = gk_value<KT>(gB[1]), gb2 = gk_value<KT>(gB[2]);
            const KT lt = tn[0], mt = tn[1], c1 = tn[2];
            const KT s = mt * (ga0 * gb0 + ga1 * gb1 + ga2 * gb2);
            const KT la[3] = {lt * ga0, lt * ga1, lt * ga2};
            const KT ma[3] = {mt * gb0, mt * gb1, mt * gb2};
            const KT gaa[3] = {ga0, ga1, ga2};
            const KT gbb[3] = {gb0, gb1, gb2};
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) k[i][j] += la[i] * gbb[j] + ma[i] * gaa[j];
#pragma unroll
            for (int i = 0; i < 3; ++i) k[i][i] += s;
            if (c1 != (KT)0) {
                const KT* n = tn + 3;
                const KT va[3] = {n[0] * ga0 + n[3] * ga1 + n[4] * ga2, n[3] * ga0 + n[1] * ga1 + n[5] * ga2,
                                  n[4] * ga0 + n[5] * ga1 + n[2] * ga2};
                const KT vb[3] = {n[0] * gb0 + n[3] * gb1 + n[4] * gb2, n[3] * gb0 + n[1] * gb1 + n[5] * gb2,
                                  n[4] * gb0 + n[5] * gb1 + n[2] * gb2};
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int j = 0; j < 3; ++j) k[i][j] -= c1 * va[i] * vb[j];
            }
        }
        if (VIJ) {
            // reference VIJ layout: value a*n+b of the element slice holds Ke[a][b]
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

// y_e = K_e x_e with the FP64 Gauss-point tangents stored by the assembly (matrix-free, FP64).
// Used for the residual of the iterative refinement, so that a mixed-precision solve is exact
// for the FP64 tangent.
template <int NN, int NQ>
struct ApplyShared {
    static constexpr int TPE = (NQ <= 8) ? 8 : 32;
    static constexpr int EPB = kBlock / TPE;
    // per-element rows padded by one entry (bank spread of the elements of a warp)
    double xv[EPB][NN * 3 + 1];
    double g[EPB][NQ * NN * 3 + 1];
    double sw[EPB][NQ * 6 + 1];
};

template <int NN, int NQ>
__global__ void __launch_bounds__(kBlock) small_strain_apply_kernel(int nEl, const int32_t* __restrict__ nodeDof,
                                                                    const double* __restrict__ geo,
                                                                    const double* __restrict__ x,
                                                                    const double* __restrict__ tang,
                                                                    double* __restrict__ ye) {
    constexpr int TPE = (NQ <= 8) ? 8 : 32;
    constexpr int EPB = kBlock / TPE;
    constexpr int ND = 3 * NN;
    constexpr int NG = 3 * NN + 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ApplyShared<NN, NQ>& sh = *reinterpret_cast<ApplyShared<NN, NQ>*>(smem_raw);
    const int tid = threadIdx.x;
    const int le = tid / TPE;
    const int lane = tid % TPE;
    const int e = blockIdx.x * EPB + le;
    const bool valid = e < nEl;
    if (valid) {
        for (int a = lane; a < NN; a += TPE) {
            const int d = nodeDof[(int64_t)e * NN + a];
            sh.xv[le][3 * a + 0] = x[d + 0];
            sh.xv[le][3 * a + 1] = x[d + 1];
            sh.xv[le][3 * a + 2] = x[d + 2];
        }
    }
    __syncthreads();
    if (valid && lane < NQ) {
        const int q = lane;
        const double* gq = geo + ((int64_t)e * NQ + q) * NG;
        double H[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
        for (int a = 0; a < NN; ++a) {
#pragma unroll
            for (int c = 0; c < 3; ++c) sh.g[le][(q * NN + a) * 3 + c] = gq[3 * a + c];
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) H[i][j] += sh.xv[le][3 * a + i] * sh.g[le][(q * NN + a) * 3 + j];
        }
        const double ep[6] = {H[0][0], H[1][1], H[2][2], H[0][1] + H[1][0], H[0][2] + H[2][0], H[1][2] + H[2][1]};
        const int64_t nQPtot = (int64_t)nEl * NQ;
        const int64_t qi = (int64_t)e * NQ + q;
        const double lt = tang[qi], mt = tang[nQPtot + qi], c1 = tang[2 * nQPtot + qi];
        const double tr = ep[0] + ep[1] + ep[2];
        double ne = 0.0, n[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) n[i] = 0.0;
        if (c1 != 0.0) {
#pragma unroll
            for (int i = 0; i < 6; ++i) {
                n[i] = tang[(3 + i) * nQPtot + qi];
                ne += n[i] * ep[i];
            }
        }
        // sigma = (lt 1x1 + 2 mt I_s - c1 n x n) eps   (weights already in lt, mt, c1)
#pragma unroll
        for (int i = 0; i < 3; ++i) sh.sw[le][6 * q + i] = lt * tr + 2.0 * mt * ep[i] - c1 * n[i] * ne;
#pragma unroll
        for (int i = 3; i < 6; ++i) sh.sw[le][6 * q + i] = mt * ep[i] - c1 * n[i] * ne;
    }
    __syncthreads();
    if (!valid) return;
    for (int a = lane; a < NN; a += TPE) {
        double f0 = 0, f1 = 0, f2 = 0;
        for (int q = 0; q < NQ; ++q) {
            const double* s = &sh.sw[le][6 * q];
            const double* gg = &sh.g[le][(q * NN + a) * 3];
            const double gx = gg[0], gy = gg[1], gz = gg[2];
            f0 += s[0] * gx + s[3] * gy + s[4] * gz;
            f1 += s[3] * gx + s[1] * gy + s[5] * gz;
            f2 += s[4] * gx + s[5] * gy + s[2] * gz;
        }
        double* o = ye + (int64_t)e * ND + 3 * a;
        o[0] = f0;
        o[1] = f1;
        o[2] = f2;
    }
}

// The same product with the contractions in double-float arithmetic on the FP32 pipe (the FP64
// pipe of this GPU executes 2 lanes per SM and cycle): x split once into FP32 pairs, the
// geometry read from the split cache, H = sum_a x_a (x) g_a and y_a = sum_q sigma_q . g_qa as
// double-float sums (about 48 significant bits, as the element kernel's strain increment and
// residual), the Gauss-point stress from the FP64 tangent in FP64.
template <int NN, int NQ>
struct ApplyDFShared {
    static constexpr int TPE = (NQ <= 8) ? 8 : 32;
    static constexpr int EPB = kBlock / TPE;
    float2 xv[EPB][NN * 3 + 1];
    float2 g[EPB][NQ * NN * 3 + 1];
    float2 sw[EPB][NQ * 6 + 1];
};

template <int NN, int NQ>
__global__ void __launch_bounds__(kBlock) small_strain_apply_df_kernel(int nEl, const int32_t* __restrict__ nodeDof,
                                                                       const float2* __restrict__ geoS,
                                                                       const double* __restrict__ x,
                                                                       const double* __restrict__ tang,
                                                                       double* __restrict__ ye, int intConv) {
    constexpr int TPE = (NQ <= 8) ? 8 : 32;
    constexpr int EPB = kBlock / TPE;
    constexpr int ND = 3 * NN;
    constexpr int NG = 3 * NN + 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ApplyDFShared<NN, NQ>& sh = *reinterpret_cast<ApplyDFShared<NN, NQ>*>(smem_raw);
    const int tid = threadIdx.x;
    const int le = tid / TPE;
    const int lane = tid % TPE;
    const int e = blockIdx.x * EPB + le;
    const bool valid = e < nEl;
    if (valid) {
        for (int a = lane; a < NN; a += TPE) {
            const int d = nodeDof[(int64_t)e * NN + a];
            sh.xv[le][3 * a + 0] = df_split_sel(x[d + 0], intConv);
            sh.xv[le][3 * a + 1] = df_split_sel(x[d + 1], intConv);
            sh.xv[le][3 * a + 2] = df_split_sel(x[d + 2], intConv);
        }
    }
    __syncthreads();
    if (valid && lane < NQ) {
        const int q = lane;
        const float2* gq = geoS + ((int64_t)e * NQ + q) * NG;
        DF H[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) H[i][j] = DF{0.f, 0.f};
#pragma unroll 4
        for (int a = 0; a < NN; ++a) {
            float2 ga[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                ga[c] = gq[3 * a + c];
                sh.g[le][(q * NN + a) * 3 + c] = ga[c];
            }
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const float2 u = sh.xv[le][3 * a + i];
#pragma unroll
                for (int j = 0; j < 3; ++j) df_fma(H[i][j], u, ga[j]);
            }
        }
        const double ep[6] = {df_value_sel(H[0][0], intConv), df_value_sel(H[1][1], intConv),
                              df_value_sel(H[2][2], intConv),
                              df_value_sel(H[0][1], intConv) + df_value_sel(H[1][0], intConv),
                              df_value_sel(H[0][2], intConv) + df_value_sel(H[2][0], intConv),
                              df_value_sel(H[1][2], intConv) + df_value_sel(H[2][1], intConv)};
        const int64_t nQPtot = (int64_t)nEl * NQ;
        const int64_t qi = (int64_t)e * NQ + q;
        const double lt = tang[qi], mt = tang[nQPtot + qi], c1 = tang[2 * nQPtot + qi];
        const double tr = ep[0] + ep[1] + ep[2];
        double ne = 0.0, n[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) n[i] = 0.0;
        if (c1 != 0.0) {
#pragma unroll
            for (int i = 0; i < 6; ++i) {
                n[i] = tang[(3 + i) * nQPtot + qi];
                ne += n[i] * ep[i];
            }
        }
        // sigma = (lt 1x1 + 2 mt I_s - c1 n x n) eps   (weights already in lt, mt, c1)
#pragma unroll
        for (int i = 0; i < 3; ++i) sh.sw[le][6 * q + i] = df_split_sel(lt * tr + 2.0 * mt * ep[i] - c1 * n[i] * ne, intConv);
#pragma unroll
        for (int i = 3; i < 6; ++i) sh.sw[le][6 * q + i] = df_split_sel(mt * ep[i] - c1 * n[i] * ne, intConv);
    }
    __syncthreads();
    if (!valid) return;
    for (int a = lane; a < NN; a += TPE) {
        DF f0{0.f, 0.f}, f1{0.f, 0.f}, f2{0.f, 0.f};
#pragma unroll 2
        for (int q = 0; q < NQ; ++q) {
            const float2* sq = &sh.sw[le][6 * q];
            const float2* gg = &sh.g[le][(q * NN + a) * 3];
            const float2 gx = gg[0], gy = gg[1], gz = gg[2];
            df_fma(f0, sq[0], gx);
            df_fma(f0, sq[3], gy);
            df_fma(f0, sq[4], gz);
            df_fma(f1, sq[3], gx);
            df_fma(f1, sq[1], gy);
            df_fma(f1, sq[5], gz);
            df_fma(f2, sq[4], gx);
            df_fma(f2, sq[5], gy);
            df_fma(f2, sq[2], gz);
        }
        double* o = ye + (int64_t)e * ND + 3 * a;
        o[0] = df_value_sel(f0, intConv);
        o[1] = df_value_sel(f1, intConv);
        o[2] = df_value_sel(f2, intConv);
    }
}

// The same product for elements with 8 Gauss points (TPE = 8 threads per element, a thread per
// Gauss point) without the per-element geometry and stress stages in shared memory (which held
// occupancy near a third): the Gauss-point thread keeps its stress, and for each node a forms
// its term sigma_q . g_qa (geometry re-read from L1) as a double-float value; the 8 threads of
// the element sum the terms by an xor butterfly of double-float additions (TwoSum of the high
// parts: its error term is exact, so both partners of a pair get the same sum and every lane
// ends with the same bits), and thread a keeps node a's result.  Only x is staged.
__device__ __forceinline__ DF df_add(DF a, DF b) {
    const float s = __fadd_rn(a.hi, b.hi);
    const float bv = __fsub_rn(s, a.hi);
    const float err = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bv)), __fsub_rn(b.hi, bv));
    return DF{s, __fadd_rn(__fadd_rn(a.lo, b.lo), err)};
}
__device__ __forceinline__ DF df_shfl_xor8(DF v, int o) {
    return DF{__shfl_xor_sync(0xffffffffu, v.hi, o, 8), __shfl_xor_sync(0xffffffffu, v.lo, o, 8)};
}

template <int NN>
__global__ void __launch_bounds__(kBlock) small_strain_apply_df8_kernel(int nEl, const int32_t* __restrict__ nodeDof,
                                                                        const float2* __restrict__ geoS,
                                                                        const double* __restrict__ x,
                                                                        const double* __restrict__ tang,
                                                                        double* __restrict__ ye, int intConv) {
    constexpr int NQ = 8, TPE = 8, EPB = kBlock / TPE;
    constexpr int ND = 3 * NN;
    constexpr int NG = 3 * NN + 1;
    __shared__ float2 xv[EPB][ND + 1];
    const int tid = threadIdx.x;
    const int le = tid / TPE;
    const int q = tid % TPE;
    const int e0 = blockIdx.x * EPB + le;
    const bool valid = e0 < nEl;
    const int e = valid ? e0 : nEl - 1;  // the last element's lanes keep the shuffles full
    for (int a = q; a < NN; a += TPE) {
        const int d = nodeDof[(int64_t)e * NN + a];
        xv[le][3 * a + 0] = df_split_sel(x[d + 0], intConv);
        xv[le][3 * a + 1] = df_split_sel(x[d + 1], intConv);
        xv[le][3 * a + 2] = df_split_sel(x[d + 2], intConv);
    }
    __syncthreads();
    const float2* gq = geoS + ((int64_t)e * NQ + q) * NG;
    DF H[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) H[i][j] = DF{0.f, 0.f};
#pragma unroll 4
    for (int a = 0; a < NN; ++a) {
        float2 ga[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) ga[c] = gq[3 * a + c];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const float2 u = xv[le][3 * a + i];
#pragma unroll
            for (int j = 0; j < 3; ++j) df_fma(H[i][j], u, ga[j]);
        }
    }
    const double ep[6] = {df_value_sel(H[0][0], intConv), df_value_sel(H[1][1], intConv),
                          df_value_sel(H[2][2], intConv),
                          df_value_sel(H[0][1], intConv) + df_value_sel(H[1][0], intConv),
                          df_value_sel(H[0][2], intConv) + df_value_sel(H[2][0], intConv),
                          df_value_sel(H[1][2], intConv) + df_value_sel(H[2][1], intConv)};
    const int64_t nQPtot = (int64_t)nEl * NQ;
    const int64_t qi = (int64_t)e * NQ + q;
    const double lt = tang[qi], mt = tang[nQPtot + qi], c1 = tang[2 * nQPtot + qi];
    const double tr = ep[0] + ep[1] + ep[2];
    double ne = 0.0, n[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) n[i] = 0.0;
    if (c1 != 0.0) {
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            n[i] = tang[(3 + i) * nQPtot + qi];
            ne += n[i] * ep[i];
        }
    }
    float2 sw[6];
#pragma unroll
    for (int i = 0; i < 3; ++i) sw[i] = df_split_sel(lt * tr + 2.0 * mt * ep[i] - c1 * n[i] * ne, intConv);
#pragma unroll
    for (int i = 3; i < 6; ++i) sw[i] = df_split_sel(mt * ep[i] - c1 * n[i] * ne, intConv);
    DF own0{0.f, 0.f}, own1{0.f, 0.f}, own2{0.f, 0.f};
#pragma unroll 2
    for (int a = 0; a < NN; ++a) {
        const float2 gx = gq[3 * a + 0], gy = gq[3 * a + 1], gz = gq[3 * a + 2];
        DF f0{0.f, 0.f}, f1{0.f, 0.f}, f2{0.f, 0.f};
        df_fma(f0, sw[0], gx);
        df_fma(f0, sw[3], gy);
        df_fma(f0, sw[4], gz);
        df_fma(f1, sw[3], gx);
        df_fma(f1, sw[1], gy);
        df_fma(f1, sw[5], gz);
        df_fma(f2, sw[4], gx);
        df_fma(f2, sw[5], gy);
        df_fma(f2, sw[2], gz);
#pragma unroll
        for (int o = 4; o > 0; o >>= 1) {
            f0 = df_add(f0, df_shfl_xor8(f0, o));
            f1 = df_add(f1, df_shfl_xor8(f1, o));
            f2 = df_add(f2, df_shfl_xor8(f2, o));
        }
        if ((a & (TPE - 1)) == q) {
            own0 = f0;
            own1 = f1;
            own2 = f2;
        }
        if ((a & (TPE - 1)) == TPE - 1 || a == NN - 1) {
            const int ao = (a & ~(TPE - 1)) + q;  // the node this lane owns in this group of 8
            if (valid && ao <= a) {
                double* o = ye + (int64_t)e * ND + 3 * ao;
                o[0] = df_value_sel(own0, intConv);
                o[1] = df_value_sel(own1, intConv);
                o[2] = df_value_sel(own2, intConv);
            }
        }
    }
}

// Consistent body force of a constant load vector (element.py:348-371): Pe[a,c] = load_c sum_q N_qa detJ_q w_q
template <int NN, int NQ>
__global__ void body_force_kernel(const ElemTables* __restrict__ T, int nEl, const double* __restrict__ geo,
                                  double l0, double l1, double l2, double* __restrict__ Pe) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nEl) return;
    constexpr int NG = 3 * NN + 1;
    double acc[NN];
    for (int a = 0; a < NN; ++a) acc[a] = 0.0;
    for (int q = 0; q < NQ; ++q) {
        const double wdet = geo[((int64_t)e * NQ + q) * NG + 3 * NN];
        for (int a = 0; a < NN; ++a) acc[a] += T->N[q][a] * wdet;
    }
    for (int a = 0; a < NN; ++a) {
        Pe[(int64_t)e * 3 * NN + 3 * a + 0] = l0 * acc[a];
        Pe[(int64_t)e * 3 * NN + 3 * a + 1] = l1 * acc[a];
        Pe[(int64_t)e * 3 * NN + 3 * a + 2] = l2 * acc[a];
    }
}

template <int NN, int NQ, typename KT, int MAT>
static ef_status launch_ss(const Group& g, const double* dU, void* K, int vij, double* Pe, double* tang, int* flags,
                           cudaStream_t s) {
    constexpr int EPB = SSShared<NN, NQ, KT>::EPB;
    const int grid = (g.nEl + EPB - 1) / EPB;
    PropsArg pa;
    for (int i = 0; i < 8; ++i) pa.v[i] = g.props[i];
    pa.cutback = g.cutback;
    const double* sIn = g.state[g.cur];
    double* sOut = g.state[1 - g.cur];
    if (grid == 0) return EF_OK;
    if (!g.geoS) {
        ef_set_error("small-strain kernel: split geometry cache missing");
        return EF_ERR_STATE;
    }
    const size_t smem = sizeof(SSShared<NN, NQ, KT>);
    if (vij) {
        auto k = small_strain_kernel<NN, NQ, KT, MAT, true>;
        EF_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k<<<grid, kBlock, smem, ef::counted(s)>>>(g.nEl, g.nodeDof, g.geoS, dU, sIn, sOut, pa, g.propsTable, g.elemRow,
                                                  (KT*)K, Pe, tang, flags, g.intConv);
    } else {
        auto k = small_strain_kernel<NN, NQ, KT, MAT, false>;
        EF_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k<<<grid, kBlock, smem, ef::counted(s)>>>(g.nEl, g.nodeDof, g.geoS, dU, sIn, sOut, pa, g.propsTable, g.elemRow,
                                                  (KT*)K, Pe, tang, flags, g.intConv);
    }
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

template <int NN, int NQ>
static ef_status dispatch_ss(const Group& g, const double* dU, void* K, int kDouble, int vij, double* Pe,
                             double* tang, int* flags, cudaStream_t s) {
    if (g.mat == MAT_VON_MISES)
        return kDouble ? launch_ss<NN, NQ, double, MAT_VON_MISES>(g, dU, K, vij, Pe, tang, flags, s)
                       : launch_ss<NN, NQ, float, MAT_VON_MISES>(g, dU, K, vij, Pe, tang, flags, s);
    if (g.mat == MAT_LINEAR_ELASTIC)
        return kDouble ? launch_ss<NN, NQ, double, MAT_LINEAR_ELASTIC>(g, dU, K, vij, Pe, tang, flags, s)
                       : launch_ss<NN, NQ, float, MAT_LINEAR_ELASTIC>(g, dU, K, vij, Pe, tang, flags, s);
    ef_set_error("material not available for small-strain elements");
    return EF_ERR_ARG;
}

template <int NN, int NQ>
static ef_status launch_apply(const Group& g, const double* x, const double* tang, double* ye, cudaStream_t s) {
    constexpr int EPB = ApplyShared<NN, NQ>::EPB;
    const int grid = (g.nEl + EPB - 1) / EPB;
    if (grid == 0) return EF_OK;
    static const bool fp64 = [] {
        const char* e = getenv("EF_APPLY_FP64");
        return e && atoi(e) != 0;
    }();
    static const bool staged = [] {
        const char* e = getenv("EF_APPLY_STAGED");
        return e && atoi(e) != 0;
    }();
    if (g.geoS && !fp64 && NQ == 8 && !staged) {  // 8 Gauss points: the butterfly form (EF_APPLY_STAGED=1: staged)
        small_strain_apply_df8_kernel<NN><<<(g.nEl + kBlock / 8 - 1) / (kBlock / 8), kBlock, 0, ef::counted(s)>>>(
            g.nEl, g.nodeDof, g.geoS, x, tang, ye, g.intConv);
        EF_CUDA(cudaGetLastError());
        return EF_OK;
    }
    if (g.geoS && !fp64) {  // double-float contractions (default); EF_APPLY_FP64=1: the FP64 kernel
        const size_t smemDF = sizeof(ApplyDFShared<NN, NQ>);
        auto kd = small_strain_apply_df_kernel<NN, NQ>;
        EF_CUDA(cudaFuncSetAttribute(kd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smemDF));
        kd<<<grid, kBlock, smemDF, ef::counted(s)>>>(g.nEl, g.nodeDof, g.geoS, x, tang, ye, g.intConv);
        EF_CUDA(cudaGetLastError());
        return EF_OK;
    }
    const size_t smem = sizeof(ApplyShared<NN, NQ>);
    auto k = small_strain_apply_kernel<NN, NQ>;
    EF_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k<<<grid, kBlock, smem, ef::counted(s)>>>(g.nEl, g.nodeDof, g.geo, x, tang, ye);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

template <int NN, int NQ>
static ef_status launch_geometry(const Group& g, const ElemTables* T, const double* X, int* flags, cudaStream_t s) {
    const int64_t n = (int64_t)g.nEl * NQ;
    if (n == 0) return EF_OK;
    geometry_kernel<NN, NQ><<<(int)((n + 127) / 128), 128, 0, ef::counted(s)>>>(T, g.nEl, g.nodeDof, X, g.geo, g.geoS,
                                                                              flags);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

}  // namespace ef

using namespace ef;

#define EF_FOR_TYPES(M) M(8, 8) M(8, 1) M(8, 27) M(20, 27) M(20, 8)

ef_status ef_launch_geometry(const Group& g, const ElemTables* T, const double* X, int* flags, cudaStream_t s) {
#define EF_G(NN_, NQ_) \
    if (g.nNodes == NN_ && g.nQP == NQ_) return launch_geometry<NN_, NQ_>(g, T, X, flags, s);
    EF_FOR_TYPES(EF_G)
#undef EF_G
    ef_set_error("unsupported element type");
    return EF_ERR_ARG;
}

ef_status ef_launch_small_strain(const Group& g, const double* dU, void* Kout, int kDouble, int kLayoutVIJ,
                                 double* Pe, double* tang, int* flags, cudaStream_t s) {
#define EF_SS(NN_, NQ_) \
    if (g.nNodes == NN_ && g.nQP == NQ_) return dispatch_ss<NN_, NQ_>(g, dU, Kout, kDouble, kLayoutVIJ, Pe, tang, flags, s);
    EF_FOR_TYPES(EF_SS)
#undef EF_SS
    ef_set_error("unsupported element type for the small-strain kernel");
    return EF_ERR_ARG;
}

ef_status ef_launch_small_strain_apply(const Group& g, const double* x, const double* tang, double* ye,
                                       cudaStream_t s) {
#define EF_AP(NN_, NQ_) \
    if (g.nNodes == NN_ && g.nQP == NQ_) return launch_apply<NN_, NQ_>(g, x, tang, ye, s);
    EF_FOR_TYPES(EF_AP)
#undef EF_AP
    ef_set_error("unsupported element type for the tangent apply");
    return EF_ERR_ARG;
}

ef_status ef_launch_body_force(const Group& g, const ElemTables* T, const double load[3], double* Pe, cudaStream_t s) {
    const int grid = (g.nEl + 127) / 128;
    if (grid == 0) return EF_OK;
#define EF_BF(NN_, NQ_)                                                                                   \
    if (g.nNodes == NN_ && g.nQP == NQ_) {                                                               \
        body_force_kernel<NN_, NQ_><<<grid, 128, 0, ef::counted(s)>>>(T, g.nEl, g.geo, load[0], load[1], load[2], Pe); \
        EF_CUDA(cudaGetLastError());                                                                     \
        return EF_OK;                                                                                    \
    }
    EF_FOR_TYPES(EF_BF)
#undef EF_BF
    ef_set_error("unsupported element type for body forces");
    return EF_ERR_ARG;
}
