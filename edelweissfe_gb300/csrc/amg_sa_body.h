// Per-thread bodies of the smoothed-aggregation kernels (amg.cu), and the tentative prolongation
// block they share with the plain aggregation kernels.
//
// The kernels are thin wrappers that map a thread (or a warp lane) to one call of these
// functions.  The functions are plain C++ on fixed-width integers and float arithmetic, so the
// same source compiles for the device and for the host, where a test runs them over every index
// of a small system and checks the results against dense products (tests/native/amg_sa_check.cpp).
//
// Notation, for one level transition (finer level of block size BF, coarser of BC = 6):
//   P_t        tentative prolongator, block (m, agg(m)) = pblock(offset of m from its centroid)
//   P          = P_t - w D^-1 A P_t on the live finer DOFs, zero on masked finer rows
//   AP         = A P,   A_c = P^T A P (compensated FP32 sums, dead coarse DOFs identity)
// with A the finer operator whose masked rows and columns are dropped.  The index maps that list
// the terms of each sum in a fixed order come from amg_sa_pattern.h.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define EF_SA_HD __host__ __device__ __forceinline__
#define EF_SA_UNROLL _Pragma("unroll")
#else
#define EF_SA_HD inline
#define EF_SA_UNROLL
#endif

namespace ef {

constexpr int BC = 6;  // DOFs of a coarse node

// rounded FP32 sum and difference that the compiler may not fuse into an FMA (TwoSum needs both
// roundings); the host build of the test compiles with -ffp-contract=off
EF_SA_HD float sa_add_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
EF_SA_HD float sa_sub_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}

// the values of one block (8-byte aligned for BF = 3, 16-byte aligned for BF = 6)
template <int BF>
EF_SA_HD void sa_load_block(const float* __restrict__ src, float P[BF * BC]) {
#if defined(__CUDA_ARCH__)
    if constexpr (BF == 6) {
        const float4* s4 = reinterpret_cast<const float4*>(src);
        EF_SA_UNROLL
        for (int q = 0; q < BF * BC / 4; ++q) {
            const float4 v = __ldg(s4 + q);
            P[4 * q] = v.x;
            P[4 * q + 1] = v.y;
            P[4 * q + 2] = v.z;
            P[4 * q + 3] = v.w;
        }
    } else {
        const float2* s2 = reinterpret_cast<const float2*>(src);
        EF_SA_UNROLL
        for (int q = 0; q < BF * BC / 2; ++q) {
            const float2 v = __ldg(s2 + q);
            P[2 * q] = v.x;
            P[2 * q + 1] = v.y;
        }
    }
#else
    for (int p = 0; p < BF * BC; ++p) P[p] = src[p];
#endif
}

// the BF x BF block at d into registers: 6 x 6 blocks (144 bytes, 16-byte aligned) as 16-byte words
// on the device, 3 x 3 blocks (36 bytes, 4-byte aligned) value by value
template <int BF>
EF_SA_HD void sa_load_ablock(const float* __restrict__ d, float A[BF * BF]) {
#if defined(__CUDA_ARCH__)
    if constexpr (BF == 6) {
        const float4* d4 = reinterpret_cast<const float4*>(d);
        EF_SA_UNROLL
        for (int u = 0; u < 9; ++u) {
            const float4 w = d4[u];
            A[4 * u] = w.x;
            A[4 * u + 1] = w.y;
            A[4 * u + 2] = w.z;
            A[4 * u + 3] = w.w;
        }
        return;
    }
#endif
    for (int u = 0; u < BF * BF; ++u) A[u] = d[u];
}

// finer-node prolongation block, BF x 6: [I | R(d)] (BF = 3) or [I R(d) ; 0 I] (BF = 6) with
// R(d) = [e_x x d, e_y x d, e_z x d] and d the node's offset from its aggregate centroid
template <int BF>
EF_SA_HD void pblock(const float* __restrict__ d, float P[BF][BC]) {
    const float dx = d[0], dy = d[1], dz = d[2];
    EF_SA_UNROLL
    for (int i = 0; i < BF; ++i)
        EF_SA_UNROLL
        for (int j = 0; j < BC; ++j) P[i][j] = 0.f;
    P[0][0] = P[1][1] = P[2][2] = 1.f;
    // rotation columns: e_x x d = (0,-dz,dy), e_y x d = (dz,0,-dx), e_z x d = (-dy,dx,0)
    P[1][3] = -dz;
    P[2][3] = dy;
    P[0][4] = dz;
    P[2][4] = -dx;
    P[0][5] = -dy;
    P[1][5] = dx;
    if (BF == 6) {
        P[3 % BF][3] = 1.f;
        P[4 % BF][4] = 1.f;
        P[5 % BF][5] = 1.f;
    }
}

// P block b = (m = pRow[b], J = pCol[b]): the finer blocks k of row m whose column lies in
// aggregate J (pSrc[pSeg[b] .. pSeg[b+1])) give sum_k A_k P_t(col k); then
//   P(m, J) = [J == agg(m)] P_t(m) - w D_m^-1 sum_k A_k P_t(col k)
template <int BF>
EF_SA_HD void sa_prolongator_block(int64_t b, const int32_t* __restrict__ pRow, const int32_t* __restrict__ pCol,
                                   const int64_t* __restrict__ pSeg, const int32_t* __restrict__ pSrc,
                                   const int32_t* __restrict__ fineCol, const float* __restrict__ fineVals,
                                   const uint8_t* __restrict__ fineMask, const float* __restrict__ offs,
                                   const int32_t* __restrict__ agg, const float* __restrict__ binv, float w,
                                   float* __restrict__ Pv) {
    const int m = pRow[b], J = pCol[b];
    float acc[BF][BC];
    EF_SA_UNROLL
    for (int i = 0; i < BF; ++i)
        EF_SA_UNROLL
        for (int j = 0; j < BC; ++j) acc[i][j] = 0.f;
    bool mr[BF];
    EF_SA_UNROLL
    for (int i = 0; i < BF; ++i) mr[i] = fineMask && fineMask[BF * (int64_t)m + i];
    for (int64_t t = pSeg[b]; t < pSeg[b + 1]; ++t) {
        const int32_t k = pSrc[t];
        const int n = fineCol[k];
        float Pn[BF][BC];
        pblock<BF>(offs + 3 * (int64_t)n, Pn);
        float v[BF * BF];
        sa_load_ablock<BF>(fineVals + (int64_t)k * BF * BF, v);
        bool mc[BF];
        EF_SA_UNROLL
        for (int q = 0; q < BF; ++q) mc[q] = fineMask && fineMask[BF * (int64_t)n + q];
        EF_SA_UNROLL
        for (int i = 0; i < BF; ++i) {
            if (mr[i]) continue;
            EF_SA_UNROLL
            for (int q = 0; q < BF; ++q) {
                if (mc[q]) continue;
                const float a = v[i * BF + q];
                EF_SA_UNROLL
                for (int j = 0; j < BC; ++j) acc[i][j] += a * Pn[q][j];
            }
        }
    }
    float Pm[BF][BC];
    pblock<BF>(offs + 3 * (int64_t)m, Pm);
    const bool own = J == agg[m];
    const float* B = binv + (int64_t)m * BF * BF;
    float* out = Pv + b * BF * BC;
    EF_SA_UNROLL
    for (int i = 0; i < BF; ++i) {
        const bool masked = fineMask && fineMask[BF * (int64_t)m + i];
        EF_SA_UNROLL
        for (int j = 0; j < BC; ++j) {
            float z = 0.f;
            EF_SA_UNROLL
            for (int q = 0; q < BF; ++q) z += B[i * BF + q] * acc[q][j];
            out[i * BC + j] = masked ? 0.f : (own ? Pm[i][j] : 0.f) - w * z;
        }
    }
}

// AP block a = (m = apRow[a], J): sum over the pairs (finer block k of row m, P block (col k, J))
// listed in apK / apP[apSeg[a] .. apSeg[a+1])
template <int BF>
EF_SA_HD void sa_ap_block(int64_t a, const int32_t* __restrict__ apRow, const int64_t* __restrict__ apSeg,
                          const int32_t* __restrict__ apK, const int32_t* __restrict__ apP,
                          const int32_t* __restrict__ fineCol, const float* __restrict__ fineVals,
                          const uint8_t* __restrict__ fineMask, const float* __restrict__ Pv, float* __restrict__ APv) {
    const int m = apRow[a];
    float acc[BF][BC];
    EF_SA_UNROLL
    for (int i = 0; i < BF; ++i)
        EF_SA_UNROLL
        for (int j = 0; j < BC; ++j) acc[i][j] = 0.f;
    for (int64_t t = apSeg[a]; t < apSeg[a + 1]; ++t) {
        const int32_t k = apK[t];
        const int n = fineCol[k];
        const float* v = fineVals + (int64_t)k * BF * BF;
        const float* P = Pv + (int64_t)apP[t] * BF * BC;
        EF_SA_UNROLL
        for (int i = 0; i < BF; ++i) {
            if (fineMask && fineMask[BF * (int64_t)m + i]) continue;
            EF_SA_UNROLL
            for (int q = 0; q < BF; ++q) {
                if (fineMask && fineMask[BF * (int64_t)n + q]) continue;
                const float av = v[i * BF + q];
                EF_SA_UNROLL
                for (int j = 0; j < BC; ++j) acc[i][j] += av * P[q * BC + j];
            }
        }
    }
    float* out = APv + a * BF * BC;
    EF_SA_UNROLL
    for (int i = 0; i < BF; ++i)
        EF_SA_UNROLL
        for (int j = 0; j < BC; ++j) out[i * BC + j] = acc[i][j];
}

// AP pair t (finer block k = apK[t] of row m, P block apP[t] of row col(k)): c = A_k P_apP[t], rows
// of masked finer DOFs of row m and columns of masked finer DOFs of col(k) dropped.  Summed over
// the pairs of an AP block in their listed order this is the block of sa_ap_block (with the
// products of one pair rounded together).
template <int BF>
EF_SA_HD void sa_ap_pair(int64_t t, int m, const int32_t* __restrict__ apK, const int32_t* __restrict__ apP,
                         const int32_t* __restrict__ fineCol, const float* __restrict__ fineVals,
                         const uint8_t* __restrict__ fineMask, const float* __restrict__ Pv, float c[BF * BC]) {
    const int32_t k = apK[t];
    const int n = fineCol[k];
    float v[BF * BF];
    sa_load_ablock<BF>(fineVals + (int64_t)k * BF * BF, v);
    float P[BF * BC];
    sa_load_block<BF>(Pv + (int64_t)apP[t] * BF * BC, P);
    bool mr[BF], mc[BF];
    EF_SA_UNROLL
    for (int i = 0; i < BF; ++i) {
        mr[i] = fineMask && fineMask[BF * (int64_t)m + i];
        mc[i] = fineMask && fineMask[BF * (int64_t)n + i];
    }
    EF_SA_UNROLL
    for (int p = 0; p < BF * BC; ++p) c[p] = 0.f;
    EF_SA_UNROLL
    for (int i = 0; i < BF; ++i) {
        if (mr[i]) continue;
        EF_SA_UNROLL
        for (int q = 0; q < BF; ++q) {
            if (mc[q]) continue;
            const float av = v[i * BF + q];
            EF_SA_UNROLL
            for (int j = 0; j < BC; ++j) c[i * BC + j] += av * P[q * BC + j];
        }
    }
}

// coarse block S = (I, J): sum over the pairs (P block (m, I), AP block (m, J)) listed in
// cP / cAP[cSeg[S] .. cSeg[S+1]) of P^T AP, TwoSum-compensated; dead coarse DOFs get identity
// rows and columns
template <int BF>
EF_SA_HD void sa_galerkin_block(int64_t S, const int64_t* __restrict__ cSeg, const int32_t* __restrict__ cP,
                                const int32_t* __restrict__ cAP, const float* __restrict__ Pv,
                                const float* __restrict__ APv, const int32_t* __restrict__ coarseRowOfBlock,
                                const int32_t* __restrict__ coarseCol, const uint8_t* __restrict__ coarseDead,
                                float* __restrict__ coarseVals) {
    float hi[BC][BC], lo[BC][BC];
    EF_SA_UNROLL
    for (int i = 0; i < BC; ++i)
        EF_SA_UNROLL
        for (int j = 0; j < BC; ++j) hi[i][j] = lo[i][j] = 0.f;
    for (int64_t t = cSeg[S]; t < cSeg[S + 1]; ++t) {
        const float* P = Pv + (int64_t)cP[t] * BF * BC;
        const float* Q = APv + (int64_t)cAP[t] * BF * BC;
        EF_SA_UNROLL
        for (int i = 0; i < BC; ++i)
            EF_SA_UNROLL
            for (int j = 0; j < BC; ++j) {
                float s = 0.f;
                EF_SA_UNROLL
                for (int q = 0; q < BF; ++q) s += P[q * BC + i] * Q[q * BC + j];
                const float tt = sa_add_rn(hi[i][j], s);
                const float bv = sa_sub_rn(tt, hi[i][j]);
                lo[i][j] = sa_add_rn(lo[i][j], sa_add_rn(sa_sub_rn(hi[i][j], sa_sub_rn(tt, bv)), sa_sub_rn(s, bv)));
                hi[i][j] = tt;
            }
    }
    const int I = coarseRowOfBlock[S], J = coarseCol[S];
    EF_SA_UNROLL
    for (int i = 0; i < BC; ++i)
        EF_SA_UNROLL
        for (int j = 0; j < BC; ++j) {
            float a = sa_add_rn(hi[i][j], lo[i][j]);
            if (coarseDead[BC * (int64_t)I + i] || coarseDead[BC * (int64_t)J + j]) a = (I == J && i == j) ? 1.f : 0.f;
            coarseVals[S * BC * BC + i * BC + j] = a;
        }
}

// restriction rc[I] = sum over the P blocks b of column I of P_b^T t[row(b)]: the partial sum of
// one of nLanes lanes, which takes the blocks tPtr[I] + lane, + 2 lane, ... (the kernel adds the
// lanes of a warp with a fixed shuffle tree and zeroes dead coarse DOFs)
template <int BF>
EF_SA_HD void sa_restrict_partial(int I, int lane, int nLanes, const int32_t* __restrict__ tPtr,
                                  const int32_t* __restrict__ tIdx, const int32_t* __restrict__ pRow,
                                  const float* __restrict__ Pv, const float* __restrict__ t, float a[BC]) {
    EF_SA_UNROLL
    for (int j = 0; j < BC; ++j) a[j] = 0.f;
    for (int k = tPtr[I] + lane; k < tPtr[I + 1]; k += nLanes) {
        const int32_t b = tIdx[k];
        const int m = pRow[b];
        const float* P = Pv + (int64_t)b * BF * BC;
        EF_SA_UNROLL
        for (int i = 0; i < BF; ++i) {
            const float ti = t[BF * (int64_t)m + i];
            EF_SA_UNROLL
            for (int j = 0; j < BC; ++j) a[j] += P[i * BC + j] * ti;
        }
    }
}

// prolongation x[m] += alpha sum over the P blocks b of row m of P_b xc[col(b)], on the finer
// DOFs that the mask leaves free
template <int BF>
EF_SA_HD void sa_prolong_row(int m, const int32_t* __restrict__ pRowPtr, const int32_t* __restrict__ pCol,
                             const float* __restrict__ Pv, const float* __restrict__ xc,
                             const uint8_t* __restrict__ mask, float* __restrict__ x, float alpha) {
    float s[BF];
    EF_SA_UNROLL
    for (int i = 0; i < BF; ++i) s[i] = 0.f;
    for (int b = pRowPtr[m]; b < pRowPtr[m + 1]; ++b) {
        const float* P = Pv + (int64_t)b * BF * BC;
        const float* c = xc + BC * (int64_t)pCol[b];
        float cv[BC];
        EF_SA_UNROLL
        for (int j = 0; j < BC; ++j) cv[j] = c[j];
        EF_SA_UNROLL
        for (int i = 0; i < BF; ++i)
            EF_SA_UNROLL
            for (int j = 0; j < BC; ++j) s[i] += P[i * BC + j] * cv[j];
    }
    EF_SA_UNROLL
    for (int i = 0; i < BF; ++i)
        if (!(mask && mask[BF * (int64_t)m + i])) x[BF * (int64_t)m + i] += alpha * s[i];
}

// Two-stage forms of the restriction and the prolongation, coalesced over the P blocks: stage 1
// maps one P block to one thread -- consecutive threads read consecutive blocks -- and stores the
// block's product (6 values for the restriction, BF for the prolongation); stage 2 sums the
// products of each coarse node over its transpose list (in the list's fixed order) or of each
// finer row over its contiguous blocks.

// restriction, stage 1: c[b][j] = sum_i P_b[i][j] t[row(b)][i]
template <int BF>
EF_SA_HD void sa_restrict_contrib(int64_t b, const int32_t* __restrict__ pRow, const float* __restrict__ Pv,
                                  const float* __restrict__ t, float* __restrict__ c) {
    const int64_t m = pRow[b];
    const float* P = Pv + b * BF * BC;
    float ti[BF];
    EF_SA_UNROLL
    for (int i = 0; i < BF; ++i) ti[i] = t[BF * m + i];
    EF_SA_UNROLL
    for (int j = 0; j < BC; ++j) {
        float a = 0.f;
        EF_SA_UNROLL
        for (int i = 0; i < BF; ++i) a += P[i * BC + j] * ti[i];
        c[b * BC + j] = a;
    }
}

// restriction, stage 2: one lane's share of coarse node I, a[j] = sum of c[tIdx[k]][j] over
// k = tPtr[I] + lane, + nLanes, ...
EF_SA_HD void sa_restrict_sum_partial(int I, int lane, int nLanes, const int32_t* __restrict__ tPtr,
                                      const int32_t* __restrict__ tIdx, const float* __restrict__ c, float a[BC]) {
    EF_SA_UNROLL
    for (int j = 0; j < BC; ++j) a[j] = 0.f;
    for (int k = tPtr[I] + lane; k < tPtr[I + 1]; k += nLanes) {
        const float* q = c + (int64_t)tIdx[k] * BC;
        EF_SA_UNROLL
        for (int j = 0; j < BC; ++j) a[j] += q[j];
    }
}

// prolongation, stage 1: q[b][i] = sum_j P_b[i][j] xc[col(b)][j]
template <int BF>
EF_SA_HD void sa_prolong_contrib(int64_t b, const int32_t* __restrict__ pCol, const float* __restrict__ Pv,
                                 const float* __restrict__ xc, float* __restrict__ q) {
    const float* P = Pv + b * BF * BC;
    const float* cv = xc + BC * (int64_t)pCol[b];
    float x[BC];
    EF_SA_UNROLL
    for (int j = 0; j < BC; ++j) x[j] = cv[j];
    EF_SA_UNROLL
    for (int i = 0; i < BF; ++i) {
        float s = 0.f;
        EF_SA_UNROLL
        for (int j = 0; j < BC; ++j) s += P[i * BC + j] * x[j];
        q[b * BF + i] = s;
    }
}

// prolongation, stage 2: x[m] += alpha sum over row m's blocks of q[b] on the free DOFs
template <int BF>
EF_SA_HD void sa_prolong_apply(int m, const int32_t* __restrict__ pRowPtr, const float* __restrict__ q,
                               const uint8_t* __restrict__ mask, float* __restrict__ x, float alpha) {
    float s[BF];
    EF_SA_UNROLL
    for (int i = 0; i < BF; ++i) s[i] = 0.f;
    for (int b = pRowPtr[m]; b < pRowPtr[m + 1]; ++b)
        EF_SA_UNROLL
        for (int i = 0; i < BF; ++i) s[i] += q[(int64_t)b * BF + i];
    EF_SA_UNROLL
    for (int i = 0; i < BF; ++i)
        if (!(mask && mask[BF * (int64_t)m + i])) x[BF * (int64_t)m + i] += alpha * s[i];
}

// Fused fine-level post-smoothing.  With one damped block-Jacobi sweep before and after the coarse
// correction and the cycle started from zero, x1 = w D^-1 r, t = r - A x1, and after the coarse
// correction e,
//     x3 = x1 + a P e + w D^-1 (r - A (x1 + a P e)) = w D^-1 (r + t) + C e,
//     C  = a (P - w D^-1 A P) = a (I - w D^-1 A) P     (the pattern of AP),
// so the prolongation and the post-sweep become one product with C.  Block a = (m, J) of C from
// AP block a and P block b = apToP[a] = (m, J) (or -1 when P has no such block).
template <int BF>
EF_SA_HD void sa_post_block(int64_t a, const int32_t* __restrict__ apRow, const int32_t* __restrict__ apToP,
                            const float* __restrict__ Pv, const float* __restrict__ APv,
                            const float* __restrict__ binv, float omega, float alpha, float C[BF * BC]) {
    const int64_t m = apRow[a];
    const int32_t b = apToP[a];
    float B[BF * BF], Q[BF * BC], P[BF * BC];
    sa_load_ablock<BF>(binv + m * BF * BF, B);
    sa_load_block<BF>(APv + a * BF * BC, Q);
    if (b >= 0) {
        sa_load_block<BF>(Pv + (int64_t)b * BF * BC, P);
    } else {
        EF_SA_UNROLL
        for (int u = 0; u < BF * BC; ++u) P[u] = 0.f;
    }
    EF_SA_UNROLL
    for (int i = 0; i < BF; ++i)
        EF_SA_UNROLL
        for (int j = 0; j < BC; ++j) {
            float z = 0.f;
            EF_SA_UNROLL
            for (int q = 0; q < BF; ++q) z += B[i * BF + q] * Q[q * BC + j];
            C[i * BC + j] = alpha * (P[i * BC + j] - omega * z);
        }
}

// One-pass transfers.  The prolongation reads P in its row order (Pv); the restriction reads a
// copy of P in the transpose order (slot k holds block tIdx[k], rowT[k] = pRow[tIdx[k]]), so the
// blocks of one coarse column are consecutive.  A thread takes one block: the BF x BC values are
// contiguous (72 bytes for BF = 3, 144 for BF = 6) and load as 8- or 16-byte words.

// transpose-order copy, slot k: dst[k] = Pv[tIdx[k]] (BF x BC values)
template <int BF>
EF_SA_HD void sa_block_copy(int64_t k, const int32_t* __restrict__ tIdx, const float* __restrict__ Pv,
                            float* __restrict__ dst) {
    const int64_t b = tIdx[k];
    EF_SA_UNROLL
    for (int p = 0; p < BF * BC; ++p) dst[k * BF * BC + p] = Pv[b * BF * BC + p];
}

// restriction, one thread's share of coarse node I from the transpose-order copy PT:
// a[j] = sum over k = tPtr[I] + lane, + nLanes, ... of sum_i PT_k[i][j] t[rowT[k]][i]
template <int BF>
EF_SA_HD void sa_restrict_onepass_partial(int I, int lane, int nLanes, const int32_t* __restrict__ tPtr,
                                          const int32_t* __restrict__ rowT, const float* __restrict__ PT,
                                          const float* __restrict__ t, float a[BC]) {
    EF_SA_UNROLL
    for (int j = 0; j < BC; ++j) a[j] = 0.f;
    for (int64_t k = tPtr[I] + lane; k < tPtr[I + 1]; k += nLanes) {
        float P[BF * BC];
        sa_load_block<BF>(PT + k * BF * BC, P);
        const int64_t m = rowT[k];
        float ti[BF];
        EF_SA_UNROLL
        for (int i = 0; i < BF; ++i) ti[i] = t[BF * m + i];
        EF_SA_UNROLL
        for (int i = 0; i < BF; ++i)
            EF_SA_UNROLL
            for (int j = 0; j < BC; ++j) a[j] += P[i * BC + j] * ti[i];
    }
}

// prolongation product of block b (row order): q[i] = sum_j P_b[i][j] xc[col(b)][j]
template <int BF>
EF_SA_HD void sa_prolong_onepass_block(int64_t b, const int32_t* __restrict__ pCol, const float* __restrict__ Pv,
                                       const float* __restrict__ xc, float q[BF]) {
    float P[BF * BC];
    sa_load_block<BF>(Pv + b * BF * BC, P);
    const float* cv = xc + BC * (int64_t)pCol[b];
    float x[BC];
    EF_SA_UNROLL
    for (int j = 0; j < BC; ++j) x[j] = cv[j];
    EF_SA_UNROLL
    for (int i = 0; i < BF; ++i) {
        float s = 0.f;
        EF_SA_UNROLL
        for (int j = 0; j < BC; ++j) s += P[i * BC + j] * x[j];
        q[i] = s;
    }
}

// prolongation sum of finer row m from the block products q of the blocks b0, b0 + 1, ... (stride
// BF): x[m] += alpha sum over row m's blocks, on the free DOFs
template <int BF>
EF_SA_HD void sa_prolong_onepass_row(int m, int64_t b0, const int32_t* __restrict__ pRowPtr, const float* q,
                                     const uint8_t* __restrict__ mask, float* __restrict__ x, float alpha) {
    float s[BF];
    EF_SA_UNROLL
    for (int i = 0; i < BF; ++i) s[i] = 0.f;
    for (int64_t b = pRowPtr[m]; b < pRowPtr[m + 1]; ++b)
        EF_SA_UNROLL
        for (int i = 0; i < BF; ++i) s[i] += q[(b - b0) * BF + i];
    EF_SA_UNROLL
    for (int i = 0; i < BF; ++i)
        if (!(mask && mask[BF * (int64_t)m + i])) x[BF * (int64_t)m + i] += alpha * s[i];
}

}  // namespace ef

#undef EF_SA_HD
#undef EF_SA_UNROLL
