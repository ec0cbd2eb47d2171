// Aggregation multigrid with rigid-body coarse spaces on the block system.
//
// Level 0 is the context's 3x3-block (displacement) system.  Every coarser node is an aggregate
// of finer nodes and carries 6 DOFs: 3 translations and 3 rotations about the aggregate
// centroid, so the coarse spaces contain the rigid-body modes that elasticity needs.  The
// tentative prolongation of a finer node m with offset d = x_m - c_I from its aggregate
// centroid is
//   level 0 -> 1 (3 DOFs):  P_m = [ I | R(d) ]               (3 x 6)
//   level l -> l+1 (6 DOFs): P_m = [ I R(d) ; 0 I ]          (6 x 6)
// with R(d) = [e_x x d, e_y x d, e_z x d].  The Galerkin operators P^T A P are sums of
// P_m^T A_mn P_n over the finer blocks, formed by an atomic-free segmented sum in compensated
// FP32.
// Smoothing is damped block Jacobi; the coarsest level is solved with a dense
// pseudo-inverse (Gauss-Jordan, pivots below a relative threshold dropped).

#include <cuda_bf16.h>

#include <algorithm>

#include "amg_sa_body.h"
#include "ef_common.cuh"

namespace ef {

// Vector loads/stores of the multigrid phases: plain, or through L2 only (CG) in the cluster
// kernel, whose CTAs read vectors that other CTAs of the cluster wrote in the same launch.
template <bool CG>
__device__ __forceinline__ float ldv(const float* p) {
    if (CG) return __ldcg(p);
    return *p;
}
template <bool CG>
__device__ __forceinline__ void stv(float* p, float v) {
    if (CG)
        __stcg(p, v);
    else
        *p = v;
}

// coarse block S = sum over finer blocks f = (m, n) of P_m^T A_f P_n (fixed order); on level 0
// masked fine rows/columns are left out; dead coarse DOFs get identity rows/columns
template <int BF>
__global__ void galerkin_kernel(int64_t nCoarseBlocks, const int64_t* __restrict__ seg, const int32_t* __restrict__ src,
                                const int32_t* __restrict__ fineRowOfBlock, const int32_t* __restrict__ fineCol,
                                const float* __restrict__ fineVals, const uint8_t* __restrict__ fineMask,
                                const float* __restrict__ offs, const int32_t* __restrict__ coarseRowOfBlock,
                                const int32_t* __restrict__ coarseCol, const uint8_t* __restrict__ coarseDead,
                                float* __restrict__ coarseVals) {
    const int64_t S = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (S >= nCoarseBlocks) return;
    // compensated FP32 sums (TwoSum: value hi + lo), no FP64: on this GPU the FP64 pipe, and in
    // particular its FP32 -> FP64 conversions, bounded this kernel
    float acc[BC][BC], lo[BC][BC];
#pragma unroll
    for (int i = 0; i < BC; ++i)
#pragma unroll
        for (int j = 0; j < BC; ++j) acc[i][j] = lo[i][j] = 0.f;
    for (int64_t t = seg[S]; t < seg[S + 1]; ++t) {
        const int32_t f = src[t];
        const int m = fineRowOfBlock[f], n = fineCol[f];
        float A[BF][BF];
        const float* v = fineVals + (int64_t)f * BF * BF;
#pragma unroll
        for (int i = 0; i < BF; ++i)
#pragma unroll
            for (int j = 0; j < BF; ++j) {
                float a = v[i * BF + j];
                if (fineMask && (fineMask[BF * m + i] || fineMask[BF * n + j])) a = 0.f;
                A[i][j] = a;
            }
        float Pm[BF][BC], Pn[BF][BC];
        pblock<BF>(offs + 3 * (int64_t)m, Pm);
        pblock<BF>(offs + 3 * (int64_t)n, Pn);
        float AP[BF][BC];
#pragma unroll
        for (int i = 0; i < BF; ++i)
#pragma unroll
            for (int j = 0; j < BC; ++j) {
                float s = 0.f;
#pragma unroll
                for (int k = 0; k < BF; ++k) s += A[i][k] * Pn[k][j];
                AP[i][j] = s;
            }
#pragma unroll
        for (int i = 0; i < BC; ++i)
#pragma unroll
            for (int j = 0; j < BC; ++j) {
                float s = 0.f;
#pragma unroll
                for (int k = 0; k < BF; ++k) s += Pm[k][i] * AP[k][j];
                const float t = __fadd_rn(acc[i][j], s);
                const float bv = __fsub_rn(t, acc[i][j]);
                lo[i][j] = __fadd_rn(lo[i][j], __fadd_rn(__fsub_rn(acc[i][j], __fsub_rn(t, bv)), __fsub_rn(s, bv)));
                acc[i][j] = t;
            }
    }
    const int I = coarseRowOfBlock[S], J = coarseCol[S];
#pragma unroll
    for (int i = 0; i < BC; ++i)
#pragma unroll
        for (int j = 0; j < BC; ++j) {
            float a = __fadd_rn(acc[i][j], lo[i][j]);
            if (coarseDead[BC * I + i] || coarseDead[BC * J + j]) a = (I == J && i == j) ? 1.f : 0.f;
            coarseVals[S * BC * BC + i * BC + j] = a;
        }
}

// ---- smoothed aggregation (index maps from amg_sa_pattern.h) -------------------------------
// P = P_t - w D^-1 A P_t on the live finer DOFs (masked finer rows of P are zero; A with masked
// rows and columns dropped, as in the Galerkin product), AP = A P, A_c = P^T A P: segmented sums
// in the fixed order of the maps, FP32 with compensated accumulation for the coarse operator.
// The per-thread bodies are in amg_sa_body.h.

// one P block per thread
template <int BF>
__global__ void sa_prolongator_kernel(int64_t nP, const int32_t* __restrict__ pRow, const int32_t* __restrict__ pCol,
                                      const int64_t* __restrict__ pSeg, const int32_t* __restrict__ pSrc,
                                      const int32_t* __restrict__ fineCol, const float* __restrict__ fineVals,
                                      const uint8_t* __restrict__ fineMask, const float* __restrict__ offs,
                                      const int32_t* __restrict__ agg, const float* __restrict__ binv,
                                      const float* __restrict__ wP, float* __restrict__ Pv) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nP) return;
    sa_prolongator_block<BF>(b, pRow, pCol, pSeg, pSrc, fineCol, fineVals, fineMask, offs, agg, binv, *wP, Pv);
}

// one AP block per thread
template <int BF>
__global__ void sa_ap_kernel(int64_t nAP, const int32_t* __restrict__ apRow, const int64_t* __restrict__ apSeg,
                             const int32_t* __restrict__ apK, const int32_t* __restrict__ apP,
                             const int32_t* __restrict__ fineCol, const float* __restrict__ fineVals,
                             const uint8_t* __restrict__ fineMask, const float* __restrict__ Pv,
                             float* __restrict__ APv) {
    const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nAP) return;
    sa_ap_block<BF>(a, apRow, apSeg, apK, apP, fineCol, fineVals, fineMask, Pv, APv);
}

// AP by groups of kSaApRows finer rows: a thread per pair (coalesced pair lists) leaves the pair's
// product in shared memory, then a thread per value of an AP block of the group sums it over the
// block's pairs in list order.
// cap >= the pairs of every group (checked on the host); a group above it is skipped.
constexpr int kSaApThreads = 256;
constexpr int kSaApRows = 2;
template <int BF>
__global__ void __launch_bounds__(kSaApThreads) sa_ap_rows_kernel(
    int nF, int cap, const int32_t* __restrict__ apRowPtr, const int64_t* __restrict__ apSeg,
    const int32_t* __restrict__ apK, const int32_t* __restrict__ apP, const int32_t* __restrict__ fineCol,
    const float* __restrict__ fineVals, const uint8_t* __restrict__ fineMask, const float* __restrict__ Pv,
    float* __restrict__ APv) {
    extern __shared__ float apC[];  // [cap][BF * BC]
    const int m0 = blockIdx.x * kSaApRows;
    const int m1 = min(m0 + kSaApRows, nF);
    const int64_t a0 = apRowPtr[m0], a1 = apRowPtr[m1];
    const int64_t t0 = apSeg[a0], t1 = apSeg[a1];
    if (t1 - t0 > cap) return;  // the same for the whole CTA
    for (int64_t t = t0 + threadIdx.x; t < t1; t += kSaApThreads) {
        int m = m0;
        while (m + 1 < m1 && apSeg[apRowPtr[m + 1]] <= t) ++m;
        float c[BF * BC];
        sa_ap_pair<BF>(t, m, apK, apP, fineCol, fineVals, fineMask, Pv, c);
        float2* d = reinterpret_cast<float2*>(apC + (t - t0) * (BF * BC));
#pragma unroll
        for (int p = 0; p < BF * BC / 2; ++p) d[p] = make_float2(c[2 * p], c[2 * p + 1]);
    }
    __syncthreads();
    // a thread per (AP block, pair of values): the block's pairs in list order (8-byte words)
    constexpr int H = BF * BC / 2;
    const int nTask = (int)(a1 - a0) * H;
    const float2* apC2 = reinterpret_cast<const float2*>(apC);
    float2* APv2 = reinterpret_cast<float2*>(APv);
    for (int task = threadIdx.x; task < nTask; task += kSaApThreads) {
        const int64_t a = a0 + task / H;
        const int p = task % H;
        float2 acc = make_float2(0.f, 0.f);
        for (int64_t t = apSeg[a]; t < apSeg[a + 1]; ++t) {
            const float2 v = apC2[(t - t0) * H + p];
            acc.x += v.x;
            acc.y += v.y;
        }
        APv2[a * H + p] = acc;
    }
}

// one coarse block per thread
template <int BF>
__global__ void sa_galerkin_kernel(int64_t nC, const int64_t* __restrict__ cSeg, const int32_t* __restrict__ cP,
                                   const int32_t* __restrict__ cAP, const float* __restrict__ Pv,
                                   const float* __restrict__ APv, const int32_t* __restrict__ coarseRowOfBlock,
                                   const int32_t* __restrict__ coarseCol, const uint8_t* __restrict__ coarseDead,
                                   float* __restrict__ coarseVals) {
    const int64_t S = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (S >= nC) return;
    sa_galerkin_block<BF>(S, cSeg, cP, cAP, Pv, APv, coarseRowOfBlock, coarseCol, coarseDead, coarseVals);
}

// A warp per coarse block (8 per CTA): the lanes form the products s_ij = sum_q P_qi Q_qj of up
// to 32 pairs at once into shared memory, then lane v (and v + 32) adds value v of each pair with
// TwoSum in list order -- the operations of sa_galerkin_block in the same order (the same bits),
// with the pairs' loads issued by 32 lanes together instead of one thread walking them.
constexpr int kGalWarps = 8;
template <int BF>
__global__ void __launch_bounds__(32 * kGalWarps) sa_galerkin_warp_kernel(
    int64_t nC, const int64_t* __restrict__ cSeg, const int32_t* __restrict__ cP, const int32_t* __restrict__ cAP,
    const float* __restrict__ Pv, const float* __restrict__ APv, const int32_t* __restrict__ coarseRowOfBlock,
    const int32_t* __restrict__ coarseCol, const uint8_t* __restrict__ coarseDead, float* __restrict__ coarseVals) {
    constexpr int NV = BC * BC;  // 36 values per coarse block
    __shared__ float sp[kGalWarps][32][NV + 1];
    const int wp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t S = (int64_t)blockIdx.x * kGalWarps + wp;
    if (S >= nC) return;  // the whole warp
    const int64_t t0 = cSeg[S], t1 = cSeg[S + 1];
    float hi0 = 0.f, lo0 = 0.f, hi1 = 0.f, lo1 = 0.f;
    auto add = [](float& hi, float& lo, float v) {
        const float tt = sa_add_rn(hi, v);
        const float bv = sa_sub_rn(tt, hi);
        lo = sa_add_rn(lo, sa_add_rn(sa_sub_rn(hi, sa_sub_rn(tt, bv)), sa_sub_rn(v, bv)));
        hi = tt;
    };
    for (int64_t tb = t0; tb < t1; tb += 32) {
        const int64_t t = tb + lane;
        if (t < t1) {
            float pr[BF * BC], qr[BF * BC];
            sa_load_block<BF>(Pv + (int64_t)cP[t] * BF * BC, pr);
            sa_load_block<BF>(APv + (int64_t)cAP[t] * BF * BC, qr);
#pragma unroll
            for (int i = 0; i < BC; ++i)
#pragma unroll
                for (int j = 0; j < BC; ++j) {
                    float s = 0.f;
#pragma unroll
                    for (int q = 0; q < BF; ++q) s += pr[q * BC + i] * qr[q * BC + j];
                    sp[wp][lane][i * BC + j] = s;
                }
        }
        __syncwarp();
        const int cnt = (t1 - tb < 32) ? (int)(t1 - tb) : 32;
        for (int u = 0; u < cnt; ++u) {
            add(hi0, lo0, sp[wp][u][lane]);
            if (lane < NV - 32) add(hi1, lo1, sp[wp][u][lane + 32]);
        }
        __syncwarp();
    }
    const int I = coarseRowOfBlock[S], J = coarseCol[S];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int v = lane + 32 * h;
        if (v >= NV) break;
        const int i = v / BC, j = v % BC;
        float a = h ? sa_add_rn(hi1, lo1) : sa_add_rn(hi0, lo0);
        if (coarseDead[BC * (int64_t)I + i] || coarseDead[BC * (int64_t)J + j]) a = (I == J && i == j) ? 1.f : 0.f;
        coarseVals[S * NV + v] = a;
    }
}

// one warp per coarse node: lane partial sums over strided P blocks, fixed shuffle tree; dead
// coarse DOFs -> 0
template <int BF>
__global__ void sa_restrict_kernel(int nC, const int32_t* __restrict__ tPtr, const int32_t* __restrict__ tIdx,
                                   const int32_t* __restrict__ pRow, const float* __restrict__ Pv,
                                   const float* __restrict__ t, const uint8_t* __restrict__ coarseDead,
                                   float* __restrict__ rc) {
    const int lane = threadIdx.x & 31;
    const int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (I >= nC) return;
    float a[BC];
    sa_restrict_partial<BF>(I, lane, 32, tPtr, tIdx, pRow, Pv, t, a);
#pragma unroll
    for (int j = 0; j < BC; ++j)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a[j] += __shfl_xor_sync(0xffffffffu, a[j], o);
    if (lane < BC) {
        float v = a[0];
#pragma unroll
        for (int j = 1; j < BC; ++j)
            if (lane == j) v = a[j];
        rc[BC * I + lane] = coarseDead[BC * I + lane] ? 0.f : v;
    }
}

// one finer node per thread
template <int BF>
__global__ void sa_prolong_kernel(int nF, const int32_t* __restrict__ pRowPtr, const int32_t* __restrict__ pCol,
                                  const float* __restrict__ Pv, const float* __restrict__ xc,
                                  const uint8_t* __restrict__ mask, float* __restrict__ x, float alpha) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nF) return;
    sa_prolong_row<BF>(m, pRowPtr, pCol, Pv, xc, mask, x, alpha);
}

// two-stage transfers (amg_sa_body.h): one P block per thread, then sums per coarse node (a warp,
// lanes over its transpose list, fixed shuffle tree) or per finer row (a thread)
template <int BF>
__global__ void sa_restrict_contrib_kernel(int64_t nP, const int32_t* __restrict__ pRow, const float* __restrict__ Pv,
                                           const float* __restrict__ t, float* __restrict__ c) {
    ef::dep_entry();
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b < nP) sa_restrict_contrib<BF>(b, pRow, Pv, t, c);
}

__global__ void sa_restrict_sum_kernel(int nC, const int32_t* __restrict__ tPtr, const int32_t* __restrict__ tIdx,
                                       const float* __restrict__ c, const uint8_t* __restrict__ coarseDead,
                                       float* __restrict__ rc) {
    ef::dep_entry();
    const int lane = threadIdx.x & 31;
    const int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (I >= nC) return;
    float a[BC];
    sa_restrict_sum_partial(I, lane, 32, tPtr, tIdx, c, a);
#pragma unroll
    for (int j = 0; j < BC; ++j)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a[j] += __shfl_xor_sync(0xffffffffu, a[j], o);
    if (lane < BC) {
        float v = a[0];
#pragma unroll
        for (int j = 1; j < BC; ++j)
            if (lane == j) v = a[j];
        rc[BC * I + lane] = coarseDead[BC * I + lane] ? 0.f : v;
    }
}

template <int BF>
__global__ void sa_prolong_contrib_kernel(int64_t nP, const int32_t* __restrict__ pCol, const float* __restrict__ Pv,
                                          const float* __restrict__ xc, float* __restrict__ q) {
    ef::dep_entry();
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b < nP) sa_prolong_contrib<BF>(b, pCol, Pv, xc, q);
}

template <int BF>
__global__ void sa_prolong_apply_kernel(int nF, const int32_t* __restrict__ pRowPtr, const float* __restrict__ q,
                                        const uint8_t* __restrict__ mask, float* __restrict__ x, float alpha) {
    ef::dep_entry();
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m < nF) sa_prolong_apply<BF>(m, pRowPtr, q, mask, x, alpha);
}

// one-pass transfers (amg_sa_body.h)
template <int BF>
__global__ void sa_block_copy_kernel(int64_t nP, const int32_t* __restrict__ tIdx, const float* __restrict__ Pv,
                                     float* __restrict__ dst) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nP) sa_block_copy<BF>(k, tIdx, Pv, dst);
}

// restriction: a CTA per coarse node, a thread per P block of its column (consecutive blocks of
// the transpose-order copy), sums in a fixed order (each thread's blocks, a shuffle tree per warp,
// the warps in order)
constexpr int kSaRestrictThreads = 128;
template <int BF>
__global__ void __launch_bounds__(kSaRestrictThreads) sa_restrict_onepass_kernel(
    int nC, const int32_t* __restrict__ tPtr, const int32_t* __restrict__ rowT,
    const float* __restrict__ PT, const float* __restrict__ t, const uint8_t* __restrict__ coarseDead,
    float* __restrict__ rc) {
    ef::dep_entry();
    __shared__ float red[kSaRestrictThreads / 32][BC];
    const int I = blockIdx.x;
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    float a[BC];
    sa_restrict_onepass_partial<BF>(I, threadIdx.x, kSaRestrictThreads, tPtr, rowT, PT, t, a);
#pragma unroll
    for (int j = 0; j < BC; ++j) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a[j] += __shfl_xor_sync(0xffffffffu, a[j], o);
        if (lane == 0) red[wp][j] = a[j];
    }
    __syncthreads();
    if (threadIdx.x < BC) {
        float v = 0.f;
#pragma unroll
        for (int w = 0; w < kSaRestrictThreads / 32; ++w) v += red[w][threadIdx.x];
        rc[BC * I + threadIdx.x] = coarseDead[BC * I + threadIdx.x] ? 0.f : v;
    }
}

// BF16 form of the fine level's transpose-order copy (3 x 6 blocks): per slot one 16-byte word with
// values 0..7, one with 8..15 and one 4-byte word with 16..17 (three arrays, consecutive slots
// consecutive), for the restriction, which then streams 36 instead of 72 bytes per block
__device__ __forceinline__ uint32_t sa_pack_bf16x2(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}
__device__ __forceinline__ float2 sa_unpack_bf16x2(uint32_t v) {
    return __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&v));
}

__global__ void sa_block_copy_h_kernel(int64_t nP, const int32_t* __restrict__ tIdx, const float* __restrict__ Pv,
                                       uint4* __restrict__ q0, uint4* __restrict__ q1, uint32_t* __restrict__ q2) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nP) return;
    const float* P = Pv + (int64_t)tIdx[k] * 18;
    q0[k] = make_uint4(sa_pack_bf16x2(P[0], P[1]), sa_pack_bf16x2(P[2], P[3]), sa_pack_bf16x2(P[4], P[5]),
                       sa_pack_bf16x2(P[6], P[7]));
    q1[k] = make_uint4(sa_pack_bf16x2(P[8], P[9]), sa_pack_bf16x2(P[10], P[11]), sa_pack_bf16x2(P[12], P[13]),
                       sa_pack_bf16x2(P[14], P[15]));
    q2[k] = sa_pack_bf16x2(P[16], P[17]);
}

// the restriction of sa_restrict_onepass_kernel<3> from the BF16 copy
__global__ void __launch_bounds__(kSaRestrictThreads) sa_restrict_onepass_h_kernel(
    int nC, const int32_t* __restrict__ tPtr, const int32_t* __restrict__ rowT, const uint4* __restrict__ q0,
    const uint4* __restrict__ q1, const uint32_t* __restrict__ q2, const float* __restrict__ t,
    const uint8_t* __restrict__ coarseDead, float* __restrict__ rc) {
    ef::dep_entry();
    __shared__ float red[kSaRestrictThreads / 32][BC];
    const int I = blockIdx.x;
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    float a[BC];
#pragma unroll
    for (int j = 0; j < BC; ++j) a[j] = 0.f;
    for (int64_t k = tPtr[I] + threadIdx.x; k < tPtr[I + 1]; k += kSaRestrictThreads) {
        const uint4 u = q0[k], v = q1[k];
        const uint32_t w = q2[k];
        float P[18];
        const uint32_t words[9] = {u.x, u.y, u.z, u.w, v.x, v.y, v.z, v.w, w};
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            const float2 f = sa_unpack_bf16x2(words[q]);
            P[2 * q] = f.x;
            P[2 * q + 1] = f.y;
        }
        const int64_t m = rowT[k];
        const float t0 = t[3 * m], t1 = t[3 * m + 1], t2 = t[3 * m + 2];
#pragma unroll
        for (int j = 0; j < BC; ++j) a[j] += P[j] * t0 + P[BC + j] * t1 + P[2 * BC + j] * t2;
    }
#pragma unroll
    for (int j = 0; j < BC; ++j) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a[j] += __shfl_xor_sync(0xffffffffu, a[j], o);
        if (lane == 0) red[wp][j] = a[j];
    }
    __syncthreads();
    if (threadIdx.x < BC) {
        float v = 0.f;
#pragma unroll
        for (int w = 0; w < kSaRestrictThreads / 32; ++w) v += red[w][threadIdx.x];
        rc[BC * I + threadIdx.x] = coarseDead[BC * I + threadIdx.x] ? 0.f : v;
    }
}

// the same restriction with a warp per coarse node (kSaRestrictWarpNodes nodes per CTA): lanes
// stride over the node's blocks, a shuffle tree per value, no shared memory or CTA barrier
constexpr int kSaRestrictWarpNodes = 4;
__global__ void __launch_bounds__(32 * kSaRestrictWarpNodes) sa_restrict_warp_h_kernel(
    int nC, const int32_t* __restrict__ tPtr, const int32_t* __restrict__ rowT, const uint4* __restrict__ q0,
    const uint4* __restrict__ q1, const uint32_t* __restrict__ q2, const float* __restrict__ t,
    const uint8_t* __restrict__ coarseDead, float* __restrict__ rc) {
    ef::dep_entry();
    const int I = blockIdx.x * kSaRestrictWarpNodes + (threadIdx.x >> 5);
    if (I >= nC) return;
    const int lane = threadIdx.x & 31;
    float a[BC];
#pragma unroll
    for (int j = 0; j < BC; ++j) a[j] = 0.f;
    const int k1 = tPtr[I + 1];
#pragma unroll 2
    for (int k = tPtr[I] + lane; k < k1; k += 32) {
        const uint4 u = __ldcs(q0 + k), v = __ldcs(q1 + k);
        const uint32_t w = __ldcs(q2 + k);
        const int64_t m = __ldcs(rowT + k);
        const float t0 = t[3 * m], t1 = t[3 * m + 1], t2 = t[3 * m + 2];
        float P[18];
        const uint32_t words[9] = {u.x, u.y, u.z, u.w, v.x, v.y, v.z, v.w, w};
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            const float2 f = sa_unpack_bf16x2(words[q]);
            P[2 * q] = f.x;
            P[2 * q + 1] = f.y;
        }
#pragma unroll
        for (int j = 0; j < BC; ++j) a[j] += P[j] * t0 + P[BC + j] * t1 + P[2 * BC + j] * t2;
    }
#pragma unroll
    for (int j = 0; j < BC; ++j)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a[j] += __shfl_xor_sync(0xffffffffu, a[j], o);
    if (lane < BC) {
        float v = a[0];
#pragma unroll
        for (int j = 1; j < BC; ++j) v = lane == j ? a[j] : v;
        rc[BC * I + lane] = coarseDead[BC * I + lane] ? 0.f : v;
    }
}

// prolongation: a CTA per kSaProlongRows consecutive finer rows; a thread per P block of those
// rows (row order) leaves the block's product in shared memory, then
// thread r sums row r's products in block order.  cap >= the block count of every such group of
// rows (checked on the host when the copy is built); a group above it is skipped.
constexpr int kSaProlongThreads = 256;
constexpr int kSaProlongRows = 64;
template <int BF>
__global__ void __launch_bounds__(kSaProlongThreads) sa_prolong_onepass_kernel(
    int nF, int cap, const int32_t* __restrict__ pRowPtr, const int32_t* __restrict__ pCol,
    const float* __restrict__ Pv, const float* __restrict__ xc, const uint8_t* __restrict__ mask,
    float* __restrict__ x, float alpha) {
    ef::dep_entry();
    extern __shared__ float saQ[];  // [cap][BF]
    const int r0 = blockIdx.x * kSaProlongRows;
    const int r1 = min(r0 + kSaProlongRows, nF);
    const int64_t b0 = pRowPtr[r0], b1 = pRowPtr[r1];
    if (b1 - b0 > cap) return;  // the same for the whole CTA
    for (int64_t b = b0 + threadIdx.x; b < b1; b += kSaProlongThreads) {
        float v[BF];
        sa_prolong_onepass_block<BF>(b, pCol, Pv, xc, v);
#pragma unroll
        for (int i = 0; i < BF; ++i) saQ[(b - b0) * BF + i] = v[i];
    }
    __syncthreads();
    if (threadIdx.x < r1 - r0) sa_prolong_onepass_row<BF>(r0 + threadIdx.x, b0, pRowPtr, saQ, mask, x, alpha);
}

// *wP = 4 / (3 lambda) with lambda = sqrt(*n2), the prolongator damping from the power iteration
__global__ void sa_damping_kernel(const double* __restrict__ n2, float* __restrict__ wP) {
    const double v = *n2;
    *wP = v > 0.0 ? (float)(4.0 / (3.0 * sqrt(v))) : 0.f;
}

// inverse of each 6x6 diagonal block (pseudo-inverse: pivots below 1e-9 of the largest
// diagonal entry are dropped), FP64 Gauss-Jordan in registers
__global__ void bj6_setup_kernel(int nN, const int64_t* __restrict__ diagPos, const float* __restrict__ vals,
                                 float* __restrict__ inv) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nN) return;
    double A[BC][2 * BC];
    const float* D = vals + diagPos[m] * BC * BC;
    double dmax = 0.0;
#pragma unroll
    for (int i = 0; i < BC; ++i) {
#pragma unroll
        for (int j = 0; j < BC; ++j) {
            A[i][j] = (double)D[i * BC + j];
            A[i][BC + j] = i == j ? 1.0 : 0.0;
        }
        dmax = fmax(dmax, fabs(A[i][i]));
    }
    bool drop[BC];
#pragma unroll
    for (int c = 0; c < BC; ++c) drop[c] = false;
    for (int c = 0; c < BC; ++c) {
        if (!(fabs(A[c][c]) > 1e-9 * dmax)) {
            drop[c] = true;
            continue;
        }
        const double p = 1.0 / A[c][c];
        for (int j = 0; j < 2 * BC; ++j) A[c][j] *= p;
        for (int r = 0; r < BC; ++r) {
            if (r == c) continue;
            const double f = A[r][c];
            for (int j = 0; j < 2 * BC; ++j) A[r][j] -= f * A[c][j];
        }
    }
    for (int i = 0; i < BC; ++i)
        for (int j = 0; j < BC; ++j)
            inv[(int64_t)m * BC * BC + i * BC + j] = (drop[i] || drop[j]) ? 0.f : (float)A[i][BC + j];
}

// x = omega * D^-1 r (+ x when accumulating); masked DOFs -> 0
template <int BS, bool CG>
__device__ __forceinline__ void bj_row(int m, const float* __restrict__ binv, const uint8_t* __restrict__ mask,
                                       float omega, const float* r, float* x, int accumulate) {
    const float* B = binv + (int64_t)m * BS * BS;
    float rv[BS];
#pragma unroll
    for (int i = 0; i < BS; ++i) rv[i] = ldv<CG>(r + BS * m + i);
#pragma unroll
    for (int i = 0; i < BS; ++i) {
        float z = 0.f;
#pragma unroll
        for (int j = 0; j < BS; ++j) z += B[i * BS + j] * rv[j];
        z *= omega;
        if (mask && mask[BS * m + i]) z = 0.f;
        if (accumulate)
            stv<CG>(x + BS * m + i, ldv<CG>(x + BS * m + i) + z);
        else
            stv<CG>(x + BS * m + i, z);
    }
}

template <int BS>
__global__ void bj_apply_kernel(int nN, const float* __restrict__ binv, const uint8_t* __restrict__ mask, float omega,
                                const float* __restrict__ r, float* __restrict__ x, int accumulate) {
    ef::dep_entry();
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nN) return;
    bj_row<BS, false>(m, binv, mask, omega, r, x, accumulate);
}

// One damped block-Jacobi sweep finished for block row m from y = (A x)_m, held by every lane:
// lane i < BS writes xout_i = x_i + omega (D_m^-1 (r - A x)_m)_i (masked entries of the
// residual count as zero, masked entries of x stay).  xout must not alias x.
template <int BS, bool CG = false>
__device__ __forceinline__ void smooth_row(int m, int lane, const float* y, const float* x, const float* r,
                                           const uint8_t* __restrict__ mask, const float* __restrict__ binv,
                                           float omega, float* xout) {
    float tv[BS];
#pragma unroll
    for (int j = 0; j < BS; ++j) tv[j] = (mask && mask[BS * m + j]) ? 0.f : ldv<CG>(r + BS * m + j) - y[j];
    const float* B = binv + (int64_t)m * BS * BS + lane * BS;
    float z = 0.f;
#pragma unroll
    for (int j = 0; j < BS; ++j) z += B[j] * tv[j];
    const int d = BS * m + lane;
    const float xd = ldv<CG>(x + d);
    stv<CG>(xout + d, (mask && mask[d]) ? xd : xd + omega * z);
}

// t = r - A x on one level (masked rows -> 0); 8 lanes per block row, batched loads.  With
// binv set it runs a whole smoothing sweep instead: t receives x + omega D^-1 (r - A x).
template <int BS>
__global__ void __launch_bounds__(256) level_residual_kernel(int nN, const int32_t* __restrict__ rowPtr,
                                                              const int32_t* __restrict__ colIdx,
                                                              const float* __restrict__ vals,
                                                              const float* __restrict__ x, const float* __restrict__ r,
                                                              const uint8_t* __restrict__ mask, float* __restrict__ t,
                                                              const float* __restrict__ binv, float omega) {
    ef::dep_entry();
    const int lane = threadIdx.x & 7;
    const int m0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 3;
    const int m = m0 < nN ? m0 : nN - 1;
    float y[BS];
#pragma unroll
    for (int i = 0; i < BS; ++i) y[i] = 0.f;
    const int s = rowPtr[m], e = rowPtr[m + 1];
    for (int base = s; base < e; base += 32) {
        int cc[4];
        float v[4][BS * BS];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int k = base + lane + 8 * j;
            if (k < e) {
                cc[j] = BS * colIdx[k];
                const float* src = vals + (int64_t)k * BS * BS;
#pragma unroll
                for (int q = 0; q < BS * BS; ++q) v[j][q] = src[q];
            } else {
                cc[j] = -1;
            }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (cc[j] >= 0) {
                float xv[BS];
#pragma unroll
                for (int i = 0; i < BS; ++i) xv[i] = x[cc[j] + i];
#pragma unroll
                for (int i = 0; i < BS; ++i) {
                    float a = 0.f;
#pragma unroll
                    for (int k = 0; k < BS; ++k) a += v[j][i * BS + k] * xv[k];
                    y[i] += a;
                }
            }
    }
#pragma unroll
    for (int i = 0; i < BS; ++i)
#pragma unroll
        for (int o = 4; o > 0; o >>= 1) y[i] += __shfl_xor_sync(0xffffffffu, y[i], o);
    if (m0 < nN && lane < BS) {
        if (binv) {
            smooth_row<BS>(m, lane, y, x, r, mask, binv, omega, t);
        } else {
            const int d = BS * m + lane;
            float yy = y[0];
#pragma unroll
            for (int i = 1; i < BS; ++i)
                if (lane == i) yy = y[i];
            t[d] = (mask && mask[d]) ? 0.f : r[d] - yy;
        }
    }
}

// t = r - A x for 6x6 blocks, one warp per block row: lane 6g + i (g < 5, i < 6) takes row i of
// the blocks g, g + 5, g + 10, ... of the row (three 8-byte loads of the block row, so that the
// warp reads five consecutive blocks per slot, three slots per step), the five slots of each i
// are combined by a fixed shuffle sequence.  With binv set: one smoothing sweep, t = x + omega D^-1 (r - A x).
template <bool CG>
__device__ __forceinline__ float2 ldv2(const float* p) {
    if (CG) return __ldcg(reinterpret_cast<const float2*>(p));
    return *reinterpret_cast<const float2*>(p);
}
// H: the block values come from a BF16 copy (valsH, 6 values = three 4-byte words per block row)
template <bool CG, bool H = false>
__device__ __forceinline__ void resid6_row(int m, int lane, const int32_t* __restrict__ rowPtr,
                                           const int32_t* __restrict__ colIdx, const float* __restrict__ vals,
                                           const float* x, const float* r, const uint8_t* __restrict__ mask, float* t,
                                           const float* __restrict__ binv, float omega,
                                           const uint32_t* __restrict__ valsH = nullptr, float ys = 1.f) {
    const int g = lane / BC, ri = lane - BC * g;
    float acc = 0.f;
    if (g < 5) {
        // three blocks per lane and step (15 per warp), their loads issued together
        const int e = rowPtr[m + 1];
        for (int k0 = rowPtr[m] + g; k0 < e; k0 += 15) {
            int c[3];
            float2 a[3][3];
#pragma unroll
            for (int u = 0; u < 3; ++u) {
                const int k = k0 + 5 * u;
                c[u] = -1;
                if (k < e) {
                    c[u] = BC * colIdx[k];
                    if (H) {
                        const uint32_t* v = valsH + ((int64_t)k * BC * BC + BC * ri) / 2;
#pragma unroll
                        for (int q = 0; q < 3; ++q) {
                            const uint32_t w = v[q];
                            a[u][q] = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&w));
                        }
                    } else {
                        const float2* v = reinterpret_cast<const float2*>(vals + (int64_t)k * BC * BC + BC * ri);
                        a[u][0] = v[0];
                        a[u][1] = v[1];
                        a[u][2] = v[2];
                    }
                }
            }
#pragma unroll
            for (int u = 0; u < 3; ++u)
                if (c[u] >= 0) {
                    const float2 x0 = ldv2<CG>(x + c[u]), x1 = ldv2<CG>(x + c[u] + 2), x2 = ldv2<CG>(x + c[u] + 4);
                    acc += a[u][0].x * x0.x + a[u][0].y * x0.y + a[u][1].x * x1.x + a[u][1].y * x1.y +
                           a[u][2].x * x2.x + a[u][2].y * x2.y;
                }
        }
    }
    // lanes i < 6: acc(i) + acc(i + 6) + acc(i + 12) + acc(i + 18) + acc(i + 24)
    const float s1 = acc + __shfl_down_sync(0xffffffffu, acc, 6);
    const float s2 = s1 + __shfl_down_sync(0xffffffffu, s1, 12);
    const float yi = s2 + __shfl_down_sync(0xffffffffu, acc, 24);
    float y[BC];
#pragma unroll
    for (int i = 0; i < BC; ++i) y[i] = __shfl_sync(0xffffffffu, yi, i);
    if (lane < BC) {
        if (binv) {
            smooth_row<BC, CG>(m, lane, y, x, r, mask, binv, omega, t);
        } else {
            const int d = BC * m + lane;
            stv<CG>(t + d, (mask && mask[d]) ? 0.f : ldv<CG>(r + d) - ys * yi);
        }
    }
}

__global__ void __launch_bounds__(256) level_residual6_kernel(int nN, const int32_t* __restrict__ rowPtr,
                                                               const int32_t* __restrict__ colIdx,
                                                               const float* __restrict__ vals,
                                                               const float* __restrict__ x, const float* __restrict__ r,
                                                               const uint8_t* __restrict__ mask, float* __restrict__ t,
                                                               const float* __restrict__ binv, float omega,
                                                               const uint32_t* __restrict__ valsH, float ys) {
    ef::dep_entry();
    const int lane = threadIdx.x & 31;
    const int m = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (m >= nN) return;
    if (valsH)
        resid6_row<false, true>(m, lane, rowPtr, colIdx, vals, x, r, mask, t, binv, omega, valsH, ys);
    else
        resid6_row<false, false>(m, lane, rowPtr, colIdx, vals, x, r, mask, t, binv, omega, nullptr, ys);
}

// B = A (M D^-1) on a 6-DOF level: block k of A times the block inverse of its column node with
// the rows of dead DOFs zeroed (the block-Jacobi sweep from zero, x1 = w M D^-1 r, then has the
// residual r - A x1 = r - w B r)
__global__ void scale_blocks6_kernel(int64_t nB, const int32_t* __restrict__ colIdx, const float* __restrict__ vals,
                                     const float* __restrict__ binv, const uint8_t* __restrict__ dead,
                                     float* __restrict__ out) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nB) return;
    const int64_t c = colIdx[k];
    float A[BC * BC], D[BC * BC];
    sa_load_ablock<BC>(vals + k * BC * BC, A);
    sa_load_ablock<BC>(binv + c * BC * BC, D);
    bool dq[BC];
#pragma unroll
    for (int q = 0; q < BC; ++q) dq[q] = dead[BC * c + q];
    float4* O = reinterpret_cast<float4*>(out + k * BC * BC);
    float o[BC * BC];
#pragma unroll
    for (int i = 0; i < BC; ++i)
#pragma unroll
        for (int j = 0; j < BC; ++j) {
            float z = 0.f;
#pragma unroll
            for (int q = 0; q < BC; ++q) z += dq[q] ? 0.f : A[i * BC + q] * D[q * BC + j];
            o[i * BC + j] = z;
        }
#pragma unroll
    for (int u = 0; u < BC * BC / 4; ++u) O[u] = make_float4(o[4 * u], o[4 * u + 1], o[4 * u + 2], o[4 * u + 3]);
}

// Fused post-smoothing of a 6-DOF level (amg_sa_body.h): C = a (I - w D^-1 A) P in the pattern of
// A P (FP32, rows in order), then x = w D^-1 (r + t) + C e with e the coarser level's correction.
__global__ void sa_post6_setup_kernel(int64_t nAP, const int32_t* __restrict__ apRow,
                                      const int32_t* __restrict__ apToP, const float* __restrict__ Pv,
                                      const float* __restrict__ APv, const float* __restrict__ binv, float omega,
                                      float alpha, float* __restrict__ C) {
    const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nAP) return;
    float c[BC * BC];
    sa_post_block<BC>(a, apRow, apToP, Pv, APv, binv, omega, alpha, c);
#pragma unroll
    for (int p = 0; p < BC * BC; ++p) C[a * BC * BC + p] = c[p];
}

// a warp per row m; lanes 6 k + i (k < 5) take component i of the row's blocks k, k + 5, ...;
// the five partial sums of a component are added in a fixed order, then lanes i < 6 form
// x[m][i] = w (D_m^-1 (r + t)_m)[i] + y[i] (dead DOFs 0)
__global__ void __launch_bounds__(256) sa_post6_fused_kernel(int nN, const int32_t* __restrict__ rowPtr,
                                                             const int32_t* __restrict__ col,
                                                             const float* __restrict__ C, const float* __restrict__ e,
                                                             const float* __restrict__ r, const float* __restrict__ t,
                                                             const float* __restrict__ binv,
                                                             const uint8_t* __restrict__ dead, float omega,
                                                             float* __restrict__ x) {
    ef::dep_entry();
    const int lane = threadIdx.x & 31;
    const int m = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (m >= nN) return;  // whole warps
    const int k0 = lane / BC, i = lane % BC;
    float y = 0.f;
    if (k0 < 5)
        for (int a = rowPtr[m] + k0; a < rowPtr[m + 1]; a += 5) {
            const float* cr = C + (int64_t)a * BC * BC + i * BC;
            const float* ev = e + BC * (int64_t)col[a];
#pragma unroll
            for (int j = 0; j < BC; ++j) y += cr[j] * ev[j];
        }
    // lane i gathers lanes i + 6, i + 12, i + 18, i + 24 in that order
    float s = y;
#pragma unroll
    for (int k = 1; k < 5; ++k) {
        const float v = __shfl_sync(0xffffffffu, y, (i + BC * k) & 31);
        if (k0 == 0) s += v;
    }
    if (lane < BC) {
        const float* B = binv + (int64_t)m * BC * BC + i * BC;
        float z = 0.f;
#pragma unroll
        for (int q = 0; q < BC; ++q) z += B[q] * (r[BC * (int64_t)m + q] + t[BC * (int64_t)m + q]);
        x[BC * (int64_t)m + i] = dead[BC * (int64_t)m + i] ? 0.f : omega * z + s;
    }
}

// BF16 copy of FP32 values (coarse-level blocks for the smoothing residuals)
__global__ void to_bf16_kernel(int64_t n, const float* __restrict__ src, __nv_bfloat16* __restrict__ dst) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = __float2bfloat16(src[i]);
}

// rc[I] = sum over members m of aggregate I of P_m^T t[m]; one warp per aggregate, members
// strided over the lanes and combined by a fixed shuffle tree
template <int BF, bool CG>
__device__ __forceinline__ void restrict_row(int I, int lane, const int32_t* __restrict__ aggPtr,
                                             const int32_t* __restrict__ aggIdx, const float* __restrict__ offs,
                                             const float* t, const uint8_t* __restrict__ coarseDead, float* rc) {
    float a[BC];
#pragma unroll
    for (int j = 0; j < BC; ++j) a[j] = 0.f;
    for (int k = aggPtr[I] + lane; k < aggPtr[I + 1]; k += 32) {
        const int m = aggIdx[k];
        float P[BF][BC];
        pblock<BF>(offs + 3 * (int64_t)m, P);
#pragma unroll
        for (int i = 0; i < BF; ++i) {
            const float ti = ldv<CG>(t + BF * m + i);
#pragma unroll
            for (int j = 0; j < BC; ++j) a[j] += P[i][j] * ti;
        }
    }
#pragma unroll
    for (int j = 0; j < BC; ++j)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a[j] += __shfl_xor_sync(0xffffffffu, a[j], o);
    if (lane < BC) {
        float v = a[0];
#pragma unroll
        for (int j = 1; j < BC; ++j)
            if (lane == j) v = a[j];
        stv<CG>(rc + BC * I + lane, coarseDead[BC * I + lane] ? 0.f : v);
    }
}

template <int BF>
__global__ void restrict_kernel(int nC, const int32_t* __restrict__ aggPtr, const int32_t* __restrict__ aggIdx,
                                const float* __restrict__ offs, const float* __restrict__ t,
                                const uint8_t* __restrict__ coarseDead, float* __restrict__ rc) {
    const int lane = threadIdx.x & 31;
    const int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (I >= nC) return;
    restrict_row<BF, false>(I, lane, aggPtr, aggIdx, offs, t, coarseDead, rc);
}

// x[m] += P_m xc[agg(m)] on free finer DOFs
template <int BF, bool CG>
__device__ __forceinline__ void prolong_row(int m, const int32_t* __restrict__ agg, const float* __restrict__ offs,
                                            const float* xc, const uint8_t* __restrict__ mask, float* x, float alpha) {
    const int I = agg[m];
    float P[BF][BC];
    pblock<BF>(offs + 3 * (int64_t)m, P);
    float c[BC];
#pragma unroll
    for (int j = 0; j < BC; ++j) c[j] = ldv<CG>(xc + BC * I + j);
#pragma unroll
    for (int i = 0; i < BF; ++i) {
        if (mask && mask[BF * m + i]) continue;
        float s = 0.f;
#pragma unroll
        for (int j = 0; j < BC; ++j) s += P[i][j] * c[j];
        stv<CG>(x + BF * m + i, ldv<CG>(x + BF * m + i) + alpha * s);
    }
}

template <int BF>
__global__ void prolong_kernel(int nN, const int32_t* __restrict__ agg, const float* __restrict__ offs,
                               const float* __restrict__ xc, const uint8_t* __restrict__ mask, float* __restrict__ x,
                               float alpha) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nN) return;
    prolong_row<BF, false>(m, agg, offs, xc, mask, x, alpha);
}

// dense pseudo-inverse of the coarsest operator (n = 6 nN <= kMaxCoarsestDof), FP32 Gauss-Jordan
// with partial pivoting in shared memory, one CTA; pivots below 1e-6 of the largest diagonal
// entry mark a null direction whose rows/columns of the inverse are zero
constexpr int kMaxCoarsestDof = 96;
__global__ void coarsest_inverse_kernel(int nN, const int32_t* __restrict__ rowPtr, const int32_t* __restrict__ colIdx,
                                        const float* __restrict__ vals, float* __restrict__ inv) {
    // FP32 Gauss-Jordan on [A | I] in shared memory (one CTA; the FP64 version spent ~1.5 ms in
    // the FP64 pipe of a single SM); pivots below 1e-6 of the largest diagonal entry mark a null
    // direction (FP32 round-off of a zero pivot is ~1e-7 of it).  Two CTA barriers per column:
    // the pivot of column col + 1 is chosen while column col is eliminated (the thread updating
    // entry (r, col + 1), r > col, posts (|value|, smallest row on ties) by a 64-bit atomic max),
    // the row swap and the scaling of the pivot row are one pass, and the left block's column col,
    // never read again, is left as it is.
    extern __shared__ float smemF[];
    const int n = BC * nN;
    const int ld = 2 * n + 1;
    auto A = [&](int r, int c) -> float& { return smemF[r * ld + c]; };
    __shared__ unsigned long long key[2];
    __shared__ float dmax;
    __shared__ unsigned char drop[kMaxCoarsestDof];
    const int tid = threadIdx.y * blockDim.x + threadIdx.x, nt = blockDim.x * blockDim.y;
    for (int r = threadIdx.y; r < n; r += blockDim.y)
        for (int c = threadIdx.x; c < 2 * n; c += blockDim.x) A(r, c) = (c >= n && c - n == r) ? 1.f : 0.f;
    __syncthreads();
    // the blocks' values spread over all threads (a value per thread and step; the row of block
    // k by a scan of the at most 16 row starts)
    const int nnzV = rowPtr[nN] * BC * BC;
    for (int v = tid; v < nnzV; v += nt) {
        const int k = v / (BC * BC), ij = v - k * (BC * BC);
        int m = 0;
        while (m + 1 < nN && rowPtr[m + 1] <= k) ++m;
        A(BC * m + ij / BC, BC * colIdx[k] + ij % BC) = vals[v];
    }
    __syncthreads();
    if (threadIdx.y == 0) {  // the largest |diagonal| by the first warp
        float d = 0.f;
        for (int i = threadIdx.x; i < n; i += 32) d = fmaxf(d, fabsf(A(i, i)));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) d = fmaxf(d, __shfl_xor_sync(0xffffffffu, d, o));
        if (threadIdx.x == 0) dmax = d;
    }
    for (int i = tid; i < n; i += nt) drop[i] = 0;
    // the pivot key of an entry: |value| bits above, the complement of the row below (the larger
    // key: the larger magnitude, then the smaller row)
    auto pkey = [](float v, int r) -> unsigned long long {
        return ((unsigned long long)__float_as_uint(fabsf(v)) << 32) | (unsigned long long)(0xFFFFFFFFu - (unsigned)r);
    };
    bool searched = false;  // the current column's key was posted by the previous elimination
    for (int col = 0; col < n; ++col) {
        if (!searched) {  // column 0, or the column after a dropped one: an explicit search
            if (tid == 0) key[col & 1] = 0ull;
            __syncthreads();
            for (int r = col + tid; r < n; r += nt) atomicMax(&key[col & 1], pkey(A(r, col), r));
        }
        __syncthreads();
        const unsigned long long kk = key[col & 1];
        const float best = __uint_as_float((unsigned)(kk >> 32));
        const int piv = (best > 1e-6f * dmax) ? (int)(0xFFFFFFFFu - (unsigned)(kk & 0xFFFFFFFFull)) : -1;
        if (piv < 0) {
            if (tid == 0) drop[col] = 1;
            searched = false;
            continue;
        }
        // swap rows col and piv and scale the pivot row by 1 / d over the live columns
        const float d = A(piv, col);
        if (tid == 0) key[(col + 1) & 1] = 0ull;
        for (int c = col + 1 + tid; c < 2 * n; c += nt) {
            const float a = A(col, c), b = A(piv, c);
            A(col, c) = b / d;
            if (piv != col) A(piv, c) = a;
        }
        __syncthreads();
        // eliminate column col from every other row (its multiplier from the unswapped column:
        // row piv now holds the old row col, whose entry is still at (col, col)): warp w takes
        // columns col + 1 + w + 32 k, lane l rows l + 32 i (a row stride of ld = 2 n + 1 words
        // keeps the lanes on distinct banks); warp 0, which holds column col + 1, picks the next
        // pivot among its rows below col by a shuffle tree
        {
            const int lane = threadIdx.x, w = threadIdx.y;
            float f[kMaxCoarsestDof / 32];
#pragma unroll
            for (int i = 0; i < kMaxCoarsestDof / 32; ++i) {
                const int r = lane + 32 * i;
                f[i] = (r < n && r != col) ? ((r == piv) ? A(col, col) : A(r, col)) : 0.f;
            }
            unsigned long long kbest = 0ull;
            for (int c = col + 1 + w; c < 2 * n; c += 32) {
                const float a = A(col, c);
#pragma unroll
                for (int i = 0; i < kMaxCoarsestDof / 32; ++i) {
                    const int r = lane + 32 * i;
                    if (r < n && r != col) {
                        const float v = A(r, c) - f[i] * a;
                        A(r, c) = v;
                        if (c == col + 1 && r > col) kbest = max(kbest, pkey(v, r));
                    }
                }
            }
            if (w == 0) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) kbest = max(kbest, __shfl_xor_sync(0xffffffffu, kbest, o));
                if (lane == 0) key[(col + 1) & 1] = kbest;
            }
        }
        searched = true;
    }
    __syncthreads();
    for (int i = tid; i < n * n; i += nt) {
        const int r = i / n, c = i % n;
        inv[i] = (drop[r] || drop[c]) ? 0.f : A(r, n + c);
    }
}

// x = Ainv r on the coarsest level (dense matvec), dead DOFs -> 0
// x = inv r on the coarsest level (dead DOFs -> 0), one warp per row (coalesced row of inv,
// fixed shuffle tree)
template <bool CG>
__device__ __forceinline__ void coarsest_row(int i, int lane, int n, const float* __restrict__ inv, const float* r,
                                             const uint8_t* __restrict__ dead, float* x) {
    float s = 0.f;
    for (int j = lane; j < n; j += 32) s += inv[(int64_t)i * n + j] * ldv<CG>(r + j);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) stv<CG>(x + i, dead[i] ? 0.f : s);
}

__global__ void coarsest_apply_kernel(int n, const float* __restrict__ inv, const float* __restrict__ r,
                                      const uint8_t* __restrict__ dead, float* __restrict__ x) {
    ef::dep_entry();
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (i >= n) return;
    coarsest_row<false>(i, threadIdx.x & 31, n, inv, r, dead, x);
}

// The multigrid cycle below a level as one launch: one cluster of kCoarseCtas CTAs runs the
// phases of a host-built program in order, with a cluster barrier (release/acquire at cluster
// scope, after a device-scope fence) between phases.  Vectors written in the launch are read
// and written through L2 only.  Every thread runs every phase loop and every barrier, so the
// barrier count is uniform over the cluster.
constexpr int kCoarseCtas = 8;
constexpr int kCoarseThreads = 512;
__global__ void __cluster_dims__(kCoarseCtas, 1, 1) __launch_bounds__(kCoarseThreads, 1)
    coarse_cycle_kernel(const CoarseOp* __restrict__ ops, int nOps) {
    const int tid = blockIdx.x * kCoarseThreads + threadIdx.x;
    const int nThreads = kCoarseCtas * kCoarseThreads;
    const int lane = threadIdx.x & 31;
    const int gw = tid >> 5;
    const int nWarps = nThreads >> 5;
    for (int o = 0; o < nOps; ++o) {
        const CoarseOp op = ops[o];
        switch (op.type) {
            case COP_BJ:
                for (int m = tid; m < op.n; m += nThreads) bj_row<BC, true>(m, op.f1, op.mask, op.omega, op.in, op.out, 0);
                break;
            case COP_SWEEP:
                for (int m = gw; m < op.n; m += nWarps)
                    resid6_row<true>(m, lane, op.p0, op.p1, op.f0, op.in, op.rhs, op.mask, op.out, op.f1, op.omega);
                break;
            case COP_RESID:
                for (int m = gw; m < op.n; m += nWarps)
                    resid6_row<true>(m, lane, op.p0, op.p1, op.f0, op.in, op.rhs, op.mask, op.out, nullptr, 0.f);
                break;
            case COP_RESTRICT:
                for (int I = gw; I < op.n; I += nWarps)
                    restrict_row<BC, true>(I, lane, op.p0, op.p1, op.f0, op.in, op.mask, op.out);
                break;
            case COP_PROLONG:
                for (int m = tid; m < op.n; m += nThreads)
                    prolong_row<BC, true>(m, op.p0, op.f0, op.in, op.mask, op.out, op.omega);
                break;
            case COP_COARSEST:
                for (int i = gw; i < op.n; i += nWarps) coarsest_row<true>(i, lane, op.n, op.f0, op.in, op.mask, op.out);
                break;
            default:
                break;
        }
        __threadfence();
        __syncwarp();
        asm volatile("barrier.cluster.arrive.release;\n" ::: "memory");
        asm volatile("barrier.cluster.wait.acquire;\n" ::: "memory");
    }
}

// x /= sqrt(*n2) (x stays when *n2 is not positive): the power iteration's normalisation with the
// norm left on the device
__global__ void scale_rnorm_kernel(int64_t n, float* __restrict__ x, const double* __restrict__ n2) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = *n2;
    if (v > 0.0) x[i] *= (float)(1.0 / sqrt(v));
}

// deterministic pseudo-random start vector in [-0.5, 0.5) (integer hash of the index)
__global__ void fill_hash_kernel(int64_t n, float* __restrict__ x) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t h = (uint32_t)i * 2654435761u + 0x9e3779b9u;
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    x[i] = (float)h * (1.0f / 4294967296.0f) - 0.5f;
}

// one Chebyshev smoothing step on D^-1 A: d = a d + b D^-1 t (a = 0: d = b D^-1 t), x += d
// (x = d when `first`); masked DOFs -> 0
template <int BS>
__global__ void cheb_step_kernel(int nN, const float* __restrict__ binv, const uint8_t* __restrict__ mask, float a,
                                 float b, const float* __restrict__ t, float* __restrict__ d, float* __restrict__ x,
                                 int first) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nN) return;
    const float* B = binv + (int64_t)m * BS * BS;
    float tv[BS];
#pragma unroll
    for (int i = 0; i < BS; ++i) tv[i] = t[BS * m + i];
#pragma unroll
    for (int i = 0; i < BS; ++i) {
        float z = 0.f;
#pragma unroll
        for (int j = 0; j < BS; ++j) z += B[i * BS + j] * tv[j];
        const int k = BS * m + i;
        float dn = (a != 0.f ? a * d[k] : 0.f) + b * z;
        if (mask && mask[k]) dn = 0.f;
        d[k] = dn;
        x[k] = first ? dn : x[k] + dn;
    }
}

// fine-level residual t = r - A x from a split BF16 copy of the 3x3 blocks: values 0..7 of block
// k in one 16-byte word, value 8 in a separate array (two loads per block instead of nine)
__global__ void __launch_bounds__(256) level_residual3_bf16_kernel(int nN, const int32_t* __restrict__ rowPtr,
                                                                    const int32_t* __restrict__ colIdx,
                                                                    const uint4* __restrict__ v8,
                                                                    const __nv_bfloat16* __restrict__ v1,
                                                                    const float* __restrict__ x,
                                                                    const float* __restrict__ r,
                                                                    const uint8_t* __restrict__ mask,
                                                                    float* __restrict__ t,
                                                                    const float* __restrict__ binv, float omega) {
    const int lane = threadIdx.x & 7;
    const int m0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 3;
    const int m = m0 < nN ? m0 : nN - 1;
    float y0 = 0.f, y1 = 0.f, y2 = 0.f;
    const int s = rowPtr[m], e = rowPtr[m + 1];
    for (int base = s; base < e; base += 32) {
        int cc[4];
        uint4 q[4];
        float w8[4];
        // the block words are loaded beside the column indices (predicated on the row bounds,
        // not on the loaded index), so only the x gathers wait for colIdx
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int k = base + lane + 8 * j;
            if (k < e) {
                cc[j] = 3 * colIdx[k];
                q[j] = v8[k];
                w8[j] = __bfloat162float(v1[k]);
            } else {
                cc[j] = -1;
            }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (cc[j] >= 0) {
                const float x0 = x[cc[j]], x1 = x[cc[j] + 1], x2 = x[cc[j] + 2];
                const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&q[j]);
                const float2 a01 = __bfloat1622float2(h[0]), a23 = __bfloat1622float2(h[1]);
                const float2 a45 = __bfloat1622float2(h[2]), a67 = __bfloat1622float2(h[3]);
                y0 += a01.x * x0 + a01.y * x1 + a23.x * x2;
                y1 += a23.y * x0 + a45.x * x1 + a45.y * x2;
                y2 += a67.x * x0 + a67.y * x1 + w8[j] * x2;
            }
    }
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) {
        y0 += __shfl_xor_sync(0xffffffffu, y0, o);
        y1 += __shfl_xor_sync(0xffffffffu, y1, o);
        y2 += __shfl_xor_sync(0xffffffffu, y2, o);
    }
    if (m0 < nN && lane < 3) {
        if (binv) {
            const float yv[3] = {y0, y1, y2};
            smooth_row<3>(m, lane, yv, x, r, mask, binv, omega, t);
        } else {
            const int d = 3 * m + lane;
            const float yy = lane == 0 ? y0 : (lane == 1 ? y1 : y2);
            t[d] = (mask && mask[d]) ? 0.f : r[d] - yy;
        }
    }
}

// Staged form of level_residual3_bf16_kernel for the fine level.  Persistent CTAs walk chunks of
// kStageRows block rows; the blocks of the next chunk (16-byte words, the ninth values and the
// column indices, contiguous in memory) are copied into shared memory with cp.async while the
// current chunk is computed, so that every CTA keeps a whole chunk of loads in flight.  Each row
// is then computed by 8 lanes from shared memory, as in the unstaged kernel (same order of
// operations, same results).  Stage layout (cap = the largest chunk's block count): cap uint4
// words | cap + 16 BF16 values | cap + 8 column indices; the index and BF16 ranges start on
// 16-byte boundaries below the chunk's first block and end on 16-byte boundaries above its last.
constexpr int kStageRows = 32;
constexpr int kStageThreads = kStageRows * 8;

__host__ __device__ inline size_t stage_v1_bytes(int cap) { return (((size_t)cap + 16) * 2 + 15) & ~(size_t)15; }
__host__ __device__ inline size_t stage_bytes_bf16(int cap) {
    return (size_t)cap * 16 + stage_v1_bytes(cap) + ((size_t)cap + 8) * 4;
}

__device__ __forceinline__ void stage_chunk_bf16(int b0, int b1, const uint4* __restrict__ v8,
                                                 const __nv_bfloat16* __restrict__ v1,
                                                 const int32_t* __restrict__ colIdx, char* stage, int cap) {
    uint4* s8 = reinterpret_cast<uint4*>(stage);
    __nv_bfloat16* s1 = reinterpret_cast<__nv_bfloat16*>(stage + (size_t)cap * 16);
    int32_t* sc = reinterpret_cast<int32_t*>(stage + (size_t)cap * 16 + stage_v1_bytes(cap));
    const int n8 = b1 - b0;
    for (int i = threadIdx.x; i < n8; i += kStageThreads) cp_async16(s8 + i, v8 + b0 + i);
    const int v1s = b0 & ~7;
    const int n1 = (b1 - v1s + 7) >> 3;  // 16-byte pieces of 8 BF16 values
    for (int i = threadIdx.x; i < n1; i += kStageThreads) cp_async16(s1 + 8 * i, v1 + v1s + 8 * i);
    const int cs = b0 & ~3;
    const int nc = (b1 - cs + 3) >> 2;  // 16-byte pieces of 4 indices
    for (int i = threadIdx.x; i < nc; i += kStageThreads) cp_async16(sc + 4 * i, colIdx + cs + 4 * i);
}

__global__ void __launch_bounds__(kStageThreads) level_residual3_bf16_staged_kernel(
    int nN, const int32_t* __restrict__ rowPtr, const int32_t* __restrict__ colIdx, const uint4* __restrict__ v8,
    const __nv_bfloat16* __restrict__ v1, const float* __restrict__ x, const float* __restrict__ r,
    const uint8_t* __restrict__ mask, float* __restrict__ t, const float* __restrict__ binv, float omega, int cap) {
    extern __shared__ __align__(16) char smem[];
    const size_t sb = (stage_bytes_bf16(cap) + 15) & ~(size_t)15;
    const int nChunks = (nN + kStageRows - 1) / kStageRows;
    const int lane = threadIdx.x & 7;
    const int rowInChunk = threadIdx.x >> 3;
    int ch = blockIdx.x;
    if (ch >= nChunks) return;
    int b0 = rowPtr[ch * kStageRows];
    int b1 = rowPtr[min((ch + 1) * kStageRows, nN)];
    stage_chunk_bf16(b0, b1, v8, v1, colIdx, smem, cap);
    cp_async_commit();
    int st = 0;
    for (; ch < nChunks; ch += gridDim.x, st ^= 1) {
        const int nx = ch + gridDim.x;
        int nb0 = 0, nb1 = 0;
        if (nx < nChunks) {
            nb0 = rowPtr[nx * kStageRows];
            nb1 = rowPtr[min((nx + 1) * kStageRows, nN)];
            stage_chunk_bf16(nb0, nb1, v8, v1, colIdx, smem + (st ^ 1) * sb, cap);
        }
        cp_async_commit();  // (an empty group when there is no next chunk)
        // this row's own entries and bounds, fetched while the stage completes
        const int m0 = ch * kStageRows + rowInChunk;
        const int m = m0 < nN ? m0 : nN - 1;
        const int s = rowPtr[m], e = rowPtr[m + 1];
        cp_async_wait<1>();
        __syncthreads();
        const char* sg = smem + st * sb;
        const uint4* s8 = reinterpret_cast<const uint4*>(sg);
        const __nv_bfloat16* s1 = reinterpret_cast<const __nv_bfloat16*>(sg + (size_t)cap * 16);
        const int32_t* sc = reinterpret_cast<const int32_t*>(sg + (size_t)cap * 16 + stage_v1_bytes(cap));
        const int o8 = b0, o1 = b0 & ~7, oc = b0 & ~3;
        float y0 = 0.f, y1 = 0.f, y2 = 0.f;
        for (int base = s; base < e; base += 32) {
            int cc[4];
            uint4 q[4];
            float w8[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int k = base + lane + 8 * j;
                if (k < e) {
                    cc[j] = 3 * sc[k - oc];
                    q[j] = s8[k - o8];
                    w8[j] = __bfloat162float(s1[k - o1]);
                } else {
                    cc[j] = -1;
                }
            }
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (cc[j] >= 0) {
                    const float x0 = x[cc[j]], x1 = x[cc[j] + 1], x2 = x[cc[j] + 2];
                    const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&q[j]);
                    const float2 a01 = __bfloat1622float2(h[0]), a23 = __bfloat1622float2(h[1]);
                    const float2 a45 = __bfloat1622float2(h[2]), a67 = __bfloat1622float2(h[3]);
                    y0 += a01.x * x0 + a01.y * x1 + a23.x * x2;
                    y1 += a23.y * x0 + a45.x * x1 + a45.y * x2;
                    y2 += a67.x * x0 + a67.y * x1 + w8[j] * x2;
                }
        }
#pragma unroll
        for (int o = 4; o > 0; o >>= 1) {
            y0 += __shfl_xor_sync(0xffffffffu, y0, o);
            y1 += __shfl_xor_sync(0xffffffffu, y1, o);
            y2 += __shfl_xor_sync(0xffffffffu, y2, o);
        }
        if (m0 < nN && lane < 3) {
            if (binv) {
                const float yv[3] = {y0, y1, y2};
                smooth_row<3>(m, lane, yv, x, r, mask, binv, omega, t);
            } else {
                const int d = 3 * m + lane;
                const float yy = lane == 0 ? y0 : (lane == 1 ? y1 : y2);
                t[d] = (mask && mask[d]) ? 0.f : r[d] - yy;
            }
        }
        __syncthreads();  // the stage is free for the chunk after next
        b0 = nb0;
        b1 = nb1;
    }
    cp_async_wait<0>();
}

// split BF16 copy of 3x3 blocks for level_residual3_bf16_kernel
__global__ void to_bf16_split_kernel(int64_t nb, const float* __restrict__ src, uint4* __restrict__ v8,
                                     __nv_bfloat16* __restrict__ v1) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nb) return;
    const float* a = src + k * 9;
    __nv_bfloat162 h[4] = {__floats2bfloat162_rn(a[0], a[1]), __floats2bfloat162_rn(a[2], a[3]),
                           __floats2bfloat162_rn(a[4], a[5]), __floats2bfloat162_rn(a[6], a[7])};
    v8[k] = *reinterpret_cast<uint4*>(h);
    v1[k] = __float2bfloat16(a[8]);
}

}  // namespace ef

using namespace ef;

size_t ef_sa_ap_rows_smem(int bf, int cap) { return (size_t)cap * bf * BC * sizeof(float); }
int ef_sa_ap_rows() { return kSaApRows; }

static inline int nb_(int64_t n, int t) { return (int)((n + t - 1) / t); }

int ef_amg_coarse_dofs() { return BC; }
int ef_max_coarsest_nodes() { return kMaxCoarsestDof / BC; }

ef_status ef_launch_galerkin(int bf, int64_t nCoarseBlocks, const int64_t* seg, const int32_t* src,
                             const int32_t* fineRowOfBlock, const int32_t* fineCol, const float* fineVals,
                             const uint8_t* fineMask, const float* offs, const int32_t* coarseRowOfBlock,
                             const int32_t* coarseCol, const uint8_t* coarseDead, float* coarseVals, cudaStream_t s) {
    if (nCoarseBlocks == 0) return EF_OK;
    if (bf == 3)
        galerkin_kernel<3><<<nb_(nCoarseBlocks, 64), 64, 0, ef::counted(s)>>>(nCoarseBlocks, seg, src, fineRowOfBlock, fineCol,
                                                                 fineVals, fineMask, offs, coarseRowOfBlock, coarseCol,
                                                                 coarseDead, coarseVals);
    else
        galerkin_kernel<6><<<nb_(nCoarseBlocks, 64), 64, 0, ef::counted(s)>>>(nCoarseBlocks, seg, src, fineRowOfBlock, fineCol,
                                                                 fineVals, fineMask, offs, coarseRowOfBlock, coarseCol,
                                                                 coarseDead, coarseVals);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_bj6_setup(int nN, const int64_t* diagPos, const float* vals, float* inv, cudaStream_t s) {
    bj6_setup_kernel<<<nb_(nN, 64), 64, 0, ef::counted(s)>>>(nN, diagPos, vals, inv);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_bj_apply(int bs, int nN, const float* binv, const uint8_t* mask, float omega, const float* r,
                             float* x, int accumulate, cudaStream_t s) {
    if (bs == 3)
        EF_CUDA(ef::launch_dep(bj_apply_kernel<3>, nb_(nN, 256), 256, 0, s, nN, binv, mask, omega, r, x, accumulate));
    else
        EF_CUDA(ef::launch_dep(bj_apply_kernel<6>, nb_(nN, 256), 256, 0, s, nN, binv, mask, omega, r, x, accumulate));
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

// binv == nullptr: t = r - A x; otherwise one smoothing sweep t = x + omega D^-1 (r - A x)
ef_status ef_launch_level_residual(int bs, int nN, const int32_t* rowPtr, const int32_t* colIdx, const float* vals,
                                   const float* x, const float* r, const uint8_t* mask, float* t, cudaStream_t s,
                                   const float* binv, float omega, const void* valsH, float ys) {
    if (bs == 3) {
        if (ys != 1.f) {
            ef_set_error("level residual: a scaled product is implemented for 6-DOF levels only");
            return EF_ERR_ARG;
        }
        EF_CUDA(ef::launch_dep(level_residual_kernel<3>, nb_((int64_t)nN * 8, 256), 256, 0, s, nN, rowPtr, colIdx, vals,
                x, r, mask, t, binv, omega));
    } else {
        EF_CUDA(ef::launch_dep(level_residual6_kernel, nb_((int64_t)nN * 32, 256), 256, 0, s, nN, rowPtr, colIdx, vals,
                x, r, mask, t, binv, omega, (const uint32_t*)valsH, ys));
    }
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_scale_blocks6(int64_t nB, const int32_t* colIdx, const float* vals, const float* binv,
                                  const uint8_t* dead, float* out, cudaStream_t s) {
    if (nB <= 0) return EF_OK;
    scale_blocks6_kernel<<<nb_(nB, 128), 128, 0, ef::counted(s)>>>(nB, colIdx, vals, binv, dead, out);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_sa_post6_setup(int64_t nAP, const int32_t* apRow, const int32_t* apToP, const float* Pv,
                                   const float* APv, const float* binv, float omega, float alpha, float* C,
                                   cudaStream_t s) {
    if (nAP <= 0) return EF_OK;
    sa_post6_setup_kernel<<<nb_(nAP, 128), 128, 0, ef::counted(s)>>>(nAP, apRow, apToP, Pv, APv, binv, omega, alpha,
                                                                     C);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_sa_post6_fused(int nN, const int32_t* rowPtr, const int32_t* col, const float* C, const float* e,
                                   const float* r, const float* t, const float* binv, const uint8_t* dead,
                                   float omega, float* x, cudaStream_t s) {
    if (nN <= 0) return EF_OK;
    EF_CUDA(ef::launch_dep(sa_post6_fused_kernel, nb_((int64_t)nN * 32, 256), 256, 0, s, nN, rowPtr, col, C, e, r, t,
                           binv, dead, omega, x));
    return EF_OK;
}

// ---- smoothed aggregation launchers ----
ef_status ef_launch_sa_damping(const double* n2, float* wP, cudaStream_t s) {
    sa_damping_kernel<<<1, 1, 0, ef::counted(s)>>>(n2, wP);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_sa_setup(int bf, int64_t nP, const int32_t* pRow, const int32_t* pCol, const int64_t* pSeg,
                             const int32_t* pSrc, int64_t nAP, const int32_t* apRow, const int64_t* apSeg,
                             const int32_t* apK, const int32_t* apP, const int32_t* fineCol, const float* fineVals,
                             const uint8_t* fineMask, const float* offs, const int32_t* agg, const float* binv,
                             const float* wP, float* Pv, float* APv, int64_t nC, const int64_t* cSeg,
                             const int32_t* cP, const int32_t* cAP, const int32_t* coarseRowOfBlock,
                             const int32_t* coarseCol, const uint8_t* coarseDead, float* coarseVals, int nF,
                             const int32_t* apRowPtr, int apCap, cudaStream_t s) {
#define EF_SA(BF_)                                                                                             \
    sa_prolongator_kernel<BF_><<<nb_(nP, 128), 128, 0, ef::counted(s)>>>(nP, pRow, pCol, pSeg, pSrc, fineCol, \
                                                                        fineVals, fineMask, offs, agg, binv,  \
                                                                        wP, Pv);                              \
    if (apRowPtr)                                                                                              \
        sa_ap_rows_kernel<BF_><<<nb_(nF, kSaApRows), kSaApThreads, ef_sa_ap_rows_smem(BF_, apCap),            \
                                 ef::counted(s)>>>(nF, apCap, apRowPtr, apSeg, apK, apP, fineCol, fineVals,    \
                                                   fineMask, Pv, APv);                                         \
    else                                                                                                       \
        sa_ap_kernel<BF_><<<nb_(nAP, 128), 128, 0, ef::counted(s)>>>(nAP, apRow, apSeg, apK, apP, fineCol,    \
                                                                    fineVals, fineMask, Pv, APv);             \
    if (galWarp)                                                                                               \
        sa_galerkin_warp_kernel<BF_><<<nb_(nC, kGalWarps), 32 * kGalWarps, 0, ef::counted(s)>>>(               \
            nC, cSeg, cP, cAP, Pv, APv, coarseRowOfBlock, coarseCol, coarseDead, coarseVals);                  \
    else                                                                                                       \
        sa_galerkin_kernel<BF_><<<nb_(nC, 64), 64, 0, ef::counted(s)>>>(nC, cSeg, cP, cAP, Pv, APv,           \
                                                                       coarseRowOfBlock, coarseCol, coarseDead, \
                                                                       coarseVals)
    if (nP == 0 || nC == 0) return EF_OK;
    const char* ge = getenv("EF_GALERKIN_WARP");  // 0: a thread per coarse block
    const bool galWarp = !ge || atoi(ge) != 0;
    if (bf == 3) {
        EF_SA(3);
    } else {
        EF_SA(6);
    }
#undef EF_SA
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_sa_restrict(int bf, int nC, const int32_t* tPtr, const int32_t* tIdx, const int32_t* pRow,
                                const float* Pv, const float* t, const uint8_t* coarseDead, float* rc,
                                cudaStream_t s) {
    if (bf == 3)
        sa_restrict_kernel<3><<<nb_((int64_t)nC * 32, 256), 256, 0, ef::counted(s)>>>(nC, tPtr, tIdx, pRow, Pv, t,
                                                                                      coarseDead, rc);
    else
        sa_restrict_kernel<6><<<nb_((int64_t)nC * 32, 256), 256, 0, ef::counted(s)>>>(nC, tPtr, tIdx, pRow, Pv, t,
                                                                                      coarseDead, rc);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

// two-stage restriction rc = P^T t through c [nP][6] and prolongation x += alpha P xc through
// c [nP][bf] (the same scratch of the level)
ef_status ef_launch_sa_restrict2(int bf, int nC, int64_t nP, const int32_t* tPtr, const int32_t* tIdx,
                                 const int32_t* pRow, const float* Pv, const float* t, const uint8_t* coarseDead,
                                 float* c, float* rc, cudaStream_t s) {
    if (nP > 0) {
        if (bf == 3)
            EF_CUDA(ef::launch_dep(sa_restrict_contrib_kernel<3>, nb_(nP, 256), 256, 0, s, nP, pRow, Pv, t, c));
        else
            EF_CUDA(ef::launch_dep(sa_restrict_contrib_kernel<6>, nb_(nP, 256), 256, 0, s, nP, pRow, Pv, t, c));
    }
    EF_CUDA(ef::launch_dep(sa_restrict_sum_kernel, nb_((int64_t)nC * 32, 256), 256, 0, s, nC, tPtr, tIdx, c, coarseDead,
            rc));
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_sa_prolong2(int bf, int nF, int64_t nP, const int32_t* pRowPtr, const int32_t* pCol,
                                const float* Pv, const float* xc, const uint8_t* mask, float* c, float* x, float alpha,
                                cudaStream_t s) {
    if (nP > 0) {
        if (bf == 3)
            EF_CUDA(ef::launch_dep(sa_prolong_contrib_kernel<3>, nb_(nP, 256), 256, 0, s, nP, pCol, Pv, xc, c));
        else
            EF_CUDA(ef::launch_dep(sa_prolong_contrib_kernel<6>, nb_(nP, 256), 256, 0, s, nP, pCol, Pv, xc, c));
    }
    if (bf == 3)
        EF_CUDA(ef::launch_dep(sa_prolong_apply_kernel<3>, nb_(nF, 256), 256, 0, s, nF, pRowPtr, c, mask, x, alpha));
    else
        EF_CUDA(ef::launch_dep(sa_prolong_apply_kernel<6>, nb_(nF, 256), 256, 0, s, nF, pRowPtr, c, mask, x, alpha));
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

// transpose-order copy of P for the one-pass restriction
ef_status ef_launch_sa_block_copy(int bf, int64_t nP, const int32_t* tIdx, const float* Pv, float* dst,
                                  cudaStream_t s) {
    if (nP <= 0) return EF_OK;
    if (bf == 3)
        sa_block_copy_kernel<3><<<nb_(nP, 256), 256, 0, ef::counted(s)>>>(nP, tIdx, Pv, dst);
    else
        sa_block_copy_kernel<6><<<nb_(nP, 256), 256, 0, ef::counted(s)>>>(nP, tIdx, Pv, dst);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_sa_block_copy_h(int64_t nP, const int32_t* tIdx, const float* Pv, void* q0, void* q1, void* q2,
                                    cudaStream_t s) {
    if (nP <= 0) return EF_OK;
    sa_block_copy_h_kernel<<<nb_(nP, 256), 256, 0, ef::counted(s)>>>(nP, tIdx, Pv, (uint4*)q0, (uint4*)q1,
                                                                      (uint32_t*)q2);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_sa_restrict_onepass_h(int nC, const int32_t* tPtr, const int32_t* rowT, const void* q0,
                                          const void* q1, const void* q2, const float* t, const uint8_t* coarseDead,
                                          float* rc, cudaStream_t s) {
    if (nC <= 0) return EF_OK;
    const char* e = getenv("EF_SA_RESTRICT_WARP");  // read at each launch site (the cycle is captured once)
    const bool warp = !e || atoi(e) != 0;
    if (warp)
        EF_CUDA(ef::launch_dep(sa_restrict_warp_h_kernel, nb_(nC, kSaRestrictWarpNodes), 32 * kSaRestrictWarpNodes,
                               0, s, nC, tPtr, rowT, (const uint4*)q0, (const uint4*)q1, (const uint32_t*)q2, t,
                               coarseDead, rc));
    else
        EF_CUDA(ef::launch_dep(sa_restrict_onepass_h_kernel, nC, kSaRestrictThreads, 0, s, nC, tPtr, rowT,
                               (const uint4*)q0, (const uint4*)q1, (const uint32_t*)q2, t, coarseDead, rc));
    return EF_OK;
}

size_t ef_sa_prolong_onepass_smem(int bf, int cap) { return (size_t)cap * bf * sizeof(float); }
int ef_sa_prolong_onepass_rows() { return kSaProlongRows; }

ef_status ef_launch_sa_restrict_onepass(int bf, int nC, const int32_t* tPtr, const int32_t* rowT, const float* PT,
                                        const float* t, const uint8_t* coarseDead, float* rc, cudaStream_t s) {
    if (nC <= 0) return EF_OK;
    if (bf == 3)
        EF_CUDA(ef::launch_dep(sa_restrict_onepass_kernel<3>, nC, kSaRestrictThreads, 0, s, nC, tPtr, rowT, PT, t,
                               coarseDead, rc));
    else
        EF_CUDA(ef::launch_dep(sa_restrict_onepass_kernel<6>, nC, kSaRestrictThreads, 0, s, nC, tPtr, rowT, PT, t,
                               coarseDead, rc));
    return EF_OK;
}

ef_status ef_launch_sa_prolong_onepass(int bf, int nF, int cap, const int32_t* pRowPtr, const int32_t* pCol,
                                       const float* Pv, const float* xc, const uint8_t* mask, float* x, float alpha,
                                       cudaStream_t s) {
    if (nF <= 0) return EF_OK;
    const int grid = nb_(nF, kSaProlongRows);
    const size_t smem = ef_sa_prolong_onepass_smem(bf, cap);
    if (bf == 3)
        EF_CUDA(ef::launch_dep(sa_prolong_onepass_kernel<3>, grid, kSaProlongThreads, smem, s, nF, cap, pRowPtr, pCol,
                               Pv, xc, mask, x, alpha));
    else
        EF_CUDA(ef::launch_dep(sa_prolong_onepass_kernel<6>, grid, kSaProlongThreads, smem, s, nF, cap, pRowPtr, pCol,
                               Pv, xc, mask, x, alpha));
    return EF_OK;
}

ef_status ef_launch_sa_prolong(int bf, int nF, const int32_t* pRowPtr, const int32_t* pCol, const float* Pv,
                               const float* xc, const uint8_t* mask, float* x, float alpha, cudaStream_t s) {
    if (bf == 3)
        sa_prolong_kernel<3><<<nb_(nF, 256), 256, 0, ef::counted(s)>>>(nF, pRowPtr, pCol, Pv, xc, mask, x, alpha);
    else
        sa_prolong_kernel<6><<<nb_(nF, 256), 256, 0, ef::counted(s)>>>(nF, pRowPtr, pCol, Pv, xc, mask, x, alpha);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_restrict(int bf, int nC, const int32_t* aggPtr, const int32_t* aggIdx, const float* offs,
                             const float* t, const uint8_t* coarseDead, float* rc, cudaStream_t s) {
    if (bf == 3)
        restrict_kernel<3><<<nb_((int64_t)nC * 32, 256), 256, 0, ef::counted(s)>>>(nC, aggPtr, aggIdx, offs, t, coarseDead, rc);
    else
        restrict_kernel<6><<<nb_((int64_t)nC * 32, 256), 256, 0, ef::counted(s)>>>(nC, aggPtr, aggIdx, offs, t, coarseDead, rc);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_prolong(int bf, int nN, const int32_t* agg, const float* offs, const float* xc,
                            const uint8_t* mask, float* x, cudaStream_t s, float alpha) {
    if (bf == 3)
        prolong_kernel<3><<<nb_(nN, 256), 256, 0, ef::counted(s)>>>(nN, agg, offs, xc, mask, x, alpha);
    else
        prolong_kernel<6><<<nb_(nN, 256), 256, 0, ef::counted(s)>>>(nN, agg, offs, xc, mask, x, alpha);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_coarsest_inverse(int nN, const int32_t* rowPtr, const int32_t* colIdx, const float* vals,
                                     float* inv, cudaStream_t s) {
    if (BC * nN > kMaxCoarsestDof) {
        ef_set_error("coarsest level too large for the dense solve");
        return EF_ERR_ARG;
    }
    const size_t smem = sizeof(float) * BC * nN * (2 * BC * nN + 1);
    EF_CUDA(cudaFuncSetAttribute(coarsest_inverse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    coarsest_inverse_kernel<<<1, dim3(32, 32), smem, ef::counted(s)>>>(nN, rowPtr, colIdx, vals, inv);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_coarsest_apply(int n, const float* inv, const float* r, const uint8_t* dead, float* x,
                                   cudaStream_t s) {
    EF_CUDA(ef::launch_dep(coarsest_apply_kernel, nb_((int64_t)n * 32, 256), 256, 0, s, n, inv, r, dead, x));
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

int ef_coarse_cycle_threads() { return kCoarseCtas * kCoarseThreads; }

ef_status ef_launch_coarse_cycle(const ef::CoarseOp* ops, int nOps, cudaStream_t s) {
    coarse_cycle_kernel<<<kCoarseCtas, kCoarseThreads, 0, ef::counted(s)>>>(ops, nOps);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_to_bf16(int64_t n, const float* src, void* dst, cudaStream_t s) {
    if (n == 0) return EF_OK;
    to_bf16_kernel<<<nb_(n, 256), 256, 0, ef::counted(s)>>>(n, src, (__nv_bfloat16*)dst);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_scale_rnorm(int64_t n, float* x, const double* n2, cudaStream_t s) {
    if (n == 0) return EF_OK;
    scale_rnorm_kernel<<<nb_(n, 256), 256, 0, ef::counted(s)>>>(n, x, n2);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

// x *= *fac (a factor left on the device in FP32)
__global__ void scale_by_kernel(int64_t n, float* __restrict__ x, const float* __restrict__ fac) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] *= *fac;
}
ef_status ef_launch_scale_by(int64_t n, float* x, const float* fac, cudaStream_t s) {
    if (n == 0) return EF_OK;
    scale_by_kernel<<<nb_(n, 256), 256, 0, ef::counted(s)>>>(n, x, fac);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_fill_hash(int64_t n, float* x, cudaStream_t s) {
    if (n == 0) return EF_OK;
    fill_hash_kernel<<<nb_(n, 256), 256, 0, ef::counted(s)>>>(n, x);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

// fine-level (3x3 blocks) residual t = r - A x with the split BF16 copy of the block values
// (vals: nBlocks uint4 words followed by nBlocks BF16 values)
ef_status ef_launch_level_residual_bf16(int nN, int64_t nBlocks, const int32_t* rowPtr, const int32_t* colIdx,
                                        const void* vals, const float* x, const float* r, const uint8_t* mask,
                                        float* t, cudaStream_t s, const float* binv, float omega) {
    const uint4* v8 = (const uint4*)vals;
    const __nv_bfloat16* v1 = (const __nv_bfloat16*)(v8 + nBlocks);
    level_residual3_bf16_kernel<<<nb_((int64_t)nN * 8, 256), 256, 0, ef::counted(s)>>>(nN, rowPtr, colIdx, v8, v1, x,
                                                                                     r, mask, t, binv, omega);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

// largest block count of a chunk of kStageRows rows (host)
int ef_stage_cap(int nN, const int32_t* rowPtrHost) {
    int cap = 0;
    for (int m0 = 0; m0 < nN; m0 += kStageRows)
        cap = std::max(cap, rowPtrHost[std::min(m0 + kStageRows, nN)] - rowPtrHost[m0]);
    return cap;
}

// staged fine-level BF16 residual / sweep; nSM CTAs x the resident count for the stage size
ef_status ef_launch_level_residual_bf16_staged(int nSM, int cap, int nN, int64_t nBlocks, const int32_t* rowPtr,
                                               const int32_t* colIdx, const void* vals, const float* x, const float* r,
                                               const uint8_t* mask, float* t, cudaStream_t s, const float* binv,
                                               float omega) {
    const uint4* v8 = (const uint4*)vals;
    const __nv_bfloat16* v1 = (const __nv_bfloat16*)(v8 + nBlocks);
    const size_t smem = 2 * ((stage_bytes_bf16(cap) + 15) & ~(size_t)15);
    static size_t attrSet = 0;
    if (smem > 48 * 1024 && smem > attrSet) {
        EF_CUDA(cudaFuncSetAttribute(level_residual3_bf16_staged_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
        attrSet = smem;
    }
    int perSM = 0;
    EF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, level_residual3_bf16_staged_kernel, kStageThreads,
                                                          smem));
    if (perSM < 1) {
        ef_set_error("staged BF16 residual: chunk does not fit in shared memory");
        return EF_ERR_ARG;
    }
    const int nChunks = (nN + kStageRows - 1) / kStageRows;
    const int grid = std::max(1, std::min(nChunks, perSM * nSM));
    level_residual3_bf16_staged_kernel<<<grid, kStageThreads, smem, ef::counted(s)>>>(
        nN, rowPtr, colIdx, v8, v1, x, r, mask, t, binv, omega, cap);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_to_bf16_split(int64_t nBlocks, const float* src, void* dst, cudaStream_t s) {
    if (nBlocks == 0) return EF_OK;
    uint4* v8 = (uint4*)dst;
    to_bf16_split_kernel<<<nb_(nBlocks, 256), 256, 0, ef::counted(s)>>>(nBlocks, src, v8,
                                                                        (__nv_bfloat16*)(v8 + nBlocks));
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_cheb_step(int bs, int nN, const float* binv, const uint8_t* mask, float a, float b, const float* t,
                              float* d, float* x, int first, cudaStream_t s) {
    if (bs == 3)
        cheb_step_kernel<3><<<nb_(nN, 256), 256, 0, ef::counted(s)>>>(nN, binv, mask, a, b, t, d, x, first);
    else
        cheb_step_kernel<6><<<nb_(nN, 256), 256, 0, ef::counted(s)>>>(nN, binv, mask, a, b, t, d, x, first);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}
