// Sliced-ELL copies of the fine 3x3-block system and the fine-level kernels that stream them.
//
// The fine system's block rows are grouped into slices of 32; a slice is as wide as its longest
// row (shorter rows are padded with zero blocks whose column is the row itself) and its entries
// are stored column-major: entry j of the slice's row i sits at slot e0 + 32 j + i.  A warp takes
// one slice, a lane one row, so at every step j the warp reads 32 consecutive column indices and
// 32 consecutive blocks -- fully coalesced, with no row-pointer load ahead of them -- and, on a
// mesh numbered along a grid line, gathers x from 32 consecutive nodes.  An optional row
// permutation (rows sorted by length within windows) keeps the padding small on meshes whose row
// lengths vary; on the structured hex8 box it is the identity and costs one coalesced load.
//
// Two value copies, refreshed from the FP32 block values after every assembly:
//  * FP32, nine planes per slot column: value k of slot t at 9 (t - i) + 32 k + i (i = t mod 32),
//    for the FGMRES product y = K z;
//  * BF16 split: one 16-byte word with values 0..7 per slot and value 8 in a second array, for the
//    multigrid's fine smoothing sweeps and residuals (a preconditioner only).
// Summation per row runs over the row's blocks in column order with one accumulator per output
// component: deterministic, not the same rounding as the CSR kernels.

#include <cuda_bf16.h>
#include <stdint.h>

#include "ef_common.cuh"

namespace ef {

constexpr int kSellThreads = 128;  // four warps per CTA
constexpr int kSellSlicesPerCta = kSellThreads / 32;  // the product: a warp per slice
// Split slices: S warps per slice, each taking a contiguous share of the slice's entries, four
// warps per CTA up to S = 4 and S warps (one slice) above

__global__ void sell_refresh_kernel(int64_t nE, const int32_t* __restrict__ src, const float* __restrict__ bsr,
                                    float* __restrict__ v9, uint4* __restrict__ v8, __nv_bfloat16* __restrict__ v1) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nE) return;
    const int64_t b = src[t];
    float a[9];
    if (b >= 0) {
#pragma unroll
        for (int k = 0; k < 9; ++k) a[k] = bsr[b * 9 + k];
    } else {
#pragma unroll
        for (int k = 0; k < 9; ++k) a[k] = 0.f;
    }
    const int64_t i = t & 31;
    float* d = v9 + 9 * (t - i) + i;
#pragma unroll
    for (int k = 0; k < 9; ++k) d[32 * k] = a[k];
    if (v8) {
        __nv_bfloat162 h[4] = {__floats2bfloat162_rn(a[0], a[1]), __floats2bfloat162_rn(a[2], a[3]),
                               __floats2bfloat162_rn(a[4], a[5]), __floats2bfloat162_rn(a[6], a[7])};
        v8[t] = *reinterpret_cast<const uint4*>(h);
        v1[t] = __float2bfloat16_rn(a[8]);
    }
}

// The slice and entry range of this warp: warp h of the S warps of a slice takes entries
// [j0, j1) = [ceil(h w / S), ceil((h + 1) w / S)) of its width w.  Returns false past the last
// slice.
struct SellPart {
    int sl, h, lane, j0, j1;
    int64_t e0;
};
constexpr int sell_split_threads(int S) { return S <= 4 ? kSellThreads : 32 * S; }
template <int S>
__device__ __forceinline__ bool sell_part(int nSlices, const int64_t* __restrict__ off, SellPart& p) {
    constexpr int spc = sell_split_threads(S) / (32 * S);
    p.lane = threadIdx.x & 31;
    const int wi = threadIdx.x >> 5;
    p.sl = blockIdx.x * spc + wi / S;
    p.h = wi % S;
    if (p.sl >= nSlices) return false;
    p.e0 = off[p.sl];
    const int w = (int)((off[p.sl + 1] - p.e0) >> 5);
    p.j0 = (p.h * w + S - 1) / S;
    p.j1 = ((p.h + 1) * w + S - 1) / S;
    return true;
}

// the partial sums of warps 1..S-1 of a slice go through shared memory to warp 0, which adds them
// after its own in warp order (a fixed order: deterministic)
template <int S>
__device__ __forceinline__ bool sell_combine(const SellPart& p, bool active, float& y0, float& y1, float& y2) {
    if constexpr (S == 1) {
        return active;
    } else {
        constexpr int spc = sell_split_threads(S) / (32 * S);
        __shared__ float part[spc][S - 1][3][32];
        const int ls = (threadIdx.x >> 5) / S;
        if (active && p.h > 0) {
            part[ls][p.h - 1][0][p.lane] = y0;
            part[ls][p.h - 1][1][p.lane] = y1;
            part[ls][p.h - 1][2][p.lane] = y2;
        }
        __syncthreads();
        if (!active || p.h != 0) return false;
#pragma unroll
        for (int q = 0; q < S - 1; ++q) {
            y0 += part[ls][q][0][p.lane];
            y1 += part[ls][q][1][p.lane];
            y2 += part[ls][q][2][p.lane];
        }
        return true;
    }
}

// y = K x on the free DOFs (0 on masked rows); COPY: xcopy = x as well; S warps per slice
template <bool COPY, int S>
__global__ void __launch_bounds__(sell_split_threads(S)) sell_spmv3_kernel(
    int nN, int nSlices, const int64_t* __restrict__ off, const int32_t* __restrict__ perm,
    const int32_t* __restrict__ col, const float* __restrict__ v9, const float* __restrict__ x,
    const uint8_t* __restrict__ mask, float* __restrict__ y, float* __restrict__ xcopy) {
    ef::dep_entry();
    SellPart p;
    const bool active = sell_part<S>(nSlices, off, p);
    float y0 = 0.f, y1 = 0.f, y2 = 0.f;
    if (active) {
        const int32_t* cs = col + p.e0 + p.lane;
        const float* vs = v9 + 9 * p.e0 + p.lane;
#pragma unroll 3
        for (int j = p.j0; j < p.j1; ++j) {
            const int c3 = 3 * __ldcs(cs + 32 * j);
            const float* vv = vs + 288 * j;
            const float a0 = __ldcs(vv), a1 = __ldcs(vv + 32), a2 = __ldcs(vv + 64);
            const float a3 = __ldcs(vv + 96), a4 = __ldcs(vv + 128), a5 = __ldcs(vv + 160);
            const float a6 = __ldcs(vv + 192), a7 = __ldcs(vv + 224), a8 = __ldcs(vv + 256);
            const float x0 = x[c3], x1 = x[c3 + 1], x2 = x[c3 + 2];
            y0 += a0 * x0 + a1 * x1 + a2 * x2;
            y1 += a3 * x0 + a4 * x1 + a5 * x2;
            y2 += a6 * x0 + a7 * x1 + a8 * x2;
        }
    }
    if (!sell_combine<S>(p, active, y0, y1, y2)) return;
    const int r = p.sl * 32 + p.lane;
    if (r >= nN) return;
    const int m = perm ? perm[r] : r;
    const int d = 3 * m;
    y[d + 0] = mask[d + 0] ? 0.f : y0;
    y[d + 1] = mask[d + 1] ? 0.f : y1;
    y[d + 2] = mask[d + 2] ? 0.f : y2;
    if (COPY) {
        xcopy[d + 0] = x[d + 0];
        xcopy[d + 1] = x[d + 1];
        xcopy[d + 2] = x[d + 2];
    }
}

// t = r - K x on the fine level (0 on masked rows), or with binv a damped block-Jacobi sweep
// t = x + omega D^-1 (r - K x) (masked DOFs keep x), from the BF16 split copy; S warps per slice
template <int S>
__global__ void __launch_bounds__(sell_split_threads(S)) sell_level3_bf16_kernel(
    int nN, int nSlices, const int64_t* __restrict__ off, const int32_t* __restrict__ perm,
    const int32_t* __restrict__ col, const uint4* __restrict__ v8, const __nv_bfloat16* __restrict__ v1,
    const float* __restrict__ x, const float* __restrict__ r, const uint8_t* __restrict__ mask, float* __restrict__ t,
    const float* __restrict__ binv, float omega) {
    ef::dep_entry();
    SellPart p;
    const bool active = sell_part<S>(nSlices, off, p);
    float y0 = 0.f, y1 = 0.f, y2 = 0.f;
    if (active) {
        const int32_t* cs = col + p.e0 + p.lane;
        const uint4* qs = v8 + p.e0 + p.lane;
        const __nv_bfloat16* ws = v1 + p.e0 + p.lane;
#pragma unroll 4
        for (int j = p.j0; j < p.j1; ++j) {
            const int c3 = 3 * __ldcs(cs + 32 * j);
            const uint4 q = __ldcs(qs + 32 * j);
            const float w8 = __bfloat162float(ws[32 * j]);
            const float x0 = x[c3], x1 = x[c3 + 1], x2 = x[c3 + 2];
            const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&q);
            const float2 a01 = __bfloat1622float2(h[0]), a23 = __bfloat1622float2(h[1]);
            const float2 a45 = __bfloat1622float2(h[2]), a67 = __bfloat1622float2(h[3]);
            y0 += a01.x * x0 + a01.y * x1 + a23.x * x2;
            y1 += a23.y * x0 + a45.x * x1 + a45.y * x2;
            y2 += a67.x * x0 + a67.y * x1 + w8 * x2;
        }
    }
    if (!sell_combine<S>(p, active, y0, y1, y2)) return;
    const int rr = p.sl * 32 + p.lane;
    if (rr >= nN) return;
    const int m = perm ? perm[rr] : rr;
    const int d = 3 * m;
    const bool k0 = mask[d], k1 = mask[d + 1], k2 = mask[d + 2];
    const float t0 = k0 ? 0.f : r[d] - y0, t1 = k1 ? 0.f : r[d + 1] - y1, t2 = k2 ? 0.f : r[d + 2] - y2;
    if (!binv) {
        t[d] = t0;
        t[d + 1] = t1;
        t[d + 2] = t2;
        return;
    }
    const float* B = binv + 9 * (int64_t)m;
    const float z0 = B[0] * t0 + B[1] * t1 + B[2] * t2;
    const float z1 = B[3] * t0 + B[4] * t1 + B[5] * t2;
    const float z2 = B[6] * t0 + B[7] * t1 + B[8] * t2;
    const float x0 = x[d], x1 = x[d + 1], x2 = x[d + 2];
    t[d] = k0 ? x0 : x0 + omega * z0;
    t[d + 1] = k1 ? x1 : x1 + omega * z1;
    t[d + 2] = k2 ? x2 : x2 + omega * z2;
}

}  // namespace ef

using namespace ef;

static inline unsigned sell_grid(int nSlices) {
    return (unsigned)((nSlices + kSellSlicesPerCta - 1) / kSellSlicesPerCta);
}
static inline unsigned sell_split_grid(int nSlices, int S) {
    const int spc = sell_split_threads(S) / (32 * S);
    return (unsigned)((nSlices + spc - 1) / spc);
}

ef_status ef_launch_sell_refresh(int64_t nE, const int32_t* src, const float* bsr, float* v9, void* v8, void* v1,
                                 cudaStream_t s) {
    if (nE <= 0) return EF_OK;
    sell_refresh_kernel<<<(unsigned)((nE + 255) / 256), 256, 0, ef::counted(s)>>>(
        nE, src, bsr, v9, (uint4*)v8, (__nv_bfloat16*)v1);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_sell_spmv3(int nN, int nSlices, const int64_t* off, const int32_t* perm, const int32_t* col,
                               const float* v9, const float* x, const uint8_t* mask, float* y, float* xcopy, int split,
                               cudaStream_t s) {
    if (nSlices <= 0) return EF_OK;
#define EF_SPMV3(C_, S_)                                                                                           \
    EF_CUDA(ef::launch_dep(sell_spmv3_kernel<C_, S_>, sell_split_grid(nSlices, S_), sell_split_threads(S_), 0, s, \
                           nN, nSlices, off, perm, col, v9, x, mask, y, xcopy))
#define EF_SPMV3_S(C_)      \
    if (split == 2)         \
        EF_SPMV3(C_, 2);    \
    else if (split == 4)    \
        EF_SPMV3(C_, 4);    \
    else if (split == 8)    \
        EF_SPMV3(C_, 8);    \
    else                    \
        EF_SPMV3(C_, 1)
    if (xcopy) {
        EF_SPMV3_S(true);
    } else {
        EF_SPMV3_S(false);
    }
#undef EF_SPMV3_S
#undef EF_SPMV3
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_sell_level3_bf16(int nN, int nSlices, const int64_t* off, const int32_t* perm, const int32_t* col,
                                     const void* v8, const void* v1, const float* x, const float* r,
                                     const uint8_t* mask, float* t, const float* binv, float omega, int split,
                                     cudaStream_t s) {
    if (nSlices <= 0) return EF_OK;
#define EF_L3(S_)                                                                                                   \
    EF_CUDA(ef::launch_dep(sell_level3_bf16_kernel<S_>, sell_split_grid(nSlices, S_), sell_split_threads(S_), 0, s, \
                           nN, nSlices, off, perm, col, (const uint4*)v8, (const __nv_bfloat16*)v1, x, r, mask, t,   \
                           binv, omega))
    if (split == 1)
        EF_L3(1);
    else if (split == 2)
        EF_L3(2);
    else if (split == 8)
        EF_L3(8);
    else
        EF_L3(4);
#undef EF_L3
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}
