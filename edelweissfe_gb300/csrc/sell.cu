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

#include "amg_sa_body.h"
#include "ef_common.cuh"

namespace ef {

constexpr int kSellThreads = 128;  // four warps per CTA
constexpr int kSellSlicesPerCta = kSellThreads / 32;  // the product: a warp per slice
// Split slices: S warps per slice, each taking a contiguous share of the slice's entries, four
// warps per CTA up to S = 4 and S warps (one slice) above

// FP32 planes of K; the BF16 copy holds K, or with binv the blocks of K (M D^-1) (the block
// inverse of the slot's column node with the rows of masked DOFs zeroed), for the residual of the
// block-Jacobi sweep from zero: r - K (w M D^-1 r) = r - w (K M D^-1) r
__global__ void sell_refresh_kernel(int64_t nE, const int32_t* __restrict__ src, const float* __restrict__ bsr,
                                    float* __restrict__ v9, uint4* __restrict__ v8, __nv_bfloat16* __restrict__ v1,
                                    const int32_t* __restrict__ col, const float* __restrict__ binv,
                                    const uint8_t* __restrict__ mask) {
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
    if (v8 && binv) {
        const int64_t c = col[t];
        const float* D = binv + 9 * c;
        float sa[9];
#pragma unroll
        for (int p = 0; p < 3; ++p)
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                float z = 0.f;
#pragma unroll
                for (int u = 0; u < 3; ++u) z += mask[3 * c + u] ? 0.f : a[3 * p + u] * D[3 * u + q];
                sa[3 * p + q] = z;
            }
#pragma unroll
        for (int k = 0; k < 9; ++k) a[k] = sa[k];
    }
    if (v8) {
        __nv_bfloat162 h[4] = {__floats2bfloat162_rn(a[0], a[1]), __floats2bfloat162_rn(a[2], a[3]),
                               __floats2bfloat162_rn(a[4], a[5]), __floats2bfloat162_rn(a[6], a[7])};
        v8[t] = *reinterpret_cast<const uint4*>(h);
        v1[t] = __float2bfloat16_rn(a[8]);
    }
}

// Diagonal form of the slices (structured meshes): every block column is its row plus one of a few
// node offsets, slot column j of every slice holding offset dia[j] (zero blocks where the row has
// no such neighbour), so the column is computed, not loaded, and the x gathers of a warp are 32
// consecutive nodes.  The rows are in natural order; a column outside the nodes is clamped (its
// block is zero).
__device__ __forceinline__ int dia_column(int row, int d, int nN) { return min(max(row + d, 0), nN - 1); }

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

// y = sc K x on the free DOFs (0 on masked rows); COPY: xcopy = sc x as well; sc = *scale (1 without
// one: the FGMRES basis vector x then carries its normalisation factor); S warps per slice
template <bool COPY, int S, bool DIA>
__global__ void __launch_bounds__(sell_split_threads(S)) sell_spmv3_kernel(
    int nN, int nSlices, const int64_t* __restrict__ off, const int32_t* __restrict__ perm,
    const int32_t* __restrict__ col, const float* __restrict__ v9, const float* __restrict__ x,
    const uint8_t* __restrict__ mask, float* __restrict__ y, float* __restrict__ xcopy,
    const float* __restrict__ scale, const int32_t* __restrict__ dia, const float* __restrict__ binv) {
    ef::dep_entry();
    SellPart p;
    const bool active = sell_part<S>(nSlices, off, p);
    float y0 = 0.f, y1 = 0.f, y2 = 0.f;
    if (active) {
        const int32_t* cs = col + p.e0 + p.lane;
        const float* vs = v9 + 9 * p.e0 + p.lane;
        const int row = p.sl * 32 + p.lane;
#pragma unroll 3
        for (int j = p.j0; j < p.j1; ++j) {
            const int c3 = 3 * (DIA ? dia_column(row, __ldg(dia + j), nN) : __ldcs(cs + 32 * j));
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
    if (scale) {
        const float sc = *scale;
        y0 *= sc;
        y1 *= sc;
        y2 *= sc;
        if (COPY) {
            xcopy[d + 0] = sc * x[d + 0];
            xcopy[d + 1] = sc * x[d + 1];
            xcopy[d + 2] = sc * x[d + 2];
        }
    } else if (COPY) {
        xcopy[d + 0] = x[d + 0];
        xcopy[d + 1] = x[d + 1];
        xcopy[d + 2] = x[d + 2];
    }
    y0 = mask[d + 0] ? 0.f : y0;
    y1 = mask[d + 1] ? 0.f : y1;
    y2 = mask[d + 2] ? 0.f : y2;
    if (binv) {  // y = D^-1 (K x) with the row's block inverse (the power iteration on D^-1 K)
        const float* B = binv + 9 * (int64_t)m;
        const float z0 = B[0] * y0 + B[1] * y1 + B[2] * y2;
        const float z1 = B[3] * y0 + B[4] * y1 + B[5] * y2;
        const float z2 = B[6] * y0 + B[7] * y1 + B[8] * y2;
        y0 = mask[d + 0] ? 0.f : z0;
        y1 = mask[d + 1] ? 0.f : z1;
        y2 = mask[d + 2] ? 0.f : z2;
    }
    y[d + 0] = y0;
    y[d + 1] = y1;
    y[d + 2] = y2;
}

// t = r - ys K x on the fine level (0 on masked rows), or with binv a damped block-Jacobi sweep
// t = x + omega D^-1 (r - K x) (masked DOFs keep x), from the BF16 split copy; S warps per slice
template <int S, bool DIA>
__global__ void __launch_bounds__(sell_split_threads(S)) sell_level3_bf16_kernel(
    int nN, int nSlices, const int64_t* __restrict__ off, const int32_t* __restrict__ perm,
    const int32_t* __restrict__ col, const uint4* __restrict__ v8, const __nv_bfloat16* __restrict__ v1,
    const float* __restrict__ x, const float* __restrict__ r, const uint8_t* __restrict__ mask, float* __restrict__ t,
    const float* __restrict__ binv, float omega, float ys, const int32_t* __restrict__ dia) {
    ef::dep_entry();
    SellPart p;
    const bool active = sell_part<S>(nSlices, off, p);
    float y0 = 0.f, y1 = 0.f, y2 = 0.f;
    if (active) {
        const int32_t* cs = col + p.e0 + p.lane;
        const uint4* qs = v8 + p.e0 + p.lane;
        const __nv_bfloat16* ws = v1 + p.e0 + p.lane;
        const int row = p.sl * 32 + p.lane;
#pragma unroll 4
        for (int j = p.j0; j < p.j1; ++j) {
            const int c3 = 3 * (DIA ? dia_column(row, __ldg(dia + j), nN) : __ldcs(cs + 32 * j));
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
    const float t0 = k0 ? 0.f : r[d] - ys * y0, t1 = k1 ? 0.f : r[d + 1] - ys * y1,
                t2 = k2 ? 0.f : r[d + 2] - ys * y2;
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

// ---- fused fine-level post-smoothing x = w D^-1 (r + t) + C e (amg_sa_body.h) ----------------
//
// C (3 x 6 blocks, the pattern of A P) in BF16, sliced like the fine system: slices of 32 finer
// rows (in the order perm: sorted by length within windows), slot e0 + 32 j + i holding slice row
// i's j-th block (padding: zero block, column 0); per slot one 16-byte word with values 0..7, one
// with values 8..15 and one 4-byte word with 16..17.

__device__ __forceinline__ uint32_t bf16x2_bits(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// slot t: C of AP block src[t] (or zeros)
__global__ void sa_post_setup_kernel(int64_t nSlot, const int32_t* __restrict__ src, const int32_t* __restrict__ apRow,
                                     const int32_t* __restrict__ apToP, const float* __restrict__ Pv,
                                     const float* __restrict__ APv, const float* __restrict__ binv, float omega,
                                     float alpha, uint4* __restrict__ q0, uint4* __restrict__ q1,
                                     uint32_t* __restrict__ q2) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nSlot) return;
    float C[18];
    const int64_t a = src[t];
    if (a >= 0) {
        sa_post_block<3>(a, apRow, apToP, Pv, APv, binv, omega, alpha, C);
    } else {
#pragma unroll
        for (int p = 0; p < 18; ++p) C[p] = 0.f;
    }
    q0[t] = make_uint4(bf16x2_bits(C[0], C[1]), bf16x2_bits(C[2], C[3]), bf16x2_bits(C[4], C[5]),
                       bf16x2_bits(C[6], C[7]));
    q1[t] = make_uint4(bf16x2_bits(C[8], C[9]), bf16x2_bits(C[10], C[11]), bf16x2_bits(C[12], C[13]),
                       bf16x2_bits(C[14], C[15]));
    q2[t] = bf16x2_bits(C[16], C[17]);
}

__device__ __forceinline__ float2 bf16x2_floats(uint32_t v) {
    return __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&v));
}

// x = w D^-1 (r + t) + sum over the row's C blocks of C e[col] (masked DOFs 0); S warps per slice
template <int S>
__global__ void __launch_bounds__(sell_split_threads(S)) sa_post_fused_kernel(
    int nN, int nSlices, const int64_t* __restrict__ off, const int32_t* __restrict__ perm,
    const int32_t* __restrict__ col,
    const uint4* __restrict__ q0, const uint4* __restrict__ q1, const uint32_t* __restrict__ q2,
    const float* __restrict__ e, const float* __restrict__ r, const float* __restrict__ t,
    const float* __restrict__ binv, const uint8_t* __restrict__ mask, float omega, float* __restrict__ x) {
    ef::dep_entry();
    SellPart p;
    const bool active = sell_part<S>(nSlices, off, p);
    float y0 = 0.f, y1 = 0.f, y2 = 0.f;
    if (active) {
        const int32_t* cs = col + p.e0 + p.lane;
        const uint4* a0 = q0 + p.e0 + p.lane;
        const uint4* a1 = q1 + p.e0 + p.lane;
        const uint32_t* a2 = q2 + p.e0 + p.lane;
#pragma unroll 2
        for (int j = p.j0; j < p.j1; ++j) {
            const float* ev = e + 6 * (int64_t)__ldcs(cs + 32 * j);
            const uint4 u = __ldcs(a0 + 32 * j), v = __ldcs(a1 + 32 * j);
            const uint32_t w2 = __ldcs(a2 + 32 * j);
            const float e0 = ev[0], e1 = ev[1], e2 = ev[2], e3 = ev[3], e4 = ev[4], e5 = ev[5];
            const float2 c01 = bf16x2_floats(u.x), c23 = bf16x2_floats(u.y), c45 = bf16x2_floats(u.z);
            const float2 c67 = bf16x2_floats(u.w), c89 = bf16x2_floats(v.x), cab = bf16x2_floats(v.y);
            const float2 ccd = bf16x2_floats(v.z), cef = bf16x2_floats(v.w), cgh = bf16x2_floats(w2);
            y0 += c01.x * e0 + c01.y * e1 + c23.x * e2 + c23.y * e3 + c45.x * e4 + c45.y * e5;
            y1 += c67.x * e0 + c67.y * e1 + c89.x * e2 + c89.y * e3 + cab.x * e4 + cab.y * e5;
            y2 += ccd.x * e0 + ccd.y * e1 + cef.x * e2 + cef.y * e3 + cgh.x * e4 + cgh.y * e5;
        }
    }
    if (!sell_combine<S>(p, active, y0, y1, y2)) return;
    const int rr = p.sl * 32 + p.lane;
    if (rr >= nN) return;
    const int m = perm ? perm[rr] : rr;
    const int d = 3 * m;
    const float s0 = r[d] + t[d], s1 = r[d + 1] + t[d + 1], s2 = r[d + 2] + t[d + 2];
    const float* B = binv + 9 * (int64_t)m;
    const float z0 = B[0] * s0 + B[1] * s1 + B[2] * s2;
    const float z1 = B[3] * s0 + B[4] * s1 + B[5] * s2;
    const float z2 = B[6] * s0 + B[7] * s1 + B[8] * s2;
    x[d] = mask[d] ? 0.f : omega * z0 + y0;
    x[d + 1] = mask[d + 1] ? 0.f : omega * z1 + y1;
    x[d + 2] = mask[d + 2] ? 0.f : omega * z2 + y2;
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
                                 const int32_t* col, const float* binv, const uint8_t* mask, cudaStream_t s) {
    if (nE <= 0) return EF_OK;
    sell_refresh_kernel<<<(unsigned)((nE + 255) / 256), 256, 0, ef::counted(s)>>>(
        nE, src, bsr, v9, (uint4*)v8, (__nv_bfloat16*)v1, col, binv, mask);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_sell_spmv3(int nN, int nSlices, const int64_t* off, const int32_t* perm, const int32_t* col,
                               const float* v9, const float* x, const uint8_t* mask, float* y, float* xcopy, int split,
                               cudaStream_t s, const float* scale, const int32_t* dia, const float* binv) {
    if (nSlices <= 0) return EF_OK;
#define EF_SPMV3(C_, S_)                                                                                              \
    do {                                                                                                              \
        if (dia)                                                                                                      \
            EF_CUDA(ef::launch_dep(sell_spmv3_kernel<C_, S_, true>, sell_split_grid(nSlices, S_),                     \
                                   sell_split_threads(S_), 0, s, nN, nSlices, off, perm, col, v9, x, mask, y, xcopy,  \
                                   scale, dia, binv));                                                                \
        else                                                                                                          \
            EF_CUDA(ef::launch_dep(sell_spmv3_kernel<C_, S_, false>, sell_split_grid(nSlices, S_),                    \
                                   sell_split_threads(S_), 0, s, nN, nSlices, off, perm, col, v9, x, mask, y, xcopy,  \
                                   scale, dia, binv));                                                                \
    } while (0)
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
                                     cudaStream_t s, float ys, const int32_t* dia) {
    if (nSlices <= 0) return EF_OK;
#define EF_L3(S_)                                                                                                    \
    do {                                                                                                             \
        if (dia)                                                                                                     \
            EF_CUDA(ef::launch_dep(sell_level3_bf16_kernel<S_, true>, sell_split_grid(nSlices, S_),                  \
                                   sell_split_threads(S_), 0, s, nN, nSlices, off, perm, col, (const uint4*)v8,      \
                                   (const __nv_bfloat16*)v1, x, r, mask, t, binv, omega, ys, dia));                  \
        else                                                                                                         \
            EF_CUDA(ef::launch_dep(sell_level3_bf16_kernel<S_, false>, sell_split_grid(nSlices, S_),                 \
                                   sell_split_threads(S_), 0, s, nN, nSlices, off, perm, col, (const uint4*)v8,      \
                                   (const __nv_bfloat16*)v1, x, r, mask, t, binv, omega, ys, dia));                  \
    } while (0)
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

ef_status ef_launch_sa_post_setup(int64_t nSlot, const int32_t* src, const int32_t* apRow, const int32_t* apToP,
                                  const float* Pv, const float* APv, const float* binv, float omega, float alpha,
                                  void* q0, void* q1, void* q2, cudaStream_t s) {
    if (nSlot <= 0) return EF_OK;
    sa_post_setup_kernel<<<(unsigned)((nSlot + 255) / 256), 256, 0, ef::counted(s)>>>(
        nSlot, src, apRow, apToP, Pv, APv, binv, omega, alpha, (uint4*)q0, (uint4*)q1, (uint32_t*)q2);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_sa_post_fused(int nN, int nSlices, const int64_t* off, const int32_t* perm, const int32_t* col,
                                  const void* q0, const void* q1, const void* q2, const float* e, const float* r,
                                  const float* t, const float* binv, const uint8_t* mask, float omega, float* x,
                                  int split, cudaStream_t s) {
    if (nSlices <= 0) return EF_OK;
#define EF_POST(S_)                                                                                              \
    EF_CUDA(ef::launch_dep(sa_post_fused_kernel<S_>, sell_split_grid(nSlices, S_), sell_split_threads(S_), 0, s, \
                           nN, nSlices, off, perm, col, (const uint4*)q0, (const uint4*)q1, (const uint32_t*)q2, e, r, \
                           t, binv, mask, omega, x))
    if (split == 1)
        EF_POST(1);
    else if (split == 2)
        EF_POST(2);
    else if (split == 8)
        EF_POST(8);
    else
        EF_POST(4);
#undef EF_POST
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}
