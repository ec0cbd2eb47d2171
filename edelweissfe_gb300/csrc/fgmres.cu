// Flexible GMRES building blocks (FP32 vectors, FP64 reductions): masked BSR SpMV, classical
// Gram-Schmidt as multi-dot products and a multi-axpy (re-orthogonalised when the DGKS test asks
// for it), normalisation and the final x += Z y.  Reductions are per-CTA partials summed in a
// fixed order, so every FGMRES run is bit-reproducible.

#include <algorithm>

#include "ef_common.cuh"

namespace ef {

constexpr int kFB = 256;
constexpr int kMaxBasis = 128;  // cap on the Krylov basis size (restart length + 1)

// y = A x on the free DOFs (masked rows -> 0); 8 lanes per block row.  The column indices and the
// block values of a row are loaded together (predicated on the row bounds only), then the x
// gathers that depend on the column indices: two dependent memory steps per row, not three.
__global__ void __launch_bounds__(kFB) spmv_f32_kernel(int nN, const int32_t* __restrict__ rowPtr,
                                                        const int32_t* __restrict__ colIdx,
                                                        const float* __restrict__ vals, const float* __restrict__ x,
                                                        const uint8_t* __restrict__ mask, float* __restrict__ y,
                                                        float* __restrict__ xcopy) {
    const int lane = threadIdx.x & 7;
    const int m0 = (blockIdx.x * kFB + threadIdx.x) >> 3;
    const int m = m0 < nN ? m0 : nN - 1;
    float y0 = 0.f, y1 = 0.f, y2 = 0.f;
    const int s = rowPtr[m], e = rowPtr[m + 1];
    for (int base = s; base < e; base += 32) {
        int cc[4];
        float v[4][9];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int k = base + lane + 8 * j;
            if (k < e) {
                cc[j] = 3 * colIdx[k];
                const float* src = vals + (int64_t)k * 9;
#pragma unroll
                for (int q = 0; q < 9; ++q) v[j][q] = src[q];
            } else {
                cc[j] = -1;
            }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (cc[j] >= 0) {
                const float x0 = x[cc[j]], x1 = x[cc[j] + 1], x2 = x[cc[j] + 2];
                y0 += v[j][0] * x0 + v[j][1] * x1 + v[j][2] * x2;
                y1 += v[j][3] * x0 + v[j][4] * x1 + v[j][5] * x2;
                y2 += v[j][6] * x0 + v[j][7] * x1 + v[j][8] * x2;
            }
    }
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) {
        y0 += __shfl_xor_sync(0xffffffffu, y0, o);
        y1 += __shfl_xor_sync(0xffffffffu, y1, o);
        y2 += __shfl_xor_sync(0xffffffffu, y2, o);
    }
    if (m0 < nN && lane < 3) {
        const int d = 3 * m + lane;
        const float yy = lane == 0 ? y0 : (lane == 1 ? y1 : y2);
        y[d] = (mask && mask[d]) ? 0.f : yy;
        if (xcopy) xcopy[d] = x[d];
    }
}

// Staged form of spmv_f32_kernel: persistent CTAs walk chunks of kSpRows block rows, copying the
// next chunk's block values and column indices (contiguous in memory) into shared memory with
// cp.async while the current one is computed; the rows are then computed by 8 lanes each from
// shared memory, with the same order of operations as the unstaged kernel.  Stage layout
// (cap = the largest chunk's block count): 9 cap + 8 floats | cap + 8 indices, both ranges
// starting on the 16-byte boundary below the chunk's first block.
constexpr int kSpRows = kFB / 8;

__host__ __device__ inline size_t sp_stage_bytes(int cap) {
    return (((size_t)9 * cap + 8) * 4 + 15) / 16 * 16 + ((size_t)cap + 8) * 4;
}

__device__ __forceinline__ void sp_stage_chunk(int b0, int b1, const float* __restrict__ vals,
                                               const int32_t* __restrict__ colIdx, char* stage, int cap) {
    float* sv = reinterpret_cast<float*>(stage);
    int32_t* sc = reinterpret_cast<int32_t*>(stage + (((size_t)9 * cap + 8) * 4 + 15) / 16 * 16);
    const int vs = (9 * b0) & ~3;
    const int nv = (9 * b1 - vs + 3) >> 2;  // 16-byte pieces of 4 values
    for (int i = threadIdx.x; i < nv; i += kFB) cp_async16(sv + 4 * i, vals + (int64_t)vs + 4 * i);
    const int cs = b0 & ~3;
    const int nc = (b1 - cs + 3) >> 2;
    for (int i = threadIdx.x; i < nc; i += kFB) cp_async16(sc + 4 * i, colIdx + cs + 4 * i);
}

__global__ void __launch_bounds__(kFB) spmv_f32_staged_kernel(int nN, const int32_t* __restrict__ rowPtr,
                                                               const int32_t* __restrict__ colIdx,
                                                               const float* __restrict__ vals,
                                                               const float* __restrict__ x,
                                                               const uint8_t* __restrict__ mask, float* __restrict__ y,
                                                               float* __restrict__ xcopy, int cap) {
    extern __shared__ __align__(16) char smem[];
    const size_t sb = (sp_stage_bytes(cap) + 15) & ~(size_t)15;
    const int nChunks = (nN + kSpRows - 1) / kSpRows;
    const int lane = threadIdx.x & 7;
    const int rowInChunk = threadIdx.x >> 3;
    int ch = blockIdx.x;
    if (ch >= nChunks) return;
    int b0 = rowPtr[ch * kSpRows];
    int b1 = rowPtr[min((ch + 1) * kSpRows, nN)];
    sp_stage_chunk(b0, b1, vals, colIdx, smem, cap);
    cp_async_commit();
    int st = 0;
    for (; ch < nChunks; ch += gridDim.x, st ^= 1) {
        const int nx = ch + gridDim.x;
        int nb0 = 0, nb1 = 0;
        if (nx < nChunks) {
            nb0 = rowPtr[nx * kSpRows];
            nb1 = rowPtr[min((nx + 1) * kSpRows, nN)];
            sp_stage_chunk(nb0, nb1, vals, colIdx, smem + (st ^ 1) * sb, cap);
        }
        cp_async_commit();
        const int m0 = ch * kSpRows + rowInChunk;
        const int m = m0 < nN ? m0 : nN - 1;
        const int s = rowPtr[m], e = rowPtr[m + 1];
        cp_async_wait<1>();
        __syncthreads();
        const char* sg = smem + st * sb;
        const float* sv = reinterpret_cast<const float*>(sg);
        const int32_t* sc = reinterpret_cast<const int32_t*>(sg + (((size_t)9 * cap + 8) * 4 + 15) / 16 * 16);
        const int vs = (9 * b0) & ~3, cs = b0 & ~3;
        float y0 = 0.f, y1 = 0.f, y2 = 0.f;
        for (int base = s; base < e; base += 32) {
            int cc[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int k = base + lane + 8 * j;
                cc[j] = k < e ? 3 * sc[k - cs] : -1;
            }
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (cc[j] >= 0) {
                    const float* v = sv + (9 * (base + lane + 8 * j) - vs);
                    const float x0 = x[cc[j]], x1 = x[cc[j] + 1], x2 = x[cc[j] + 2];
                    y0 += v[0] * x0 + v[1] * x1 + v[2] * x2;
                    y1 += v[3] * x0 + v[4] * x1 + v[5] * x2;
                    y2 += v[6] * x0 + v[7] * x1 + v[8] * x2;
                }
        }
#pragma unroll
        for (int o = 4; o > 0; o >>= 1) {
            y0 += __shfl_xor_sync(0xffffffffu, y0, o);
            y1 += __shfl_xor_sync(0xffffffffu, y1, o);
            y2 += __shfl_xor_sync(0xffffffffu, y2, o);
        }
        if (m0 < nN && lane < 3) {
            const int d = 3 * m + lane;
            const float yy = lane == 0 ? y0 : (lane == 1 ? y1 : y2);
            y[d] = (mask && mask[d]) ? 0.f : yy;
            if (xcopy) xcopy[d] = x[d];
        }
        __syncthreads();
        b0 = nb0;
        b1 = nb1;
    }
    cp_async_wait<0>();
}

// DGKS test (Daniel, Gragg, Kaufman, Stewart 1976) of classical Gram-Schmidt: after the first
// projection w' = w - V h of w (|w|^2 = h[nv]), re-orthogonalise only when the Pythagorean
// estimate |w'|^2 = |w|^2 - |h|^2 shows cancellation, |w'|^2 < eta2 |w|^2.  Every thread that
// asks computes the same sum in the same order, so all kernels of one column agree.
__device__ __forceinline__ bool dgks_reorth(const double* __restrict__ h, int nv, double eta2) {
    if (!(eta2 > 0.0)) return false;
    double hh = 0.0;
    for (int k = 0; k < nv; ++k) hh += h[k] * h[k];
    const double w2 = h[nv];
    return w2 - hh < eta2 * w2;
}

// FP64 is a narrow pipe on this GPU (2 lanes per SM and cycle), so the reductions below run in
// FP32 inside a CTA (the vectors themselves are FP32) and in FP64 only across CTAs, where the
// sums are long.  All orders are fixed.

// fixed-order FP64 sum of v[0..n) over the CTA, returned to thread 0: thread-strided partial sums
// (their loads in flight together), a shuffle tree per warp, the warps' sums in order by thread 0
// (the other threads' FP64 work ends at their warp's tree)
__device__ __forceinline__ double cta_sum_fixed(const double* __restrict__ v, int n, double* red) {
    double t = 0.0;
    for (int c = threadIdx.x; c < n; c += kFB) t += v[c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
#pragma unroll
        for (int q = 0; q < kFB / 32; ++q) s += red[q];
    return s;
}

// fixed-order FP32 sum over a warp (every lane gets it)
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// part[k * gridDim.x + cta] = sum over this CTA's elements of V[k] . w, k < nv.  The vectors go
// in groups of 8 (8 accumulators per thread), two elements per thread and step, so that 16
// independent loads are in flight per thread.
__global__ void __launch_bounds__(kFB, 4) multidot_partial_kernel(int64_t n, int nv, const float* __restrict__ V,
                                                                int64_t ldv, const float* __restrict__ w,
                                                                double* __restrict__ part,
                                                                const double* __restrict__ gate, int gateNv,
                                                                double eta2) {
    ef::dep_entry();
    if (gate && !dgks_reorth(gate, gateNv, eta2)) return;
    __shared__ float red[kFB / 32][kMaxBasis];
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const int64_t stride = (int64_t)gridDim.x * kFB;
    for (int k0 = 0; k0 < nv; k0 += 8) {
        const int kn = min(8, nv - k0);
        float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        int64_t i = (int64_t)blockIdx.x * kFB + threadIdx.x;
        for (; i + stride < n; i += 2 * stride) {
            const float wa = w[i], wb = w[i + stride];
            float va[8], vb[8];
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (k < kn) {
                    va[k] = V[(k0 + k) * ldv + i];
                    vb[k] = V[(k0 + k) * ldv + i + stride];
                }
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (k < kn) acc[k] = fmaf(vb[k], wb, fmaf(va[k], wa, acc[k]));
        }
        if (i < n) {
            const float wa = w[i];
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (k < kn) acc[k] = fmaf(V[(k0 + k) * ldv + i], wa, acc[k]);
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const float a = warp_sum(acc[k]);
            if (lane == 0 && k < kn) red[wp][k0 + k] = a;
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nv; k += kFB) {
        float s = 0.f;
#pragma unroll
        for (int q = 0; q < kFB / 32; ++q) s += red[q][k];
        part[(int64_t)k * gridDim.x + blockIdx.x] = (double)s;
    }
}

// h[k] = sum_c part[k * nPart + c], one CTA per k, fixed order
__global__ void __launch_bounds__(kFB) multidot_final_kernel(int nPart, int nv, const double* __restrict__ part,
                                                              double* __restrict__ h, const double* __restrict__ gate,
                                                              int gateNv, double eta2) {
    ef::dep_entry();
    if (gate && !dgks_reorth(gate, gateNv, eta2)) return;
    __shared__ double red[kFB / 32];
    const int k = blockIdx.x;
    if (k >= nv) return;
    const double s = cta_sum_fixed(part + (int64_t)k * nPart, nPart, red);
    if (threadIdx.x == 0) h[k] = s;
}

// w -= sum_k h[k] V[k] over a fixed grid, and partN[cta] = this CTA's part of |w|^2 (fixed
// order).  With a gate (the first-pass coefficients and |w|^2) the pass runs only when the DGKS
// test asks for re-orthogonalisation.
__global__ void __launch_bounds__(kFB) cgs_axpy_kernel(int64_t n, int nv, const float* __restrict__ V, int64_t ldv,
                                                        const double* __restrict__ h, float* __restrict__ w,
                                                        double* __restrict__ partN, const double* __restrict__ gate,
                                                        double eta2) {
    ef::dep_entry();
    if (gate && !dgks_reorth(gate, nv, eta2)) return;
    __shared__ float hs[kMaxBasis];
    __shared__ float red[kFB / 32];
    for (int k = threadIdx.x; k < nv; k += kFB) hs[k] = (float)h[k];
    __syncthreads();
    float nrm = 0.f;
    for (int64_t i = (int64_t)blockIdx.x * kFB + threadIdx.x; i < n; i += (int64_t)gridDim.x * kFB) {
        float s = w[i];
        int k = 0;
        for (; k + 8 <= nv; k += 8) {
            float v[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) v[q] = V[(k + q) * ldv + i];
#pragma unroll
            for (int q = 0; q < 8; ++q) s -= hs[k + q] * v[q];
        }
        for (; k < nv; ++k) s -= hs[k] * V[k * ldv + i];
        w[i] = s;
        nrm = fmaf(s, s, nrm);
    }
    nrm = warp_sum(nrm);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = nrm;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
#pragma unroll
        for (int q = 0; q < kFB / 32; ++q) t += red[q];
        partN[blockIdx.x] = (double)t;
    }
}

// hAcc = hG + hTmp when the DGKS test on hG fired, else hG (k < nv)
__global__ void cgs_accumulate_kernel(int nv, const double* __restrict__ hG, const double* __restrict__ hTmp,
                                      double* __restrict__ hAcc, double eta2) {
    ef::dep_entry();
    const bool re = dgks_reorth(hG, nv, eta2);
    for (int k = threadIdx.x; k < nv; k += blockDim.x) hAcc[k] = re ? hG[k] + hTmp[k] : hG[k];
}

// Normalisation of the new basis vector: every CTA sums the |w|^2 parts np[0..nParts) in the
// same order, w *= 1/|w|, copy to w2 (the preconditioner's input buffer).  CTA 0 publishes |w|^2
// and the column's coefficients hAcc[0..nv) to host-mapped memory: hostOut[0..nv) = hAcc,
// hostOut[slotNorm] = |w|^2, hostOut[slotNorm - 1] = 1 when the column was re-orthogonalised
// (gate, eta2: the DGKS test of cgs_axpy_kernel).
__global__ void __launch_bounds__(kFB) normalize_kernel(int64_t n, float* __restrict__ w, float* __restrict__ w2,
                                                         const double* __restrict__ np, int nParts,
                                                         const double* __restrict__ hAcc, int nv,
                                                         volatile double* hostOut, int slotNorm,
                                                         const double* __restrict__ gate, double eta2,
                                                         float* __restrict__ scOut) {
    ef::dep_entry();
    if (scOut && blockIdx.x == 0 && threadIdx.x == 0) *scOut = 1.f;
    // |w|^2 over the CTA, 1/|w| by thread 0 (FP64), handed to the CTA through shared memory
    __shared__ double red[kFB / 32];
    __shared__ float sInv;
    const double t = cta_sum_fixed(np, nParts, red);
    if (threadIdx.x == 0) {
        sInv = t > 0.0 ? (float)(1.0 / sqrt(t)) : 0.f;
        if (blockIdx.x == 0 && hostOut) {
            hostOut[slotNorm] = t;
            if (gate) hostOut[slotNorm - 1] = dgks_reorth(gate, nv, eta2) ? 1.0 : 0.0;
        }
    }
    if (blockIdx.x == 0 && hostOut && hAcc)
        for (int k = threadIdx.x; k < nv; k += kFB) hostOut[k] = hAcc[k];
    __syncthreads();
    const float inv = sInv;
#pragma unroll 4
    for (int64_t i = (int64_t)blockIdx.x * kFB + threadIdx.x; i < n; i += (int64_t)gridDim.x * kFB) {
        const float v = w[i] * inv;
        w[i] = v;
        if (w2) w2[i] = v;
    }
}

// ---- Gram-Schmidt column with deferred normalisation (two kernels per column) ---------------
// The basis is kept as unnormalised vectors u_k with factors sc[k] = 1 / |u_k| (v_k = sc[k] u_k):
// the new vector is never rescaled in place.  The product that makes w = K z_j applies sc[j] to
// its result and to the stored z_j (the preconditioner is linear, so M^-1 (sc u) = sc M^-1 u).
//   gs_dot:  part[k][cta] = u_k . w over the CTA's elements (k < nv), FP32;
//   gs_axpy: every CTA sums part[k][0..nParts) in the same order (h_k = sc[k] sum), then
//            w -= sum_k h_k sc[k] u_k, a copy of w to the preconditioner's input, |w|^2 parts;
//            the last CTA to finish (an atomic ticket, no waiting) sums the |w|^2 parts in order,
//            sets sc[nv] = 1 / |w| and publishes h and |w|^2 to host-mapped memory.
// One CTA per SM of kGsThreads threads, so that a CTA's sum over the parts stays short.
constexpr int kGsThreads = 1024;

__global__ void __launch_bounds__(kGsThreads, 1) gs_dot_kernel(int64_t n, int nv, const float* __restrict__ V,
                                                               int64_t ldv, const float* __restrict__ w,
                                                               float* __restrict__ part) {
    ef::dep_entry();
    __shared__ float red[kGsThreads / 32][kMaxBasis];
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const int64_t stride = (int64_t)gridDim.x * kGsThreads;
    for (int k0 = 0; k0 < nv; k0 += 8) {
        const int kn = min(8, nv - k0);
        float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        int64_t i = (int64_t)blockIdx.x * kGsThreads + threadIdx.x;
        for (; i + stride < n; i += 2 * stride) {
            const float wa = w[i], wb = w[i + stride];
            float va[8], vb[8];
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (k < kn) {
                    va[k] = V[(k0 + k) * ldv + i];
                    vb[k] = V[(k0 + k) * ldv + i + stride];
                }
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (k < kn) acc[k] = fmaf(vb[k], wb, fmaf(va[k], wa, acc[k]));
        }
        if (i < n) {
            const float wa = w[i];
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (k < kn) acc[k] = fmaf(V[(k0 + k) * ldv + i], wa, acc[k]);
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const float a = warp_sum(acc[k]);
            if (lane == 0 && k < kn) red[wp][k0 + k] = a;
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nv; k += kGsThreads) {
        float s = 0.f;
#pragma unroll 8
        for (int q = 0; q < kGsThreads / 32; ++q) s += red[q][k];
        part[(int64_t)k * gridDim.x + blockIdx.x] = s;
    }
}

__global__ void __launch_bounds__(kGsThreads, 1) gs_axpy_kernel(int64_t n, int nv, const float* __restrict__ V,
                                                                int64_t ldv, const float* __restrict__ part,
                                                                float* __restrict__ sc, float* __restrict__ w,
                                                                float* __restrict__ w2, double* __restrict__ partN,
                                                                unsigned* __restrict__ ticket,
                                                                volatile double* hostOut, int slotNorm) {
    ef::dep_entry();
    __shared__ float hk[kMaxBasis];  // h_k (Hessenberg entries)
    __shared__ float ck[kMaxBasis];  // h_k sc[k] (coefficients of u_k)
    __shared__ float red[kGsThreads / 32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const int nP = gridDim.x;
    for (int k = wp; k < nv; k += kGsThreads / 32) {
        float t = 0.f;
        for (int c = lane; c < nP; c += 32) t += part[(int64_t)k * nP + c];
        t = warp_sum(t);
        if (lane == 0) {
            const float f = sc[k];
            const float h = t * f;
            hk[k] = h;
            ck[k] = h * f;
        }
    }
    __syncthreads();
    float nrm = 0.f;
    for (int64_t i = (int64_t)blockIdx.x * kGsThreads + threadIdx.x; i < n; i += (int64_t)nP * kGsThreads) {
        float s = w[i];
        int k = 0;
        for (; k + 8 <= nv; k += 8) {
            float v[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) v[q] = V[(k + q) * ldv + i];
#pragma unroll
            for (int q = 0; q < 8; ++q) s -= ck[k + q] * v[q];
        }
        for (; k < nv; ++k) s -= ck[k] * V[k * ldv + i];
        w[i] = s;
        w2[i] = s;
        nrm = fmaf(s, s, nrm);
    }
    nrm = warp_sum(nrm);
    if (lane == 0) red[wp] = nrm;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
#pragma unroll 8
        for (int q = 0; q < kGsThreads / 32; ++q) t += red[q];
        partN[blockIdx.x] = (double)t;
        __threadfence();
        last = atomicAdd(ticket, 1u) == (unsigned)nP - 1;
    }
    __syncthreads();
    if (!last || wp != 0) return;
    __threadfence();
    double t = 0.0;
    for (int c = lane; c < nP; c += 32) t += __ldcg(partN + c);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    for (int k = lane; k < nv; k += 32) hostOut[k] = (double)hk[k];
    if (lane == 0) {
        sc[nv] = t > 0.0 ? (float)(1.0 / sqrt(t)) : 0.f;
        hostOut[slotNorm] = t;
        hostOut[slotNorm - 1] = 0.0;  // never re-orthogonalised
        *ticket = 0u;
    }
}

// x += sum_k y[k] Z[k]   (y in FP64)
__global__ void combine_kernel(int64_t n, int nv, const float* __restrict__ Z, int64_t ldz, const double* __restrict__ y,
                               float* __restrict__ x) {
    __shared__ double ys[kMaxBasis];
    for (int k = threadIdx.x; k < nv; k += blockDim.x) ys[k] = y[k];
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = (double)x[i];
    for (int k = 0; k < nv; ++k) s += ys[k] * (double)Z[k * ldz + i];
    x[i] = (float)s;
}

// r = b - y (float)
__global__ void sub_kernel(int64_t n, const float* __restrict__ b, const float* __restrict__ y, float* __restrict__ r) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) r[i] = b[i] - y[i];
}

}  // namespace ef

using namespace ef;

static inline int nbf(int64_t n, int t) { return (int)((n + t - 1) / t); }

int ef_fgmres_max_basis() { return kMaxBasis; }

ef_status ef_launch_spmv_f32(int nN, const int32_t* rowPtr, const int32_t* colIdx, const float* vals, const float* x,
                             const uint8_t* mask, float* y, cudaStream_t s) {
    spmv_f32_kernel<<<nbf((int64_t)nN * 8, kFB), kFB, 0, ef::counted(s)>>>(nN, rowPtr, colIdx, vals, x, mask, y,
                                                                           nullptr);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

// y = A x and xcopy = x (the FGMRES product that also stores the preconditioned vector)
ef_status ef_launch_spmv_f32_copy(int nN, const int32_t* rowPtr, const int32_t* colIdx, const float* vals,
                                  const float* x, const uint8_t* mask, float* y, float* xcopy, cudaStream_t s) {
    spmv_f32_kernel<<<nbf((int64_t)nN * 8, kFB), kFB, 0, ef::counted(s)>>>(nN, rowPtr, colIdx, vals, x, mask, y,
                                                                           xcopy);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

// staged SpMV (cap: the largest block count of a chunk of kSpRows rows, ef_sp_stage_cap)
int ef_sp_stage_cap(int nN, const int32_t* rowPtrHost) {
    int cap = 0;
    for (int m0 = 0; m0 < nN; m0 += kSpRows) cap = std::max(cap, rowPtrHost[std::min(m0 + kSpRows, nN)] - rowPtrHost[m0]);
    return cap;
}

ef_status ef_launch_spmv_f32_staged(int nSM, int cap, int nN, const int32_t* rowPtr, const int32_t* colIdx,
                                    const float* vals, const float* x, const uint8_t* mask, float* y, float* xcopy,
                                    cudaStream_t s) {
    const size_t smem = 2 * ((sp_stage_bytes(cap) + 15) & ~(size_t)15);
    static size_t attrSet = 0;
    if (smem > 48 * 1024 && smem > attrSet) {
        EF_CUDA(cudaFuncSetAttribute(spmv_f32_staged_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attrSet = smem;
    }
    int perSM = 0;
    EF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, spmv_f32_staged_kernel, kFB, smem));
    if (perSM < 1) {
        ef_set_error("staged SpMV: chunk does not fit in shared memory");
        return EF_ERR_ARG;
    }
    const int nChunks = (nN + kSpRows - 1) / kSpRows;
    const int grid = std::max(1, std::min(nChunks, perSM * nSM));
    spmv_f32_staged_kernel<<<grid, kFB, smem, ef::counted(s)>>>(nN, rowPtr, colIdx, vals, x, mask, y, xcopy, cap);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

// One Gram-Schmidt step of column j (nv = j + 1 basis vectors V[0..nv), the new vector w =
// V[nv] in place), classical with DGKS-selective re-orthogonalisation:
//   hG = [V^T w, |w|^2] (one pass, nv + 1 products), w -= V hG (+ |w|^2 parts),
//   when the DGKS test on hG fires: hTmp = V^T w, w -= V hTmp (+ |w|^2 parts),
//   hAcc = hG (+ hTmp), w /= |w|, w2 = w, hAcc and |w|^2 to hostOut.
// With eta2 > 0 the re-orthogonalisation kernels are always launched (a fixed launch sequence)
// and return at once when the test does not fire; eta2 = 0 leaves them out.  part:
// [kMaxBasis][nPart], partN: [nPart], hG, hTmp, hAcc: [kMaxBasis].
ef_status ef_launch_cgs_column(int64_t n, int nv, float* V, int64_t ldv, double* part, double* partN, int nPart,
                               double* hG, double* hTmp, double* hAcc, double eta2, float* w2, double* hostOut,
                               int slotNorm, cudaStream_t s) {
    if (nv + 1 > kMaxBasis) {
        ef_set_error("FGMRES: basis larger than the compiled maximum");
        return EF_ERR_ARG;
    }
    float* w = V + (int64_t)nv * ldv;
    const bool re = eta2 > 0.0;
    EF_CUDA(ef::launch_dep(multidot_partial_kernel, nPart, kFB, 0, s, n, nv + 1, V, ldv, w, part, nullptr, 0, 0.0));
    EF_CUDA(ef::launch_dep(multidot_final_kernel, nv + 1, kFB, 0, s, nPart, nv + 1, part, hG, nullptr, 0, 0.0));
    EF_CUDA(ef::launch_dep(cgs_axpy_kernel, nPart, kFB, 0, s, n, nv, V, ldv, hG, w, partN, nullptr, 0.0));
    if (re) {
        EF_CUDA(ef::launch_dep(multidot_partial_kernel, nPart, kFB, 0, s, n, nv, V, ldv, w, part, hG, nv, eta2));
        EF_CUDA(ef::launch_dep(multidot_final_kernel, nv, kFB, 0, s, nPart, nv, part, hTmp, hG, nv, eta2));
        EF_CUDA(ef::launch_dep(cgs_axpy_kernel, nPart, kFB, 0, s, n, nv, V, ldv, hTmp, w, partN, hG, eta2));
        EF_CUDA(ef::launch_dep(cgs_accumulate_kernel, 1, kMaxBasis, 0, s, nv, hG, hTmp, hAcc, eta2));
    }
    // every normalisation CTA sums all nPart parts (from L2) and scales its share of w
    EF_CUDA(ef::launch_dep(normalize_kernel, nPart, kFB, 0, s, n, w, w2, partN, nPart, re ? hAcc : hG,
            nv, hostOut, slotNorm, re ? hG : nullptr, eta2, (float*)nullptr));
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

// One Gram-Schmidt step of column j with deferred normalisation (gs_dot_kernel, gs_axpy_kernel):
// nv = j + 1 basis vectors u_0..u_j in V with factors sc[0..nv), the new vector w = u_nv in
// place (already scaled by sc[j] through the product); w2 = w; sc[nv], h and |w|^2 to hostOut.
// part: [kMaxBasis][nPart] floats, partN: [nPart], ticket: one counter, zero between launches.
ef_status ef_launch_gs_column(int64_t n, int nv, float* V, int64_t ldv, float* part, double* partN, int nPart,
                              float* sc, unsigned* ticket, float* w2, double* hostOut, int slotNorm, cudaStream_t s) {
    if (nv + 1 > kMaxBasis) {
        ef_set_error("FGMRES: basis larger than the compiled maximum");
        return EF_ERR_ARG;
    }
    float* w = V + (int64_t)nv * ldv;
    EF_CUDA(ef::launch_dep(gs_dot_kernel, nPart, kGsThreads, 0, s, n, nv, V, ldv, w, part));
    EF_CUDA(ef::launch_dep(gs_axpy_kernel, nPart, kGsThreads, 0, s, n, nv, V, ldv, part, sc, w, w2, partN, ticket,
                           hostOut, slotNorm));
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

// w /= |w| with |w|^2 from a one-vector multidot (the restart vector); w2 = w; |w|^2 to hostOut;
// scOut (optional): the vector's factor, 1
ef_status ef_launch_normalize_first(int64_t n, float* w, double* part, int nPart, float* w2, double* hostOut,
                                    int slotNorm, cudaStream_t s, float* scOut) {
    EF_CUDA(ef::launch_dep(multidot_partial_kernel, nPart, kFB, 0, s, n, 1, w, n, w, part, nullptr, 0, 0.0));
    EF_CUDA(ef::launch_dep(normalize_kernel, nPart, kFB, 0, s, n, w, w2, part, nPart, nullptr, 0,
            hostOut, slotNorm, nullptr, 0.0, scOut));
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_combine(int64_t n, int nv, const float* Z, int64_t ldz, const double* y, float* x,
                            cudaStream_t s) {
    combine_kernel<<<nbf(n, 256), 256, 0, ef::counted(s)>>>(n, nv, Z, ldz, y, x);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_sub(int64_t n, const float* b, const float* y, float* r, cudaStream_t s) {
    sub_kernel<<<nbf(n, 256), 256, 0, ef::counted(s)>>>(n, b, y, r);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}
