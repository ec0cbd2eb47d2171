// Flexible GMRES building blocks (FP32 vectors, FP64 reductions): masked BSR SpMV, classical
// Gram-Schmidt with re-orthogonalisation as two passes of multi-dot products and a multi-axpy,
// normalisation and the final x += Z y.  Reductions are per-CTA partials summed in a fixed
// order, so every FGMRES run is bit-reproducible.

#include "ef_common.cuh"

namespace ef {

constexpr int kFB = 256;
constexpr int kMaxBasis = 128;  // cap on the Krylov basis size (restart length + 1)

// y = A x on the free DOFs (masked rows -> 0); 8 lanes per block row, batched loads
__global__ void __launch_bounds__(kFB) spmv_f32_kernel(int nN, const int32_t* __restrict__ rowPtr,
                                                        const int32_t* __restrict__ colIdx,
                                                        const float* __restrict__ vals, const float* __restrict__ x,
                                                        const uint8_t* __restrict__ mask, float* __restrict__ y) {
    const int lane = threadIdx.x & 7;
    const int m0 = (blockIdx.x * kFB + threadIdx.x) >> 3;
    const int m = m0 < nN ? m0 : nN - 1;
    float y0 = 0.f, y1 = 0.f, y2 = 0.f;
    const int s = rowPtr[m], e = rowPtr[m + 1];
    for (int base = s; base < e; base += 32) {
        int cc[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int k = base + lane + 8 * j;
            cc[j] = k < e ? 3 * colIdx[k] : -1;
        }
        float xv[4][3];
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (cc[j] >= 0) {
                xv[j][0] = x[cc[j]];
                xv[j][1] = x[cc[j] + 1];
                xv[j][2] = x[cc[j] + 2];
            }
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (cc[j] >= 0) {
                const float* v = vals + (int64_t)(base + lane + 8 * j) * 9;
                y0 += v[0] * xv[j][0] + v[1] * xv[j][1] + v[2] * xv[j][2];
                y1 += v[3] * xv[j][0] + v[4] * xv[j][1] + v[5] * xv[j][2];
                y2 += v[6] * xv[j][0] + v[7] * xv[j][1] + v[8] * xv[j][2];
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
    }
}

// part[cta * kMaxBasis + k] = sum over this CTA's chunk of V[k] . w, k < nv.  Each thread
// accumulates all nv products of its elements (nv <= kMaxBasis, in registers in groups of 8).
__global__ void __launch_bounds__(kFB) multidot_partial_kernel(int64_t n, int nv, const float* __restrict__ V,
                                                                int64_t ldv, const float* __restrict__ w,
                                                                double* __restrict__ part) {
    __shared__ double red[kFB / 32][kMaxBasis];
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    for (int k0 = 0; k0 < nv; k0 += 8) {
        float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int64_t i = (int64_t)blockIdx.x * kFB + threadIdx.x; i < n; i += (int64_t)gridDim.x * kFB) {
            const float wi = w[i];
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (k0 + k < nv) acc[k] = fmaf(V[(k0 + k) * ldv + i], wi, acc[k]);
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            double a = (double)acc[k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
            if (lane == 0 && k0 + k < nv) red[wp][k0 + k] = a;
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nv; k += kFB) {
        double s = 0.0;
        for (int q = 0; q < kFB / 32; ++q) s += red[q][k];
        part[(int64_t)blockIdx.x * kMaxBasis + k] = s;
    }
}

// h[k] = sum_c part[c][k] (fixed order, one warp per k); also accumulates into hAcc[k];
// optionally writes 1/sqrt(h[0]) as a float to invNorm (normalisation factor)
__global__ void multidot_final_kernel(int nPart, int nv, const double* __restrict__ part, double* __restrict__ h,
                                      double* __restrict__ hAcc, float* __restrict__ invNorm) {
    const int lane = threadIdx.x & 31;
    const int k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (k >= nv) return;
    double s = 0.0;
    for (int c = lane; c < nPart; c += 32) s += part[(int64_t)c * kMaxBasis + k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
        h[k] = s;
        if (hAcc) hAcc[k] += s;
        if (invNorm && k == 0) invNorm[0] = s > 0.0 ? (float)(1.0 / sqrt(s)) : 0.f;
    }
}

// w -= sum_k h[k] V[k]
__global__ void multiaxpy_kernel(int64_t n, int nv, const float* __restrict__ V, int64_t ldv,
                                 const double* __restrict__ h, float* __restrict__ w) {
    __shared__ float hs[kMaxBasis];
    for (int k = threadIdx.x; k < nv; k += blockDim.x) hs[k] = (float)h[k];
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float s = w[i];
    for (int k = 0; k < nv; ++k) s -= hs[k] * V[k * ldv + i];
    w[i] = s;
}

// v = w * invNorm
__global__ void scale_kernel(int64_t n, const float* __restrict__ w, const float* __restrict__ invNorm,
                             float* __restrict__ v) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    v[i] = w[i] * invNorm[0];
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
    spmv_f32_kernel<<<nbf((int64_t)nN * 8, kFB), kFB, 0, ef::counted(s)>>>(nN, rowPtr, colIdx, vals, x, mask, y);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

// h[0..nv) = V^T w (deterministic); part: [nPart][kMaxBasis] doubles
ef_status ef_launch_multidot(int64_t n, int nv, const float* V, int64_t ldv, const float* w, double* part, int nPart,
                             double* h, double* hAcc, float* invNorm, cudaStream_t s) {
    multidot_partial_kernel<<<nPart, kFB, 0, ef::counted(s)>>>(n, nv, V, ldv, w, part);
    multidot_final_kernel<<<(nv + 7) / 8, 256, 0, ef::counted(s)>>>(nPart, nv, part, h, hAcc, invNorm);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_multiaxpy(int64_t n, int nv, const float* V, int64_t ldv, const double* h, float* w,
                              cudaStream_t s) {
    multiaxpy_kernel<<<nbf(n, 256), 256, 0, ef::counted(s)>>>(n, nv, V, ldv, h, w);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_scale(int64_t n, const float* w, const float* invNorm, float* v, cudaStream_t s) {
    scale_kernel<<<nbf(n, 256), 256, 0, ef::counted(s)>>>(n, w, invNorm, v);
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
