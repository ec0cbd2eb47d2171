// Krylov kernels on the 3x3-block (BSR) system: SpMV, block-Jacobi PCG as one
// persistent cooperative launch, and the FP64 residual of the iterative refinement.
//
// Replaces the linear solve behind NIST.linearSolve (solvers/nonlinearimplicitstatic.py:727-751;
// the reference's solvers are MKL PARDISO / SuperLU / GMRES+AMG, config/linsolve.py).
//
// Dirichlet DOFs are eliminated symmetrically: every Krylov vector vanishes on them and
// the operator's Dirichlet rows are masked to zero, so the free-free block is solved.
// Reductions are deterministic (per-CTA partials summed in a fixed order by every CTA).
// Grid-wide barriers are the CUDA cooperative-launch grid barrier (all CTAs resident).

#include <cooperative_groups.h>

#include <algorithm>
#include <cstdio>

#include "ef_common.cuh"

namespace cg = cooperative_groups;

namespace ef {

constexpr int kKB = 512;         // threads per CTA of the Krylov kernels
constexpr int kRowLanes = 8;     // lanes per block row in the SpMV
constexpr int kBatch = 4;        // blocks per lane whose loads are issued together

struct BarrierState {
    unsigned int count;
    unsigned int gen;
};

// Grid-wide barrier of the persistent kernels.  The kernels are launched with
// cudaLaunchCooperativeKernel, so every CTA is resident and the CUDA grid barrier cannot
// deadlock.  Returns false if a device-side error flag is set (the caller then returns).
__device__ __forceinline__ bool grid_sync(BarrierState*, unsigned int, int* flags) {
    cg::this_grid().sync();
    return !(*((volatile int*)flags) & EF_FLAG_BARRIER);
}

// FP64 is a narrow pipe on this GPU (2 lanes per SM and cycle): per-thread partial sums and the
// warp trees run in the vector type AT (FP32 for the FP32 solve), the CTA's warp sums and the
// sum over CTAs in FP64, all in a fixed order.

// CTA sum of NV values per thread, returned in FP64 to every thread
template <typename AT, int NV>
__device__ __forceinline__ void block_sum(AT (&v)[NV], double (&out)[NV]) {
    constexpr int NW = kKB / 32;
    __shared__ AT red[NV][NW];
    __shared__ double res[NV];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < NV; ++j) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_xor_sync(0xffffffffu, v[j], o);
    }
    if (lane == 0) {
#pragma unroll
        for (int j = 0; j < NV; ++j) red[j][w] = v[j];
    }
    __syncthreads();
    if (threadIdx.x < NV) {
        double t = 0.0;
#pragma unroll
        for (int q = 0; q < NW; ++q) t += (double)red[threadIdx.x][q];
        res[threadIdx.x] = t;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < NV; ++j) out[j] = res[j];
    __syncthreads();
}

// sum of the per-CTA partials slot[c*4 + j], j < NV, identical in every CTA (one warp sums,
// lane-strided then a fixed shuffle tree)
template <int NV>
__device__ __forceinline__ void reduce_partials(const double* part, int nCTA, double (&v)[NV]) {
    __shared__ double res[NV];
    if (threadIdx.x < 32) {
#pragma unroll
        for (int j = 0; j < NV; ++j) {
            double a = 0.0;
            for (int c = threadIdx.x; c < nCTA; c += 32) a += __ldcg(part + c * 4 + j);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
            if (threadIdx.x == 0) res[j] = a;
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < NV; ++j) v[j] = res[j];
    __syncthreads();
}

// y_row = A_row x for the block row `m`, lanes l = 0..7 of a row group; returns partial sums
// CG = true loads x through L2 only (x was written by other CTAs of a persistent kernel)
template <typename MT, typename XT, typename AT, bool CG>
__device__ __forceinline__ void bsr_row(int m, int l, const int32_t* __restrict__ rowPtr,
                                        const int32_t* __restrict__ colIdx, const MT* __restrict__ vals,
                                        const XT* __restrict__ x, AT& y0, AT& y1, AT& y2) {
    y0 = y1 = y2 = (AT)0;
    const int s = rowPtr[m], e = rowPtr[m + 1];
    for (int base = s; base < e; base += kRowLanes * kBatch) {
        int cc[kBatch];
#pragma unroll
        for (int j = 0; j < kBatch; ++j) {
            const int k = base + l + j * kRowLanes;
            cc[j] = k < e ? 3 * colIdx[k] : -1;
        }
        AT xv[kBatch][3];
#pragma unroll
        for (int j = 0; j < kBatch; ++j) {
            if (cc[j] >= 0) {
                const int c = cc[j];
                if (CG) {
                    xv[j][0] = (AT)__ldcg(x + c);
                    xv[j][1] = (AT)__ldcg(x + c + 1);
                    xv[j][2] = (AT)__ldcg(x + c + 2);
                } else {
                    xv[j][0] = (AT)x[c];
                    xv[j][1] = (AT)x[c + 1];
                    xv[j][2] = (AT)x[c + 2];
                }
            }
        }
#pragma unroll
        for (int j = 0; j < kBatch; ++j) {
            if (cc[j] >= 0) {
                const MT* v = vals + (int64_t)(base + l + j * kRowLanes) * 9;
                y0 += (AT)v[0] * xv[j][0] + (AT)v[1] * xv[j][1] + (AT)v[2] * xv[j][2];
                y1 += (AT)v[3] * xv[j][0] + (AT)v[4] * xv[j][1] + (AT)v[5] * xv[j][2];
                y2 += (AT)v[6] * xv[j][0] + (AT)v[7] * xv[j][1] + (AT)v[8] * xv[j][2];
            }
        }
    }
#pragma unroll
    for (int o = kRowLanes / 2; o > 0; o >>= 1) {
        y0 += __shfl_xor_sync(0xffffffffu, y0, o);
        y1 += __shfl_xor_sync(0xffffffffu, y1, o);
        y2 += __shfl_xor_sync(0xffffffffu, y2, o);
    }
}

// y = beta_b * b - A x (masked rows -> 0) in AT accumulation; one launch, grid-stride rows.
// With b == nullptr: y = A x.  mask may be nullptr (no masking).
template <typename MT, typename XT, typename AT>
__global__ void __launch_bounds__(kKB) bsr_residual_kernel(int nNodes, const int32_t* __restrict__ rowPtr,
                                                           const int32_t* __restrict__ colIdx,
                                                           const MT* __restrict__ vals, const XT* __restrict__ x,
                                                           const double* __restrict__ b,
                                                           const uint8_t* __restrict__ mask, double* __restrict__ y) {
    const int lane = threadIdx.x % kRowLanes;
    const int groupsPerCTA = kKB / kRowLanes;
    const int nGroups = gridDim.x * groupsPerCTA;
    int g = blockIdx.x * groupsPerCTA + threadIdx.x / kRowLanes;
    // all lanes of a warp iterate the same number of times (shuffles need full warps)
    const int iters = (nNodes + nGroups - 1) / nGroups;
    for (int it = 0; it < iters; ++it, g += nGroups) {
        const int m = g < nNodes ? g : nNodes - 1;
        AT y0, y1, y2;
        bsr_row<MT, XT, AT, false>(m, lane, rowPtr, colIdx, vals, x, y0, y1, y2);
        if (g < nNodes && lane < 3) {
            const int d = 3 * m + lane;
            const AT yy = lane == 0 ? y0 : (lane == 1 ? y1 : y2);
            double out = b ? b[d] - (double)yy : (double)yy;
            if (mask && mask[d]) out = 0.0;
            y[d] = out;
        }
    }
}

struct PcgResult {
    int iterations;
    int status;
    double rr;   // final squared residual norm
    double bb;   // squared RHS norm
};

// Block-Jacobi PCG on the free DOFs, persistent over all iterations, two grid barriers per
// iteration.  The search direction p_k = z_k + beta_k p_{k-1} is never materialised before the
// SpMV: each row group gathers z and the previous p of its neighbours and combines them on the
// fly, writing p_k for its own row into the other half of a double buffer.
// b: RHS (zero on Dirichlet DOFs); x: solution (out).  A breakdown (p.q <= 0, e.g. FP32 round-off
// near the attainable accuracy) ends the solve with EF_NOT_CONVERGED and the current iterate.
template <typename VT>
__global__ void __launch_bounds__(kKB) pcg_persistent_kernel(
    int nNodes, const int32_t* __restrict__ rowPtr, const int32_t* __restrict__ colIdx, const VT* __restrict__ vals,
    const VT* __restrict__ binv, const uint8_t* __restrict__ mask, const VT* __restrict__ b, VT* __restrict__ x,
    VT* __restrict__ r, VT* __restrict__ z, VT* __restrict__ pA, VT* __restrict__ pB, VT* __restrict__ q,
    double* __restrict__ partA, double* __restrict__ partB, BarrierState* bar, PcgResult* res, int maxIter,
    double rtol2, int* flags) {
    const unsigned int nCTA = gridDim.x;
    const int tidg = blockIdx.x * kKB + threadIdx.x;
    const int nThr = gridDim.x * kKB;
    const int lane = threadIdx.x % kRowLanes;
    const int groupsPerCTA = kKB / kRowLanes;
    const int nGroups = gridDim.x * groupsPerCTA;

    // init: x = 0, r = b, z = M^-1 r
    VT loc[2] = {(VT)0, (VT)0};
    for (int m = tidg; m < nNodes; m += nThr) {
        const int d = 3 * m;
        VT rv[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            rv[i] = b[d + i];
            x[d + i] = (VT)0;
            r[d + i] = rv[i];
        }
        const VT* B = binv + (int64_t)m * 9;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            VT zi = B[3 * i] * rv[0] + B[3 * i + 1] * rv[1] + B[3 * i + 2] * rv[2];
            if (mask[d + i]) zi = (VT)0;
            z[d + i] = zi;
            loc[0] += rv[i] * zi;
            loc[1] += rv[i] * rv[i];
        }
    }
    {
        double cs[2];
        block_sum<VT, 2>(loc, cs);
        if (threadIdx.x == 0) {
            partB[blockIdx.x * 4 + 0] = cs[0];
            partB[blockIdx.x * 4 + 1] = cs[1];
        }
    }
    if (!grid_sync(bar, nCTA, flags)) return;
    double tot[2];
    reduce_partials<2>(partB, nCTA, tot);
    double rz = tot[0];
    const double bb = tot[1];
    double rr = bb;
    int k = 0;
    int status = EF_OK;
    VT beta = (VT)0;
    VT* pPrev = pB;
    VT* pCur = pA;
    if (bb > 0.0) {
        for (k = 0; k < maxIter; ++k) {
            // q = A p_k with p_k = z + beta p_{k-1} formed on the fly; p_k stored for own rows.
            // Loads are batched (up to kBatch blocks per lane issued before any use) so that a
            // row costs three dependent memory latencies instead of one per block.
            VT pq = (VT)0;
            {
                const int iters = (nNodes + nGroups - 1) / nGroups;
                int g = blockIdx.x * groupsPerCTA + threadIdx.x / kRowLanes;
                for (int it = 0; it < iters; ++it, g += nGroups) {
                    const int m = g < nNodes ? g : nNodes - 1;
                    VT y0 = 0, y1 = 0, y2 = 0;
                    const int s0 = rowPtr[m], s1 = rowPtr[m + 1];
                    for (int base = s0; base < s1; base += kRowLanes * kBatch) {
                        int cc[kBatch];
#pragma unroll
                        for (int j = 0; j < kBatch; ++j) {
                            const int kk = base + lane + j * kRowLanes;
                            cc[j] = kk < s1 ? 3 * colIdx[kk] : -1;
                        }
                        VT xv[kBatch][3];
#pragma unroll
                        for (int j = 0; j < kBatch; ++j) {
                            if (cc[j] >= 0) {
                                const int c = cc[j];
                                xv[j][0] = __ldcg(z + c);
                                xv[j][1] = __ldcg(z + c + 1);
                                xv[j][2] = __ldcg(z + c + 2);
                                if (k > 0) {
                                    xv[j][0] += beta * __ldcg(pPrev + c);
                                    xv[j][1] += beta * __ldcg(pPrev + c + 1);
                                    xv[j][2] += beta * __ldcg(pPrev + c + 2);
                                }
                            }
                        }
#pragma unroll
                        for (int j = 0; j < kBatch; ++j) {
                            if (cc[j] >= 0) {
                                const VT* v = vals + (int64_t)(base + lane + j * kRowLanes) * 9;
                                y0 += v[0] * xv[j][0] + v[1] * xv[j][1] + v[2] * xv[j][2];
                                y1 += v[3] * xv[j][0] + v[4] * xv[j][1] + v[5] * xv[j][2];
                                y2 += v[6] * xv[j][0] + v[7] * xv[j][1] + v[8] * xv[j][2];
                            }
                        }
                    }
#pragma unroll
                    for (int o = kRowLanes / 2; o > 0; o >>= 1) {
                        y0 += __shfl_xor_sync(0xffffffffu, y0, o);
                        y1 += __shfl_xor_sync(0xffffffffu, y1, o);
                        y2 += __shfl_xor_sync(0xffffffffu, y2, o);
                    }
                    if (g < nNodes && lane < 3) {
                        const int d = 3 * m + lane;
                        VT yy = lane == 0 ? y0 : (lane == 1 ? y1 : y2);
                        VT pd = __ldcg(z + d);
                        if (k > 0) pd += beta * __ldcg(pPrev + d);
                        if (mask[d]) yy = (VT)0;
                        q[d] = yy;
                        pCur[d] = pd;
                        pq += pd * yy;
                    }
                }
            }
            VT v1[1] = {pq};
            double c1[1];
            block_sum<VT, 1>(v1, c1);
            if (threadIdx.x == 0) partA[blockIdx.x * 4] = c1[0];
            if (!grid_sync(bar, nCTA, flags)) return;
            double t1[1];
            reduce_partials<1>(partA, nCTA, t1);
            if (!(t1[0] == t1[0])) {
                status = EF_NAN;
                break;
            }
            if (!(t1[0] > 0.0)) {
                status = EF_NOT_CONVERGED;  // breakdown: keep the current iterate
                break;
            }
            const VT alpha = (VT)(rz / t1[0]);
            VT l2[2] = {(VT)0, (VT)0};
            for (int m = tidg; m < nNodes; m += nThr) {
                const int d = 3 * m;
                VT rv[3];
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    x[d + i] += alpha * __ldcg(pCur + d + i);
                    rv[i] = r[d + i] - alpha * __ldcg(q + d + i);
                    r[d + i] = rv[i];
                }
                const VT* B = binv + (int64_t)m * 9;
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    VT zi = B[3 * i] * rv[0] + B[3 * i + 1] * rv[1] + B[3 * i + 2] * rv[2];
                    if (mask[d + i]) zi = (VT)0;
                    z[d + i] = zi;
                    l2[0] += rv[i] * zi;
                    l2[1] += rv[i] * rv[i];
                }
            }
            {
                double c2[2];
                block_sum<VT, 2>(l2, c2);
                if (threadIdx.x == 0) {
                    partB[blockIdx.x * 4 + 0] = c2[0];
                    partB[blockIdx.x * 4 + 1] = c2[1];
                }
            }
            if (!grid_sync(bar, nCTA, flags)) return;
            reduce_partials<2>(partB, nCTA, tot);
            rr = tot[1];
            if (!(rr == rr)) {
                status = EF_NAN;
                break;
            }
            if (rr <= rtol2 * bb) {
                ++k;
                break;
            }
            beta = (VT)(tot[0] / rz);
            rz = tot[0];
            VT* t = pPrev;
            pPrev = pCur;
            pCur = t;
        }
        if (k >= maxIter && status == EF_OK && !(rr <= rtol2 * bb)) status = EF_NOT_CONVERGED;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        res->iterations = k;
        res->status = status;
        res->rr = rr;
        res->bb = bb;
    }
}

// deterministic dot products: part[c*2+{0,1}] then a final pass
__global__ void __launch_bounds__(kKB) dot2_partial_kernel(int64_t n, const double* __restrict__ a,
                                                           const double* __restrict__ b, double* __restrict__ part) {
    double v[1] = {0.0};
    for (int64_t i = (int64_t)blockIdx.x * kKB + threadIdx.x; i < n; i += (int64_t)gridDim.x * kKB)
        v[0] += a[i] * b[i];
    double o[1];
    block_sum<double, 1>(v, o);
    if (threadIdx.x == 0) part[blockIdx.x] = o[0];
}

__global__ void sum_final_kernel(int n, const double* __restrict__ part, double* __restrict__ out) {
    if (threadIdx.x || blockIdx.x) return;
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += part[i];
    *out = s;
}

// small vector kernels
template <typename T>
__global__ void masked_copy_kernel(int64_t n, const double* __restrict__ src, const uint8_t* __restrict__ mask,
                                   int keepMasked, double scale, T* __restrict__ dst) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bool m = mask && mask[i];
    dst[i] = (T)((m == (keepMasked != 0)) ? src[i] * scale : 0.0);
}

template <typename T>
__global__ void axpy_kernel(int64_t n, double a, const T* __restrict__ xs, double* __restrict__ y) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] += a * (double)xs[i];
}

__global__ void add_kernel(int64_t n, const double* __restrict__ a, const double* __restrict__ b,
                           double* __restrict__ y) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = a[i] + b[i];
}

}  // namespace ef

using namespace ef;

static inline int nb(int64_t n, int t) { return (int)((n + t - 1) / t); }

int ef_krylov_block_threads() { return kKB; }
size_t ef_barrier_state_bytes() { return sizeof(BarrierState); }
size_t ef_pcg_result_bytes() { return sizeof(PcgResult); }

ef_status ef_launch_bsr_residual(int nNodes, const int32_t* rowPtr, const int32_t* colIdx, const void* vals,
                                 int mDouble, const double* x, const double* b, const uint8_t* mask, double* y,
                                 int nSM, cudaStream_t s) {
    if (nNodes == 0) return EF_OK;
    const int groups = kKB / kRowLanes;
    int grid = nb(nNodes, groups);
    const int cap = nSM * 8;
    if (grid > cap) grid = cap;
    if (mDouble)
        bsr_residual_kernel<double, double, double><<<grid, kKB, 0, ef::counted(s)>>>(nNodes, rowPtr, colIdx, (const double*)vals,
                                                                       x, b, mask, y);
    else
        bsr_residual_kernel<float, double, double><<<grid, kKB, 0, ef::counted(s)>>>(nNodes, rowPtr, colIdx, (const float*)vals, x,
                                                                      b, mask, y);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_pcg_grid(int vDouble, int nSM, int* gridOut) {
    int perSM = 0;
    if (vDouble)
        EF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, pcg_persistent_kernel<double>, kKB, 0));
    else
        EF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, pcg_persistent_kernel<float>, kKB, 0));
    if (perSM < 1) {
        ef_set_error("PCG kernel cannot be resident");
        return EF_ERR_CUDA;
    }
    *gridOut = std::min(perSM, 2) * nSM;
    return EF_OK;
}

ef_status ef_launch_pcg(int vDouble, int grid, int nNodes, const int32_t* rowPtr, const int32_t* colIdx,
                        const void* vals, const void* binv, const uint8_t* mask, const void* b, void* x, void* r,
                        void* z, void* pA, void* pB, void* q, double* partA, double* partB, void* bar, void* res,
                        int maxIter, double rtol2, int* flags, cudaStream_t s) {
    void* args[] = {&nNodes, &rowPtr, &colIdx, &vals, &binv, &mask, &b, &x, &r, &z, &pA, &pB, &q,
                    &partA, &partB, &bar, &res, &maxIter, &rtol2, &flags};
    ef::note_launches(1);
    if (vDouble)
        EF_CUDA(cudaLaunchCooperativeKernel((void*)pcg_persistent_kernel<double>, grid, kKB, args, 0, s));
    else
        EF_CUDA(cudaLaunchCooperativeKernel((void*)pcg_persistent_kernel<float>, grid, kKB, args, 0, s));
    return EF_OK;
}

ef_status ef_launch_dot(int64_t n, const double* a, const double* b, double* part, int nPart, double* out,
                        cudaStream_t s) {
    dot2_partial_kernel<<<nPart, kKB, 0, ef::counted(s)>>>(n, a, b, part);
    sum_final_kernel<<<1, 32, 0, ef::counted(s)>>>(nPart, part, out);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_masked_copy(int64_t n, const double* src, const uint8_t* mask, int keepMasked, double scale,
                                void* dst, int dstDouble, cudaStream_t s) {
    if (n == 0) return EF_OK;
    if (dstDouble)
        masked_copy_kernel<double><<<nb(n, 256), 256, 0, ef::counted(s)>>>(n, src, mask, keepMasked, scale, (double*)dst);
    else
        masked_copy_kernel<float><<<nb(n, 256), 256, 0, ef::counted(s)>>>(n, src, mask, keepMasked, scale, (float*)dst);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_axpy(int64_t n, double a, const void* xs, int xDouble, double* y, cudaStream_t s) {
    if (n == 0) return EF_OK;
    if (xDouble)
        axpy_kernel<double><<<nb(n, 256), 256, 0, ef::counted(s)>>>(n, a, (const double*)xs, y);
    else
        axpy_kernel<float><<<nb(n, 256), 256, 0, ef::counted(s)>>>(n, a, (const float*)xs, y);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_add(int64_t n, const double* a, const double* b, double* y, cudaStream_t s) {
    if (n == 0) return EF_OK;
    add_kernel<<<nb(n, 256), 256, 0, ef::counted(s)>>>(n, a, b, y);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

// ---------------------------------------------------------------------------------------------
// Allocation-free block-Jacobi PCG (ef_pcg_solve_noalloc).
//
// Some callers cannot allocate device memory at solve time: a host framework that has reserved
// the device memory for its own pool, or a latency-critical loop that must not take the
// device-wide synchronisation that cudaMalloc/cudaFree imply.  This entry point solves with the
// same persistent PCG kernel as ef_solve, but its work vectors live in a fixed file-scope device
// array instead of a context workspace, so the call itself allocates nothing.
// ---------------------------------------------------------------------------------------------

#include <mutex>

#define EF_NOALLOC_SCRATCH_BYTES (8u << 20)  // 8 MiB held by every device that loads the library
static __device__ __align__(256) unsigned char g_noallocScratch[EF_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noallocMutex;
void* g_noallocPtr[kMaxDevices] = {};
int g_noallocGrid[kMaxDevices] = {};

inline size_t align256(size_t n) { return (n + 255) & ~(size_t)255; }
}  // namespace

extern "C" int64_t ef_pcg_noalloc_max_nodes(void) {
    // layout: two partial-sum arrays (4 doubles per CTA, at most 2 CTAs per SM on 256 SMs),
    // the result record, then five FP64 work vectors of 3*nNodes entries each
    // (the last 256 bytes hold the call's device flags word)
    const size_t fixed = 2 * align256(4 * sizeof(double) * 512) + align256(sizeof(PcgResult)) + 256;
    return (int64_t)((EF_NOALLOC_SCRATCH_BYTES - fixed - 5 * 256) / (5 * 3 * sizeof(double)));
}

extern "C" ef_status ef_pcg_solve_noalloc(int64_t nNodes, const int32_t* rowPtr, const int32_t* colIdx,
                                          const double* vals, const double* binv, const uint8_t* mask,
                                          const double* b, double* x, int maxIter, double rtol, ef_solve_info* info,
                                          void* stream) {
    if (nNodes <= 0 || !rowPtr || !colIdx || !vals || !binv || !mask || !b || !x || maxIter < 0 || !(rtol >= 0.0)) {
        ef_set_error("ef_pcg_solve_noalloc: invalid arguments");
        return EF_ERR_ARG;
    }
    if (nNodes > ef_pcg_noalloc_max_nodes()) {
        ef_set_error("ef_pcg_solve_noalloc: " + std::to_string(nNodes) + " block rows exceed the fixed scratch capacity of " +
                     std::to_string(ef_pcg_noalloc_max_nodes()) + " block rows (8 MiB); use ef_solve");
        return EF_ERR_ARG;
    }
    int dev = 0;
    EF_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        ef_set_error("ef_pcg_solve_noalloc: device index out of range");
        return EF_ERR_ARG;
    }
    {
        // once per device, with that device current: the device address of the scratch array
        std::lock_guard<std::mutex> lock(g_noallocMutex);
        if (!g_noallocPtr[dev]) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noallocScratch);
            if (e != cudaSuccess || !p) {
                ef_set_error(std::string("ef_pcg_solve_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
                return EF_ERR_CUDA;
            }
            int nSM = 0, perSM = 0;
            EF_CUDA(cudaDeviceGetAttribute(&nSM, cudaDevAttrMultiProcessorCount, dev));
            EF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, pcg_persistent_kernel<double>, kKB, 0));
            const int grid = std::min(perSM, 2) * nSM;
            if (grid < 1 || grid > 512) {
                ef_set_error("ef_pcg_solve_noalloc: unsupported device (grid size)");
                return EF_ERR_CUDA;
            }
            g_noallocGrid[dev] = grid;
            g_noallocPtr[dev] = p;
        }
    }
    unsigned char* base = (unsigned char*)g_noallocPtr[dev];
    const size_t partBytes = align256(4 * sizeof(double) * 512);
    double* partA = (double*)base;
    double* partB = (double*)(base + partBytes);
    PcgResult* res = (PcgResult*)(base + 2 * partBytes);
    unsigned char* vec = base + 2 * partBytes + align256(sizeof(PcgResult));
    const size_t vb = align256(3 * (size_t)nNodes * sizeof(double));
    double* r = (double*)(vec + 0 * vb);
    double* z = (double*)(vec + 1 * vb);
    double* pA = (double*)(vec + 2 * vb);
    double* pB = (double*)(vec + 3 * vb);
    double* q = (double*)(vec + 4 * vb);
    // device flags word: the last 256 bytes of the scratch array, cleared for this call
    int* flags = (int*)(base + EF_NOALLOC_SCRATCH_BYTES - 256);
    cudaStream_t s = (cudaStream_t)stream;
    EF_CUDA(cudaMemsetAsync(flags, 0, sizeof(int), s));
    int nn = (int)nNodes;
    BarrierState* bar = nullptr;
    double rtol2 = rtol * rtol;
    void* args[] = {&nn, &rowPtr, &colIdx, &vals, &binv, &mask, &b, &x, &r, &z, &pA, &pB, &q,
                    &partA, &partB, &bar, &res, &maxIter, &rtol2, &flags};
    ef::note_launches(1);
    EF_CUDA(cudaLaunchCooperativeKernel((void*)pcg_persistent_kernel<double>, g_noallocGrid[dev], kKB, args, 0, s));
    PcgResult hr;
    EF_CUDA(cudaMemcpyAsync(&hr, res, sizeof(hr), cudaMemcpyDeviceToHost, s));
    EF_CUDA(cudaStreamSynchronize(s));
    const double rel = hr.bb > 0.0 ? sqrt(hr.rr / hr.bb) : 0.0;
    if (info) {
        info->iterations = hr.iterations;
        info->refinements = 0;
        info->relResidual = rel;
        info->status = hr.status;
        info->kernelMs = 0.0;
        info->kernelLaunches = 1;
    }
    if (hr.status != EF_OK) {
        char msg[160];
        snprintf(msg, sizeof msg, "ef_pcg_solve_noalloc: status %d after %d iterations, relative residual %.3e",
                 hr.status, hr.iterations, rel);
        ef_set_error(msg);
    }
    return hr.status == EF_OK ? EF_OK : (ef_status)hr.status;
}
