// Batched solve of many independent small problems held in one context.
//
// The problems are disjoint meshes whose nodes occupy contiguous ranges [nodePtr[p],
// nodePtr[p+1]) of the context's 3x3-block system, so the assembled system is block diagonal by
// problem.  One persistent launch solves all of them: each CTA takes problems from a list sorted
// by decreasing size (CTA k solves problems k, k + grid, ...) and runs block-Jacobi PCG on its
// problem with CTA-wide reductions only, so problems of uneven size need no grid barrier and a
// small problem never waits for a large one.  Each problem has its own step lengths, its own
// stopping test (|r| <= rtol |b| on the problem's own right-hand side) and its own iteration
// count.  Reductions are fixed shuffle trees plus a fixed-order sum over warps: deterministic for
// a given tile shape (threads per CTA, lanes per block row), which a timing autotuner picks.
//
// The per-problem Newton checks of the reference's NIST driver (solvers/nonlinearimplicitstatic.py
// :625-725) need max|R|, sum|F| and max|ddU| per problem: batch_norms_kernel, one CTA per problem.

#include <algorithm>

#include "ef_common.cuh"

namespace ef {

// CTA sums of NV values per thread in a fixed order.  FP64 is a narrow pipe on this GPU, so one
// warp does the adds (TPB / 32 strided adds per lane and value, then a shuffle tree) instead of
// every warp; red holds NV * TPB doubles.
template <int TPB, int NV>
__device__ __forceinline__ void cta_sum(double (&v)[NV], double* red) {
    __syncthreads();  // red is free again (previous readers are done)
#pragma unroll
    for (int j = 0; j < NV; ++j) red[j * TPB + threadIdx.x] = v[j];
    __syncthreads();
    if (threadIdx.x < 32) {
#pragma unroll
        for (int j = 0; j < NV; ++j) {
            double s = 0.0;
#pragma unroll
            for (int i = 0; i < TPB / 32; ++i) s += red[j * TPB + 32 * i + threadIdx.x];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (threadIdx.x == 0) red[NV * TPB + j] = s;
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < NV; ++j) v[j] = red[NV * TPB + j];
}

// TPB threads per CTA; the products use LPR lanes per block row (strided over the row's blocks,
// combined by a fixed shuffle tree), the vector updates one thread per block row.
template <int TPB, int LPR>
__global__ void __launch_bounds__(TPB) batched_pcg_kernel(
    int nProb, const int32_t* __restrict__ nodePtr, const int32_t* __restrict__ order,
    const int32_t* __restrict__ rowPtr, const int32_t* __restrict__ colIdx, const double* __restrict__ vals,
    const double* __restrict__ binv, const uint8_t* __restrict__ mask, const double* __restrict__ b,
    double* __restrict__ x, double* __restrict__ r, double* __restrict__ z, double* __restrict__ p,
    double* __restrict__ q, int maxIter, double rtol2, int* __restrict__ itersOut, double* __restrict__ relOut) {
    __shared__ double red[2 * TPB + 2];
    constexpr int RPI = TPB / LPR;  // block rows per pass of the product
    const int sub = threadIdx.x % LPR, grp = threadIdx.x / LPR;
    for (int k = blockIdx.x; k < nProb; k += gridDim.x) {
        const int pid = order[k];
        const int n0 = nodePtr[pid], n1 = nodePtr[pid + 1];
        double lrz = 0.0, lbb = 0.0;
        for (int m = n0 + (int)threadIdx.x; m < n1; m += TPB) {
            double rv[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const int d = 3 * m + i;
                rv[i] = mask[d] ? 0.0 : b[d];
                x[d] = 0.0;
                r[d] = rv[i];
            }
            const double* B = binv + (int64_t)m * 9;
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const int d = 3 * m + i;
                const double zi = mask[d] ? 0.0 : B[3 * i] * rv[0] + B[3 * i + 1] * rv[1] + B[3 * i + 2] * rv[2];
                z[d] = zi;
                p[d] = zi;
                lrz += rv[i] * zi;
                lbb += rv[i] * rv[i];
            }
        }
        double t0[2] = {lrz, lbb};
        cta_sum<TPB, 2>(t0, red);
        double rz = t0[0];
        const double bb = t0[1];
        int it = 0;
        double rr = bb;
        bool ok = true;
        if (bb > 0.0) {
            while (it < maxIter && rr > rtol2 * bb) {
                // q = A p on free rows; p.q
                double lpq = 0.0;
                for (int m0 = n0; m0 < n1; m0 += RPI) {
                    const int m = m0 + grp;
                    double y0 = 0.0, y1 = 0.0, y2 = 0.0;
                    if (m < n1)
                        for (int kk = rowPtr[m] + sub; kk < rowPtr[m + 1]; kk += LPR) {
                            const int c = 3 * colIdx[kk];
                            const double* v = vals + (int64_t)kk * 9;
                            const double p0 = p[c], p1 = p[c + 1], p2 = p[c + 2];
                            y0 += v[0] * p0 + v[1] * p1 + v[2] * p2;
                            y1 += v[3] * p0 + v[4] * p1 + v[5] * p2;
                            y2 += v[6] * p0 + v[7] * p1 + v[8] * p2;
                        }
#pragma unroll
                    for (int o = LPR / 2; o > 0; o >>= 1) {
                        y0 += __shfl_xor_sync(0xffffffffu, y0, o);
                        y1 += __shfl_xor_sync(0xffffffffu, y1, o);
                        y2 += __shfl_xor_sync(0xffffffffu, y2, o);
                    }
                    if (m < n1 && sub == 0) {
                        const double yy[3] = {y0, y1, y2};
#pragma unroll
                        for (int i = 0; i < 3; ++i) {
                            const int d = 3 * m + i;
                            const double qi = mask[d] ? 0.0 : yy[i];
                            q[d] = qi;
                            lpq += p[d] * qi;
                        }
                    }
                }
                double t1[1] = {lpq};
                cta_sum<TPB, 1>(t1, red);
                const double pq = t1[0];
                if (!(pq > 0.0)) {  // breakdown or NaN: stop with the current iterate
                    ok = pq == pq;
                    break;
                }
                const double alpha = rz / pq;
                double lrr = 0.0, lrz2 = 0.0;
                for (int m = n0 + (int)threadIdx.x; m < n1; m += TPB) {
                    double rv[3];
#pragma unroll
                    for (int i = 0; i < 3; ++i) {
                        const int d = 3 * m + i;
                        x[d] += alpha * p[d];
                        rv[i] = r[d] - alpha * q[d];
                        r[d] = rv[i];
                        lrr += rv[i] * rv[i];
                    }
                    const double* B = binv + (int64_t)m * 9;
#pragma unroll
                    for (int i = 0; i < 3; ++i) {
                        const int d = 3 * m + i;
                        const double zi =
                            mask[d] ? 0.0 : B[3 * i] * rv[0] + B[3 * i + 1] * rv[1] + B[3 * i + 2] * rv[2];
                        z[d] = zi;
                        lrz2 += rv[i] * zi;
                    }
                }
                double t2[2] = {lrr, lrz2};
                cta_sum<TPB, 2>(t2, red);
                rr = t2[0];
                const double rz2 = t2[1];
                const double beta = rz2 / rz;
                rz = rz2;
                for (int m = n0 + (int)threadIdx.x; m < n1; m += TPB)
#pragma unroll
                    for (int i = 0; i < 3; ++i) {
                        const int d = 3 * m + i;
                        p[d] = z[d] + beta * p[d];
                    }
                __syncthreads();  // p complete before the next product
                ++it;
            }
        }
        if (threadIdx.x == 0) {
            itersOut[pid] = it;
            relOut[pid] = !ok ? __longlong_as_double(0x7ff8000000000000LL) : (bb > 0.0 ? sqrt(rr / bb) : 0.0);
        }
        __syncthreads();
    }
}

// out[p] = {max |R|, sum |F|, max |ddU|} over the DOFs of problem p (ddU may be null)
__global__ void __launch_bounds__(256) batch_norms_kernel(int nProb, const int32_t* __restrict__ nodePtr,
                                                          const double* __restrict__ R, const double* __restrict__ F,
                                                          const double* __restrict__ D, double* __restrict__ out) {
    __shared__ double red[3][8];
    const int pid = blockIdx.x;
    if (pid >= nProb) return;
    const int d0 = 3 * nodePtr[pid], d1 = 3 * nodePtr[pid + 1];
    double a = 0.0, s = 0.0, c = 0.0;
    for (int d = d0 + (int)threadIdx.x; d < d1; d += 256) {
        a = fmax(a, fabs(R[d]));
        s += fabs(F[d]);
        if (D) c = fmax(c, fabs(D[d]));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a = fmax(a, __shfl_xor_sync(0xffffffffu, a, o));
        s += __shfl_xor_sync(0xffffffffu, s, o);
        c = fmax(c, __shfl_xor_sync(0xffffffffu, c, o));
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        red[0][w] = a;
        red[1][w] = s;
        red[2][w] = c;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double A = 0.0, S = 0.0, C = 0.0;
        for (int i = 0; i < 8; ++i) {
            A = fmax(A, red[0][i]);
            S += red[1][i];
            C = fmax(C, red[2][i]);
        }
        out[3 * pid] = A;
        out[3 * pid + 1] = S;
        out[3 * pid + 2] = C;
    }
}

template <int TPB, int LPR>
static ef_status launch_batched(int nSM, int nProb, const int32_t* nodePtr, const int32_t* order,
                                const int32_t* rowPtr, const int32_t* colIdx, const double* vals, const double* binv,
                                const uint8_t* mask, const double* b, double* x, double* r, double* z, double* p,
                                double* q, int maxIter, double rtol2, int* iters, double* rel, cudaStream_t s) {
    int perSM = 0;
    EF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, batched_pcg_kernel<TPB, LPR>, TPB, 0));
    const int grid = std::max(1, std::min(nProb, std::max(1, perSM) * nSM));
    batched_pcg_kernel<TPB, LPR><<<grid, TPB, 0, ef::counted(s)>>>(nProb, nodePtr, order, rowPtr, colIdx, vals, binv,
                                                                   mask, b, x, r, z, p, q, maxIter, rtol2, iters, rel);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

}  // namespace ef

using namespace ef;

// tile shapes of the batched PCG: (threads per CTA, lanes per block row in the products)
static const int kBatchTiles[][2] = {{128, 1}, {128, 4}, {128, 8}, {256, 4}, {256, 8}, {512, 8}};
int ef_batch_num_tiles() { return (int)(sizeof(kBatchTiles) / sizeof(kBatchTiles[0])); }
void ef_batch_tile_shape(int tile, int* tpb, int* lpr) {
    *tpb = kBatchTiles[tile][0];
    *lpr = kBatchTiles[tile][1];
}

ef_status ef_launch_batched_pcg(int tile, int nSM, int nProb, const int32_t* nodePtr, const int32_t* order,
                                const int32_t* rowPtr, const int32_t* colIdx, const double* vals, const double* binv,
                                const uint8_t* mask, const double* b, double* x, double* r, double* z, double* p,
                                double* q, int maxIter, double rtol2, int* iters, double* rel, cudaStream_t s) {
    if (nProb == 0) return EF_OK;
#define EF_BT(T, L)                                                                                              \
    return launch_batched<T, L>(nSM, nProb, nodePtr, order, rowPtr, colIdx, vals, binv, mask, b, x, r, z, p, q, \
                                maxIter, rtol2, iters, rel, s)
    switch (tile) {
        case 0: EF_BT(128, 1);
        case 1: EF_BT(128, 4);
        case 2: EF_BT(128, 8);
        case 3: EF_BT(256, 4);
        case 4: EF_BT(256, 8);
        case 5: EF_BT(512, 8);
        default:
            ef_set_error("batched PCG: unknown tile shape");
            return EF_ERR_ARG;
    }
#undef EF_BT
}

ef_status ef_launch_batch_norms(int nProb, const int32_t* nodePtr, const double* R, const double* F, const double* D,
                                double* out, cudaStream_t s) {
    if (nProb == 0) return EF_OK;
    batch_norms_kernel<<<nProb, 256, 0, ef::counted(s)>>>(nProb, nodePtr, R, F, D, out);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}
