// Assembly kernels: residual condensation, VIJ export, reference-order CSR scatter,
// Dirichlet rows, atomic-free 3x3-block (BSR) scatter, and deterministic norms.
//
// Reference semantics (EdelweissFE):
//   solvers/nonlinearimplicitstaticparallelmk2.pyx:186-193  P[I] += Pe, F[I] += |Pe| (element order)
//   numerics/dofmanager.py:47-82,522-557                      VIJ layout
//   numerics/csrgenerator.pyx:100-115                         data[x[k]] += V[k], increasing k
//   solvers/nonlinearimplicitstaticparallelmk2.pyx:66-109     Dirichlet rows
//
// No float atomics anywhere: every output element is owned by one thread that
// sums its contributions in a fixed (reference) order, so results are
// bit-reproducible run to run.

#include "ef_common.cuh"

namespace ef {

// P[d0+c] = sum_k Pe[src_k + c], F likewise with |.|; one thread per node (DOF triplet)
__global__ void condense_kernel(int64_t nNodes, const int32_t* __restrict__ nodeDof, const int64_t* __restrict__ ptr,
                                const int64_t* __restrict__ src, const float* __restrict__ w,
                                const double* __restrict__ Pe, double* __restrict__ P, double* __restrict__ F) {
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nNodes) return;
    double p0 = 0.0, p1 = 0.0, p2 = 0.0, f0 = 0.0, f1 = 0.0, f2 = 0.0;
    for (int64_t k = ptr[m]; k < ptr[m + 1]; ++k) {
        const double* pe = Pe + src[k];
        double a = pe[0], b = pe[1], c = pe[2];
        if (w) {  // tied node: weighted share of the slave's element vectors
            const double wk = w[k];
            a *= wk;
            b *= wk;
            c *= wk;
        }
        p0 += a;
        p1 += b;
        p2 += c;
        f0 += fabs(a);
        f1 += fabs(b);
        f2 += fabs(c);
    }
    const int d = nodeDof[m];
    P[d] = p0;
    P[d + 1] = p1;
    P[d + 2] = p2;
    if (F) {
        F[d] = f0;
        F[d + 1] = f1;
        F[d + 2] = f2;
    }
}

// adds the condensed element vectors into V (V[d] += sum), used for body forces
__global__ void condense_add_kernel(int64_t nNodes, const int32_t* __restrict__ nodeDof,
                                    const int64_t* __restrict__ ptr, const int64_t* __restrict__ src,
                                    const float* __restrict__ w, const double* __restrict__ Pe, int64_t lo, int64_t hi,
                                    double* __restrict__ V) {
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nNodes) return;
    double p0 = 0.0, p1 = 0.0, p2 = 0.0;
    bool any = false;
    for (int64_t k = ptr[m]; k < ptr[m + 1]; ++k) {
        const int64_t s = src[k];
        if (s < lo || s >= hi) continue;
        const double* pe = Pe + s;
        const double wk = w ? (double)w[k] : 1.0;
        p0 += wk * pe[0];
        p1 += wk * pe[1];
        p2 += wk * pe[2];
        any = true;
    }
    if (!any) return;
    const int d = nodeDof[m];
    V[d] += p0;
    V[d + 1] += p1;
    V[d + 2] += p2;
}

// element blocks (symmetric storage, pair p(a,b), a<=b) -> reference VIJ layout in FP64
template <typename KT>
__global__ void vij_export_kernel(int nEl, int nn, int np, const KT* __restrict__ Kblk, double* __restrict__ Kvij) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)nEl * np) return;
    const int e = (int)(t / np);
    const int p = (int)(t % np);
    int a = 0, start = 0;
    while (start + (nn - a) <= p) {
        start += nn - a;
        ++a;
    }
    const int b = a + (p - start);
    const int nd = 3 * nn;
    const KT* kb = Kblk + t * 9;
    double* ke = Kvij + (int64_t)e * nd * nd;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            const double v = (double)kb[i * 3 + j];
            ke[(3 * a + i) * nd + 3 * b + j] = v;
            if (a != b) ke[(3 * b + j) * nd + 3 * a + i] = v;
        }
}

// reference-order scalar scatter: data[s] = ((0 + V[k0]) + V[k1]) + ... for k0 < k1 < ...
__global__ void csr_scatter_kernel(int64_t nnz, const int64_t* __restrict__ seg, const int32_t* __restrict__ perm,
                                   const double* __restrict__ V, double* __restrict__ data) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nnz) return;
    double acc = 0.0;
    for (int64_t t = seg[s]; t < seg[s + 1]; ++t) acc += V[perm[t]];
    data[s] = acc;
}

__global__ void csr_dirichlet_rows_kernel(int64_t nRows, const int64_t* __restrict__ rows,
                                          const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                                          double* __restrict__ data) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nRows) return;
    const int64_t r = rows[t];
    for (int32_t j = indptr[r]; j < indptr[r + 1]; ++j) data[j] = (indices[j] == r) ? 1.0 : 0.0;
}

// BSR block s = sum over its element-block contributions (element order); src encodes
// (global element-block index << 1) | transpose
template <typename KT>
__global__ void bsr_scatter_kernel(int64_t nBlocks, const int64_t* __restrict__ seg, const int64_t* __restrict__ src,
                                   const float* __restrict__ w, const KT* __restrict__ Kblk, KT* __restrict__ vals) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nBlocks) return;
    KT acc[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) acc[i] = (KT)0;
    for (int64_t t = seg[s]; t < seg[s + 1]; ++t) {
        const int64_t c = src[t];
        const KT* kb = Kblk + (c >> 1) * 9;
        const KT wt = w ? (KT)w[t] : (KT)1;  // tie weight (products of 1/2), exact in either type
        KT v[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) v[i] = wt * kb[i];
        if (c & 1) {
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) acc[i * 3 + j] += v[j * 3 + i];
        } else {
#pragma unroll
            for (int i = 0; i < 9; ++i) acc[i] += v[i];
        }
    }
    KT* o = vals + s * 9;
#pragma unroll
    for (int i = 0; i < 9; ++i) o[i] = acc[i];
}

// block-Jacobi setup: inverse of each diagonal 3x3 block with Dirichlet rows/columns
// replaced by the identity (inverted in FP64)
template <typename KT>
__global__ void bj_setup_kernel(int64_t nNodes, const int64_t* __restrict__ diagPos, const int32_t* __restrict__ nodeDof,
                                const uint8_t* __restrict__ mask, const KT* __restrict__ vals, KT* __restrict__ inv,
                                int* __restrict__ flags) {
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nNodes) return;
    const KT* D = vals + diagPos[m] * 9;
    const int d = nodeDof[m];
    const bool f[3] = {mask[d] != 0, mask[d + 1] != 0, mask[d + 2] != 0};
    double A[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) A[i][j] = (f[i] || f[j]) ? (i == j ? 1.0 : 0.0) : (double)D[i * 3 + j];
    const double c00 = A[1][1] * A[2][2] - A[1][2] * A[2][1];
    const double c01 = A[1][2] * A[2][0] - A[1][0] * A[2][2];
    const double c02 = A[1][0] * A[2][1] - A[1][1] * A[2][0];
    const double det = A[0][0] * c00 + A[0][1] * c01 + A[0][2] * c02;
    if (!(fabs(det) > 0.0)) {
        atomicOr(flags, EF_FLAG_NAN);
    }
    const double id = 1.0 / det;
    KT* o = inv + m * 9;
    o[0] = (KT)(c00 * id);
    o[3] = (KT)(c01 * id);
    o[6] = (KT)(c02 * id);
    o[1] = (KT)((A[0][2] * A[2][1] - A[0][1] * A[2][2]) * id);
    o[4] = (KT)((A[0][0] * A[2][2] - A[0][2] * A[2][0]) * id);
    o[7] = (KT)((A[0][1] * A[2][0] - A[0][0] * A[2][1]) * id);
    o[2] = (KT)((A[0][1] * A[1][2] - A[0][2] * A[1][1]) * id);
    o[5] = (KT)((A[0][2] * A[1][0] - A[0][0] * A[1][2]) * id);
    o[8] = (KT)((A[0][0] * A[1][1] - A[0][1] * A[1][0]) * id);
}

// deterministic norms: per-block partials in a fixed order, then one block reduces them
__global__ void norms_partial_kernel(int64_t n, const double* __restrict__ R, const double* __restrict__ F,
                                     const double* __restrict__ D, double* __restrict__ part) {
    __shared__ double s0[256], s1[256], s2[256];
    double a = 0.0, b = 0.0, c = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (R) a = fmax(a, fabs(R[i]));
        if (F) b += fabs(F[i]);
        if (D) c = fmax(c, fabs(D[i]));
    }
    s0[threadIdx.x] = a;
    s1[threadIdx.x] = b;
    s2[threadIdx.x] = c;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            s0[threadIdx.x] = fmax(s0[threadIdx.x], s0[threadIdx.x + w]);
            s1[threadIdx.x] += s1[threadIdx.x + w];
            s2[threadIdx.x] = fmax(s2[threadIdx.x], s2[threadIdx.x + w]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[3 * blockIdx.x + 0] = s0[0];
        part[3 * blockIdx.x + 1] = s1[0];
        part[3 * blockIdx.x + 2] = s2[0];
    }
}

__global__ void norms_final_kernel(int nPart, const double* __restrict__ part, double* __restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double a = 0.0, b = 0.0, c = 0.0;
    for (int i = 0; i < nPart; ++i) {
        a = fmax(a, part[3 * i]);
        b += part[3 * i + 1];
        c = fmax(c, part[3 * i + 2]);
    }
    out[0] = a;
    out[1] = b;
    out[2] = c;
}

// R = P + PExt with the Dirichlet rows set to 0 (dir[i] != 0), and the partial norms of the
// convergence check: max |R|, sum |F|, max |ddU| (solvers/nonlinearimplicitstatic.py:418-436,
// :625-725)
__global__ void newton_residual_kernel(int64_t n, const double* __restrict__ P, const double* __restrict__ PExt,
                                       const uint8_t* __restrict__ dir, const double* __restrict__ F,
                                       const double* __restrict__ D, double* __restrict__ R,
                                       double* __restrict__ part) {
    __shared__ double s0[256], s1[256], s2[256];
    double a = 0.0, b = 0.0, c = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double r = dir[i] ? 0.0 : (PExt ? P[i] + PExt[i] : P[i]);
        R[i] = r;
        a = fmax(a, fabs(r));
        b += fabs(F[i]);
        if (D) c = fmax(c, fabs(D[i]));
    }
    s0[threadIdx.x] = a;
    s1[threadIdx.x] = b;
    s2[threadIdx.x] = c;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            s0[threadIdx.x] = fmax(s0[threadIdx.x], s0[threadIdx.x + w]);
            s1[threadIdx.x] += s1[threadIdx.x + w];
            s2[threadIdx.x] = fmax(s2[threadIdx.x], s2[threadIdx.x + w]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[3 * blockIdx.x + 0] = s0[0];
        part[3 * blockIdx.x + 1] = s1[0];
        part[3 * blockIdx.x + 2] = s2[0];
    }
}

// The reference's convergence test for the displacement field (solvers/nonlinearimplicitstatic.py
// :656-682, computeSpatialAveragedFluxes :771-792), decided on the device from the partial norms:
// q = {fluxTol, fluxTolAlt, corrTol, fluxFloor, nAccFluxes, prevResidual, iteration, nGrew, hasDdU}
// out = {converged, nGrew, fluxResidual, fieldCorrection, spatialAveragedFlux}
__global__ void newton_decide_kernel(int nPart, const double* __restrict__ part, const double* __restrict__ q,
                                     double* __restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double a = 0.0, b = 0.0, c = 0.0;
    for (int i = 0; i < nPart; ++i) {
        a = fmax(a, part[3 * i]);
        b += part[3 * i + 1];
        c = fmax(c, part[3 * i + 2]);
    }
    const double avg = fmax(1e-10, b / q[4]);
    const double tol = q[6] < 15.0 ? q[0] : q[1];
    const double corr = q[8] != 0.0 ? c : 0.0;
    const bool convCorr = corr < q[2];
    const bool convFlux = a <= fmax(tol * avg, q[3]);
    out[0] = (convCorr && convFlux) ? 1.0 : 0.0;
    out[1] = q[7] + (a > q[5] ? 1.0 : 0.0);
    out[2] = a;
    out[3] = corr;
    out[4] = avg;
}

// R = P + PExt, then R[dofs[k]] = values[k] (the prescribed increments of the first iteration)
__global__ void newton_first_residual_kernel(int64_t n, const double* __restrict__ P, const double* __restrict__ PExt,
                                             double* __restrict__ R) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) R[i] = PExt ? P[i] + PExt[i] : P[i];
}
__global__ void scatter_values_kernel(int64_t n, const int64_t* __restrict__ dofs, const double* __restrict__ v,
                                      double* __restrict__ R) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) R[dofs[k]] = v[k];
}

// x[slave] = (x[a] + x[b]) / 2 per component (tied nodes)
__global__ void tie_fill_kernel(int64_t n, const int32_t* __restrict__ slave, const int32_t* __restrict__ ma,
                                const int32_t* __restrict__ mb, double* __restrict__ x) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * n) return;
    const int64_t k = t / 3;
    const int c = (int)(t % 3);
    x[3 * (int64_t)slave[k] + c] = 0.5 * (x[3 * (int64_t)ma[k] + c] + x[3 * (int64_t)mb[k] + c]);
}

}  // namespace ef

using namespace ef;

static inline int nblk(int64_t n, int t) { return (int)((n + t - 1) / t); }

ef_status ef_launch_condense(int64_t nNodes, const int32_t* nodeDof, const int64_t* ptr, const int64_t* src,
                             const float* w, const double* Pe, double* P, double* F, cudaStream_t s) {
    if (nNodes == 0) return EF_OK;
    condense_kernel<<<nblk(nNodes, 256), 256, 0, ef::counted(s)>>>(nNodes, nodeDof, ptr, src, w, Pe, P, F);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_condense_add(int64_t nNodes, const int32_t* nodeDof, const int64_t* ptr, const int64_t* src,
                                 const float* w, const double* Pe, int64_t lo, int64_t hi, double* V, cudaStream_t s) {
    if (nNodes == 0) return EF_OK;
    condense_add_kernel<<<nblk(nNodes, 256), 256, 0, ef::counted(s)>>>(nNodes, nodeDof, ptr, src, w, Pe, lo, hi, V);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_vij_export(int nEl, int nn, int np, const void* Kblk, int kDouble, double* Kvij, cudaStream_t s) {
    const int64_t n = (int64_t)nEl * np;
    if (n == 0) return EF_OK;
    if (kDouble)
        vij_export_kernel<double><<<nblk(n, 256), 256, 0, ef::counted(s)>>>(nEl, nn, np, (const double*)Kblk, Kvij);
    else
        vij_export_kernel<float><<<nblk(n, 256), 256, 0, ef::counted(s)>>>(nEl, nn, np, (const float*)Kblk, Kvij);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_csr_scatter(int64_t nnz, const int64_t* seg, const int32_t* perm, const double* V, double* data,
                                cudaStream_t s) {
    if (nnz == 0) return EF_OK;
    csr_scatter_kernel<<<nblk(nnz, 256), 256, 0, ef::counted(s)>>>(nnz, seg, perm, V, data);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_csr_dirichlet_rows(int64_t nRows, const int64_t* rows, const int32_t* indptr,
                                       const int32_t* indices, double* data, cudaStream_t s) {
    if (nRows == 0) return EF_OK;
    csr_dirichlet_rows_kernel<<<nblk(nRows, 256), 256, 0, ef::counted(s)>>>(nRows, rows, indptr, indices, data);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_bsr_scatter(int64_t nBlocks, const int64_t* seg, const int64_t* src, const float* w,
                                const void* Kblk, int kDouble, void* vals, cudaStream_t s) {
    if (nBlocks == 0) return EF_OK;
    if (kDouble)
        bsr_scatter_kernel<double><<<nblk(nBlocks, 256), 256, 0, ef::counted(s)>>>(nBlocks, seg, src, w,
                                                                                   (const double*)Kblk, (double*)vals);
    else
        bsr_scatter_kernel<float><<<nblk(nBlocks, 256), 256, 0, ef::counted(s)>>>(nBlocks, seg, src, w,
                                                                                  (const float*)Kblk, (float*)vals);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_bj_setup(int64_t nNodes, const int64_t* diagPos, const int32_t* nodeDof, const uint8_t* mask,
                             const void* vals, int kDouble, void* inv, int* flags, cudaStream_t s) {
    if (nNodes == 0) return EF_OK;
    if (kDouble)
        bj_setup_kernel<double><<<nblk(nNodes, 256), 256, 0, ef::counted(s)>>>(nNodes, diagPos, nodeDof, mask,
                                                                   (const double*)vals, (double*)inv, flags);
    else
        bj_setup_kernel<float><<<nblk(nNodes, 256), 256, 0, ef::counted(s)>>>(nNodes, diagPos, nodeDof, mask, (const float*)vals,
                                                                  (float*)inv, flags);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

__global__ void residual_from_kernel(int64_t n, const double* __restrict__ b, const double* __restrict__ y,
                                     const uint8_t* __restrict__ mask, double* __restrict__ r) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    r[i] = (mask && mask[i]) ? 0.0 : (b ? b[i] - y[i] : y[i]);
}

ef_status ef_launch_residual_from(int64_t n, const double* b, const double* y, const uint8_t* mask, double* r,
                                  cudaStream_t s) {
    if (n == 0) return EF_OK;
    residual_from_kernel<<<nblk(n, 256), 256, 0, ef::counted(s)>>>(n, b, y, mask, r);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_norms(int64_t n, const double* R, const double* F, const double* D, double* part, int nPart,
                          double* out, cudaStream_t s) {
    norms_partial_kernel<<<nPart, 256, 0, ef::counted(s)>>>(n, R, F, D, part);
    norms_final_kernel<<<1, 32, 0, ef::counted(s)>>>(nPart, part, out);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_newton_check(int64_t n, const double* P, const double* PExt, const uint8_t* dir, const double* F,
                                 const double* D, double* R, double* part, int nPart, const double* q, double* out,
                                 cudaStream_t s) {
    newton_residual_kernel<<<nPart, 256, 0, ef::counted(s)>>>(n, P, PExt, dir, F, D, R, part);
    newton_decide_kernel<<<1, 32, 0, ef::counted(s)>>>(nPart, part, q, out);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_newton_first(int64_t n, const double* P, const double* PExt, int64_t nDir, const int64_t* dofs,
                                 const double* values, double* R, cudaStream_t s) {
    if (n > 0) newton_first_residual_kernel<<<nblk(n, 256), 256, 0, ef::counted(s)>>>(n, P, PExt, R);
    if (nDir > 0) scatter_values_kernel<<<nblk(nDir, 256), 256, 0, ef::counted(s)>>>(nDir, dofs, values, R);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

ef_status ef_launch_tie_fill(int64_t n, const int32_t* slave, const int32_t* ma, const int32_t* mb, double* x,
                             cudaStream_t s) {
    if (n == 0) return EF_OK;
    tie_fill_kernel<<<nblk(3 * n, 256), 256, 0, ef::counted(s)>>>(n, slave, ma, mb, x);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}

// element results (utils/elementresultcollector.pyx:38-120): one thread per requested
// (element, quadrature point) p = i * nQ + j, table[p * count + k] = state var first + k of point
// elements[i] * nQP + qps[j]; the SoA state makes the reads of a warp contiguous for consecutive
// points, the strided writes of a thread merge in L2
__global__ void results_gather_kernel(int64_t nPts, int nQ, int nQP, int64_t nq, int first, int count,
                                      const int32_t* __restrict__ elements, const int32_t* __restrict__ qps,
                                      const double* __restrict__ state, double* __restrict__ table) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nPts) return;
    const int64_t i = p / nQ;
    const int j = (int)(p - i * nQ);
    const double* src = state + (int64_t)first * nq + (int64_t)elements[i] * nQP + qps[j];
    double* out = table + p * count;
    for (int k = 0; k < count; ++k) out[k] = src[(int64_t)k * nq];
}

ef_status ef_launch_results_gather(int64_t nPts, int nQ, int nQP, int64_t nq, int first, int count,
                                   const int32_t* elements, const int32_t* qps, const double* state, double* table,
                                   cudaStream_t s) {
    if (nPts == 0) return EF_OK;
    results_gather_kernel<<<nblk(nPts, 256), 256, 0, ef::counted(s)>>>(nPts, nQ, nQP, nq, first, count, elements, qps,
                                                                        state, table);
    EF_CUDA(cudaGetLastError());
    return EF_OK;
}
