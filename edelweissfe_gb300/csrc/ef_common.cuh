// Shared definitions of the efgpu CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/efgpu.h"

#define EF_MAX_GROUPS 16

// Status flags written by device code (OR-ed into a per-context int).
#define EF_FLAG_RETURNMAP 1    // J2 Newton did not converge (reference: CutbackRequest(0.5))
#define EF_FLAG_NAN 2          // NaN in an element result
#define EF_FLAG_BARRIER 4      // a grid barrier gave up (bounded spin exhausted)
#define EF_FLAG_BADDET 8       // non-positive Jacobian determinant
#define EF_FLAG_TCWAIT 16      // a tensor-core tile of the network gave up waiting for its accumulator

namespace ef {

// Running count of the kernels this library has put on the GPU (host side): every launch site
// passes its stream through counted(); a CUDA-graph launch adds the kernels captured in it.
void note_launches(long long n);
long long launches();
inline cudaStream_t counted(cudaStream_t s) {
    note_launches(1);
    return s;
}

// Programmatic dependent launch of the kernels of the Krylov iteration and the multigrid cycle
// (chains of short dependent kernels).  A kernel launched by launch_dep() may be scheduled while
// the kernel before it in the stream is still running, so its launch latency and CTA
// rasterisation overlap the predecessor's tail.  Such a kernel starts with dep_entry(): it waits
// until the predecessor grid has completed and its writes are visible, before any load or
// store, and then lets its own successor be scheduled.  Launched without the attribute (EF_PDL=0
// or a predecessor that is not a kernel), both instructions return at once.
bool dep_launch_enabled();
__device__ __forceinline__ void dep_entry() {
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
}
template <typename... KArgs, typename... Args>
inline cudaError_t launch_dep(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = counted(s);
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = dep_launch_enabled() ? 1 : 0;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

enum MatKind { MAT_LINEAR_ELASTIC = 0, MAT_VON_MISES = 1, MAT_NEOHOOKE_WA = 2 };

// Constant tables of one element type (shape-function derivatives at the B/J
// evaluation points, body-force shape functions, weights, hex20 Jacobian quirk).
struct ElemTables {
    int nNodes, nQP, totalLagrange, quirk;
    float dNdS_f[27][3][20];
    double dNdS_d[27][3][20];
    double N[27][20];
    double w[27];
    double quirkFac[27];  // (zeta - xi) of the B/J point (C3D20 small strain only)
};

// A homogeneous element group (one element type, one material) on the device.
struct Group {
    int elType;   // index into the element table registry
    int nEl, nNodes, nQP, nDofEl, nPair;
    int mat;
    int tl;       // 1: total-Lagrange (hyperelastic) element family
    int nState;   // per Gauss point: 12 + material state (J2: kappa, NeoHookeWa: energy density)
    double props[8];
    int32_t* nodeDof;     // [nEl][nNodes]  first global DOF of each element node
    double* state[2];     // SoA [nState][nEl*nQP]; state[cur] committed, state[1-cur] trial
    int cur;
    int64_t peOffset;     // offset of this group's Pe block (doubles) in the context Pe buffer
    int64_t keOffset;     // offset of this group's Ke blocks (units of 3x3 blocks)
    int tablesSlot;       // index of the group's element table
    double* geo;          // geometry cache [nEl*nQP][3*nNodes + 1]: dN/dx and w*detJ (FP64)
    float2* geoS;         // the same values split into FP32 pairs (hi, lo = d - hi), small-strain groups
    int intConv;          // 1: the element kernel converts FP64 <-> FP32 pairs by integer operations
    const double* propsTable;  // optional per-element material rows [nRows][8] (null: props)
    const int32_t* elemRow;    // element -> row of propsTable
    float cutback;             // increment scale an element of this group asks for when its material fails
};

struct PropsArg {
    double v[8];
    float cutback;  // the group's increment scale on a material failure (atomic min into flags[1])
};

// flags[1] holds the smallest increment scale requested by a failing element (float bits; positive
// floats order like their bit patterns, so an integer atomicMin gives the minimum); this value
// means "no request"
#define EF_PNEWDT_NONE 1.0e30f

#ifdef __CUDACC__
// 16-byte asynchronous global -> shared copy (cp.async, cached in L2 only) and its group waits;
// both addresses 16-byte aligned
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}
#endif

// One phase of the multigrid cycle below a level, run by coarse_cycle_kernel (amg.cu) with a
// cluster barrier after each phase.  All coarse nodes carry 6 DOFs.
enum CoarseOpType {
    COP_BJ = 0,        // out = omega D^-1 in (masked -> 0)                 thread per row
    COP_SWEEP = 1,     // out = in + omega D^-1 (rhs - A in)                warp per row
    COP_RESID = 2,     // out = rhs - A in (masked -> 0)                    warp per row
    COP_RESTRICT = 3,  // out[I] = sum_{m in I} P_m^T in[m] (dead -> 0)     warp per aggregate
    COP_PROLONG = 4,   // out[m] += omega P_m in[agg(m)] (free DOFs)       thread per row
    COP_COARSEST = 5,  // out = inv in (dead -> 0)                          warp per DOF
};
struct CoarseOp {
    int type, n;
    const int32_t *p0, *p1;  // rowPtr, colIdx | aggPtr, aggIdx | agg
    const float *f0, *f1;    // vals, binv | offs | inv
    const uint8_t* mask;     // row mask / dead coarse DOFs
    const float* in;
    const float* rhs;
    float* out;
    float omega;
};

}  // namespace ef

#define EF_CUDA(call)                                                     \
    do {                                                                  \
        cudaError_t _e = (call);                                          \
        if (_e != cudaSuccess) {                                          \
            ef_set_error(std::string(#call) + ": " + cudaGetErrorString(_e)); \
            return EF_ERR_CUDA;                                           \
        }                                                                 \
    } while (0)

void ef_set_error(const std::string& s);

// Element kernels (elements.cu)
ef_status ef_launch_geometry(const ef::Group& g, const ef::ElemTables* T, const double* X, int* flags, cudaStream_t s);
ef_status ef_launch_small_strain(const ef::Group& g, const double* dU, void* Kout, int kDouble, int kLayoutVIJ,
                                 double* Pe, double* tang, int* flags, cudaStream_t s);
ef_status ef_launch_total_lagrange(const ef::Group& g, const double* U, void* Kout, int kDouble, int kLayoutVIJ,
                                   double* Pe, double* tang, int* flags, cudaStream_t s);
ef_status ef_launch_total_lagrange_apply(const ef::Group& g, const double* x, const double* tang, double* ye,
                                         cudaStream_t s);
int ef_tl_tangent_size();
ef_status ef_launch_small_strain_apply(const ef::Group& g, const double* x, const double* tang, double* ye,
                                       cudaStream_t s);
ef_status ef_launch_body_force(const ef::Group& g, const ef::ElemTables* T, const double load[3], double* Pe,
                               cudaStream_t s);

// Assembly launchers (assembly.cu)
ef_status ef_launch_condense(int64_t nNodes, const int32_t* nodeDof, const int64_t* ptr, const int64_t* src,
                             const float* w, const double* Pe, double* P, double* F, cudaStream_t s);
ef_status ef_launch_condense_add(int64_t nNodes, const int32_t* nodeDof, const int64_t* ptr, const int64_t* src,
                                 const float* w, const double* Pe, int64_t lo, int64_t hi, double* V, cudaStream_t s);
ef_status ef_launch_vij_export(int nEl, int nn, int np, const void* Kblk, int kDouble, double* Kvij, cudaStream_t s);
ef_status ef_launch_results_gather(int64_t nPts, int nQ, int nQP, int64_t nq, int first, int count,
                                   const int32_t* elements, const int32_t* qps, const double* state, double* table,
                                   cudaStream_t s);
ef_status ef_launch_csr_scatter(int64_t nnz, const int64_t* seg, const int32_t* perm, const double* V, double* data,
                                cudaStream_t s);
ef_status ef_launch_csr_dirichlet_rows(int64_t nRows, const int64_t* rows, const int32_t* indptr,
                                       const int32_t* indices, double* data, cudaStream_t s);
ef_status ef_launch_tie_fill(int64_t n, const int32_t* slave, const int32_t* ma, const int32_t* mb, double* x,
                             cudaStream_t s);
ef_status ef_launch_bsr_scatter(int64_t nBlocks, const int64_t* seg, const int64_t* src, const float* w,
                                const void* Kblk, int kDouble, void* vals, cudaStream_t s);
ef_status ef_launch_bj_setup(int64_t nNodes, const int64_t* diagPos, const int32_t* nodeDof, const uint8_t* mask,
                             const void* vals, int kDouble, void* inv, int* flags, cudaStream_t s);
ef_status ef_launch_residual_from(int64_t n, const double* b, const double* y, const uint8_t* mask, double* r,
                                  cudaStream_t s);
ef_status ef_launch_norms(int64_t n, const double* R, const double* F, const double* D, double* part, int nPart,
                          double* out, cudaStream_t s);
