// Internal declarations shared by the host-side translation units of the library: the context
// (struct ef_ctx) with its multigrid levels and result collectors, the kernel launchers of the
// device translation units, error and allocation helpers, and the functions one host unit calls
// in another.  Not part of the C ABI (that is include/efgpu.h).
#pragma once

#include <math.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <numeric>
#include <random>
#include <string>
#include <thread>
#include <vector>

#include "ef_common.cuh"

// krylov.cu
int ef_krylov_block_threads();
size_t ef_barrier_state_bytes();
size_t ef_pcg_result_bytes();
ef_status ef_launch_bsr_residual(int nNodes, const int32_t* rowPtr, const int32_t* colIdx, const void* vals,
                                 int mDouble, const double* x, const double* b, const uint8_t* mask, double* y,
                                 int nSM, cudaStream_t s);
ef_status ef_pcg_grid(int vDouble, int nSM, int* gridOut);
ef_status ef_launch_pcg(int vDouble, int grid, int nNodes, const int32_t* rowPtr, const int32_t* colIdx,
                        const void* vals, const void* binv, const uint8_t* mask, const void* b, void* x, void* r,
                        void* z, void* pA, void* pB, void* q, double* partA, double* partB, void* bar, void* res,
                        int maxIter, double rtol2, int* flags, cudaStream_t s);
ef_status ef_launch_dot(int64_t n, const double* a, const double* b, double* part, int nPart, double* out,
                        cudaStream_t s);
ef_status ef_launch_masked_copy(int64_t n, const double* src, const uint8_t* mask, int keepMasked, double scale,
                                void* dst, int dstDouble, cudaStream_t s);
ef_status ef_launch_axpy(int64_t n, double a, const void* xs, int xDouble, double* y, cudaStream_t s);
ef_status ef_launch_add(int64_t n, const double* a, const double* b, double* y, cudaStream_t s);

// amg.cu
int ef_amg_coarse_dofs();
int ef_max_coarsest_nodes();
ef_status ef_launch_galerkin(int bf, int64_t nCoarseBlocks, const int64_t* seg, const int32_t* src,
                             const int32_t* fineRowOfBlock, const int32_t* fineCol, const float* fineVals,
                             const uint8_t* fineMask, const float* offs, const int32_t* coarseRowOfBlock,
                             const int32_t* coarseCol, const uint8_t* coarseDead, float* coarseVals, cudaStream_t s);
ef_status ef_launch_bj6_setup(int nN, const int64_t* diagPos, const float* vals, float* inv, cudaStream_t s);
ef_status ef_launch_bj_apply(int bs, int nN, const float* binv, const uint8_t* mask, float omega, const float* r,
                             float* x, int accumulate, cudaStream_t s);
// binv null: t = r - ys A x (ys != 1 on 6-DOF levels only); else one sweep t = x + omega D^-1 (r - A x)
ef_status ef_launch_level_residual(int bs, int nN, const int32_t* rowPtr, const int32_t* colIdx, const float* vals,
                                   const float* x, const float* r, const uint8_t* mask, float* t, cudaStream_t s,
                                   const float* binv = nullptr, float omega = 0.f, const void* valsH = nullptr,
                                   float ys = 1.f);
// out = A (M D^-1) blockwise on a 6-DOF level (M: dead DOFs of the column node zeroed)
ef_status ef_launch_scale_blocks6(int64_t nB, const int32_t* colIdx, const float* vals, const float* binv,
                                  const uint8_t* dead, float* out, cudaStream_t s);
ef_status ef_launch_to_bf16(int64_t n, const float* src, void* dst, cudaStream_t s);
ef_status ef_launch_sa_damping(const double* n2, float* wP, cudaStream_t s);
ef_status ef_launch_sa_setup(int bf, int64_t nP, const int32_t* pRow, const int32_t* pCol, const int64_t* pSeg,
                             const int32_t* pSrc, int64_t nAP, const int32_t* apRow, const int64_t* apSeg,
                             const int32_t* apK, const int32_t* apP, const int32_t* fineCol, const float* fineVals,
                             const uint8_t* fineMask, const float* offs, const int32_t* agg, const float* binv,
                             const float* wP, float* Pv, float* APv, int64_t nC, const int64_t* cSeg,
                             const int32_t* cP, const int32_t* cAP, const int32_t* coarseRowOfBlock,
                             const int32_t* coarseCol, const uint8_t* coarseDead, float* coarseVals, int nF,
                             const int32_t* apRowPtr, int apCap, cudaStream_t s);
// AP by groups of ef_sa_ap_rows() finer rows (apRowPtr non-null in ef_launch_sa_setup) needs
// ef_sa_ap_rows_smem(bf, apCap) bytes of shared memory, apCap >= the pairs of every group
size_t ef_sa_ap_rows_smem(int bf, int cap);
int ef_sa_ap_rows();
ef_status ef_launch_sa_restrict(int bf, int nC, const int32_t* tPtr, const int32_t* tIdx, const int32_t* pRow,
                                const float* Pv, const float* t, const uint8_t* coarseDead, float* rc,
                                cudaStream_t s);
ef_status ef_launch_sa_restrict2(int bf, int nC, int64_t nP, const int32_t* tPtr, const int32_t* tIdx,
                                 const int32_t* pRow, const float* Pv, const float* t, const uint8_t* coarseDead,
                                 float* c, float* rc, cudaStream_t s);
ef_status ef_launch_sa_prolong2(int bf, int nF, int64_t nP, const int32_t* pRowPtr, const int32_t* pCol,
                                const float* Pv, const float* xc, const uint8_t* mask, float* c, float* x, float alpha,
                                cudaStream_t s);
// one-pass transfers: the restriction from a transpose-order copy of P, the prolongation from P
// in groups of ef_sa_prolong_onepass_rows() consecutive finer rows with
// ef_sa_prolong_onepass_smem(bf, cap) bytes of shared memory, cap >= the P blocks of every group
ef_status ef_launch_sa_block_copy(int bf, int64_t nP, const int32_t* tIdx, const float* Pv, float* dst,
                                  cudaStream_t s);
// the fine level's transpose-order copy of P in BF16 (three word arrays) and its restriction
ef_status ef_launch_sa_block_copy_h(int64_t nP, const int32_t* tIdx, const float* Pv, void* q0, void* q1, void* q2,
                                    cudaStream_t s);
ef_status ef_launch_sa_restrict_onepass_h(int nC, const int32_t* tPtr, const int32_t* rowT, const void* q0,
                                          const void* q1, const void* q2, const float* t, const uint8_t* coarseDead,
                                          float* rc, cudaStream_t s);
size_t ef_sa_prolong_onepass_smem(int bf, int cap);
int ef_sa_prolong_onepass_rows();
ef_status ef_launch_sa_restrict_onepass(int bf, int nC, const int32_t* tPtr, const int32_t* rowT, const float* PT,
                                        const float* t, const uint8_t* coarseDead, float* rc, cudaStream_t s);
ef_status ef_launch_sa_prolong_onepass(int bf, int nF, int cap, const int32_t* pRowPtr, const int32_t* pCol,
                                       const float* Pv, const float* xc, const uint8_t* mask, float* x, float alpha,
                                       cudaStream_t s);
ef_status ef_launch_sa_prolong(int bf, int nF, const int32_t* pRowPtr, const int32_t* pCol, const float* Pv,
                               const float* xc, const uint8_t* mask, float* x, float alpha, cudaStream_t s);
ef_status ef_launch_restrict(int bf, int nC, const int32_t* aggPtr, const int32_t* aggIdx, const float* offs,
                             const float* t, const uint8_t* coarseDead, float* rc, cudaStream_t s);
ef_status ef_launch_prolong(int bf, int nN, const int32_t* agg, const float* offs, const float* xc,
                            const uint8_t* mask, float* x, cudaStream_t s, float alpha);
ef_status ef_launch_coarsest_inverse(int nN, const int32_t* rowPtr, const int32_t* colIdx, const float* vals,
                                     float* inv, cudaStream_t s);
ef_status ef_launch_fill_hash(int64_t n, float* x, cudaStream_t s);
ef_status ef_launch_scale_rnorm(int64_t n, float* x, const double* n2, cudaStream_t s);
ef_status ef_launch_scale_by(int64_t n, float* x, const float* fac, cudaStream_t s);
ef_status ef_launch_cheb_step(int bs, int nN, const float* binv, const uint8_t* mask, float a, float b, const float* t,
                              float* d, float* x, int first, cudaStream_t s);
ef_status ef_launch_level_residual_bf16(int nN, int64_t nBlocks, const int32_t* rowPtr, const int32_t* colIdx,
                                        const void* vals, const float* x, const float* r, const uint8_t* mask,
                                        float* t, cudaStream_t s, const float* binv = nullptr, float omega = 0.f);
ef_status ef_launch_to_bf16_split(int64_t nBlocks, const float* src, void* dst, cudaStream_t s);
int ef_stage_cap(int nN, const int32_t* rowPtrHost);
ef_status ef_launch_level_residual_bf16_staged(int nSM, int cap, int nN, int64_t nBlocks, const int32_t* rowPtr,
                                               const int32_t* colIdx, const void* vals, const float* x, const float* r,
                                               const uint8_t* mask, float* t, cudaStream_t s, const float* binv,
                                               float omega);
ef_status ef_launch_coarse_cycle(const ef::CoarseOp* ops, int nOps, cudaStream_t s);
ef_status ef_launch_coarsest_apply(int n, const float* inv, const float* r, const uint8_t* dead, float* x,
                                   cudaStream_t s);
// mpnn.cu
int ef_mpnn_nparam();
int ef_mpnn_hidden();
int ef_mpnn_layer_offset(int l);
int ef_mpnn_out_offset();
ef_status ef_mpnn_setup_kernels();
ef_status ef_launch_edge_weights(int nN, const int32_t* rowPtr, const int32_t* colIdx, const float* vals, float* a,
                                 cudaStream_t s);
ef_status ef_launch_gather_f32(int64_t n, const int64_t* idx, const float* src, float* dst, cudaStream_t s);
ef_status ef_mpnn_forward(int nN, const int32_t* rowPtr, const int32_t* colIdx, const float* a, const float* P,
                          const float* f, const float* base, const uint8_t* mask, float so, float* acts, float* z,
                          int tc, int* flags, cudaStream_t s);
ef_status ef_mpnn_backward(int nN, const int32_t* rowPtr, const int32_t* colIdx, const float* aT, const float* P,
                           const float* f, const float* acts, const float* z, const float* e, const uint8_t* mask,
                           float scale, float so, float* grad, float* work, float* part, int nPart, cudaStream_t s);
ef_status ef_mpnn_adam(int n, float* p, const float* g, float* m1, float* m2, float lr, float b1, float b2, float eps,
                       int step, void* pb, float* pf, cudaStream_t s);
ef_status ef_launch_features(int nN, const float* Mv, const float* v, const float* binv, float s0, float s1, float s2,
                             float* f, cudaStream_t s);
ef_status ef_mpnn_bf16_to_f32(int n, const void* pb, float* pf, cudaStream_t s);
ef_status ef_mpnn_refresh(int n, const float* p, void* pb, float* pf, cudaStream_t s);
ef_status ef_mpnn_sumsq(int64_t n, int groups, const float* z, const float* e, const uint8_t* mask, double* part,
                        int nPart, double* out, cudaStream_t s, float* fac = nullptr);
ef_status ef_mpnn_scale(int64_t n, float* x, float a, cudaStream_t s);
ef_status ef_mpnn_dense_eval_host(int tc, int nN, const float* h, const float* agg, const float* W, float* q,
                                  float* hout, int* flagsOut, cudaStream_t s);
ef_status ef_mpnn_scale_features(int nN, const float* f, float s0, float s1, float s2, float* fs, cudaStream_t s);
ef_status ef_mpnn_alpha_combine(int64_t n, const float* Mv, const float* N, const double* dots, const uint8_t* mask,
                                float* z, cudaStream_t s);
// batch.cu
int ef_batch_num_tiles();
void ef_batch_tile_shape(int tile, int* tpb, int* lpr);
ef_status ef_launch_batched_pcg(int tile, int nSM, int nProb, const int32_t* nodePtr, const int32_t* order,
                                const int32_t* rowPtr, const int32_t* colIdx, const double* vals, const double* binv,
                                const uint8_t* mask, const double* b, double* x, double* r, double* z, double* p,
                                double* q, int maxIter, double rtol2, int* iters, double* rel, cudaStream_t s);
ef_status ef_launch_batch_norms(int nProb, const int32_t* nodePtr, const double* R, const double* F, const double* D,
                                double* out, cudaStream_t s);
// fgmres.cu
int ef_fgmres_max_basis();
ef_status ef_launch_spmv_f32(int nN, const int32_t* rowPtr, const int32_t* colIdx, const float* vals, const float* x,
                             const uint8_t* mask, float* y, cudaStream_t s);
ef_status ef_launch_spmv_f32_copy(int nN, const int32_t* rowPtr, const int32_t* colIdx, const float* vals,
                                  const float* x, const uint8_t* mask, float* y, float* xcopy, cudaStream_t s);
ef_status ef_launch_cgs_column(int64_t n, int nv, float* V, int64_t ldv, double* part, double* partN, int nPart,
                               double* hG, double* hTmp, double* hAcc, double eta2, float* w2, double* hostOut,
                               int slotNorm, cudaStream_t s);
ef_status ef_launch_normalize_first(int64_t n, float* w, double* part, int nPart, float* w2, double* hostOut,
                                    int slotNorm, cudaStream_t s, float* scOut = nullptr);
ef_status ef_launch_gs_column(int64_t n, int nv, float* V, int64_t ldv, float* part, double* partN, int nPart,
                              float* sc, unsigned* ticket, float* w2, double* hostOut, int slotNorm, cudaStream_t s);
int ef_sp_stage_cap(int nN, const int32_t* rowPtrHost);
ef_status ef_launch_spmv_f32_staged(int nSM, int cap, int nN, const int32_t* rowPtr, const int32_t* colIdx,
                                    const float* vals, const float* x, const uint8_t* mask, float* y, float* xcopy,
                                    cudaStream_t s);
ef_status ef_launch_combine(int64_t n, int nv, const float* Z, int64_t ldz, const double* y, float* x, cudaStream_t s);
ef_status ef_launch_sub(int64_t n, const float* b, const float* y, float* r, cudaStream_t s);
ef_status ef_launch_newton_check(int64_t n, const double* P, const double* PExt, const uint8_t* dir, const double* F,
                                 const double* D, double* R, double* part, int nPart, const double* q, double* out,
                                 cudaStream_t s);
ef_status ef_launch_newton_first(int64_t n, const double* P, const double* PExt, int64_t nDir, const int64_t* dofs,
                                 const double* values, double* R, cudaStream_t s);
ef_status ef_launch_sell_refresh(int64_t nE, const int32_t* src, const float* bsr, float* v9, void* v8, void* v1,
                                 const int32_t* col, const float* binv, const uint8_t* mask, cudaStream_t s);
ef_status ef_launch_sell_spmv3(int nN, int nSlices, const int64_t* off, const int32_t* perm, const int32_t* col,
                               const float* v9, const float* x, const uint8_t* mask, float* y, float* xcopy, int split,
                               cudaStream_t s, const float* scale = nullptr, const int32_t* dia = nullptr,
                               const float* binv = nullptr);
ef_status ef_launch_sell_level3_bf16(int nN, int nSlices, const int64_t* off, const int32_t* perm, const int32_t* col,
                                     const void* v8, const void* v1, const float* x, const float* r,
                                     const uint8_t* mask, float* t, const float* binv, float omega, int split,
                                     cudaStream_t s, float ys = 1.f, const int32_t* dia = nullptr);

// the same on a 6-DOF level (amg.cu): C FP32 in the pattern of A P, a warp per row
ef_status ef_launch_sa_post6_setup(int64_t nAP, const int32_t* apRow, const int32_t* apToP, const float* Pv,
                                   const float* APv, const float* binv, float omega, float alpha, float* C,
                                   cudaStream_t s);
ef_status ef_launch_sa_post6_fused(int nN, const int32_t* rowPtr, const int32_t* col, const float* C, const float* e,
                                   const float* r, const float* t, const float* binv, const uint8_t* dead,
                                   float omega, float* x, cudaStream_t s);
// fused fine-level post-smoothing x = w D^-1 (r + t) + C e with C = a (I - w D^-1 A) P (sell.cu):
// C blocks per slot from the AP / P blocks, then the product
ef_status ef_launch_sa_post_setup(int64_t nSlot, const int32_t* src, const int32_t* apRow, const int32_t* apToP,
                                  const float* Pv, const float* APv, const float* binv, float omega, float alpha,
                                  void* q0, void* q1, void* q2, cudaStream_t s);
ef_status ef_launch_sa_post_fused(int nN, int nSlices, const int64_t* off, const int32_t* perm, const int32_t* col,
                                  const void* q0, const void* q1, const void* q2, const float* e, const float* r,
                                  const float* t, const float* binv, const uint8_t* mask, float omega, float* x,
                                  int split, cudaStream_t s);

using namespace ef;

// error message of the calling thread (ef_last_error)
void ef_set_error(const std::string& s);
// launches issued during a stream capture are credited to the graph captured on this thread
extern thread_local long long* t_captureCount;

#define EF_CHECK(call)                   \
    do {                                 \
        ef_status _s = (call);           \
        if (_s != EF_OK) return _s;      \
    } while (0)

#define EF_REQUIRE_FINALIZED(c)                                  \
    do {                                                         \
        if (!(c) || !(c)->finalized) {                           \
            ef_set_error("context missing or not finalized");    \
            return EF_ERR_STATE;                                 \
        }                                                        \
    } while (0)

namespace efh {

struct PcgResultHost {
    int iterations;
    int status;
    double rr;
    double bb;
};

struct HostGroup {
    std::string elType;
    int mat;
    std::vector<double> props;
    int nEl, nNodes, nQP, tl;
    std::vector<int32_t> nodeDof;  // [nEl][nNodes]
    std::vector<double> propsTable;  // optional per-element material rows [nRows][8]
    std::vector<int32_t> elemRow;    // element -> row
    double cutback = 0.5;            // increment scale requested on a material failure (vonmises.py:231)
};

template <typename T>
inline T* dalloc(size_t n, ef_status* st) {
    T* p = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc(&p, n * sizeof(T));
    if (e != cudaSuccess) {
        ef_set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
        *st = EF_ERR_CUDA;
        return nullptr;
    }
    return p;
}

// run f(lo, hi) over [0, n) on the host cores
template <typename F>
inline void parallel_for(int64_t n, F f) {
    unsigned nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    if (n < 100000) nt = 1;
    std::vector<std::thread> th;
    const int64_t chunk = (n + nt - 1) / nt;
    for (unsigned t = 0; t < nt; ++t) {
        const int64_t lo = t * chunk, hi = std::min<int64_t>(n, lo + chunk);
        if (lo >= hi) break;
        th.emplace_back([=]() { f(lo, hi); });
    }
    for (auto& x : th) x.join();
}


template <typename T>
inline ef_status upload(T** dst, const std::vector<T>& v) {
    ef_status st = EF_OK;
    *dst = dalloc<T>(std::max<size_t>(1, v.size()), &st);
    if (!*dst) return st;
    if (!v.empty()) EF_CUDA(cudaMemcpy(*dst, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
    return EF_OK;
}

}  // namespace efh

using namespace efh;

// one coarse level of the aggregation multigrid (level 0 is the context's own BSR system)
struct AmgLevel {
    int nN = 0;
    int64_t nBlocks = 0;
    int32_t *rowPtr = nullptr, *colIdx = nullptr, *rowOfBlock = nullptr;
    int64_t* diagPos = nullptr;
    float *vals = nullptr, *binv = nullptr;
    uint8_t* dead = nullptr;                // coarse DOFs without a free fine DOF
    int32_t *agg = nullptr;                 // finer node -> this level's node
    float* offs = nullptr;                  // finer node position relative to its aggregate centroid [nFiner][3]
    std::vector<float> hOffs;
    std::vector<double> hCentroid;          // [nN][3]
    int32_t *aggPtr = nullptr, *aggIdx = nullptr;  // members of each node of this level
    int64_t* gseg = nullptr;                // Galerkin map: blocks of the finer level per block here
    int32_t* gsrc = nullptr;
    float *x = nullptr, *r = nullptr, *t = nullptr;  // V-cycle work vectors of this level
    float* x2 = nullptr;                             // second smoothing iterate (sweeps alternate)
    uint16_t* valsH = nullptr;                       // BF16 copy of vals for the smoothing residuals
    float* valsB = nullptr;  // A (M D^-1) blockwise, for the fused cycle's residual without a pre-sweep launch
    // smoothed aggregation (transition from the finer level to this one): index maps and values
    int64_t saNP = 0, saNAP = 0;
    int32_t *saPRowPtr = nullptr, *saPCol = nullptr, *saPRow = nullptr, *saPSrc = nullptr;
    int32_t *saTPtr = nullptr, *saTIdx = nullptr, *saApRow = nullptr, *saApK = nullptr, *saApP = nullptr;
    int32_t *saCP = nullptr, *saCAP = nullptr;
    int64_t *saPSeg = nullptr, *saApSeg = nullptr, *saCSeg = nullptr;
    float *saPv = nullptr, *saAPv = nullptr, *saW = nullptr;
    float* saC = nullptr;  // [saNP][6] block products of the two-stage restriction / prolongation
    // one-pass transfers: transpose-order copy of P with the block row of each slot; saCap bounds
    // the blocks of a prolongation group of finer rows
    float* saPT = nullptr;
    void *saPTh0 = nullptr, *saPTh1 = nullptr, *saPTh2 = nullptr;  // BF16 form (fine level, EF_SA_PT_BF16)
    int32_t* saRowT = nullptr;
    int saCap = 0;
    // fused post-smoothing of the finer level when it has 6 DOFs: C = a (I - w D^-1 A) P in the
    // pattern of A P (rows, columns, C values, the P block of each AP block)
    int32_t *postRowPtr = nullptr, *postCol = nullptr, *postApToP = nullptr;
    float* postC = nullptr;
    int32_t* saApRowPtr = nullptr;  // AP row pointer, for the AP product by groups of rows (null: a thread
    int saApCap = 0;                // per AP block); saApCap bounds the pairs of a group
    bool saOnePass = false;  // this level's transfers run in one pass
    std::vector<int32_t> hRowPtr, hColIdx, hAgg, hAggPtr, hAggIdx;
    std::vector<uint8_t> hDead;

    // device arrays of the level (null ones are skipped)
    void free_device() {
        for (void* p : {(void*)rowPtr, (void*)colIdx, (void*)rowOfBlock, (void*)diagPos, (void*)vals, (void*)binv,
                        (void*)dead, (void*)agg, (void*)offs, (void*)aggPtr, (void*)aggIdx, (void*)gseg, (void*)gsrc,
                        (void*)x, (void*)x2, (void*)valsH, (void*)r, (void*)t, (void*)saPRowPtr, (void*)saPCol,
                        (void*)saPRow, (void*)saPSrc, (void*)saTPtr, (void*)saTIdx, (void*)saApRow, (void*)saApK,
                        (void*)saApP, (void*)saCP, (void*)saCAP, (void*)saPSeg, (void*)saApSeg, (void*)saCSeg,
                        (void*)saPv, (void*)saAPv, (void*)saW, (void*)saC, (void*)saPT,
                        (void*)saRowT, (void*)saPTh0, (void*)saPTh1, (void*)saPTh2, (void*)saApRowPtr, (void*)postRowPtr, (void*)postCol, (void*)valsB,
                        (void*)postApToP, (void*)postC})
            if (p) cudaFree(p);
    }
};

// element result collector: device lists of elements and quadrature points of one group, the
// state slice [first, first + count) and the gathered table [nEls][nQ][count]
struct ResultCollector {
    int group = -1;  // -1: free slot
    int nEls = 0, nQ = 0, first = 0, count = 0;
    int32_t* dEl = nullptr;
    int32_t* dQp = nullptr;
    double* dTable = nullptr;
};

struct ef_ctx {
    int64_t nDof = 0, nNodes = 0, nElements = 0;
    std::vector<double> hX;
    double* dX = nullptr;
    std::vector<HostGroup> hg;
    std::vector<Group> groups;
    std::vector<ElemTables*> dTables;
    std::vector<ResultCollector> results;
    bool finalized = false;
    int keFp64 = 0;
    int nSM = 0;
    // element outputs
    double* Pe = nullptr;
    int64_t nPe = 0;
    void* Kblk = nullptr;
    int64_t nKblk = 0;
    int* dFlags = nullptr;
    // node ties u_s = (u_a + u_b) / 2 (eliminated: K^ = T^T K T, P^ = T^T P, x_s filled after solves)
    std::vector<int32_t> hTieS, hTieA, hTieB;
    int32_t *dTieS = nullptr, *dTieA = nullptr, *dTieB = nullptr;
    float *dCondW = nullptr, *dBsrW = nullptr;  // tie weights of the condensation / BSR sources (null: 1)
    double* dTieTmp = nullptr;
    // condensation map
    int32_t* dNodeDof = nullptr;
    int64_t* dCondPtr = nullptr;
    int64_t* dCondSrc = nullptr;
    // BSR system
    int64_t nBlocks = 0;
    int32_t* dRowPtr = nullptr;
    int32_t* dColIdx = nullptr;
    int64_t* dBsrSeg = nullptr;
    int64_t* dBsrSrc = nullptr;
    int64_t* dDiagPos = nullptr;
    void* dBsrVals = nullptr;
    void* dBinv = nullptr;
    uint8_t* dMask = nullptr;
    bool anyDirichlet = false;
    // the Dirichlet DOFs of ef_set_dirichlet (without tied DOFs) for the residual of the Newton check
    int64_t nDir = 0;
    int64_t* dDirIdx = nullptr;
    uint8_t* dDirMask = nullptr;
    double* dNewton = nullptr;  // [16]: decision inputs (9) and outputs (5) of ef_newton_residual
    // scalar CSR (reference layout)
    bool scalar = false;
    int64_t nVIJ = 0, nnz = 0;
    std::vector<int32_t> hIndptr, hIndices;
    int32_t* dIndptr = nullptr;
    int32_t* dIndices = nullptr;
    int64_t* dCsrSeg = nullptr;
    int32_t* dCsrPerm = nullptr;
    double* dKvijTmp = nullptr;
    // reductions / Krylov workspace
    double* dPart = nullptr;
    int nPart = 0;
    double* dRed = nullptr;  // small result buffer
    int pcgGrid[2] = {0, 0};
    double *dPartA = nullptr, *dPartB = nullptr;
    void* dBar = nullptr;
    void* dPcgRes = nullptr;
    void* w32[7] = {};  // FP32 Krylov vectors: b, x, r, z, p (two buffers), q
    double* w64[5] = {};  // FP64: xd, xf, r64, tmp, y
    // exact refinement: FP64 Gauss-point tangents per group and an element-vector buffer
    std::vector<double*> dTang;
    double* dYe = nullptr;
    bool exact = false;
    void* w64k[7] = {};   // FP64 Krylov vectors for the all-FP64 mode
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaEvent_t evS[2] = {nullptr, nullptr};  // FGMRES SpMV timing
    // aggregation multigrid for the FGMRES preconditioner
    std::vector<AmgLevel> amg;           // levels 1..L-1
    float* amgCoarsestInv = nullptr;
    int32_t* dRowOfBlock0 = nullptr;     // fine-level block -> block row
    float *fineX = nullptr, *fineT = nullptr;  // level-0 V-cycle work vectors
    bool amgStale = true;                // coarse values need a refresh (new system or mask)
    bool amgMaskChanged = true;          // the Dirichlet mask changed since the coarse levels were built
    int amgMaxReuse = 0;                 // new systems that may reuse the coarse levels (ef_fgmres_set_reuse)
    int amgReuseLeft = 0;                // reuses left before the next rebuild
    bool amgPowerDue = true;             // the next build re-estimates the damping (power iterations)
    bool nnEdgeStale = true;             // the learned correction's edge weights need a refresh
    std::vector<uint8_t> hMask;
    std::vector<int32_t> hRowPtr0, hColIdx0;  // host copy of the fine block pattern
    // sliced-ELL copy of the fine system (sell.cu): FGMRES product and fine smoothing
    int sellMode = -1;                     // -1 not decided, 0 off (EF_SELL=0 or too much padding), 1 on
    bool sellStale = true;                 // values need a refresh from the assembled blocks
    int sellSlices = 0;
    int64_t sellE = 0;                     // slots (32 x the sum of the slice widths)
    int64_t* dSellOff = nullptr;           // [sellSlices + 1] first slot of each slice
    // fused fine-level post-smoothing (EF_AMG_FUSED_POST): sliced layout of C over the fine rows
    bool postFused = true;
    bool sellScaled = false;  // the BF16 fine copy holds K (M D^-1) (fused cycle: no pre-sweep launch)
    int postSlices = 0;
    int64_t postSlots = 0;
    int64_t* dPostOff = nullptr;
    int32_t* dPostPerm = nullptr;  // fine row of each slot row (rows sorted by length within windows)
    int32_t *dPostCol = nullptr, *dPostSrc = nullptr, *dPostApToP = nullptr;
    void *dPostQ0 = nullptr, *dPostQ1 = nullptr, *dPostQ2 = nullptr;
    int sellSplit = 4;                     // warps per slice of the BF16 sweep: 1, 2, 4 or 8 (EF_SELL_SPLIT)
    int sellSplitProduct = 4;              // the same for the FP32 product (EF_SELL_SPLIT_PRODUCT)
    int32_t* dSellPerm = nullptr;          // [nNodes] block row of each SELL row (null: identity)
    int32_t* dSellCol = nullptr;           // [sellE] block column (padding: the row itself)
    // diagonal form (EF_SELL_DIA): every slice has the same slot columns, slot column j at node
    // offset dSellDia[j] from the row (no column array read by the fine kernels); null: off
    int32_t* dSellDia = nullptr;
    int sellDiaN = 0;
    int32_t* dSellSrc = nullptr;           // [sellE] source block in the BSR values (-1: padding)
    float* dSellV9 = nullptr;              // FP32 values, nine planes per slot column
    void* dSellV8 = nullptr;               // BF16 values 0..7 per slot (16-byte words)
    void* dSellV1 = nullptr;               // BF16 value 8 per slot
    // V-cycle parameters: damping, smoothing sweeps per side, coarse over-correction, cycle type
    float amgOmega = 1.0f;                  // upper bound of the smoothing damping
    std::vector<float> levelOmega;          // per smoothed level: amgOmega, or 4 / (3 lambda_max(D^-1 A)) when smaller
    float* amgPow[2] = {nullptr, nullptr};  // power-iteration vectors (fine size)
    float* amgPowFac = nullptr;             // 1 / |a| of the power iteration (FP32, on the device)
    float* amgZero = nullptr;
    bool amgBf16 = true;                    // fine-level smoothing residuals from a BF16 copy of the blocks
    bool amgCheb = false;                   // Chebyshev smoothing (degree amgSweeps) instead of damped block Jacobi
    bool amgBf16Coarse = false;             // coarse smoothing residuals from BF16 copies (EF_AMG_BF16_COARSE)
    double refineAim = 0.5;  // an inner solve aims at this fraction of the remaining target (EF_REFINE_AIM)
    // the tightest relative tolerance of an inner solve after the first (EF_REFINE_FLOOR; 0: none):
    // an FP32 solve lowers the FP64 residual of its right-hand side by about 3e-3 at best (the
    // rounding of the FP32 products), so iterating it further buys nothing
    double refineFloor = 1e-2;
    double fgHold = 2.0;     // FGMRES: no column enqueued ahead when the trend reaches hold x target (EF_FGMRES_HOLD)
    bool amgDeadValid = false;  // the levels' dead-DOF masks match the current Dirichlet mask
    bool amgSmoothed = true;                // smoothed-aggregation prolongators (EF_AMG_SMOOTHED=0: plain aggregation)
    int saTransfer = 2;                     // SA transfers: 0 a thread per coarse node / finer row, 1 block
                                            // products + sums, 2 one pass, a thread per block (EF_SA_TRANSFER)
    bool amgCluster = false;                // levels below clusterLevel as one cluster launch (EF_AMG_CLUSTER=1)
    int stageCap = 0;                       // > 0: fine BF16 smoothing through shared-memory staging (EF_AMG_STAGED=1)
    int clusterLevel = -1;                  // level whose coarse correction runs in coarse_cycle_kernel
    ef::CoarseOp* dCoarseOps = nullptr;     // its phase program (device)
    int nCoarseOps = 0, nCoarseOpsCap = 0;
    float* clusterCur = nullptr;            // level clusterLevel's iterate that the program updates
    double* amgNorms = nullptr;             // power-iteration norms of the damping estimate
    int amgNormsCap = 0;
    std::vector<float> levelLam;            // per smoothed level: estimated lambda_max(D^-1 A), quantised
    std::vector<float*> chebD;              // per smoothed level: Chebyshev direction vector
    void* dBsrValsH = nullptr;
    int amgSweeps = 2;
    float amgAlpha = 1.5f;
    int amgCycle = 2;  // 1: V-cycle, 2: W-cycle below the finest level
    int amgPre = 2, amgPost = 2;  // block-Jacobi sweeps before / after the coarse correction
    int amgPreC = 2, amgPostC = 2;  // the same on the coarse levels
    int amgWLevels = 1;           // coarse levels 1..amgWLevels repeat their coarse correction
    // the whole preconditioner application captured once as a CUDA graph (fixed in/out buffers)
    float *vcIn = nullptr, *vcOut = nullptr;
    cudaStream_t capStream = nullptr;
    cudaGraphExec_t vcGraph = nullptr;
    // captured element pass (several groups): the vectors it was captured for and its kernels
    bool elemGraphs = true;
    const void* egKey[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaGraphExec_t egExec = nullptr;
    long long egKernels = 0;
    long long vcGraphKernels = 0, nnGraphKernels = 0;
    // learned correction (message-passing network) on top of the V-cycle
    struct NNSystem {                       // a system the training pairs were taken from
        float *K = nullptr, *a = nullptr;   // BSR values, edge weights
        int64_t version = -1;
    };
    struct NNSample {
        float *f = nullptr, *base = nullptr, *r = nullptr, *e = nullptr;  // raw features [nN][9], Mv, input, target
        bool hasE = false;                                                // (scaled to rms(e) = 1, else rms(r) = 1)
        int sys = -1;                                                     // -1: empty slot
        double ee = 0.0, er = 0.0, rr = 0.0;                              // e.e, e.r, r.r
    };
    bool nnInit = false, nnOn = false;
    int nnTensorCores = 1;                  // dense layers on tcgen05 (0: FP32 CUDA cores)
    float *nnP = nullptr, *nnPf = nullptr, *nnM1 = nullptr, *nnM2 = nullptr, *nnG = nullptr;  // FP32 masters, BF16 view,
    void* nnPb = nullptr;                                                                   // Adam moments, gradient;
    float *nnActs = nullptr, *nnF = nullptr, *nnWork = nullptr, *nnPart = nullptr;          // BF16 inference copy
    float *nnA = nullptr, *nnAT = nullptr;  // edge weights of the current system and their transpose
    int64_t* nnTpos = nullptr;              // block (m, n) -> position of block (n, m)
    double* nnRed = nullptr;                // FP64 reduction partials (3 per CTA) and results
    int nnPartN = 0;
    float nnS[3] = {1.f, 1.f, 1.f};         // feature group scales
    float nnSo = 1.f;                       // output scale
    bool nnScalesSet = false;
    int nnStep = 0;                         // Adam step counter
    int nnMaxSamples = 0, nnMaxSystems = 0;
    int64_t nnAdded = 0;                    // samples added so far (ring position)
    int64_t nnVersion = 0;                  // bumped by every assembly
    std::vector<NNSample> nnSamples;
    std::vector<NNSystem> nnSystems;
    float *nnD = nullptr, *nnKd = nullptr;  // loss work vectors
    float *nnRho = nullptr, *nnN = nullptr, *nnKN = nullptr;  // inference: v - K Mv, network output, K N
    int nnKind = 0;                         // collected pairs: 0 iterate errors (r, e), 1 Krylov vectors (r)
    int nnEvery = 0, nnMaxPerSolve = 0;     // FGMRES iterate snapshots for training pairs (0: off)
    std::vector<float*> nnSnaps;
    int nnSnapCount = 0;
    cudaGraphExec_t nnGraph = nullptr;
    float* vcOut2 = nullptr;
    // batch of independent problems (contiguous node ranges), see ef_batch_setup
    int batchN = 0;
    int32_t *dBatchNodePtr = nullptr, *dBatchOrder = nullptr;
    int batchTile = 1;  // index into the batched-PCG tile shapes
    // FGMRES workspace
    float* fgV = nullptr;                // [restart+1][nDof]
    float* fgZ = nullptr;                // [restart][nDof]
    float* fgW = nullptr;
    double* fgPart = nullptr;
    double* fgH = nullptr;               // device scratch: [hG | hTmp | hAcc | y], 128 each
    double* fgPartN = nullptr;           // per-CTA parts of |w|^2
    int fgNPart = 0;                     // CTAs of the orthogonalisation kernels
    // deferred normalisation of the basis (two Gram-Schmidt kernels per column; EF_FGMRES_DEFER)
    bool fgDefer = true;
    float* fgPartF = nullptr;            // [kMaxBasis][nSM] per-CTA dot products
    float* fgSc = nullptr;               // [kMaxBasis] 1 / |u_k| of the unnormalised basis vectors
    unsigned* fgTicket = nullptr;        // last-CTA counter of gs_axpy_kernel (0 between launches)
    int spCap = 0;                       // > 0: FGMRES SpMV through shared-memory staging (EF_SPMV_STAGED=1)
    int fgPc = 0;                        // FGMRES base preconditioner: EF_FGMRES_PC_MULTIGRID / _JACOBI
    double* fgPinDev = nullptr;          // device address of fgPin
    bool vcInStale = true;               // vcIn does not hold the next basis vector
    double fgEta2 = 0.0;                 // DGKS threshold squared (EF_FGMRES_ETA; 0: one pass)
    int fgRestart = 0;
    double* fgPin = nullptr;                   // pinned host copies of two columns' coefficients
    cudaEvent_t fgDone[2] = {nullptr, nullptr};
    cudaEvent_t fgNormDone = nullptr;  // the starting vector's norm is in host-mapped memory
    cudaEvent_t fgEv[2][4] = {};               // per column slot: iteration start/end, SpMV start/end
};

// ---- functions of one host unit called from another ----------------------------------------
// system.cu
ef_status residual64(ef_ctx* c, const double* x, const double* b, double* r, cudaStream_t s);
ef_status dot_host(ef_ctx* c, const double* a, const double* b, double* out, cudaStream_t s);
ef_status run_pcg(ef_ctx* c, int vDouble, const void* rhs, void* sol, int maxIter, double rtol, PcgResultHost* out,
                  ef_solve_info* prof, cudaStream_t s);
// precond.cu
ef_status amg_workspace(ef_ctx* c);
ef_status amg_build(ef_ctx* c);
ef_status amg_refresh(ef_ctx* c, cudaStream_t s);
ef_status amg_vcycle(ef_ctx* c, int l, const float* r, float* x, cudaStream_t s);
ef_status amg_capture(ef_ctx* c);
ef_status sell_refresh(ef_ctx* c, cudaStream_t s);
ef_status nn_edge_refresh(ef_ctx* c, cudaStream_t s, bool force = false);
// solve.cu
ef_status nn_apply(ef_ctx* c, cudaStream_t s);
ef_status nn_capture(ef_ctx* c);
ef_status apply_base(ef_ctx* c, cudaStream_t s);
ef_status fgmres_precond(ef_ctx* c, const float* v, const float** out, cudaStream_t s);
// learned_api.cu
ef_status nn_add_sample(ef_ctx* c, const float* r, const float* e, cudaStream_t s);
ef_status nn_collect_snapshots(ef_ctx* c, const float* x, cudaStream_t s);
ef_status nn_snapshot_buffer(ef_ctx* c, float** out);
ef_status nn_current_system(ef_ctx* c, cudaStream_t s, int* out);
