// C ABI of the efgpu library: context, model setup (element groups, DOF maps, VIJ->CSR
// slot maps built on the host), and the hot-path entry points declared in include/efgpu.h.

#include <math.h>
#include <string.h>

#include <algorithm>
#include <numeric>
#include <random>
#include <string>
#include <thread>
#include <vector>

#include "amg_sa_pattern.h"
#include "ef_common.cuh"

#include <atomic>

// launch counter (see ef_common.cuh); launches issued during a stream capture are credited to the
// graph being captured on this thread instead
static std::atomic<long long> g_launchCount{0};
static thread_local long long* t_captureCount = nullptr;
void ef::note_launches(long long n) {
    if (t_captureCount)
        *t_captureCount += n;
    else
        g_launchCount.fetch_add(n, std::memory_order_relaxed);
}
long long ef::launches() { return g_launchCount.load(std::memory_order_relaxed); }

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
ef_status ef_launch_level_residual(int bs, int nN, const int32_t* rowPtr, const int32_t* colIdx, const float* vals,
                                   const float* x, const float* r, const uint8_t* mask, float* t, cudaStream_t s,
                                   const float* binv = nullptr, float omega = 0.f, const void* valsH = nullptr);
ef_status ef_launch_to_bf16(int64_t n, const float* src, void* dst, cudaStream_t s);
ef_status ef_launch_sa_damping(const double* n2, float* wP, cudaStream_t s);
ef_status ef_launch_sa_setup(int bf, int64_t nP, const int32_t* pRow, const int32_t* pCol, const int64_t* pSeg,
                             const int32_t* pSrc, int64_t nAP, const int32_t* apRow, const int64_t* apSeg,
                             const int32_t* apK, const int32_t* apP, const int32_t* fineCol, const float* fineVals,
                             const uint8_t* fineMask, const float* offs, const int32_t* agg, const float* binv,
                             const float* wP, float* Pv, float* APv, int64_t nC, const int64_t* cSeg,
                             const int32_t* cP, const int32_t* cAP, const int32_t* coarseRowOfBlock,
                             const int32_t* coarseCol, const uint8_t* coarseDead, float* coarseVals,
                             cudaStream_t s);
ef_status ef_launch_sa_restrict(int bf, int nC, const int32_t* tPtr, const int32_t* tIdx, const int32_t* pRow,
                                const float* Pv, const float* t, const uint8_t* coarseDead, float* rc,
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
                        int nPart, double* out, cudaStream_t s);
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
                                    int slotNorm, cudaStream_t s);
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
                                 cudaStream_t s);
ef_status ef_launch_sell_spmv3(int nN, int nSlices, const int64_t* off, const int32_t* perm, const int32_t* col,
                               const float* v9, const float* x, const uint8_t* mask, float* y, float* xcopy,
                               cudaStream_t s);
ef_status ef_launch_sell_level3_bf16(int nN, int nSlices, const int64_t* off, const int32_t* perm, const int32_t* col,
                                     const void* v8, const void* v1, const float* x, const float* r,
                                     const uint8_t* mask, float* t, const float* binv, float omega, cudaStream_t s);

using namespace ef;

static thread_local std::string g_err;
void ef_set_error(const std::string& s) { g_err = s; }

#define EF_CHECK(call)                   \
    do {                                 \
        ef_status _s = (call);           \
        if (_s != EF_OK) return _s;      \
    } while (0)

namespace {

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

struct TypeInfo {
    const char* name;
    int nNodes;
    int rule;  // 0: 1 point, 1: 2x2x2, 2: 3x3x3
    int tl;
};

// elements/library.py:212-291 (small strain), :453-532 (total Lagrange) and the aliases of :535-551
const TypeInfo kTypes[] = {
    {"C3D8", 8, 1, 0},    {"C3D8R", 8, 0, 0},   {"C3D8E", 8, 2, 0},    {"C3D20", 20, 2, 0},
    {"C3D20R", 20, 1, 0}, {"C3D8TL", 8, 1, 1},  {"C3D20TL", 20, 2, 1}, {"C3D8RTL", 8, 0, 1},
    {"C3D8ETL", 8, 2, 1}, {"C3D20RTL", 20, 1, 1}, {"C3D8N", 8, 1, 0},  {"C3D20N", 20, 2, 0},
    {"C3D8NTL", 8, 1, 1}, {"C3D20NTL", 20, 2, 1},
};

bool ieq(const char* a, const char* b) {
    for (; *a && *b; ++a, ++b)
        if (tolower(*a) != tolower(*b)) return false;
    return *a == *b;
}

// parametric node tables (S1, S2, S3) -- elements/displacementelement/_elementcomputationmatrices.py _J3D8/_J3D20
const int kHex8[8][3] = {{-1, -1, -1}, {-1, -1, 1}, {1, -1, 1}, {1, -1, -1},
                         {-1, 1, -1},  {-1, 1, 1},  {1, 1, 1},  {1, 1, -1}};
const int kHex20[20][3] = {{-1, -1, -1}, {-1, -1, 1}, {1, -1, 1}, {1, -1, -1}, {-1, 1, -1}, {-1, 1, 1}, {1, 1, 1},
                           {1, 1, -1},   {-1, -1, 0}, {0, -1, 1}, {1, -1, 0},  {0, -1, -1}, {-1, 1, 0}, {0, 1, 1},
                           {1, 1, 0},    {0, 1, -1},  {-1, 0, -1}, {-1, 0, 1}, {1, 0, 1},   {1, 0, -1}};

// Gauss rules of elements/library.py (xi, eta, zeta, w)
void gauss_rule(int rule, std::vector<double>& xi, std::vector<double>& eta, std::vector<double>& zeta,
                std::vector<double>& w) {
    xi.clear();
    eta.clear();
    zeta.clear();
    w.clear();
    if (rule == 0) {
        xi = {0.0};
        eta = {0.0};
        zeta = {0.0};
        w = {8.0};
    } else if (rule == 1) {
        const double g = 1.0 / sqrt(3.0);
        const double s8[4] = {-1, 1, 1, -1}, t8[4] = {-1, -1, 1, 1};
        for (int h = 0; h < 2; ++h)
            for (int i = 0; i < 4; ++i) {
                xi.push_back(h ? g : -g);
                eta.push_back(g * t8[i]);
                zeta.push_back(g * s8[i]);
                w.push_back(1.0);
            }
    } else {
        const double r = sqrt(0.6);
        const double t20[9] = {-1, -1, -1, 0, 0, 0, 1, 1, 1};
        const double s20[3] = {-1, 0, 1};
        const double w1 = pow(5.0 / 9.0, 3), w2 = pow(5.0 / 9.0, 2) * (8.0 / 9.0), w3 = (5.0 / 9.0) * pow(8.0 / 9.0, 2),
                     w4 = pow(8.0 / 9.0, 3);
        const double wI[3] = {w1, w2, w1}, wII[3] = {w2, w3, w2}, wIII[3] = {w3, w4, w3};
        const double* wrows[9] = {wI, wII, wI, wII, wIII, wII, wI, wII, wI};
        for (int h = 0; h < 3; ++h)
            for (int i = 0; i < 9; ++i) {
                xi.push_back(r * (h - 1));
                eta.push_back(r * t20[i]);
                zeta.push_back(r * s20[i % 3]);
                w.push_back(wrows[(9 * h + i) / 3][i % 3]);  // 9 groups of 3 over the 27 points
            }
    }
}

void shape(int nn, const double* S, double* N, double dN[3][20]) {
    for (int a = 0; a < nn; ++a) {
        const int* sa = nn == 8 ? kHex8[a] : kHex20[a];
        double f[3], df[3];
        for (int k = 0; k < 3; ++k) {
            if (sa[k] != 0) {
                f[k] = 1.0 + sa[k] * S[k];
                df[k] = sa[k];
            } else {
                f[k] = 1.0 - S[k] * S[k];
                df[k] = -2.0 * S[k];
            }
        }
        const bool corner = sa[0] != 0 && sa[1] != 0 && sa[2] != 0;
        if (nn == 8) {
            N[a] = f[0] * f[1] * f[2] / 8.0;
            dN[0][a] = df[0] * f[1] * f[2] / 8.0;
            dN[1][a] = f[0] * df[1] * f[2] / 8.0;
            dN[2][a] = f[0] * f[1] * df[2] / 8.0;
        } else if (corner) {
            const double lin = sa[0] * S[0] + sa[1] * S[1] + sa[2] * S[2] - 2.0;
            N[a] = f[0] * f[1] * f[2] * lin / 8.0;
            dN[0][a] = (df[0] * f[1] * f[2] * lin + f[0] * f[1] * f[2] * sa[0]) / 8.0;
            dN[1][a] = (f[0] * df[1] * f[2] * lin + f[0] * f[1] * f[2] * sa[1]) / 8.0;
            dN[2][a] = (f[0] * f[1] * df[2] * lin + f[0] * f[1] * f[2] * sa[2]) / 8.0;
        } else {
            N[a] = f[0] * f[1] * f[2] / 4.0;
            dN[0][a] = df[0] * f[1] * f[2] / 4.0;
            dN[1][a] = f[0] * df[1] * f[2] / 4.0;
            dN[2][a] = f[0] * f[1] * df[2] / 4.0;
        }
    }
}

void build_tables(const TypeInfo& t, ElemTables& T) {
    memset(&T, 0, sizeof(T));
    std::vector<double> xi, eta, zeta, w;
    gauss_rule(t.rule, xi, eta, zeta, w);
    T.nNodes = t.nNodes;
    T.nQP = (int)w.size();
    T.totalLagrange = t.tl;
    T.quirk = t.nNodes == 20 ? 1 : 0;  // both element families use _J3D20 with its row-2 term
    for (int q = 0; q < T.nQP; ++q) {
        double N[20], dN[3][20];
        const double Sb[3] = {eta[q], xi[q], zeta[q]};  // B/J evaluation point
        shape(t.nNodes, Sb, N, dN);
        for (int r = 0; r < 3; ++r)
            for (int a = 0; a < t.nNodes; ++a) {
                T.dNdS_d[q][r][a] = dN[r][a];
                T.dNdS_f[q][r][a] = (float)dN[r][a];
            }
        const double Sn[3] = {xi[q], eta[q], zeta[q]};  // computeNOperator evaluation point
        double dN2[3][20];
        shape(t.nNodes, Sn, N, dN2);
        for (int a = 0; a < t.nNodes; ++a) T.N[q][a] = N[a];
        T.w[q] = w[q];
        T.quirkFac[q] = zeta[q] - xi[q];
    }
}

int material_kind(const char* m, int* nProps) {
    if (ieq(m, "linearelastic")) {
        *nProps = 2;
        return MAT_LINEAR_ELASTIC;
    }
    if (ieq(m, "vonmises")) {
        *nProps = 6;
        return MAT_VON_MISES;
    }
    if (ieq(m, "neohookewa")) {
        *nProps = 2;
        return MAT_NEOHOOKE_WA;
    }
    return -1;
}

template <typename T>
T* dalloc(size_t n, ef_status* st) {
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
void parallel_for(int64_t n, F f) {
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

}  // namespace

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
    // smoothed aggregation (transition from the finer level to this one): index maps and values
    int64_t saNP = 0, saNAP = 0;
    int32_t *saPRowPtr = nullptr, *saPCol = nullptr, *saPRow = nullptr, *saPSrc = nullptr;
    int32_t *saTPtr = nullptr, *saTIdx = nullptr, *saApRow = nullptr, *saApK = nullptr, *saApP = nullptr;
    int32_t *saCP = nullptr, *saCAP = nullptr;
    int64_t *saPSeg = nullptr, *saApSeg = nullptr, *saCSeg = nullptr;
    float *saPv = nullptr, *saAPv = nullptr, *saW = nullptr;
    std::vector<int32_t> hRowPtr, hColIdx, hAgg, hAggPtr, hAggIdx;
    std::vector<uint8_t> hDead;

    // device arrays of the level (null ones are skipped)
    void free_device() {
        for (void* p : {(void*)rowPtr, (void*)colIdx, (void*)rowOfBlock, (void*)diagPos, (void*)vals, (void*)binv,
                        (void*)dead, (void*)agg, (void*)offs, (void*)aggPtr, (void*)aggIdx, (void*)gseg, (void*)gsrc,
                        (void*)x, (void*)x2, (void*)valsH, (void*)r, (void*)t, (void*)saPRowPtr, (void*)saPCol,
                        (void*)saPRow, (void*)saPSrc, (void*)saTPtr, (void*)saTIdx, (void*)saApRow, (void*)saApK,
                        (void*)saApP, (void*)saCP, (void*)saCAP, (void*)saPSeg, (void*)saApSeg, (void*)saCSeg,
                        (void*)saPv, (void*)saAPv, (void*)saW})
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
    bool nnEdgeStale = true;             // the learned correction's edge weights need a refresh
    std::vector<uint8_t> hMask;
    std::vector<int32_t> hRowPtr0, hColIdx0;  // host copy of the fine block pattern
    // sliced-ELL copy of the fine system (sell.cu): FGMRES product and fine smoothing
    int sellMode = -1;                     // -1 not decided, 0 off (EF_SELL=0 or too much padding), 1 on
    bool sellStale = true;                 // values need a refresh from the assembled blocks
    int sellSlices = 0;
    int64_t sellE = 0;                     // slots (32 x the sum of the slice widths)
    int64_t* dSellOff = nullptr;           // [sellSlices + 1] first slot of each slice
    int32_t* dSellPerm = nullptr;          // [nNodes] block row of each SELL row (null: identity)
    int32_t* dSellCol = nullptr;           // [sellE] block column (padding: the row itself)
    int32_t* dSellSrc = nullptr;           // [sellE] source block in the BSR values (-1: padding)
    float* dSellV9 = nullptr;              // FP32 values, nine planes per slot column
    void* dSellV8 = nullptr;               // BF16 values 0..7 per slot (16-byte words)
    void* dSellV1 = nullptr;               // BF16 value 8 per slot
    // V-cycle parameters: damping, smoothing sweeps per side, coarse over-correction, cycle type
    float amgOmega = 1.0f;                  // upper bound of the smoothing damping
    std::vector<float> levelOmega;          // per smoothed level: amgOmega, or 4 / (3 lambda_max(D^-1 A)) when smaller
    float* amgPow[2] = {nullptr, nullptr};  // power-iteration vectors (fine size)
    float* amgZero = nullptr;
    bool amgBf16 = true;                    // fine-level smoothing residuals from a BF16 copy of the blocks
    bool amgCheb = false;                   // Chebyshev smoothing (degree amgSweeps) instead of damped block Jacobi
    bool amgBf16Coarse = false;             // coarse smoothing residuals from BF16 copies (EF_AMG_BF16_COARSE)
    bool amgSmoothed = true;                // smoothed-aggregation prolongators (EF_AMG_SMOOTHED=0: plain aggregation)
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
    int spCap = 0;                       // > 0: FGMRES SpMV through shared-memory staging (EF_SPMV_STAGED=1)
    int fgPc = 0;                        // FGMRES base preconditioner: EF_FGMRES_PC_MULTIGRID / _JACOBI
    double* fgPinDev = nullptr;          // device address of fgPin
    bool vcInStale = true;               // vcIn does not hold the next basis vector
    double fgEta2 = 0.0;                 // DGKS threshold squared (EF_FGMRES_ETA; 0: one pass)
    int fgRestart = 0;
    double* fgPin = nullptr;                   // pinned host copies of two columns' coefficients
    cudaEvent_t fgDone[2] = {nullptr, nullptr};
    cudaEvent_t fgEv[2][4] = {};               // per column slot: iteration start/end, SpMV start/end
};

extern "C" {

int ef_abi_version(void) { return 3; }

const char* ef_last_error(void) { return g_err.c_str(); }

ef_status ef_create(int64_t nDof, const double* nodeCoords, ef_ctx** out) {
    if (!out || nDof <= 0 || !nodeCoords) {
        ef_set_error("ef_create: invalid arguments");
        return EF_ERR_ARG;
    }
    if (nDof % 3 != 0 || nDof >= (int64_t)1 << 31) {
        ef_set_error("ef_create: nDof must be a multiple of 3 (displacement triplets) and < 2^31");
        return EF_ERR_ARG;
    }
    ef_ctx* c = new ef_ctx();
    c->nDof = nDof;
    c->nNodes = nDof / 3;
    c->hX.assign(nodeCoords, nodeCoords + nDof);
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&c->nSM, cudaDevAttrMultiProcessorCount, dev);
    *out = c;
    return EF_OK;
}

void ef_destroy(ef_ctx* c) {
    if (!c) return;
    auto F = [](void* p) {
        if (p) cudaFree(p);
    };
    F(c->dX);
    for (auto& g : c->groups) {
        F(g.nodeDof);
        F(g.state[0]);
        F(g.state[1]);
        F((void*)g.propsTable);
        F((void*)g.elemRow);
        F(g.geo);
        F(g.geoS);
    }
    for (auto* t : c->dTables) F(t);
    for (auto& r : c->results) {
        F(r.dEl);
        F(r.dQp);
        F(r.dTable);
    }
    F(c->Pe);
    F(c->Kblk);
    F(c->dFlags);
    F(c->dDirIdx);
    F(c->dDirMask);
    F(c->dNewton);
    F(c->dSellOff);
    F(c->dSellPerm);
    F(c->dSellCol);
    F(c->dSellSrc);
    F(c->dSellV9);
    F(c->dSellV8);
    F(c->dSellV1);
    F(c->dNodeDof);
    F(c->dCondPtr);
    F(c->dCondSrc);
    F(c->dCondW);
    F(c->dBsrW);
    F(c->dTieS);
    F(c->dTieA);
    F(c->dTieB);
    F(c->dTieTmp);
    F(c->dRowPtr);
    F(c->dColIdx);
    F(c->dBsrSeg);
    F(c->dBsrSrc);
    F(c->dDiagPos);
    F(c->dBsrVals);
    F(c->dBinv);
    F(c->dMask);
    F(c->dIndptr);
    F(c->dIndices);
    F(c->dCsrSeg);
    F(c->dCsrPerm);
    F(c->dKvijTmp);
    F(c->dPart);
    F(c->dRed);
    F(c->dPartA);
    F(c->dPartB);
    F(c->dBar);
    F(c->dPcgRes);
    for (auto* p : c->w32) F(p);
    for (auto* p : c->w64) F(p);
    for (auto* p : c->w64k) F(p);
    for (auto* p : c->dTang) F(p);
    F(c->dYe);
    for (auto& L : c->amg) L.free_device();
    F(c->amgCoarsestInv);
    F(c->amgPow[0]);
    F(c->amgPow[1]);
    F(c->amgZero);
    F(c->dBsrValsH);
    for (float* p : c->chebD) F(p);
    F(c->dBatchNodePtr);
    F(c->dBatchOrder);
    F(c->vcIn);
    F(c->vcOut);
    if (c->vcGraph) cudaGraphExecDestroy(c->vcGraph);
    if (c->dCoarseOps) cudaFree(c->dCoarseOps);
    if (c->amgNorms) cudaFree(c->amgNorms);
    if (c->egExec) cudaGraphExecDestroy(c->egExec);
    if (c->nnGraph) cudaGraphExecDestroy(c->nnGraph);
    for (void* p : {(void*)c->nnP, (void*)c->nnPf, (void*)c->nnM1, (void*)c->nnM2, (void*)c->nnG, c->nnPb,
                    (void*)c->nnActs, (void*)c->nnF, (void*)c->nnWork, (void*)c->nnPart, (void*)c->nnA,
                    (void*)c->nnAT, (void*)c->nnTpos, (void*)c->nnRed, (void*)c->vcOut2})
        F(p);
    for (auto& smp : c->nnSamples)
        for (void* p : {(void*)smp.f, (void*)smp.base, (void*)smp.r, (void*)smp.e}) F(p);
    F(c->nnRho);
    F(c->nnN);
    F(c->nnKN);
    for (auto& sy : c->nnSystems) {
        F(sy.K);
        F(sy.a);
    }
    F(c->nnD);
    F(c->nnKd);
    for (float* p : c->nnSnaps) F(p);
    if (c->capStream) cudaStreamDestroy(c->capStream);
    F(c->dRowOfBlock0);
    F(c->fineX);
    F(c->fineT);
    if (c->fgPin) cudaFreeHost(c->fgPin);
    for (int k = 0; k < 2; ++k) {
        if (c->fgDone[k]) cudaEventDestroy(c->fgDone[k]);
        for (int e = 0; e < 4; ++e)
            if (c->fgEv[k][e]) cudaEventDestroy(c->fgEv[k][e]);
    }
    F(c->fgV);
    F(c->fgZ);
    F(c->fgW);
    F(c->fgPart);
    F(c->fgH);
    F(c->fgPartN);
    for (auto e : c->ev)
        if (e) cudaEventDestroy(e);
    for (auto e : c->evS)
        if (e) cudaEventDestroy(e);
    delete c;
}

ef_status ef_add_group(ef_ctx* c, const char* elType, const char* material, const double* props, int nProps,
                       int nEl, const int32_t* elDofs, int* groupId) {
    if (!c || !elType || !material || nEl < 0 || (nEl > 0 && !elDofs)) {
        ef_set_error("ef_add_group: invalid arguments");
        return EF_ERR_ARG;
    }
    if (c->finalized) {
        ef_set_error("ef_add_group: context already finalized");
        return EF_ERR_STATE;
    }
    if ((int)c->hg.size() >= EF_MAX_GROUPS) {
        ef_set_error("ef_add_group: too many groups");
        return EF_ERR_ARG;
    }
    const TypeInfo* ti = nullptr;
    for (const auto& t : kTypes)
        if (ieq(t.name, elType)) ti = &t;
    if (!ti) {
        ef_set_error(std::string("ef_add_group: unknown element type ") + elType);
        return EF_ERR_ARG;
    }
    int need = 0;
    const int mk = material_kind(material, &need);
    if (mk < 0) {
        ef_set_error(std::string("ef_add_group: unknown material ") + material);
        return EF_ERR_ARG;
    }
    if (nProps < need || nProps > 8 || !props) {
        ef_set_error("ef_add_group: wrong number of material properties");
        return EF_ERR_ARG;
    }
    if ((ti->tl && mk != MAT_NEOHOOKE_WA) || (!ti->tl && mk == MAT_NEOHOOKE_WA)) {
        ef_set_error("ef_add_group: total-Lagrange elements need a hyperelastic material and vice versa");
        return EF_ERR_ARG;
    }
    HostGroup g;
    g.elType = ti->name;
    g.mat = mk;
    g.props.assign(props, props + nProps);
    g.nEl = nEl;
    g.nNodes = ti->nNodes;
    g.tl = ti->tl;
    ElemTables T;
    build_tables(*ti, T);
    g.nQP = T.nQP;
    const int nd = 3 * ti->nNodes;
    g.nodeDof.resize((size_t)nEl * ti->nNodes);
    for (int64_t e = 0; e < nEl; ++e)
        for (int a = 0; a < ti->nNodes; ++a) {
            const int32_t d0 = elDofs[e * nd + 3 * a];
            if (d0 < 0 || d0 + 2 >= c->nDof || d0 % 3 != 0 || elDofs[e * nd + 3 * a + 1] != d0 + 1 ||
                elDofs[e * nd + 3 * a + 2] != d0 + 2) {
                ef_set_error("ef_add_group: element DOFs must be in-range node triplets (3n, 3n+1, 3n+2)");
                return EF_ERR_ARG;
            }
            g.nodeDof[e * ti->nNodes + a] = d0;
        }
    ef_status st = EF_OK;
    ElemTables* dT = dalloc<ElemTables>(1, &st);
    if (!dT) return st;
    EF_CUDA(cudaMemcpy(dT, &T, sizeof(T), cudaMemcpyHostToDevice));
    c->dTables.push_back(dT);
    if (groupId) *groupId = (int)c->hg.size();
    c->hg.push_back(std::move(g));
    return EF_OK;
}

ef_status ef_set_ties(ef_ctx* c, const int64_t* slave, const int64_t* masterA, const int64_t* masterB, int64_t n) {
    if (!c) return EF_ERR_ARG;
    if (c->finalized) {
        ef_set_error("ef_set_ties: context already finalized");
        return EF_ERR_STATE;
    }
    if (n < 0 || (n > 0 && (!slave || !masterA || !masterB))) return EF_ERR_ARG;
    const int64_t nN = c->nNodes;
    std::vector<uint8_t> isSlave(nN, 0);
    for (int64_t i = 0; i < n; ++i) {
        const int64_t s_ = slave[i], a = masterA[i], b = masterB[i];
        if (s_ < 0 || s_ >= nN || a < 0 || a >= nN || b < 0 || b >= nN || s_ == a || s_ == b || isSlave[s_]) {
            ef_set_error("ef_set_ties: node out of range, self-tied or tied twice");
            return EF_ERR_ARG;
        }
        isSlave[s_] = 1;
    }
    for (int64_t i = 0; i < n; ++i)
        if (isSlave[masterA[i]] || isSlave[masterB[i]]) {
            ef_set_error("ef_set_ties: a master node is itself tied");
            return EF_ERR_ARG;
        }
    c->hTieS.assign(slave, slave + n);
    c->hTieA.assign(masterA, masterA + n);
    c->hTieB.assign(masterB, masterB + n);
    return EF_OK;
}

// slots 6 and 7 of a small-strain material's property row: lambda and G of (E, nu), formed once
// (the element kernel reads them instead of dividing per Gauss point)
static void derived_props(int mat, double* p) {
    if (mat != MAT_LINEAR_ELASTIC && mat != MAT_VON_MISES) return;
    const double E = p[0], nu = p[1];
    p[6] = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
    p[7] = E / (2.0 * (1.0 + nu));
}

ef_status ef_set_group_cutback(ef_ctx* c, int groupId, double scale) {
    if (!c) return EF_ERR_ARG;
    if (c->finalized) {
        ef_set_error("ef_set_group_cutback: context already finalized");
        return EF_ERR_STATE;
    }
    if (groupId < 0 || groupId >= (int)c->hg.size() || !(scale > 0.0 && scale < 1.0)) {
        ef_set_error("ef_set_group_cutback: needs a group and a scale in (0, 1)");
        return EF_ERR_ARG;
    }
    c->hg[groupId].cutback = scale;
    return EF_OK;
}

ef_status ef_set_group_props(ef_ctx* c, int groupId, const double* table, int nRows, int nProps,
                             const int32_t* elemRow) {
    if (!c) return EF_ERR_ARG;
    if (c->finalized) {
        ef_set_error("ef_set_group_props: context already finalized");
        return EF_ERR_STATE;
    }
    if (groupId < 0 || groupId >= (int)c->hg.size() || !table || !elemRow || nRows <= 0 || nProps <= 0 ||
        nProps > 8) {
        ef_set_error("ef_set_group_props: bad arguments");
        return EF_ERR_ARG;
    }
    HostGroup& h = c->hg[groupId];
    int need = 0;
    const char* names[3] = {"linearelastic", "vonmises", "neohookewa"};
    material_kind(names[h.mat], &need);
    if (nProps < need) {
        ef_set_error("ef_set_group_props: too few material properties per row");
        return EF_ERR_ARG;
    }
    h.propsTable.assign((size_t)nRows * 8, 0.0);
    for (int r = 0; r < nRows; ++r) {
        for (int i = 0; i < nProps; ++i) h.propsTable[(size_t)r * 8 + i] = table[(size_t)r * nProps + i];
        derived_props(h.mat, &h.propsTable[(size_t)r * 8]);
    }
    h.elemRow.assign(elemRow, elemRow + h.nEl);
    for (int32_t r : h.elemRow)
        if (r < 0 || r >= nRows) {
            ef_set_error("ef_set_group_props: element row out of range");
            h.propsTable.clear();
            h.elemRow.clear();
            return EF_ERR_ARG;
        }
    return EF_OK;
}

ef_status ef_finalize(ef_ctx* c, int options) {
    if (!c) return EF_ERR_ARG;
    if (c->finalized) {
        ef_set_error("ef_finalize: called twice");
        return EF_ERR_STATE;
    }
    c->keFp64 = (options & EF_OPT_KE_FP64) ? 1 : 0;
    c->scalar = !(options & EF_OPT_NO_SCALAR_CSR) && c->hTieS.empty();  // the reference CSR has no ties
    if (const char* e = getenv("EF_ELEM_GRAPH")) c->elemGraphs = atoi(e) != 0;
    if (const char* e = getenv("EF_MPNN_TC")) c->nnTensorCores = atoi(e) != 0;
    const size_t ks = c->keFp64 ? sizeof(double) : sizeof(float);
    ef_status st = EF_OK;
    const int64_t nNodes = c->nNodes;
    c->dX = dalloc<double>(c->nDof, &st);
    if (!c->dX) return st;
    EF_CUDA(cudaMemcpy(c->dX, c->hX.data(), sizeof(double) * c->nDof, cudaMemcpyHostToDevice));

    c->dFlags = dalloc<int>(4, &st);
    if (!c->dFlags) return st;
    {
        const float none = EF_PNEWDT_NONE;
        int hf[4] = {0, 0, 0, 0};
        memcpy(&hf[1], &none, sizeof(float));
        EF_CUDA(cudaMemcpy(c->dFlags, hf, sizeof(hf), cudaMemcpyHostToDevice));
    }

    // groups: device node maps and double-buffered SoA state
    int64_t peOff = 0, keOff = 0, nEl = 0, nVIJ = 0;
    for (size_t gi = 0; gi < c->hg.size(); ++gi) {
        const HostGroup& h = c->hg[gi];
        Group g;
        memset(&g, 0, sizeof(g));
        g.nEl = h.nEl;
        g.nNodes = h.nNodes;
        g.nQP = h.nQP;
        g.nDofEl = 3 * h.nNodes;
        g.nPair = h.nNodes * (h.nNodes + 1) / 2;
        g.mat = h.mat;
        g.tl = h.tl;
        if (const char* e = getenv("EF_ELEM_INTCONV")) g.intConv = atoi(e) != 0;
        g.cutback = (float)h.cutback;
        g.nState = 12 + ((h.mat == MAT_VON_MISES || h.mat == MAT_NEOHOOKE_WA) ? 1 : 0);
        for (size_t i = 0; i < h.props.size() && i < 8; ++i) g.props[i] = h.props[i];
        derived_props(h.mat, g.props);
        g.nodeDof = dalloc<int32_t>(h.nodeDof.size(), &st);
        if (!g.nodeDof) return st;
        EF_CUDA(cudaMemcpy(g.nodeDof, h.nodeDof.data(), sizeof(int32_t) * h.nodeDof.size(), cudaMemcpyHostToDevice));
        const size_t ns = (size_t)g.nState * h.nEl * h.nQP;
        for (int k = 0; k < 2; ++k) {
            g.state[k] = dalloc<double>(ns, &st);
            if (!g.state[k]) return st;
            EF_CUDA(cudaMemset(g.state[k], 0, sizeof(double) * ns));
        }
        g.cur = 0;
        if (!h.propsTable.empty()) {
            double* pt = dalloc<double>(h.propsTable.size(), &st);
            int32_t* er = dalloc<int32_t>(h.elemRow.size(), &st);
            if (!pt || !er) return st;
            EF_CUDA(cudaMemcpy(pt, h.propsTable.data(), sizeof(double) * h.propsTable.size(), cudaMemcpyHostToDevice));
            EF_CUDA(cudaMemcpy(er, h.elemRow.data(), sizeof(int32_t) * h.elemRow.size(), cudaMemcpyHostToDevice));
            g.propsTable = pt;
            g.elemRow = er;
        }
        g.geo = dalloc<double>((size_t)h.nEl * h.nQP * (3 * h.nNodes + 1), &st);
        if (!g.geo) return st;
        if (!g.tl) {
            g.geoS = dalloc<float2>((size_t)h.nEl * h.nQP * (3 * h.nNodes + 1), &st);
            if (!g.geoS) return st;
        }
        EF_CHECK(ef_launch_geometry(g, c->dTables[gi], c->dX, c->dFlags, 0));
        g.peOffset = peOff;
        g.keOffset = keOff;
        g.tablesSlot = (int)gi;
        peOff += (int64_t)h.nEl * g.nDofEl;
        keOff += (int64_t)h.nEl * g.nPair;
        nEl += h.nEl;
        nVIJ += (int64_t)h.nEl * g.nDofEl * g.nDofEl;
        c->groups.push_back(g);
    }
    c->nElements = nEl;
    c->nPe = peOff;
    c->nKblk = keOff;
    c->nVIJ = nVIJ;
    c->Pe = dalloc<double>(peOff, &st);
    if (!c->Pe) return st;
    c->Kblk = dalloc<char>((size_t)keOff * 9 * ks, &st);
    if (!c->Kblk) return st;

    // node -> first DOF
    std::vector<int32_t> nodeDof(nNodes);
    for (int64_t m = 0; m < nNodes; ++m) nodeDof[m] = (int32_t)(3 * m);
    c->dNodeDof = dalloc<int32_t>(nNodes, &st);
    if (!c->dNodeDof) return st;
    EF_CUDA(cudaMemcpy(c->dNodeDof, nodeDof.data(), sizeof(int32_t) * nNodes, cudaMemcpyHostToDevice));

    // ties: every node maps to target nodes with weights (itself with 1; a tied node to its two
    // masters with 1/2 each)
    const bool ties = !c->hTieS.empty();
    std::vector<int32_t> tieOf(nNodes, -1);
    for (size_t i = 0; i < c->hTieS.size(); ++i) tieOf[c->hTieS[i]] = (int32_t)i;
    auto targets = [&](int64_t m, int64_t* t, float* w) -> int {
        const int32_t k = tieOf[m];
        if (k < 0) {
            t[0] = m;
            w[0] = 1.f;
            return 1;
        }
        t[0] = c->hTieA[k];
        t[1] = c->hTieB[k];
        w[0] = w[1] = 0.5f;
        return 2;
    };
    if (ties) {
        const int64_t nt = (int64_t)c->hTieS.size();
        c->dTieS = dalloc<int32_t>(nt, &st);
        c->dTieA = dalloc<int32_t>(nt, &st);
        c->dTieB = dalloc<int32_t>(nt, &st);
        c->dTieTmp = dalloc<double>(c->nDof, &st);
        if (st != EF_OK) return st;
        EF_CUDA(cudaMemcpy(c->dTieS, c->hTieS.data(), sizeof(int32_t) * nt, cudaMemcpyHostToDevice));
        EF_CUDA(cudaMemcpy(c->dTieA, c->hTieA.data(), sizeof(int32_t) * nt, cudaMemcpyHostToDevice));
        EF_CUDA(cudaMemcpy(c->dTieB, c->hTieB.data(), sizeof(int32_t) * nt, cudaMemcpyHostToDevice));
    }

    // condensation map: node m <- Pe slices of (group, element, local node) in element order
    // (with ties: the slices of the nodes tied to m, weighted; a tied node itself gets none)
    std::vector<int64_t> cptr(nNodes + 1, 0);
    for (const auto& h : c->hg)
        for (int32_t d : h.nodeDof) {
            int64_t t[2];
            float w[2];
            const int nt = targets(d / 3, t, w);
            for (int i = 0; i < nt; ++i) cptr[t[i] + 1]++;
        }
    for (int64_t m = 0; m < nNodes; ++m) cptr[m + 1] += cptr[m];
    std::vector<int64_t> csrc(cptr[nNodes]);
    std::vector<float> cw(ties ? cptr[nNodes] : 0);
    {
        std::vector<int64_t> fill(cptr.begin(), cptr.end() - 1);
        for (size_t gi = 0; gi < c->hg.size(); ++gi) {
            const auto& h = c->hg[gi];
            const Group& g = c->groups[gi];
            for (int64_t e = 0; e < h.nEl; ++e)
                for (int a = 0; a < h.nNodes; ++a) {
                    int64_t t[2];
                    float w[2];
                    const int nt = targets(h.nodeDof[e * h.nNodes + a] / 3, t, w);
                    for (int i = 0; i < nt; ++i) {
                        const int64_t pos = fill[t[i]]++;
                        csrc[pos] = g.peOffset + e * g.nDofEl + 3 * a;
                        if (ties) cw[pos] = w[i];
                    }
                }
        }
    }
    c->dCondPtr = dalloc<int64_t>(nNodes + 1, &st);
    c->dCondSrc = dalloc<int64_t>(csrc.size(), &st);
    if (!c->dCondPtr || !c->dCondSrc) return st;
    EF_CUDA(cudaMemcpy(c->dCondPtr, cptr.data(), sizeof(int64_t) * (nNodes + 1), cudaMemcpyHostToDevice));
    EF_CUDA(cudaMemcpy(c->dCondSrc, csrc.data(), sizeof(int64_t) * csrc.size(), cudaMemcpyHostToDevice));
    if (ties) {
        c->dCondW = dalloc<float>(cw.size(), &st);
        if (!c->dCondW) return st;
        EF_CUDA(cudaMemcpy(c->dCondW, cw.data(), sizeof(float) * cw.size(), cudaMemcpyHostToDevice));
    }

    // BSR pattern + block scatter map.  Global block (m, n) = sum over elements (in order) of
    // K_ab with node(a) = m, node(b) = n; stored pair p(min,max) with a transpose flag if a > b.
    {
        std::vector<int64_t> rcount(nNodes + 1, 0);
        for (const auto& h : c->hg)
            for (int64_t e = 0; e < h.nEl; ++e) {
                int nb = 0;  // element nodes counted with their targets
                for (int b = 0; b < h.nNodes; ++b) nb += tieOf[h.nodeDof[e * h.nNodes + b] / 3] < 0 ? 1 : 2;
                for (int a = 0; a < h.nNodes; ++a) {
                    int64_t t[2];
                    float w[2];
                    const int nt = targets(h.nodeDof[e * h.nNodes + a] / 3, t, w);
                    for (int i = 0; i < nt; ++i) rcount[t[i] + 1] += nb;
                }
            }
        for (int64_t m = 0; m < nNodes; ++m)
            if (tieOf[m] >= 0) rcount[m + 1] += 1;  // the tied node's own (empty) diagonal block
        for (int64_t m = 0; m < nNodes; ++m) rcount[m + 1] += rcount[m];
        const int64_t nEnt = rcount[nNodes];
        // entries per row: (col node, element-block code); element order is preserved by the fill order
        std::vector<int32_t> ecol(nEnt);
        std::vector<int64_t> esrc(nEnt);
        std::vector<float> ew(ties ? nEnt : 0);
        std::vector<int64_t> fill(rcount.begin(), rcount.end() - 1);
        for (size_t gi = 0; gi < c->hg.size(); ++gi) {
            const auto& h = c->hg[gi];
            const Group& g = c->groups[gi];
            const int nn = h.nNodes;
            for (int64_t e = 0; e < h.nEl; ++e)
                for (int a = 0; a < nn; ++a) {
                    int64_t ta[2], tb[2];
                    float wa[2], wb[2];
                    const int na = targets(h.nodeDof[e * nn + a] / 3, ta, wa);
                    for (int ia = 0; ia < na; ++ia)
                        for (int b = 0; b < nn; ++b) {
                            const int nb = targets(h.nodeDof[e * nn + b] / 3, tb, wb);
                            const int lo = std::min(a, b), hi = std::max(a, b);
                            const int p = lo * nn - lo * (lo - 1) / 2 + (hi - lo);
                            const int64_t blk = g.keOffset + e * g.nPair + p;
                            for (int ib = 0; ib < nb; ++ib) {
                                const int64_t pos = fill[ta[ia]]++;
                                ecol[pos] = (int32_t)tb[ib];
                                esrc[pos] = (blk << 1) | (a > b ? 1 : 0);
                                if (ties) ew[pos] = wa[ia] * wb[ib];
                            }
                        }
                }
        }
        for (int64_t m = 0; m < nNodes; ++m)
            if (tieOf[m] >= 0) {  // marker of the tied node's diagonal block: no source
                const int64_t pos = fill[m]++;
                ecol[pos] = (int32_t)m;
                esrc[pos] = -1;
            }
        // per row: stable sort by column, unique columns -> blocks
        std::vector<int64_t> rowBlocks(nNodes + 1, 0);
        std::vector<int64_t> order(nEnt);
        parallel_for(nNodes, [&](int64_t lo, int64_t hi) {
            for (int64_t m = lo; m < hi; ++m) {
                const int64_t s = rcount[m], e = rcount[m + 1];
                for (int64_t i = s; i < e; ++i) order[i] = i;
                std::stable_sort(order.begin() + s, order.begin() + e,
                                 [&](int64_t x, int64_t y) { return ecol[x] < ecol[y]; });
                int64_t nb = 0;
                for (int64_t i = s; i < e; ++i)
                    if (i == s || ecol[order[i]] != ecol[order[i - 1]]) ++nb;
                rowBlocks[m + 1] = nb;
            }
        });
        for (int64_t m = 0; m < nNodes; ++m) rowBlocks[m + 1] += rowBlocks[m];
        const int64_t nBlocks = rowBlocks[nNodes];
        if (nBlocks >= ((int64_t)1 << 31)) {
            ef_set_error("ef_finalize: too many blocks");
            return EF_ERR_ARG;
        }
        c->nBlocks = nBlocks;
        std::vector<int32_t> rowPtr(nNodes + 1), colIdx(nBlocks);
        std::vector<int64_t> seg(nBlocks + 1), src(nEnt), diag(nNodes, -1);
        std::vector<float> sw(ties ? nEnt : 0);
        for (int64_t m = 0; m <= nNodes; ++m) rowPtr[m] = (int32_t)rowBlocks[m];
        parallel_for(nNodes, [&](int64_t lo, int64_t hi) {
            for (int64_t m = lo; m < hi; ++m) {
                int64_t b = rowBlocks[m] - 1;
                for (int64_t i = rcount[m]; i < rcount[m + 1]; ++i) {
                    const int64_t o = order[i];
                    if (i == rcount[m] || ecol[o] != ecol[order[i - 1]]) {
                        ++b;
                        colIdx[b] = ecol[o];
                        seg[b] = i;
                        if (ecol[o] == m) diag[m] = b;
                    }
                    src[i] = esrc[o];
                    if (ties) sw[i] = ew[o];
                }
            }
        });
        seg[nBlocks] = nEnt;
        if (ties) {
            // drop the markers of tied nodes' diagonal blocks (those blocks have no source: zero)
            std::vector<int64_t> seg2(nBlocks + 1);
            std::vector<int64_t> src2;
            std::vector<float> sw2;
            src2.reserve(nEnt);
            sw2.reserve(nEnt);
            for (int64_t b = 0; b < nBlocks; ++b) {
                seg2[b] = (int64_t)src2.size();
                for (int64_t i = seg[b]; i < seg[b + 1]; ++i)
                    if (src[i] >= 0) {
                        src2.push_back(src[i]);
                        sw2.push_back(sw[i]);
                    }
            }
            seg2[nBlocks] = (int64_t)src2.size();
            seg.swap(seg2);
            src.swap(src2);
            sw.swap(sw2);
        }
        const int64_t nSrc = (int64_t)src.size();
        for (int64_t m = 0; m < nNodes; ++m)
            if (diag[m] < 0) {
                ef_set_error("ef_finalize: a DOF triplet belongs to no element (no diagonal block)");
                return EF_ERR_ARG;
            }
        c->dRowPtr = dalloc<int32_t>(nNodes + 1, &st);
        c->dColIdx = dalloc<int32_t>(nBlocks + 16, &st);  // padding: staged loads round the end up to 16 bytes
        c->dBsrSeg = dalloc<int64_t>(nBlocks + 1, &st);
        c->dBsrSrc = dalloc<int64_t>(nSrc, &st);
        c->dDiagPos = dalloc<int64_t>(nNodes, &st);
        c->dBsrVals = dalloc<char>((size_t)nBlocks * 9 * ks + 64, &st);  // + padding for staged loads
        c->dBinv = dalloc<char>((size_t)nNodes * 9 * ks, &st);
        c->dMask = dalloc<uint8_t>(c->nDof, &st);
        if (!c->dRowPtr || !c->dColIdx || !c->dBsrSeg || !c->dBsrSrc || !c->dDiagPos || !c->dBsrVals || !c->dBinv ||
            !c->dMask)
            return st;
        EF_CUDA(cudaMemcpy(c->dRowPtr, rowPtr.data(), sizeof(int32_t) * (nNodes + 1), cudaMemcpyHostToDevice));
        EF_CUDA(cudaMemcpy(c->dColIdx, colIdx.data(), sizeof(int32_t) * nBlocks, cudaMemcpyHostToDevice));
        EF_CUDA(cudaMemcpy(c->dBsrSeg, seg.data(), sizeof(int64_t) * (nBlocks + 1), cudaMemcpyHostToDevice));
        EF_CUDA(cudaMemcpy(c->dBsrSrc, src.data(), sizeof(int64_t) * nSrc, cudaMemcpyHostToDevice));
        if (ties) {
            c->dBsrW = dalloc<float>(nSrc, &st);
            if (!c->dBsrW) return st;
            EF_CUDA(cudaMemcpy(c->dBsrW, sw.data(), sizeof(float) * nSrc, cudaMemcpyHostToDevice));
        }
        EF_CUDA(cudaMemcpy(c->dDiagPos, diag.data(), sizeof(int64_t) * nNodes, cudaMemcpyHostToDevice));
        c->hMask.assign(c->nDof, 0);
        for (int32_t sN : c->hTieS)
            for (int k = 0; k < 3; ++k) c->hMask[3 * (int64_t)sN + k] = 1;  // tied DOFs are eliminated
        EF_CUDA(cudaMemcpy(c->dMask, c->hMask.data(), c->nDof, cudaMemcpyHostToDevice));
        c->hRowPtr0 = rowPtr;
        c->hColIdx0 = colIdx;
    }

    // scalar CSR of the reference (SciPy canonical pattern) + reference-order scatter map
    if (c->scalar) {
        if (c->nVIJ >= ((int64_t)1 << 31)) {
            ef_set_error("ef_finalize: VIJ too long for the scalar CSR map; use EF_OPT_NO_SCALAR_CSR");
            return EF_ERR_ARG;
        }
        // per DOF row r: (element, local index i) occurrences in element order
        const int64_t nDof = c->nDof;
        std::vector<int64_t> rptr(nDof + 1, 0);
        for (const auto& h : c->hg)
            for (int64_t e = 0; e < h.nEl; ++e)
                for (int a = 0; a < h.nNodes; ++a)
                    for (int k = 0; k < 3; ++k) rptr[h.nodeDof[e * h.nNodes + a] + k + 1] += 3 * h.nNodes;
        for (int64_t r = 0; r < nDof; ++r) rptr[r + 1] += rptr[r];
        const int64_t nEnt = rptr[nDof];
        std::vector<int32_t> col(nEnt);
        std::vector<int32_t> kk(nEnt);
        std::vector<int64_t> fill(rptr.begin(), rptr.end() - 1);
        int64_t vijOff = 0;
        for (size_t gi = 0; gi < c->hg.size(); ++gi) {
            const auto& h = c->hg[gi];
            const int nd = 3 * h.nNodes;
            for (int64_t e = 0; e < h.nEl; ++e) {
                const int32_t* nd0 = &h.nodeDof[e * h.nNodes];
                for (int i = 0; i < nd; ++i) {
                    const int64_t r = nd0[i / 3] + i % 3;  // VIJ value p = i + j*nd -> (row d[i], col d[j])
                    for (int j = 0; j < nd; ++j) {
                        const int64_t pos = fill[r]++;
                        col[pos] = nd0[j / 3] + j % 3;
                        kk[pos] = (int32_t)(vijOff + e * (int64_t)nd * nd + i + (int64_t)j * nd);
                    }
                }
            }
            vijOff += (int64_t)h.nEl * nd * nd;
        }
        std::vector<int64_t> rowNnz(nDof + 1, 0);
        parallel_for(nDof, [&](int64_t lo, int64_t hi) {
            std::vector<std::pair<int32_t, int32_t>> tmp;
            for (int64_t r = lo; r < hi; ++r) {
                const int64_t s = rptr[r], e = rptr[r + 1];
                tmp.resize(e - s);
                for (int64_t i = s; i < e; ++i) tmp[i - s] = {col[i], kk[i]};
                std::sort(tmp.begin(), tmp.end());
                int64_t nb = 0;
                for (int64_t i = s; i < e; ++i) {
                    col[i] = tmp[i - s].first;
                    kk[i] = tmp[i - s].second;
                    if (i == s || col[i] != col[i - 1]) ++nb;
                }
                rowNnz[r + 1] = nb;
            }
        });
        for (int64_t r = 0; r < nDof; ++r) rowNnz[r + 1] += rowNnz[r];
        const int64_t nnz = rowNnz[nDof];
        c->nnz = nnz;
        c->hIndptr.resize(nDof + 1);
        c->hIndices.resize(nnz);
        std::vector<int64_t> seg(nnz + 1);
        for (int64_t r = 0; r <= nDof; ++r) c->hIndptr[r] = (int32_t)rowNnz[r];
        parallel_for(nDof, [&](int64_t lo, int64_t hi) {
            for (int64_t r = lo; r < hi; ++r) {
                int64_t sl = rowNnz[r] - 1;
                for (int64_t i = rptr[r]; i < rptr[r + 1]; ++i) {
                    if (i == rptr[r] || col[i] != col[i - 1]) {
                        ++sl;
                        c->hIndices[sl] = col[i];
                        seg[sl] = i;
                    }
                }
            }
        });
        seg[nnz] = nEnt;
        c->dIndptr = dalloc<int32_t>(nDof + 1, &st);
        c->dIndices = dalloc<int32_t>(nnz, &st);
        c->dCsrSeg = dalloc<int64_t>(nnz + 1, &st);
        c->dCsrPerm = dalloc<int32_t>(nEnt, &st);
        if (!c->dIndptr || !c->dIndices || !c->dCsrSeg || !c->dCsrPerm) return st;
        EF_CUDA(cudaMemcpy(c->dIndptr, c->hIndptr.data(), sizeof(int32_t) * (nDof + 1), cudaMemcpyHostToDevice));
        EF_CUDA(cudaMemcpy(c->dIndices, c->hIndices.data(), sizeof(int32_t) * nnz, cudaMemcpyHostToDevice));
        EF_CUDA(cudaMemcpy(c->dCsrSeg, seg.data(), sizeof(int64_t) * (nnz + 1), cudaMemcpyHostToDevice));
        EF_CUDA(cudaMemcpy(c->dCsrPerm, kk.data(), sizeof(int32_t) * nEnt, cudaMemcpyHostToDevice));
    }

    // reduction and Krylov workspaces
    c->nPart = 2 * c->nSM;
    c->dPart = dalloc<double>(4 * c->nPart, &st);
    c->dRed = dalloc<double>(16, &st);
    if (!c->dPart || !c->dRed) return st;
    EF_CHECK(ef_pcg_grid(0, c->nSM, &c->pcgGrid[0]));
    EF_CHECK(ef_pcg_grid(1, c->nSM, &c->pcgGrid[1]));
    const int maxGrid = std::max(c->pcgGrid[0], c->pcgGrid[1]);
    c->dPartA = dalloc<double>(4 * (size_t)maxGrid, &st);
    c->dPartB = dalloc<double>(4 * (size_t)maxGrid, &st);
    c->dBar = dalloc<char>(ef_barrier_state_bytes(), &st);
    c->dPcgRes = dalloc<char>(ef_pcg_result_bytes(), &st);
    if (!c->dPartA || !c->dPartB || !c->dBar || !c->dPcgRes) return st;
    EF_CUDA(cudaMemset(c->dBar, 0, ef_barrier_state_bytes()));
    for (int i = 0; i < 7; ++i) {
        c->w32[i] = dalloc<float>(c->nDof, &st);
        if (!c->w32[i]) return st;
    }
    for (int i = 0; i < 5; ++i) {
        c->w64[i] = dalloc<double>(c->nDof, &st);
        if (!c->w64[i]) return st;
    }
    if (!c->keFp64) {
        // FP32 system: keep the FP64 tangent for a matrix-free refinement residual
        for (const auto& g : c->groups) {
            const size_t nt = (size_t)(g.tl ? ef_tl_tangent_size() : 9) * g.nEl * g.nQP;
            double* t = dalloc<double>(nt, &st);
            if (!t) return st;
            EF_CUDA(cudaMemset(t, 0, sizeof(double) * nt));
            c->dTang.push_back(t);
        }
        c->dYe = dalloc<double>(c->nPe, &st);
        if (!c->dYe) return st;
        c->exact = true;
    }
    for (int i = 0; i < 7; ++i) {
        c->w64k[i] = dalloc<double>(c->nDof, &st);
        if (!c->w64k[i]) return st;
    }
    EF_CUDA(cudaEventCreate(&c->ev[0]));
    EF_CUDA(cudaEventCreate(&c->ev[1]));
    EF_CUDA(cudaEventCreate(&c->evS[0]));
    EF_CUDA(cudaEventCreate(&c->evS[1]));
    c->finalized = true;
    return EF_OK;
}

ef_status ef_get_info(const ef_ctx* c, ef_info* out) {
    if (!c || !out) return EF_ERR_ARG;
    out->nDof = c->nDof;
    out->nNodes = c->nNodes;
    out->nElements = c->nElements;
    out->nVIJ = c->nVIJ;
    out->nnz = c->nnz;
    out->nBlocks = c->nBlocks;
    out->nPe = c->nPe;
    out->keFp64 = c->keFp64;
    return EF_OK;
}

#define EF_REQUIRE_FINALIZED(c)                                  \
    do {                                                         \
        if (!(c) || !(c)->finalized) {                           \
            ef_set_error("context missing or not finalized");    \
            return EF_ERR_STATE;                                 \
        }                                                        \
    } while (0)

}  // extern "C"

// one element pass: every group's kernel, then the condensation into P and F
static ef_status element_step(ef_ctx* c, const double* U_np, const double* dU, double* P, double* F, cudaStream_t s) {
    const size_t ks = c->keFp64 ? sizeof(double) : sizeof(float);
    for (size_t gi = 0; gi < c->groups.size(); ++gi) {
        const Group& g = c->groups[gi];
        void* K = (char*)c->Kblk + (size_t)g.keOffset * 9 * ks;
        double* tang = c->exact ? c->dTang[gi] : nullptr;
        if (g.tl)
            EF_CHECK(ef_launch_total_lagrange(g, U_np, K, c->keFp64, 0, c->Pe + g.peOffset, tang, c->dFlags, s));
        else
            EF_CHECK(ef_launch_small_strain(g, dU, K, c->keFp64, 0, c->Pe + g.peOffset, tang, c->dFlags, s));
    }
    EF_CHECK(ef_launch_condense(c->nNodes, c->dNodeDof, c->dCondPtr, c->dCondSrc, c->dCondW, c->Pe, P, F, s));
    return EF_OK;
}

extern "C" {

// With several element groups (element types), the pass is captured as one CUDA graph the second
// time it runs on the same vectors and replayed from then on.
ef_status ef_compute_elements(ef_ctx* c, const double* U_np, const double* dU, const double* time2, double dT,
                              double* P, double* F, void* stream) {
    EF_REQUIRE_FINALIZED(c);
    (void)time2;
    (void)dT;
    if (!dU || !P) {
        ef_set_error("ef_compute_elements: null vector");
        return EF_ERR_ARG;
    }
    for (const auto& g : c->groups)
        if (g.tl && !U_np) {
            ef_set_error("ef_compute_elements: total-Lagrange elements need U_np");
            return EF_ERR_ARG;
        }
    cudaStream_t s = (cudaStream_t)stream;
    if (c->groups.size() < 2 || !c->elemGraphs) return element_step(c, U_np, dU, P, F, s);
    const void* key[4] = {U_np, dU, P, F};
    const bool same = memcmp(key, c->egKey, sizeof(key)) == 0;
    if (same && c->egExec) {
        ef::note_launches(c->egKernels);
        EF_CUDA(cudaGraphLaunch(c->egExec, s));
        return EF_OK;
    }
    if (!same) {  // new vectors: run eagerly and remember them
        if (c->egExec) cudaGraphExecDestroy(c->egExec);
        c->egExec = nullptr;
        memcpy(c->egKey, key, sizeof(key));
        return element_step(c, U_np, dU, P, F, s);
    }
    if (!c->capStream) EF_CUDA(cudaStreamCreateWithFlags(&c->capStream, cudaStreamNonBlocking));
    EF_CUDA(cudaStreamBeginCapture(c->capStream, cudaStreamCaptureModeThreadLocal));
    long long captured = 0;
    t_captureCount = &captured;
    const ef_status st = element_step(c, U_np, dU, P, F, c->capStream);
    t_captureCount = nullptr;
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(c->capStream, &g);
    if (st != EF_OK) return st;
    if (e != cudaSuccess) {
        ef_set_error(std::string("element-pass capture: ") + cudaGetErrorString(e));
        return EF_ERR_CUDA;
    }
    EF_CUDA(cudaGraphInstantiate(&c->egExec, g, 0));
    cudaGraphDestroy(g);
    c->egKernels = captured;
    ef::note_launches(c->egKernels);
    EF_CUDA(cudaGraphLaunch(c->egExec, s));
    return EF_OK;
}

ef_status ef_element_status(ef_ctx* c, void* stream, double* pNewDT) {
    EF_REQUIRE_FINALIZED(c);
    int hf[2] = {0, 0};
    EF_CUDA(cudaMemcpyAsync(hf, c->dFlags, sizeof(hf), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    EF_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    const int f = hf[0];
    float req = EF_PNEWDT_NONE;
    memcpy(&req, &hf[1], sizeof(float));
    {
        const float none = EF_PNEWDT_NONE;
        int reset[2] = {0, 0};
        memcpy(&reset[1], &none, sizeof(float));
        EF_CUDA(cudaMemcpy(c->dFlags, reset, sizeof(reset), cudaMemcpyHostToDevice));
    }
    if (pNewDT) *pNewDT = 1.0;
    if (f & EF_FLAG_NAN) return EF_NAN;
    if (f & EF_FLAG_RETURNMAP) {
        // the smallest scale any failing element asked for (min over elements, as the Marmot
        // element loop's min over its threads' pNewDT, solvers/nonlinearimplicitstaticparallel.pyx:145-150)
        if (pNewDT) *pNewDT = req < EF_PNEWDT_NONE ? (double)req : 0.5;
        return EF_CUTBACK;
    }
    if (f & EF_FLAG_BADDET) {
        ef_set_error("non-positive Jacobian determinant in an element");
        return EF_ERR_DEVICE;
    }
    if (f & EF_FLAG_BARRIER) {
        ef_set_error("a device-side grid barrier timed out");
        return EF_ERR_DEVICE;
    }
    return EF_OK;
}

ef_status ef_get_state_size(const ef_ctx* c, int groupId, int* nQP, int* nState) {
    if (!c || !c->finalized || groupId < 0 || groupId >= (int)c->groups.size()) return EF_ERR_ARG;
    if (nQP) *nQP = c->groups[groupId].nQP;
    if (nState) *nState = c->groups[groupId].nState;
    return EF_OK;
}

// host AoS [nEl][nQP][nState] <-> device SoA [nState][nEl*nQP]
ef_status ef_set_state(ef_ctx* c, int groupId, const double* state) {
    EF_REQUIRE_FINALIZED(c);
    if (groupId < 0 || groupId >= (int)c->groups.size() || !state) return EF_ERR_ARG;
    const Group& g = c->groups[groupId];
    const int64_t nq = (int64_t)g.nEl * g.nQP;
    std::vector<double> soa((size_t)nq * g.nState);
    for (int64_t i = 0; i < nq; ++i)
        for (int v = 0; v < g.nState; ++v) soa[v * nq + i] = state[i * g.nState + v];
    EF_CUDA(cudaMemcpy(g.state[g.cur], soa.data(), sizeof(double) * soa.size(), cudaMemcpyHostToDevice));
    return EF_OK;
}

ef_status ef_get_state(ef_ctx* c, int groupId, int trial, double* state) {
    EF_REQUIRE_FINALIZED(c);
    if (groupId < 0 || groupId >= (int)c->groups.size() || !state) return EF_ERR_ARG;
    const Group& g = c->groups[groupId];
    const int64_t nq = (int64_t)g.nEl * g.nQP;
    std::vector<double> soa((size_t)nq * g.nState);
    EF_CUDA(cudaDeviceSynchronize());
    EF_CUDA(cudaMemcpy(soa.data(), g.state[trial ? 1 - g.cur : g.cur], sizeof(double) * soa.size(),
                       cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < nq; ++i)
        for (int v = 0; v < g.nState; ++v) state[i * g.nState + v] = soa[v * nq + i];
    return EF_OK;
}

ef_status ef_accept_state(ef_ctx* c) {
    EF_REQUIRE_FINALIZED(c);
    // copy trial -> committed (acceptLastState copies stateTemp into stateRef); the buffers keep
    // their roles, so launches captured in CUDA graphs stay valid across increments
    for (auto& g : c->groups)
        EF_CUDA(cudaMemcpy(g.state[g.cur], g.state[1 - g.cur], sizeof(double) * g.nState * g.nEl * g.nQP,
                           cudaMemcpyDeviceToDevice));
    return EF_OK;
}

ef_status ef_reset_state(ef_ctx* c) {
    EF_REQUIRE_FINALIZED(c);
    for (auto& g : c->groups)
        EF_CUDA(cudaMemcpy(g.state[1 - g.cur], g.state[g.cur], sizeof(double) * g.nState * g.nEl * g.nQP,
                           cudaMemcpyDeviceToDevice));
    return EF_OK;
}

ef_status ef_add_body_force(ef_ctx* c, int groupId, const double* load3, double* PExt, void* stream) {
    EF_REQUIRE_FINALIZED(c);
    if (groupId < 0 || groupId >= (int)c->groups.size() || !load3 || !PExt) {
        ef_set_error("ef_add_body_force: invalid arguments");
        return EF_ERR_ARG;
    }
    const Group& g = c->groups[groupId];
    cudaStream_t s = (cudaStream_t)stream;
    EF_CHECK(ef_launch_body_force(g, c->dTables[groupId], load3, c->Pe + g.peOffset, s));
    EF_CHECK(ef_launch_condense_add(c->nNodes, c->dNodeDof, c->dCondPtr, c->dCondSrc, c->dCondW, c->Pe, g.peOffset,
                                    g.peOffset + (int64_t)g.nEl * g.nDofEl, PExt, s));
    return EF_OK;
}

ef_status ef_export_vij(ef_ctx* c, double* Kvij, void* stream) {
    EF_REQUIRE_FINALIZED(c);
    if (!Kvij) return EF_ERR_ARG;
    const size_t ks = c->keFp64 ? sizeof(double) : sizeof(float);
    int64_t vijOff = 0;
    for (const auto& g : c->groups) {
        const void* K = (const char*)c->Kblk + (size_t)g.keOffset * 9 * ks;
        EF_CHECK(ef_launch_vij_export(g.nEl, g.nNodes, g.nPair, K, c->keFp64, Kvij + vijOff, (cudaStream_t)stream));
        vijOff += (int64_t)g.nEl * g.nDofEl * g.nDofEl;
    }
    return EF_OK;
}

ef_status ef_csr_pattern(ef_ctx* c, int32_t* indptr, int32_t* indices) {
    EF_REQUIRE_FINALIZED(c);
    if (!c->scalar) {
        ef_set_error("ef_csr_pattern: context finalized with EF_OPT_NO_SCALAR_CSR");
        return EF_ERR_STATE;
    }
    if (indptr) EF_CUDA(cudaMemcpy(indptr, c->hIndptr.data(), sizeof(int32_t) * (c->nDof + 1), cudaMemcpyDefault));
    if (indices) EF_CUDA(cudaMemcpy(indices, c->hIndices.data(), sizeof(int32_t) * c->nnz, cudaMemcpyDefault));
    return EF_OK;
}

ef_status ef_update_csr(ef_ctx* c, const double* Kvij, double* csrData, void* stream) {
    EF_REQUIRE_FINALIZED(c);
    if (!c->scalar || !csrData) {
        ef_set_error("ef_update_csr: no scalar CSR map or null output");
        return EF_ERR_STATE;
    }
    cudaStream_t s = (cudaStream_t)stream;
    if (!Kvij) {
        if (!c->dKvijTmp) {
            ef_status st = EF_OK;
            c->dKvijTmp = dalloc<double>(c->nVIJ, &st);
            if (!c->dKvijTmp) return st;
        }
        EF_CHECK(ef_export_vij(c, c->dKvijTmp, stream));
        Kvij = c->dKvijTmp;
    }
    return ef_launch_csr_scatter(c->nnz, c->dCsrSeg, c->dCsrPerm, Kvij, csrData, s);
}

ef_status ef_csr_dirichlet_rows(ef_ctx* c, double* csrData, const int64_t* rows, int64_t nRows, void* stream) {
    EF_REQUIRE_FINALIZED(c);
    if (!c->scalar || !csrData || (nRows > 0 && !rows)) return EF_ERR_ARG;
    if (nRows == 0) return EF_OK;
    for (int64_t i = 0; i < nRows; ++i)
        if (rows[i] < 0 || rows[i] >= c->nDof) {
            ef_set_error("ef_csr_dirichlet_rows: row out of range");
            return EF_ERR_ARG;
        }
    ef_status st = EF_OK;
    int64_t* d = dalloc<int64_t>(nRows, &st);
    if (!d) return st;
    cudaStream_t s = (cudaStream_t)stream;
    cudaMemcpyAsync(d, rows, sizeof(int64_t) * nRows, cudaMemcpyHostToDevice, s);
    st = ef_launch_csr_dirichlet_rows(nRows, d, c->dIndptr, c->dIndices, csrData, s);
    cudaStreamSynchronize(s);
    cudaFree(d);
    return st;
}

ef_status ef_set_dirichlet(ef_ctx* c, const int64_t* dofs, int64_t n) {
    EF_REQUIRE_FINALIZED(c);
    std::vector<uint8_t> m(c->nDof, 0);
    for (int64_t i = 0; i < n; ++i) {
        if (dofs[i] < 0 || dofs[i] >= c->nDof) {
            ef_set_error("ef_set_dirichlet: DOF out of range");
            return EF_ERR_ARG;
        }
        m[dofs[i]] = 1;
    }
    {
        ef_status st = EF_OK;
        if (c->dDirIdx) cudaFree(c->dDirIdx);
        if (c->dDirMask) cudaFree(c->dDirMask);
        c->dDirIdx = nullptr;
        c->dDirMask = nullptr;
        c->nDir = n;
        if (n > 0) {
            c->dDirIdx = dalloc<int64_t>((size_t)n, &st);
            if (!c->dDirIdx) return st;
            EF_CUDA(cudaMemcpy(c->dDirIdx, dofs, sizeof(int64_t) * n, cudaMemcpyHostToDevice));
        }
        c->dDirMask = dalloc<uint8_t>((size_t)c->nDof, &st);
        if (!c->dDirMask) return st;
        EF_CUDA(cudaMemcpy(c->dDirMask, m.data(), c->nDof, cudaMemcpyHostToDevice));
    }
    for (int32_t sN : c->hTieS)
        for (int k = 0; k < 3; ++k) m[3 * (int64_t)sN + k] = 1;
    c->anyDirichlet = n > 0 || !c->hTieS.empty();
    EF_CUDA(cudaMemcpy(c->dMask, m.data(), c->nDof, cudaMemcpyHostToDevice));
    c->hMask = std::move(m);
    c->amgStale = true;
    c->amgMaskChanged = true;
    c->nnEdgeStale = true;
    c->nnVersion++;
    return EF_OK;
}

ef_status ef_assemble_bsr(ef_ctx* c, void* stream) {
    EF_REQUIRE_FINALIZED(c);
    cudaStream_t s = (cudaStream_t)stream;
    c->sellStale = true;
    EF_CHECK(ef_launch_bsr_scatter(c->nBlocks, c->dBsrSeg, c->dBsrSrc, c->dBsrW, c->Kblk, c->keFp64, c->dBsrVals, s));
    EF_CHECK(ef_launch_bj_setup(c->nNodes, c->dDiagPos, c->dNodeDof, c->dMask, c->dBsrVals, c->keFp64, c->dBinv,
                                c->dFlags, s));
    c->amgStale = true;
    c->nnEdgeStale = true;
    c->nnVersion++;
    return EF_OK;
}

ef_status ef_bsr_matvec(ef_ctx* c, const double* x, double* y, void* stream) {
    EF_REQUIRE_FINALIZED(c);
    return ef_launch_bsr_residual((int)c->nNodes, c->dRowPtr, c->dColIdx, c->dBsrVals, c->keFp64, x, nullptr,
                                  c->anyDirichlet ? c->dMask : nullptr, y, c->nSM, (cudaStream_t)stream);
}

// r = b - K x on free rows (0 on Dirichlet rows): with the exact FP64 tangent (matrix-free element
// apply) when the system is stored in FP32, else with the stored system
static ef_status residual64(ef_ctx* c, const double* x, const double* b, double* r, cudaStream_t s) {
    if (!c->exact)
        return ef_launch_bsr_residual((int)c->nNodes, c->dRowPtr, c->dColIdx, c->dBsrVals, c->keFp64, x, b, c->dMask,
                                      r, c->nSM, s);
    double* y = c->w64[4];
    if (c->dTieS) {  // the element apply needs the tied DOFs filled from their masters
        EF_CUDA(cudaMemcpyAsync(c->dTieTmp, x, sizeof(double) * c->nDof, cudaMemcpyDeviceToDevice, s));
        EF_CHECK(ef_launch_tie_fill((int64_t)c->hTieS.size(), c->dTieS, c->dTieA, c->dTieB, c->dTieTmp, s));
        x = c->dTieTmp;
    }
    for (size_t gi = 0; gi < c->groups.size(); ++gi) {
        const Group& g = c->groups[gi];
        if (g.tl)
            EF_CHECK(ef_launch_total_lagrange_apply(g, x, c->dTang[gi], c->dYe + g.peOffset, s));
        else
            EF_CHECK(ef_launch_small_strain_apply(g, x, c->dTang[gi], c->dYe + g.peOffset, s));
    }
    EF_CHECK(ef_launch_condense(c->nNodes, c->dNodeDof, c->dCondPtr, c->dCondSrc, c->dCondW, c->dYe, y, nullptr, s));
    return ef_launch_residual_from(c->nDof, b, y, c->dMask, r, s);
}

static ef_status dot_host(ef_ctx* c, const double* a, const double* b, double* out, cudaStream_t s) {
    EF_CHECK(ef_launch_dot(c->nDof, a, b, c->dPart, c->nPart, c->dRed, s));
    EF_CUDA(cudaMemcpyAsync(out, c->dRed, sizeof(double), cudaMemcpyDeviceToHost, s));
    EF_CUDA(cudaStreamSynchronize(s));
    return EF_OK;
}

// one PCG launch on the free DOFs: solves K d = rhs (rhs zero on Dirichlet DOFs)
static ef_status run_pcg(ef_ctx* c, int vDouble, const void* rhs, void* sol, int maxIter, double rtol,
                         PcgResultHost* out, ef_solve_info* prof, cudaStream_t s) {
    void** w = vDouble ? c->w64k : c->w32;
    EF_CUDA(cudaMemsetAsync(c->dBar, 0, ef_barrier_state_bytes(), s));
    if (prof) EF_CUDA(cudaEventRecord(c->ev[0], s));
    EF_CHECK(ef_launch_pcg(vDouble, c->pcgGrid[vDouble], (int)c->nNodes, c->dRowPtr, c->dColIdx, c->dBsrVals, c->dBinv,
                           c->dMask, rhs, sol, w[2], w[3], w[4], w[5], w[6], c->dPartA, c->dPartB, c->dBar,
                           c->dPcgRes, maxIter, rtol * rtol, c->dFlags, s));
    if (prof) EF_CUDA(cudaEventRecord(c->ev[1], s));
    EF_CUDA(cudaMemcpyAsync(out, c->dPcgRes, sizeof(PcgResultHost), cudaMemcpyDeviceToHost, s));
    EF_CUDA(cudaStreamSynchronize(s));
    if (prof) {
        float ms = 0.f;
        EF_CUDA(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
        prof->kernelMs += ms;
        prof->kernelLaunches += 1;
    }
    int f = 0;
    EF_CUDA(cudaMemcpy(&f, c->dFlags, sizeof(int), cudaMemcpyDeviceToHost));
    if (f & EF_FLAG_BARRIER) {
        ef_set_error("PCG: grid barrier timed out");
        return EF_ERR_DEVICE;
    }
    return EF_OK;
}


}  // extern "C"

// ---- aggregation multigrid (host setup, device refresh and V-cycle) -------------------------

// greedy aggregation of a block graph: seeds take their whole (unaggregated) neighbourhood,
// left-over nodes join a neighbouring seed aggregate; nodes coupled to nothing but themselves
// (tied nodes, whose DOFs are eliminated) all share one aggregate, so they coarsen away
static int aggregate(int n, const std::vector<int32_t>& rowPtr, const std::vector<int32_t>& colIdx,
                     std::vector<int32_t>& agg) {
    agg.assign(n, -1);
    int nAgg = 0;
    int iso = -1;
    for (int m = 0; m < n; ++m)
        if (rowPtr[m + 1] - rowPtr[m] <= 1) {
            if (iso < 0) iso = nAgg++;
            agg[m] = iso;
        }
    for (int m = 0; m < n; ++m) {
        if (agg[m] != -1) continue;
        bool free = true;
        for (int k = rowPtr[m]; k < rowPtr[m + 1]; ++k)
            if (agg[colIdx[k]] != -1) {
                free = false;
                break;
            }
        if (!free) continue;
        for (int k = rowPtr[m]; k < rowPtr[m + 1]; ++k) agg[colIdx[k]] = nAgg;
        agg[m] = nAgg++;
    }
    std::vector<int32_t> first = agg;
    for (int m = 0; m < n; ++m) {
        if (agg[m] != -1) continue;
        for (int k = rowPtr[m]; k < rowPtr[m + 1]; ++k)
            if (first[colIdx[k]] != -1) {
                agg[m] = first[colIdx[k]];
                break;
            }
    }
    for (int m = 0; m < n; ++m)
        if (agg[m] == -1) agg[m] = nAgg++;
    return nAgg;
}

template <typename T>
static ef_status upload(T** dst, const std::vector<T>& v) {
    ef_status st = EF_OK;
    *dst = dalloc<T>(std::max<size_t>(1, v.size()), &st);
    if (!*dst) return st;
    if (!v.empty()) EF_CUDA(cudaMemcpy(*dst, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
    return EF_OK;
}

// vectors of the FGMRES preconditioner (input, output) and the fine-level work vectors (also
// the FGMRES restart residual), whichever base preconditioner runs
static ef_status amg_workspace(ef_ctx* c) {
    ef_status st = EF_OK;
    if (!c->vcIn) c->vcIn = dalloc<float>(c->nDof, &st);
    if (!c->vcOut) c->vcOut = dalloc<float>(c->nDof, &st);
    if (!c->fineX) c->fineX = dalloc<float>(c->nDof, &st);
    if (!c->fineT) c->fineT = dalloc<float>(c->nDof, &st);
    return (c->vcIn && c->vcOut && c->fineX && c->fineT) ? EF_OK : st;
}

// ---- sliced-ELL copy of the fine system (kernels in sell.cu) ---------------------------------

// Layout, decided once: slices of 32 block rows in their natural order; when that pads the slots
// by more than 15 % over the blocks, rows are sorted by length (longest first) within windows of
// 4096 rows and the permutation is kept if it pads less; above 50 % padding after that (or with
// EF_SELL=0, or an FP64 system) the CSR kernels stay in use.
static ef_status sell_build(ef_ctx* c) {
    if (c->sellMode >= 0) return EF_OK;
    c->sellMode = 0;
    if (const char* e = getenv("EF_SELL"))
        if (atoi(e) == 0) return EF_OK;
    const int n0 = (int)c->nNodes;
    const std::vector<int32_t>& rp = c->hRowPtr0;
    const std::vector<int32_t>& ci = c->hColIdx0;
    if (c->keFp64 || n0 <= 0 || (int64_t)rp.size() != (int64_t)n0 + 1) return EF_OK;
    auto len = [&](int m) { return rp[m + 1] - rp[m]; };
    auto slots = [&](const std::vector<int32_t>& order) {
        int64_t tot = 0;
        for (int s0 = 0; s0 < n0; s0 += 32) {
            int w = 0;
            for (int r = s0; r < std::min(s0 + 32, n0); ++r) w = std::max(w, len(order.empty() ? r : order[r]));
            tot += 32 * (int64_t)w;
        }
        return tot;
    };
    std::vector<int32_t> perm;
    int64_t nE = slots(perm);
    const double nb = (double)c->nBlocks;
    if (nE > 1.15 * nb) {
        std::vector<int32_t> p(n0);
        for (int m = 0; m < n0; ++m) p[m] = m;
        const int W = 4096;
        for (int w0 = 0; w0 < n0; w0 += W)
            std::stable_sort(p.begin() + w0, p.begin() + std::min(w0 + W, n0),
                             [&](int a, int b) { return len(a) > len(b); });
        const int64_t nE2 = slots(p);
        if (nE2 < nE) {
            nE = nE2;
            perm.swap(p);
        }
    }
    if (nE > 1.5 * nb || nE >= ((int64_t)1 << 31) / 9) return EF_OK;
    const int nS = (n0 + 31) / 32;
    std::vector<int64_t> off(nS + 1, 0);
    std::vector<int32_t> col(nE), src(nE);
    for (int s = 0; s < nS; ++s) {
        int w = 0;
        for (int r = 32 * s; r < std::min(32 * s + 32, n0); ++r) w = std::max(w, len(perm.empty() ? r : perm[r]));
        off[s + 1] = off[s] + 32 * (int64_t)w;
        for (int j = 0; j < w; ++j)
            for (int i = 0; i < 32; ++i) {
                const int r = 32 * s + i;
                const int64_t t = off[s] + 32 * (int64_t)j + i;
                if (r < n0) {
                    const int m = perm.empty() ? r : perm[r];
                    const bool real = j < len(m);
                    src[t] = real ? rp[m] + j : -1;
                    col[t] = real ? ci[rp[m] + j] : m;
                } else {
                    src[t] = -1;
                    col[t] = n0 - 1;
                }
            }
    }
    ef_status st = EF_OK;
    EF_CHECK(upload(&c->dSellOff, off));
    EF_CHECK(upload(&c->dSellCol, col));
    EF_CHECK(upload(&c->dSellSrc, src));
    if (!perm.empty()) EF_CHECK(upload(&c->dSellPerm, perm));
    c->dSellV9 = dalloc<float>(9 * (size_t)nE, &st);
    if (!c->dSellV9) return st;
    if (c->amgBf16) {
        c->dSellV8 = dalloc<uint4>((size_t)nE, &st);
        c->dSellV1 = dalloc<uint16_t>((size_t)nE, &st);
        if (!c->dSellV8 || !c->dSellV1) return st;
    }
    c->sellSlices = nS;
    c->sellE = nE;
    c->sellMode = 1;
    c->sellStale = true;
    return EF_OK;
}

// the SELL values from the assembled FP32 blocks (after every assembly)
static ef_status sell_refresh(ef_ctx* c, cudaStream_t s) {
    EF_CHECK(sell_build(c));
    if (c->sellMode != 1 || !c->sellStale) return EF_OK;
    EF_CHECK(ef_launch_sell_refresh(c->sellE, c->dSellSrc, (const float*)c->dBsrVals, c->dSellV9, c->dSellV8,
                                    c->dSellV1, s));
    c->sellStale = false;
    return EF_OK;
}

static ef_status amg_build(ef_ctx* c) {
    if (!c->amg.empty()) return EF_OK;
    if (const char* e = getenv("EF_AMG_SMOOTHED")) c->amgSmoothed = atoi(e) != 0;
    // smoothed prolongators: one sweep before and after, V-cycle (the fastest cfg 2 load step of
    // 1/1, 2/2 x V, W on level 1); plain aggregation: two sweeps and a W-cycle on level 1
    if (c->amgSmoothed) {
        c->amgSweeps = 1;
        c->amgWLevels = 0;
    }
    if (const char* e = getenv("EF_AMG_OMEGA")) c->amgOmega = (float)atof(e);
    if (const char* e = getenv("EF_AMG_SWEEPS")) c->amgSweeps = std::max(1, atoi(e));
    c->amgPre = c->amgPost = c->amgSweeps;
    if (const char* e = getenv("EF_AMG_PRE")) c->amgPre = std::max(1, atoi(e));
    if (const char* e = getenv("EF_AMG_POST")) c->amgPost = std::max(1, atoi(e));
    if (const char* e = getenv("EF_AMG_WLEVELS")) c->amgWLevels = std::max(0, atoi(e));
    c->amgPreC = c->amgPre;
    c->amgPostC = c->amgPost;
    if (const char* e = getenv("EF_AMG_PRE_COARSE")) c->amgPreC = std::max(1, atoi(e));
    if (const char* e = getenv("EF_AMG_POST_COARSE")) c->amgPostC = std::max(1, atoi(e));
    if (const char* e = getenv("EF_AMG_ALPHA")) c->amgAlpha = (float)atof(e);
    if (const char* e = getenv("EF_AMG_CYCLE")) c->amgCycle = std::max(1, atoi(e));
    if (const char* e = getenv("EF_AMG_BF16")) c->amgBf16 = atoi(e) != 0;
    if (const char* e = getenv("EF_AMG_SMOOTHER")) c->amgCheb = strcmp(e, "cheb") == 0;
    if (const char* e = getenv("EF_AMG_CLUSTER")) c->amgCluster = atoi(e) != 0;
    if (const char* e = getenv("EF_AMG_BF16_COARSE")) c->amgBf16Coarse = atoi(e) != 0;
    if (c->amgSmoothed && !getenv("EF_AMG_ALPHA")) c->amgAlpha = 1.0f;  // smoothed prolongators need no over-correction
    ef_status st = EF_OK;
    const int n0 = (int)c->nNodes;
    const int BCo = ef_amg_coarse_dofs();
    // fine block -> block row
    std::vector<int32_t> rob0(c->nBlocks);
    for (int m = 0; m < n0; ++m)
        for (int k = c->hRowPtr0[m]; k < c->hRowPtr0[m + 1]; ++k) rob0[k] = m;
    EF_CHECK(upload(&c->dRowOfBlock0, rob0));
    EF_CHECK(amg_workspace(c));
    EF_CHECK(sell_build(c));
    if (c->amgBf16 && c->sellMode != 1) {  // (with the SELL copy the fine level reads its BF16 values)
        c->dBsrValsH = dalloc<uint16_t>((size_t)c->nBlocks * 9 + 32, &st);  // 16-byte words + 1 value per block (+ padding)
        if (!c->dBsrValsH) return st;
        bool staged = false;  // measured slower than the unstaged kernel (EF_AMG_STAGED=1 turns it on)
        if (const char* e = getenv("EF_AMG_STAGED")) staged = atoi(e) != 0;
        c->stageCap = staged ? ef_stage_cap(n0, c->hRowPtr0.data()) : 0;
        if (c->stageCap > 4096) c->stageCap = 0;  // rows too long for a shared-memory stage: unstaged kernel
    }
    const std::vector<int32_t>* pRow = &c->hRowPtr0;
    const std::vector<int32_t>* pCol = &c->hColIdx0;
    std::vector<double> finePos(3 * (size_t)n0);
    for (int m = 0; m < n0; ++m)
        for (int k = 0; k < 3; ++k) finePos[3 * m + k] = c->hX[3 * m + k];
    const std::vector<double>* pPos = &finePos;
    int nFine = n0;
    while (nFine > ef_max_coarsest_nodes()) {
        AmgLevel L;
        // frees the level's device arrays on an early error return, until the context owns them
        struct Guard {
            AmgLevel* L;
            ~Guard() {
                if (L) L->free_device();
            }
        } guard{&L};
        const int nC = aggregate(nFine, *pRow, *pCol, L.hAgg);
        if (nC >= nFine) break;  // no coarsening progress
        L.nN = nC;
        // members of each coarse node (increasing finer index), centroids and offsets
        L.hAggPtr.assign(nC + 1, 0);
        for (int m = 0; m < nFine; ++m) L.hAggPtr[L.hAgg[m] + 1]++;
        for (int I = 0; I < nC; ++I) L.hAggPtr[I + 1] += L.hAggPtr[I];
        L.hAggIdx.resize(nFine);
        {
            std::vector<int32_t> fill(L.hAggPtr.begin(), L.hAggPtr.end() - 1);
            for (int m = 0; m < nFine; ++m) L.hAggIdx[fill[L.hAgg[m]]++] = m;
        }
        L.hCentroid.assign(3 * (size_t)nC, 0.0);
        for (int m = 0; m < nFine; ++m)
            for (int k = 0; k < 3; ++k) L.hCentroid[3 * L.hAgg[m] + k] += (*pPos)[3 * m + k];
        for (int I = 0; I < nC; ++I) {
            const double cnt = (double)(L.hAggPtr[I + 1] - L.hAggPtr[I]);
            for (int k = 0; k < 3; ++k) L.hCentroid[3 * I + k] /= cnt;
        }
        L.hOffs.resize(3 * (size_t)nFine);
        for (int m = 0; m < nFine; ++m)
            for (int k = 0; k < 3; ++k) L.hOffs[3 * m + k] = (float)((*pPos)[3 * m + k] - L.hCentroid[3 * L.hAgg[m] + k]);
        // coarse pattern: aggregate adjacency, or with smoothed prolongators the pattern of P^T A P
        // (a superset)
        std::vector<std::vector<int32_t>> cols(nC);
        SAPattern SA;
        if (c->amgSmoothed) {
            build_sa_pattern(nFine, pRow->data(), pCol->data(), L.hAgg.data(), nC, SA);
            for (int I = 0; I < nC; ++I) cols[I].assign(SA.cCol.begin() + SA.cRowPtr[I], SA.cCol.begin() + SA.cRowPtr[I + 1]);
        } else {
            for (int m = 0; m < nFine; ++m)
                for (int k = (*pRow)[m]; k < (*pRow)[m + 1]; ++k) cols[L.hAgg[m]].push_back(L.hAgg[(*pCol)[k]]);
        }
        L.hRowPtr.assign(nC + 1, 0);
        for (int I = 0; I < nC; ++I) {
            auto& v = cols[I];
            std::sort(v.begin(), v.end());
            v.erase(std::unique(v.begin(), v.end()), v.end());
            L.hRowPtr[I + 1] = L.hRowPtr[I] + (int32_t)v.size();
        }
        L.nBlocks = L.hRowPtr[nC];
        L.hColIdx.resize(L.nBlocks);
        std::vector<int32_t> rob(L.nBlocks);
        std::vector<int64_t> diag(nC, -1);
        for (int I = 0; I < nC; ++I)
            for (size_t j = 0; j < cols[I].size(); ++j) {
                const int64_t k = L.hRowPtr[I] + (int64_t)j;
                L.hColIdx[k] = cols[I][j];
                rob[k] = I;
                if (cols[I][j] == I) diag[I] = k;
            }
        // Galerkin map: finer blocks in increasing order, grouped by their coarse block
        const int64_t nFineBlocks = (*pRow)[nFine];
        std::vector<int64_t> gcount(L.nBlocks + 1, 0);
        std::vector<int32_t> target(nFineBlocks);
        for (int m = 0; m < nFine; ++m) {
            const int I = L.hAgg[m];
            for (int k = (*pRow)[m]; k < (*pRow)[m + 1]; ++k) {
                const int J = L.hAgg[(*pCol)[k]];
                const int32_t* b = L.hColIdx.data() + L.hRowPtr[I];
                const int32_t* e = L.hColIdx.data() + L.hRowPtr[I + 1];
                const int64_t S = L.hRowPtr[I] + (std::lower_bound(b, e, J) - b);
                target[k] = (int32_t)S;
                gcount[S + 1]++;
            }
        }
        for (int64_t S = 0; S < L.nBlocks; ++S) gcount[S + 1] += gcount[S];
        std::vector<int32_t> gsrc(nFineBlocks);
        {
            std::vector<int64_t> fill(gcount.begin(), gcount.end() - 1);
            for (int64_t f = 0; f < nFineBlocks; ++f) gsrc[fill[target[f]]++] = (int32_t)f;
        }
        EF_CHECK(upload(&L.rowPtr, L.hRowPtr));
        EF_CHECK(upload(&L.colIdx, L.hColIdx));
        EF_CHECK(upload(&L.rowOfBlock, rob));
        EF_CHECK(upload(&L.diagPos, diag));
        EF_CHECK(upload(&L.agg, L.hAgg));
        EF_CHECK(upload(&L.offs, L.hOffs));
        EF_CHECK(upload(&L.aggPtr, L.hAggPtr));
        EF_CHECK(upload(&L.aggIdx, L.hAggIdx));
        EF_CHECK(upload(&L.gseg, gcount));
        EF_CHECK(upload(&L.gsrc, gsrc));
        if (c->amgSmoothed) {
            L.saNP = (int64_t)SA.pCol.size();
            L.saNAP = (int64_t)SA.apCol.size();
            std::vector<int32_t> apRow(L.saNAP);
            for (int m = 0; m < nFine; ++m)
                for (int32_t a = SA.apRowPtr[m]; a < SA.apRowPtr[m + 1]; ++a) apRow[a] = m;
            EF_CHECK(upload(&L.saPRowPtr, SA.pRowPtr));
            EF_CHECK(upload(&L.saPCol, SA.pCol));
            EF_CHECK(upload(&L.saPRow, SA.pRow));
            EF_CHECK(upload(&L.saPSeg, SA.pSeg));
            EF_CHECK(upload(&L.saPSrc, SA.pSrc));
            EF_CHECK(upload(&L.saTPtr, SA.tPtr));
            EF_CHECK(upload(&L.saTIdx, SA.tIdx));
            EF_CHECK(upload(&L.saApRow, apRow));
            EF_CHECK(upload(&L.saApSeg, SA.apSeg));
            EF_CHECK(upload(&L.saApK, SA.apK));
            EF_CHECK(upload(&L.saApP, SA.apP));
            EF_CHECK(upload(&L.saCSeg, SA.cSeg));
            EF_CHECK(upload(&L.saCP, SA.cP));
            EF_CHECK(upload(&L.saCAP, SA.cAP));
            const int bfL = c->amg.empty() ? 3 : BCo;
            L.saPv = dalloc<float>((size_t)std::max<int64_t>(1, L.saNP) * bfL * BCo, &st);
            L.saAPv = dalloc<float>((size_t)std::max<int64_t>(1, L.saNAP) * bfL * BCo, &st);
            L.saW = dalloc<float>(1, &st);
            if (!L.saPv || !L.saAPv || !L.saW) return st;
        }
        L.vals = dalloc<float>((size_t)L.nBlocks * BCo * BCo, &st);
        L.binv = dalloc<float>((size_t)nC * BCo * BCo, &st);
        L.dead = dalloc<uint8_t>((size_t)BCo * nC, &st);
        L.x = dalloc<float>((size_t)BCo * nC, &st);
        L.r = dalloc<float>((size_t)BCo * nC, &st);
        L.t = dalloc<float>((size_t)BCo * nC, &st);
        L.x2 = dalloc<float>((size_t)BCo * nC, &st);
        if (!L.vals || !L.binv || !L.dead || !L.x || !L.r || !L.t || !L.x2) return st;
        if (c->amgBf16Coarse) {
            L.valsH = dalloc<uint16_t>((size_t)L.nBlocks * BCo * BCo, &st);
            if (!L.valsH) return st;
        }
        guard.L = nullptr;
        c->amg.push_back(std::move(L));
        pRow = &c->amg.back().hRowPtr;
        pCol = &c->amg.back().hColIdx;
        pPos = &c->amg.back().hCentroid;
        nFine = nC;
    }
    c->chebD.assign(c->amg.size(), nullptr);  // Chebyshev directions of the smoothed levels
    for (size_t l = 0; l < c->amg.size(); ++l) {
        const size_t nl = l == 0 ? (size_t)c->nDof : (size_t)BCo * c->amg[l - 1].nN;
        c->chebD[l] = dalloc<float>(nl, &st);
        if (!c->chebD[l]) return st;
    }
    if (c->amg.empty() || c->amg.back().nN > ef_max_coarsest_nodes()) {
        ef_set_error("multigrid: the block graph does not coarsen to a dense-solvable size");
        return EF_ERR_ARG;
    }
    const int nc = BCo * c->amg.back().nN;
    c->amgCoarsestInv = dalloc<float>((size_t)nc * nc, &st);
    if (!c->amgCoarsestInv) return st;
    EF_CHECK(amg_workspace(c));
    c->amgStale = true;
    return EF_OK;
}

static ef_status amg_vcycle(ef_ctx* c, int l, const float* r, float* x, cudaStream_t s);

// capture the preconditioner application (fixed device pointers; values may change later)
// Phase program of the cycle at level l >= 1 (6-DOF nodes) from right-hand side r into x: the
// same operations, order and buffers as amg_vcycle's block-Jacobi path.
static void amg_cycle_ops(const ef_ctx* c, int l, const float* r, float* x, std::vector<ef::CoarseOp>& ops) {
    const int nL = (int)c->amg.size();
    const int BCo = ef_amg_coarse_dofs();
    auto op = [](int type, int n) {
        ef::CoarseOp o{};
        o.type = type;
        o.n = n;
        return o;
    };
    if (l == nL) {
        const AmgLevel& C = c->amg.back();
        ef::CoarseOp o = op(ef::COP_COARSEST, BCo * C.nN);
        o.f0 = c->amgCoarsestInv;
        o.in = r;
        o.mask = C.dead;
        o.out = x;
        ops.push_back(o);
        return;
    }
    const AmgLevel& L = c->amg[l - 1];
    const AmgLevel& Cn = c->amg[l];
    const float omega = l < (int)c->levelOmega.size() ? c->levelOmega[l] : c->amgOmega;
    auto sweep = [&](const float* xin, float* xout) {
        ef::CoarseOp o = op(ef::COP_SWEEP, L.nN);
        o.p0 = L.rowPtr;
        o.p1 = L.colIdx;
        o.f0 = L.vals;
        o.f1 = L.binv;
        o.mask = L.dead;
        o.in = xin;
        o.rhs = r;
        o.out = xout;
        o.omega = omega;
        ops.push_back(o);
    };
    float* x2 = L.x2;
    float* cur = ((c->amgPreC + c->amgPostC) & 1) ? x : x2;
    {
        ef::CoarseOp o = op(ef::COP_BJ, L.nN);
        o.f1 = L.binv;
        o.mask = L.dead;
        o.in = r;
        o.out = cur;
        o.omega = omega;
        ops.push_back(o);
    }
    for (int k = 1; k < c->amgPreC; ++k) {
        float* nxt = cur == x ? x2 : x;
        sweep(cur, nxt);
        cur = nxt;
    }
    const int reps = (c->amgCycle > 1 && l <= c->amgWLevels) ? c->amgCycle : 1;
    for (int rep = 0; rep < reps; ++rep) {
        ef::CoarseOp o = op(ef::COP_RESID, L.nN);
        o.p0 = L.rowPtr;
        o.p1 = L.colIdx;
        o.f0 = L.vals;
        o.mask = L.dead;
        o.in = cur;
        o.rhs = r;
        o.out = L.t;
        ops.push_back(o);
        ef::CoarseOp rs = op(ef::COP_RESTRICT, Cn.nN);
        rs.p0 = Cn.aggPtr;
        rs.p1 = Cn.aggIdx;
        rs.f0 = Cn.offs;
        rs.mask = Cn.dead;
        rs.in = L.t;
        rs.out = Cn.r;
        ops.push_back(rs);
        amg_cycle_ops(c, l + 1, Cn.r, Cn.x, ops);
        ef::CoarseOp pr = op(ef::COP_PROLONG, L.nN);
        pr.p0 = Cn.agg;
        pr.f0 = Cn.offs;
        pr.mask = L.dead;
        pr.in = Cn.x;
        pr.out = cur;
        pr.omega = c->amgAlpha;
        ops.push_back(pr);
    }
    for (int k = 0; k < c->amgPostC; ++k) {
        float* nxt = cur == x ? x2 : x;
        sweep(cur, nxt);
        cur = nxt;
    }
}

// Chooses the level whose coarse correction (restriction, the whole cycle below, prolongation)
// runs as one coarse_cycle_kernel launch: the first level >= 1 whose next coarser level has at
// most kClusterMaxNodes nodes; builds and uploads its phase program (before a graph capture).
static ef_status amg_prepare_cluster(ef_ctx* c) {
    constexpr int kClusterMaxNodes = 2048;
    c->clusterLevel = -1;
    c->nCoarseOps = 0;
    const int nL = (int)c->amg.size();
    if (!c->amgCluster || c->amgCheb || c->amgSmoothed) return EF_OK;
    int lc = -1;
    for (int l = 1; l < nL; ++l)
        if (c->amg[l].nN <= kClusterMaxNodes) {
            lc = l;
            break;
        }
    if (lc < 0) return EF_OK;
    const AmgLevel& L = c->amg[lc - 1];
    const AmgLevel& Cn = c->amg[lc];
    // level lc's iterate at its coarse correction: amg_vcycle's buffer alternation of the
    // pre-smoothing replayed (level lc's output vector is L.x, its second vector L.x2)
    float* x = L.x;
    float* cur = ((c->amgPreC + c->amgPostC) & 1) ? x : L.x2;
    for (int k = 1; k < c->amgPreC; ++k) cur = cur == x ? L.x2 : x;
    std::vector<ef::CoarseOp> ops;
    ef::CoarseOp rs{};
    rs.type = ef::COP_RESTRICT;
    rs.n = Cn.nN;
    rs.p0 = Cn.aggPtr;
    rs.p1 = Cn.aggIdx;
    rs.f0 = Cn.offs;
    rs.mask = Cn.dead;
    rs.in = L.t;
    rs.out = Cn.r;
    ops.push_back(rs);
    amg_cycle_ops(c, lc + 1, Cn.r, Cn.x, ops);
    ef::CoarseOp pr{};
    pr.type = ef::COP_PROLONG;
    pr.n = L.nN;
    pr.p0 = Cn.agg;
    pr.f0 = Cn.offs;
    pr.mask = L.dead;
    pr.in = Cn.x;
    pr.out = cur;
    pr.omega = c->amgAlpha;
    ops.push_back(pr);
    if (!c->dCoarseOps || (int)ops.size() > c->nCoarseOpsCap) {
        if (c->dCoarseOps) cudaFree(c->dCoarseOps);
        c->dCoarseOps = nullptr;
        ef_status st = EF_OK;
        c->dCoarseOps = dalloc<ef::CoarseOp>(ops.size(), &st);
        if (!c->dCoarseOps) return st;
        c->nCoarseOpsCap = (int)ops.size();
    }
    EF_CUDA(cudaMemcpy(c->dCoarseOps, ops.data(), sizeof(ef::CoarseOp) * ops.size(), cudaMemcpyHostToDevice));
    c->nCoarseOps = (int)ops.size();
    c->clusterLevel = lc;
    c->clusterCur = cur;
    return EF_OK;
}

static ef_status amg_capture(ef_ctx* c) {
    if (c->vcGraph) return EF_OK;
    EF_CHECK(amg_prepare_cluster(c));
    if (!c->capStream) EF_CUDA(cudaStreamCreateWithFlags(&c->capStream, cudaStreamNonBlocking));
    EF_CUDA(cudaStreamBeginCapture(c->capStream, cudaStreamCaptureModeThreadLocal));
    long long captured = 0;
    t_captureCount = &captured;
    const ef_status st = amg_vcycle(c, 0, c->vcIn, c->vcOut, c->capStream);
    t_captureCount = nullptr;
    c->vcGraphKernels = captured;
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(c->capStream, &g);
    if (st != EF_OK) return st;
    if (e != cudaSuccess) {
        ef_set_error(std::string("V-cycle capture: ") + cudaGetErrorString(e));
        return EF_ERR_CUDA;
    }
    EF_CUDA(cudaGraphInstantiate(&c->vcGraph, g, 0));
    cudaGraphDestroy(g);
    return EF_OK;
}

// A coarse DOF (translation or rotation of an aggregate) is dead when its prolongation column
// vanishes on every live finer DOF (all members clamped, or a rotation about an axis through
// all free members).
static void amg_dead_mask(const AmgLevel& L, int bf, const uint8_t* fineDead, std::vector<uint8_t>& dead) {
    const int BCo = ef_amg_coarse_dofs();
    dead.assign((size_t)BCo * L.nN, 1);
    for (int I = 0; I < L.nN; ++I) {
        double colNorm[6] = {0, 0, 0, 0, 0, 0};
        double scale = 0.0;
        for (int k = L.hAggPtr[I]; k < L.hAggPtr[I + 1]; ++k) {
            const int m = L.hAggIdx[k];
            const double dx = L.hOffs[3 * m], dy = L.hOffs[3 * m + 1], dz = L.hOffs[3 * m + 2];
            scale = std::max(scale, dx * dx + dy * dy + dz * dz);
            // rows of P_m (bf x 6)
            double P[6][6] = {};
            P[0][0] = P[1][1] = P[2][2] = 1.0;
            P[1][3] = -dz;
            P[2][3] = dy;
            P[0][4] = dz;
            P[2][4] = -dx;
            P[0][5] = -dy;
            P[1][5] = dx;
            if (bf == 6) P[3][3] = P[4][4] = P[5][5] = 1.0;
            for (int i = 0; i < bf; ++i) {
                if (fineDead[(size_t)bf * m + i]) continue;
                for (int j = 0; j < 6; ++j) colNorm[j] += P[i][j] * P[i][j];
            }
        }
        const double tol = 1e-12 * std::max(scale, 1e-300);
        for (int j = 0; j < 3; ++j) dead[BCo * I + j] = colNorm[j] > 0.5 ? 0 : 1;
        for (int j = 3; j < 6; ++j) dead[BCo * I + j] = colNorm[j] > tol && scale > 0.0 ? 0 : 1;
    }
}

// Damping of the block-Jacobi smoother on every smoothed level.  lambda, the largest eigenvalue of
// D^-1 A, is estimated by 12 power iterations from a fixed pseudo-random vector; damped Jacobi
// smoothing is stable for omega lambda < 2.  Where amgOmega lambda exceeds 1.85 (quadratic
// elements raise lambda well above its hex8 value of about 2) the level uses 4 / (3 lambda),
// quantised to 1/64 so that small changes keep the captured cycle; any change re-captures it.
static constexpr int kPowerSteps = 13;  // power-iteration steps per level

// scratch of the damping estimate (allocated once)
static ef_status amg_power_alloc(ef_ctx* c) {
    ef_status st = EF_OK;
    if (!c->amgPow[0]) {
        c->amgPow[0] = dalloc<float>(c->nDof, &st);
        c->amgPow[1] = dalloc<float>(c->nDof, &st);
        c->amgZero = dalloc<float>(c->nDof, &st);
        if (st != EF_OK) return st;
        EF_CUDA(cudaMemset(c->amgZero, 0, sizeof(float) * c->nDof));
    }
    if (!c->nnRed) {  // reduction scratch shared with the learned correction
        c->nnPartN = 2 * c->nSM;
        c->nnRed = dalloc<double>(3 * (size_t)c->nnPartN + 8, &st);
        if (!c->nnRed) return st;
    }
    const int nL = (int)c->amg.size();
    if (!c->amgNorms || c->amgNormsCap < 3 * kPowerSteps * nL) {
        if (c->amgNorms) cudaFree(c->amgNorms);
        c->amgNorms = dalloc<double>((size_t)3 * kPowerSteps * nL, &st);
        if (!c->amgNorms) return st;
        c->amgNormsCap = 3 * kPowerSteps * nL;
    }
    return EF_OK;
}

// lambda_max(D^-1 A) of level l by power iteration, entirely on the device (normalised by the
// device-side norm); the last step's squared norm, lambda^2, is left at
// amgNorms[3 (l kPowerSteps + kPowerSteps - 1)]
static ef_status amg_power(ef_ctx* c, int l, cudaStream_t s) {
    const int BCo = ef_amg_coarse_dofs();
    const bool fine = l == 0;
    const int bs = fine ? 3 : BCo;
    const int nN = fine ? (int)c->nNodes : c->amg[l - 1].nN;
    const int32_t* rowPtr = fine ? c->dRowPtr : c->amg[l - 1].rowPtr;
    const int32_t* colIdx = fine ? c->dColIdx : c->amg[l - 1].colIdx;
    const float* vals = fine ? (const float*)c->dBsrVals : c->amg[l - 1].vals;
    const float* binv = fine ? (const float*)c->dBinv : c->amg[l - 1].binv;
    const uint8_t* mask = fine ? c->dMask : c->amg[l - 1].dead;
    const int64_t n = (int64_t)bs * nN;
    float* a = c->amgPow[0];
    float* b = c->amgPow[1];
    EF_CHECK(ef_launch_fill_hash(n, a, s));
    for (int it = 0; it < kPowerSteps; ++it) {
        double* n2 = c->amgNorms + 3 * (l * kPowerSteps + it);
        EF_CHECK(ef_mpnn_sumsq(n, 1, a, nullptr, mask, c->nnRed, c->nnPartN, n2, s));
        if (it + 1 == kPowerSteps) break;
        EF_CHECK(ef_launch_scale_rnorm(n, a, n2, s));
        EF_CHECK(ef_launch_level_residual(bs, nN, rowPtr, colIdx, vals, a, c->amgZero, mask, b, s));  // -A a
        EF_CHECK(ef_launch_bj_apply(bs, nN, binv, mask, 1.f, b, a, 0, s));                            // D^-1
    }
    return EF_OK;
}

// per-level smoothing damping from the power-iteration norms (one transfer); the captured cycle
// graphs are dropped when a damping changes
static ef_status amg_damping_finish(ef_ctx* c, cudaStream_t s) {
    const int nL = (int)c->amg.size();
    std::vector<float> om(nL), lamq(nL);
    std::vector<double> hn(3 * (size_t)kPowerSteps * nL);
    EF_CUDA(cudaMemcpyAsync(hn.data(), c->amgNorms, sizeof(double) * hn.size(), cudaMemcpyDeviceToHost, s));
    EF_CUDA(cudaStreamSynchronize(s));
    for (int l = 0; l < nL; ++l) {
        // lambda: |D^-1 A a| for the unit vector a of the last step
        const double n2 = hn[3 * (l * kPowerSteps + kPowerSteps - 1)];
        const double lam = n2 > 0.0 ? sqrt(n2) : 0.0;
        float w = c->amgOmega;
        if (lam > 0.0 && lam == lam && c->amgOmega * lam > 1.85)  // close to the stability limit 2
            w = std::max(1.f, std::round((float)(4.0 / (3.0 * lam)) * 64.f)) / 64.f;
        om[l] = w;
        // lambda on a grid of 2^(1/16) steps for the Chebyshev bounds (stable captured cycles)
        lamq[l] = lam > 0.0 && lam == lam ? (float)exp2(std::ceil(16.0 * log2(lam)) / 16.0) : 2.f;
    }
    if (om != c->levelOmega || (c->amgCheb && lamq != c->levelLam)) {
        c->levelOmega = om;
        c->levelLam = lamq;
        if (c->vcGraph) {
            cudaGraphExecDestroy(c->vcGraph);
            c->vcGraph = nullptr;
        }
        if (c->nnGraph) {
            cudaGraphExecDestroy(c->nnGraph);
            c->nnGraph = nullptr;
        }
    }
    return EF_OK;
}

static ef_status amg_damping(ef_ctx* c, cudaStream_t s) {
    EF_CHECK(amg_power_alloc(c));
    for (int l = 0; l < (int)c->amg.size(); ++l) EF_CHECK(amg_power(c, l, s));
    return amg_damping_finish(c, s);
}

// edge weights of the learned correction for the current system
static ef_status nn_edge_refresh(ef_ctx* c, cudaStream_t s) {
    if (!c->nnInit || !c->nnEdgeStale) return EF_OK;
    EF_CHECK(ef_launch_edge_weights((int)c->nNodes, c->dRowPtr, c->dColIdx, (const float*)c->dBsrVals, c->nnA, s));
    EF_CHECK(ef_launch_gather_f32(c->nBlocks, c->nnTpos, c->nnA, c->nnAT, s));
    c->nnEdgeStale = false;
    return EF_OK;
}

// dead coarse DOFs from the current Dirichlet mask, then Galerkin values, block inverses, the
// coarsest inverse and the smoothing damping for the current fine system
static ef_status amg_refresh(ef_ctx* c, cudaStream_t s) {
    EF_CHECK(sell_refresh(c, s));
    if (!c->amgStale) return EF_OK;
    if (!c->amgMaskChanged && c->amgReuseLeft > 0) {
        // lagged coarse levels: the prolongators, coarse operators and damping of an earlier system
        // of the same pattern and mask; the fine level (blocks, block inverses, BF16 copy) is the
        // current system's
        c->amgReuseLeft--;
        if (c->dBsrValsH)
            EF_CHECK(ef_launch_to_bf16_split(c->nBlocks, (const float*)c->dBsrVals, c->dBsrValsH, s));
        c->amgStale = false;
        return nn_edge_refresh(c, s);
    }
    c->amgReuseLeft = c->amgMaxReuse;
    c->amgMaskChanged = false;
    const int BCo = ef_amg_coarse_dofs();
    const uint8_t* fineDead = c->hMask.data();
    for (size_t l = 0; l < c->amg.size(); ++l) {
        AmgLevel& L = c->amg[l];
        amg_dead_mask(L, l == 0 ? 3 : BCo, fineDead, L.hDead);
        EF_CUDA(cudaMemcpyAsync(L.dead, L.hDead.data(), L.hDead.size(), cudaMemcpyHostToDevice, s));
        fineDead = L.hDead.data();
    }
    if (c->amgSmoothed) EF_CHECK(amg_power_alloc(c));
    for (size_t l = 0; l < c->amg.size(); ++l) {
        AmgLevel& L = c->amg[l];
        const bool fine = l == 0;
        const int32_t* fRob = fine ? c->dRowOfBlock0 : c->amg[l - 1].rowOfBlock;
        const int32_t* fCol = fine ? c->dColIdx : c->amg[l - 1].colIdx;
        const float* fVals = fine ? (const float*)c->dBsrVals : c->amg[l - 1].vals;
        const uint8_t* fMask = fine ? c->dMask : c->amg[l - 1].dead;
        if (c->amgSmoothed) {
            // smoothed prolongator P = P_t - 4 / (3 lambda) D^-1 A P_t of the finer level (its lambda
            // from the power iteration on the device), then A P and P^T A P
            const float* fBinv = fine ? (const float*)c->dBinv : c->amg[l - 1].binv;
            EF_CHECK(amg_power(c, (int)l, s));
            EF_CHECK(ef_launch_sa_damping(c->amgNorms + 3 * ((int)l * kPowerSteps + kPowerSteps - 1), L.saW, s));
            EF_CHECK(ef_launch_sa_setup(fine ? 3 : BCo, L.saNP, L.saPRow, L.saPCol, L.saPSeg, L.saPSrc, L.saNAP,
                                        L.saApRow, L.saApSeg, L.saApK, L.saApP, fCol, fVals, fMask, L.offs, L.agg,
                                        fBinv, L.saW, L.saPv, L.saAPv, L.nBlocks, L.saCSeg, L.saCP, L.saCAP,
                                        L.rowOfBlock, L.colIdx, L.dead, L.vals, s));
        } else {
            EF_CHECK(ef_launch_galerkin(fine ? 3 : BCo, L.nBlocks, L.gseg, L.gsrc, fRob, fCol, fVals, fMask, L.offs,
                                        L.rowOfBlock, L.colIdx, L.dead, L.vals, s));
        }
        EF_CHECK(ef_launch_bj6_setup(L.nN, L.diagPos, L.vals, L.binv, s));
        if (L.valsH) EF_CHECK(ef_launch_to_bf16(L.nBlocks * BCo * BCo, L.vals, L.valsH, s));
    }
    const AmgLevel& C = c->amg.back();
    EF_CHECK(ef_launch_coarsest_inverse(C.nN, C.rowPtr, C.colIdx, C.vals, c->amgCoarsestInv, s));
    if (c->dBsrValsH)
        EF_CHECK(ef_launch_to_bf16_split(c->nBlocks, (const float*)c->dBsrVals, c->dBsrValsH, s));
    if (c->amgSmoothed) {
        EF_CHECK(amg_damping_finish(c, s));  // every level's power iteration ran above
    } else {
        EF_CHECK(amg_damping(c, s));
    }
    c->amgStale = false;
    return nn_edge_refresh(c, s);
}

// x = V-cycle(r) on level l (l = 0: the fine system); one damped block-Jacobi sweep before and
// after the coarse correction, dense solve on the coarsest level
static ef_status amg_vcycle(ef_ctx* c, int l, const float* r, float* x, cudaStream_t s) {
    const float omega = l < (int)c->levelOmega.size() ? c->levelOmega[l] : c->amgOmega;
    const int nL = (int)c->amg.size();
    const int BCo = ef_amg_coarse_dofs();
    if (l == nL) {
        const AmgLevel& C = c->amg.back();
        return ef_launch_coarsest_apply(BCo * C.nN, c->amgCoarsestInv, r, C.dead, x, s);
    }
    const bool fine = l == 0;
    const int bs = fine ? 3 : BCo;
    const int nN = fine ? (int)c->nNodes : c->amg[l - 1].nN;
    const int32_t* rowPtr = fine ? c->dRowPtr : c->amg[l - 1].rowPtr;
    const int32_t* colIdx = fine ? c->dColIdx : c->amg[l - 1].colIdx;
    const float* vals = fine ? (const float*)c->dBsrVals : c->amg[l - 1].vals;
    const float* binv = fine ? (const float*)c->dBinv : c->amg[l - 1].binv;
    const uint8_t* mask = fine ? c->dMask : c->amg[l - 1].dead;
    float* t = fine ? c->fineT : c->amg[l - 1].t;
    const void* valsH = fine ? nullptr : c->amg[l - 1].valsH;
    AmgLevel& Cn = c->amg[l];
    // fine level from a BF16 copy: the sliced-ELL one, else the BSR split copy (staged through
    // shared memory when the chunks fit)
    const bool fineH = fine && c->amgBf16 && (c->sellMode == 1 || c->dBsrValsH);
    auto fine_bf16 = [&](const float* xin, float* out, const float* bj, float om) -> ef_status {
        if (c->sellMode == 1)
            return ef_launch_sell_level3_bf16(nN, c->sellSlices, c->dSellOff, c->dSellPerm, c->dSellCol, c->dSellV8,
                                              c->dSellV1, xin, r, mask, out, bj, om, s);
        if (c->stageCap > 0)
            return ef_launch_level_residual_bf16_staged(c->nSM, c->stageCap, nN, c->nBlocks, rowPtr, colIdx,
                                                        c->dBsrValsH, xin, r, mask, out, s, bj, om);
        return ef_launch_level_residual_bf16(nN, c->nBlocks, rowPtr, colIdx, c->dBsrValsH, xin, r, mask, out, s, bj,
                                             om);
    };
    auto residual = [&]() -> ef_status {
        if (fineH) return fine_bf16(x, t, nullptr, 0.f);
        return ef_launch_level_residual(bs, nN, rowPtr, colIdx, vals, x, r, mask, t, s, nullptr, 0.f, valsH);
    };
    // Chebyshev smoothing of degree amgSweeps on [lmax / 30, 1.1 lmax] of D^-1 A; from zero the
    // first residual is r itself
    auto chebyshev = [&](bool fromZero) -> ef_status {
        const double up = 1.1 * (l < (int)c->levelLam.size() ? c->levelLam[l] : 2.0), lo = up / 30.0;
        const double theta = 0.5 * (up + lo), delta = 0.5 * (up - lo), sigma = theta / delta;
        double rhoOld = 1.0 / sigma;
        float* d = c->chebD[l];
        if (fromZero) {
            EF_CHECK(ef_launch_cheb_step(bs, nN, binv, mask, 0.f, (float)(1.0 / theta), r, d, x, 1, s));
        } else {
            EF_CHECK(residual());
            EF_CHECK(ef_launch_cheb_step(bs, nN, binv, mask, 0.f, (float)(1.0 / theta), t, d, x, 0, s));
        }
        for (int k = 1; k < c->amgSweeps; ++k) {
            const double rho = 1.0 / (2.0 * sigma - rhoOld);
            EF_CHECK(residual());
            EF_CHECK(ef_launch_cheb_step(bs, nN, binv, mask, (float)(rho * rhoOld), (float)(2.0 * rho / delta), t, d,
                                         x, 0, s));
            rhoOld = rho;
        }
        return EF_OK;
    };
    // one fused damped block-Jacobi sweep xout = xin + omega D^-1 (r - A xin)
    auto sweep = [&](const float* xin, float* xout) -> ef_status {
        if (fineH) return fine_bf16(xin, xout, binv, omega);
        return ef_launch_level_residual(bs, nN, rowPtr, colIdx, vals, xin, r, mask, xout, s, binv, omega, valsH);
    };
    // The sweeps (the first from zero) alternate between x and a second vector; the first goes
    // to the second vector when their total count is even, so that the last one lands in x.
    float* x2 = fine ? c->fineX : c->amg[l - 1].x2;
    const int nPre = fine ? c->amgPre : c->amgPreC, nPost = fine ? c->amgPost : c->amgPostC;
    float* cur = x;
    if (!c->amgCheb) cur = ((nPre + nPost) & 1) ? x : x2;
    // pre-smoothing from zero
    if (c->amgCheb) {
        EF_CHECK(chebyshev(true));
    } else {
        EF_CHECK(ef_launch_bj_apply(bs, nN, binv, mask, omega, r, cur, 0, s));
        for (int k = 1; k < nPre; ++k) {
            float* nxt = cur == x ? x2 : x;
            EF_CHECK(sweep(cur, nxt));
            cur = nxt;
        }
    }
    // coarse correction (repeated for a W-cycle below the finest level)
    const int reps = (l > 0 && l <= c->amgWLevels && c->amgCycle > 1) ? c->amgCycle : 1;
    for (int rep = 0; rep < reps; ++rep) {
        if (!c->amgCheb) {
            EF_CHECK(fineH ? fine_bf16(cur, t, nullptr, 0.f)
                                          : ef_launch_level_residual(bs, nN, rowPtr, colIdx, vals, cur, r, mask, t, s,
                                                                     nullptr, 0.f, valsH));
        } else {
            EF_CHECK(residual());
        }
        if (l == c->clusterLevel) {
            // restriction, the whole cycle below and the prolongation as one cluster launch
            if (cur != c->clusterCur || x != c->amg[l - 1].x) {
                ef_set_error("multigrid: cluster program built for other buffers");
                return EF_ERR_ARG;
            }
            EF_CHECK(ef_launch_coarse_cycle(c->dCoarseOps, c->nCoarseOps, s));
            continue;
        }
        if (c->amgSmoothed)
            EF_CHECK(ef_launch_sa_restrict(bs, Cn.nN, Cn.saTPtr, Cn.saTIdx, Cn.saPRow, Cn.saPv, t, Cn.dead, Cn.r, s));
        else
            EF_CHECK(ef_launch_restrict(bs, Cn.nN, Cn.aggPtr, Cn.aggIdx, Cn.offs, t, Cn.dead, Cn.r, s));
        EF_CHECK(amg_vcycle(c, l + 1, Cn.r, Cn.x, s));
        if (c->amgSmoothed)
            EF_CHECK(ef_launch_sa_prolong(bs, nN, Cn.saPRowPtr, Cn.saPCol, Cn.saPv, Cn.x, mask, cur, c->amgAlpha, s));
        else
            EF_CHECK(ef_launch_prolong(bs, nN, Cn.agg, Cn.offs, Cn.x, mask, cur, s, c->amgAlpha));
    }
    // post-smoothing
    if (c->amgCheb) {
        EF_CHECK(chebyshev(false));
    } else {
        for (int k = 0; k < nPost; ++k) {
            float* nxt = cur == x ? x2 : x;
            EF_CHECK(sweep(cur, nxt));
            cur = nxt;
        }
        if (cur != x) {
            ef_set_error("multigrid: smoothing sweeps did not end in the output vector");
            return EF_ERR_ARG;
        }
    }
    return EF_OK;
}

// preconditioner of FGMRES: z = V-cycle(v) (+ the learned correction when enabled)
// learned correction with Mv in vcOut and v in vcIn: rho = v - K Mv, N = NN([Mv, rho, D^-1 rho]),
// z = Mv + alpha N with the alpha that minimises |v - K z| (never worse than Mv alone in that
// norm); z in vcOut2
static ef_status nn_apply(ef_ctx* c, cudaStream_t s) {
    const int64_t n = c->nDof;
    const int nN = (int)c->nNodes;
    const float* K = (const float*)c->dBsrVals;
    double* out = c->nnRed + 3 * c->nnPartN;
    EF_CHECK(ef_launch_spmv_f32(nN, c->dRowPtr, c->dColIdx, K, c->vcOut, c->dMask, c->nnKd, s));
    EF_CHECK(ef_launch_sub(n, c->vcIn, c->nnKd, c->nnRho, s));
    EF_CHECK(ef_launch_features(nN, c->vcOut, c->nnRho, (const float*)c->dBinv, c->nnS[0], c->nnS[1], c->nnS[2],
                                c->nnF, s));
    EF_CHECK(ef_mpnn_forward(nN, c->dRowPtr, c->dColIdx, c->nnA, c->nnPf, c->nnF, nullptr, c->dMask, c->nnSo,
                             c->nnActs, c->nnN, c->nnTensorCores, c->dFlags, s));
    EF_CHECK(ef_launch_spmv_f32(nN, c->dRowPtr, c->dColIdx, K, c->nnN, c->dMask, c->nnKN, s));
    EF_CHECK(ef_mpnn_sumsq(n, 0, c->nnRho, c->nnKN, c->dMask, c->nnRed, c->nnPartN, out, s));
    EF_CHECK(ef_mpnn_sumsq(n, 1, c->nnKN, nullptr, c->dMask, c->nnRed, c->nnPartN, out + 3, s));
    return ef_mpnn_alpha_combine(n, c->vcOut, c->nnN, out, c->dMask, c->vcOut2, s);
}

static ef_status nn_capture(ef_ctx* c) {
    if (c->nnGraph) return EF_OK;
    if (!c->capStream) EF_CUDA(cudaStreamCreateWithFlags(&c->capStream, cudaStreamNonBlocking));
    EF_CUDA(cudaStreamBeginCapture(c->capStream, cudaStreamCaptureModeThreadLocal));
    long long captured = 0;
    t_captureCount = &captured;
    const ef_status st = nn_apply(c, c->capStream);
    t_captureCount = nullptr;
    c->nnGraphKernels = captured;
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(c->capStream, &g);
    if (st != EF_OK) return st;
    if (e != cudaSuccess) {
        ef_set_error(std::string("network capture: ") + cudaGetErrorString(e));
        return EF_ERR_CUDA;
    }
    EF_CUDA(cudaGraphInstantiate(&c->nnGraph, g, 0));
    cudaGraphDestroy(g);
    return EF_OK;
}

// vcOut = M vcIn with the base preconditioner: the multigrid cycle (captured graph) or one
// block-Jacobi step D^-1 (free DOFs)
static ef_status apply_base(ef_ctx* c, cudaStream_t s) {
    if (c->fgPc == EF_FGMRES_PC_JACOBI)
        return ef_launch_bj_apply(3, (int)c->nNodes, (const float*)c->dBinv, c->dMask, 1.f, c->vcIn, c->vcOut, 0, s);
    EF_CHECK(amg_capture(c));
    ef::note_launches(c->vcGraphKernels);
    EF_CUDA(cudaGraphLaunch(c->vcGraph, s));
    return EF_OK;
}

static ef_status fgmres_precond(ef_ctx* c, const float* v, const float** out, cudaStream_t s) {
    if (c->vcInStale) {  // otherwise the previous column's normalisation wrote v into vcIn
        EF_CUDA(cudaMemcpyAsync(c->vcIn, v, sizeof(float) * c->nDof, cudaMemcpyDeviceToDevice, s));
        c->vcInStale = false;
    }
    EF_CHECK(apply_base(c, s));
    *out = c->vcOut;
    if (c->nnOn) {
        EF_CHECK(nn_capture(c));
        ef::note_launches(c->nnGraphKernels);
        EF_CUDA(cudaGraphLaunch(c->nnGraph, s));
        *out = c->vcOut2;
    }
    return EF_OK;
}

// ---- learned correction: weights, training pairs, training -----------------------------------

// deterministic normal variates (Box-Muller on a 64-bit Mersenne twister)
static void nn_normal(std::mt19937_64& g, float sd, float* out, int n) {
    const double two_pi = 6.283185307179586;
    for (int i = 0; i < n; i += 2) {
        const double u1 = ((g() >> 11) + 1.0) * (1.0 / 9007199254740993.0);
        const double u2 = (g() >> 11) * (1.0 / 9007199254740992.0);
        const double rad = sqrt(-2.0 * log(u1));
        out[i] = (float)(sd * rad * cos(two_pi * u2));
        if (i + 1 < n) out[i + 1] = (float)(sd * rad * sin(two_pi * u2));
    }
}

// block (m, n) -> position of block (n, m) in the (structurally symmetric) block pattern
static ef_status nn_transpose_map(const std::vector<int32_t>& rowPtr, const std::vector<int32_t>& colIdx,
                                  std::vector<int64_t>& tpos) {
    const int64_t nN = (int64_t)rowPtr.size() - 1;
    tpos.assign(colIdx.size(), -1);
    for (int64_t m = 0; m < nN; ++m)
        for (int32_t k = rowPtr[m]; k < rowPtr[m + 1]; ++k) {
            const int32_t n = colIdx[k];
            const auto b = colIdx.begin() + rowPtr[n], e = colIdx.begin() + rowPtr[n + 1];
            const auto it = std::lower_bound(b, e, (int32_t)m);
            if (it == e || *it != (int32_t)m) {
                ef_set_error("learned correction: block pattern is not structurally symmetric");
                return EF_ERR_STATE;
            }
            tpos[k] = it - colIdx.begin();
        }
    return EF_OK;
}

static ef_status nn_upload_params(ef_ctx* c, const float* hp, cudaStream_t s) {
    const int np = ef_mpnn_nparam();
    EF_CUDA(cudaMemcpyAsync(c->nnP, hp, sizeof(float) * np, cudaMemcpyHostToDevice, s));
    EF_CUDA(cudaMemsetAsync(c->nnM1, 0, sizeof(float) * np, s));
    EF_CUDA(cudaMemsetAsync(c->nnM2, 0, sizeof(float) * np, s));
    EF_CHECK(ef_mpnn_refresh(np, c->nnP, c->nnPb, c->nnPf, s));
    EF_CUDA(cudaStreamSynchronize(s));
    c->nnStep = 0;
    return EF_OK;
}

// the stored copy of the current system (K values and edge weights), evicting the oldest one
// (and the pairs taken from it) when the store is full
static ef_status nn_current_system(ef_ctx* c, cudaStream_t s, int* out) {
    for (size_t i = 0; i < c->nnSystems.size(); ++i)
        if (c->nnSystems[i].version == c->nnVersion) {
            *out = (int)i;
            return EF_OK;
        }
    int slot = -1;
    std::vector<int> used(c->nnSystems.size(), 0);
    for (const auto& S : c->nnSamples)
        if (S.sys >= 0) used[S.sys] = 1;
    for (size_t i = 0; i < c->nnSystems.size() && slot < 0; ++i)
        if (!used[i]) slot = (int)i;
    if (slot < 0 && (int)c->nnSystems.size() < c->nnMaxSystems) {
        ef_status st = EF_OK;
        ef_ctx::NNSystem Y;
        Y.K = dalloc<float>((size_t)c->nBlocks * 9, &st);
        Y.a = dalloc<float>(c->nBlocks, &st);
        c->nnSystems.push_back(Y);
        if (st != EF_OK) return st;
        slot = (int)c->nnSystems.size() - 1;
    }
    if (slot < 0) {  // evict the oldest system
        slot = 0;
        for (size_t i = 1; i < c->nnSystems.size(); ++i)
            if (c->nnSystems[i].version < c->nnSystems[slot].version) slot = (int)i;
        for (auto& S : c->nnSamples)
            if (S.sys == slot) S.sys = -1;
    }
    ef_ctx::NNSystem& Y = c->nnSystems[slot];
    EF_CUDA(cudaMemcpyAsync(Y.K, c->dBsrVals, sizeof(float) * 9 * c->nBlocks, cudaMemcpyDeviceToDevice, s));
    EF_CUDA(cudaMemcpyAsync(Y.a, c->nnA, sizeof(float) * c->nBlocks, cudaMemcpyDeviceToDevice, s));
    Y.version = c->nnVersion;
    *out = slot;
    return EF_OK;
}

// adds the training pair (r, e) with K e = r (free DOFs, FP32 device vectors; e may be null:
// an input without its correction), scaled to rms(e) = 1 (rms(r) = 1 without e); the multigrid
// hierarchy and edge weights must be current.  Features: [Mv, rho, D^-1 rho], rho = r - K Mv.
static ef_status nn_add_sample(ef_ctx* c, const float* r, const float* e, cudaStream_t s) {
    const int64_t n = c->nDof;
    const int64_t nN = c->nNodes;
    if (c->nnMaxSamples == 0) return EF_OK;
    double* out = c->nnRed + 3 * c->nnPartN;
    double h[3] = {0, 0, 0};
    if (e) {
        EF_CHECK(ef_mpnn_sumsq(n, 1, e, nullptr, c->dMask, c->nnRed, c->nnPartN, out, s));
        EF_CUDA(cudaMemcpyAsync(&h[0], out, sizeof(double), cudaMemcpyDeviceToHost, s));
        EF_CHECK(ef_mpnn_sumsq(n, 0, e, r, c->dMask, c->nnRed, c->nnPartN, out + 3, s));
        EF_CUDA(cudaMemcpyAsync(&h[1], out + 3, sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    EF_CHECK(ef_mpnn_sumsq(n, 1, r, nullptr, c->dMask, c->nnRed, c->nnPartN, out, s));
    EF_CUDA(cudaMemcpyAsync(&h[2], out, sizeof(double), cudaMemcpyDeviceToHost, s));
    EF_CUDA(cudaStreamSynchronize(s));
    const double ss = e ? h[0] : h[2];
    if (!(ss > 0.0) || !(ss < 1e300) || !(h[2] > 0.0) || (e && !(h[1] > 0.0))) return EF_OK;  // nothing to learn
    int sys = -1;
    EF_CHECK(nn_current_system(c, s, &sys));
    size_t slot = c->nnSamples.size();
    for (size_t i = 0; i < c->nnSamples.size(); ++i)
        if (c->nnSamples[i].sys < 0) {
            slot = i;
            break;
        }
    if (slot == c->nnSamples.size()) {
        if ((int)c->nnSamples.size() < c->nnMaxSamples) {
            ef_status st = EF_OK;
            ef_ctx::NNSample S;
            S.f = dalloc<float>(9 * nN, &st);
            S.base = dalloc<float>(n, &st);
            S.r = dalloc<float>(n, &st);
            S.e = dalloc<float>(n, &st);
            c->nnSamples.push_back(S);
            if (st != EF_OK) return st;
        } else {
            slot = (size_t)(c->nnAdded % c->nnMaxSamples);
        }
    }
    c->nnAdded++;
    ef_ctx::NNSample& S = c->nnSamples[slot];
    const double inv2 = (double)n / ss;
    S.sys = sys;
    S.hasE = e != nullptr;
    S.ee = h[0] * inv2;
    S.er = h[1] * inv2;
    S.rr = h[2] * inv2;
    const float inv = (float)sqrt(inv2);
    EF_CUDA(cudaMemcpyAsync(c->vcIn, r, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
    c->vcInStale = true;
    EF_CHECK(apply_base(c, s));
    EF_CHECK(ef_launch_spmv_f32((int)nN, c->dRowPtr, c->dColIdx, (const float*)c->dBsrVals, c->vcOut, c->dMask,
                                c->nnKd, s));
    EF_CHECK(ef_launch_sub(n, c->vcIn, c->nnKd, c->nnRho, s));
    EF_CHECK(ef_launch_features((int)nN, c->vcOut, c->nnRho, (const float*)c->dBinv, 1.f, 1.f, 1.f, S.f, s));
    EF_CUDA(cudaMemcpyAsync(S.base, c->vcOut, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
    EF_CUDA(cudaMemcpyAsync(S.r, c->vcIn, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
    if (e) EF_CUDA(cudaMemcpyAsync(S.e, e, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
    EF_CHECK(ef_mpnn_scale(9 * nN, S.f, inv, s));
    EF_CHECK(ef_mpnn_scale(n, S.base, inv, s));
    EF_CHECK(ef_mpnn_scale(n, S.r, inv, s));
    if (e) EF_CHECK(ef_mpnn_scale(n, S.e, inv, s));
    return EF_OK;
}

// pairs from the iterates of a converged FGMRES solve: e_k = x - x_k, r_k = K e_k
static ef_status nn_collect_snapshots(ef_ctx* c, const float* x, cudaStream_t s) {
    const int64_t n = c->nDof;
    for (int k = 0; k < c->nnSnapCount; ++k) {
        float* ek = c->nnSnaps[k];
        EF_CHECK(ef_launch_sub(n, x, ek, ek, s));
        EF_CHECK(ef_launch_spmv_f32((int)c->nNodes, c->dRowPtr, c->dColIdx, (const float*)c->dBsrVals, ek, c->dMask,
                                    c->fgW, s));
        EF_CHECK(nn_add_sample(c, c->fgW, ek, s));
    }
    c->nnSnapCount = 0;
    return EF_OK;
}

static ef_status nn_snapshot_buffer(ef_ctx* c, float** out) {
    if (c->nnSnapCount >= (int)c->nnSnaps.size()) {
        ef_status st = EF_OK;
        float* p = dalloc<float>(c->nDof, &st);
        if (!p) return st;
        c->nnSnaps.push_back(p);
    }
    *out = c->nnSnaps[c->nnSnapCount++];
    return EF_OK;
}

// epochs of Adam over the stored pairs (shuffled deterministically); epochs = 0 only evaluates.
// Loss of a pair with d = z - e, relative to the same norm of e:
//   norm 0: |d|^2 / |e|^2,  norm 1: d.K d / e.K e,  norm 2: |K d|^2 / |K e|^2
// (K the system the pair was taken from); the mean over the pairs is reported.
static ef_status nn_train(ef_ctx* c, int epochs, float lr, int norm, double* lossFirst, double* lossLast,
                          cudaStream_t s) {
    std::vector<int> valid;
    for (size_t i = 0; i < c->nnSamples.size(); ++i)
        if (c->nnSamples[i].sys >= 0 && (norm == 2 || c->nnSamples[i].hasE)) valid.push_back((int)i);
    const int nS = (int)valid.size();
    if (nS == 0) {
        ef_set_error("ef_mpnn_train: no training pairs");
        return EF_ERR_STATE;
    }
    const int64_t n = c->nDof, nN = c->nNodes;
    double* out = c->nnRed + 3 * c->nnPartN;
    if (!c->nnScalesSet) {
        // feature group scales: 1 / rms of each group over the stored pairs
        double acc[3] = {0, 0, 0};
        for (int i : valid) {
            EF_CHECK(ef_mpnn_sumsq(9 * nN, 3, c->nnSamples[i].f, nullptr, nullptr, c->nnRed, c->nnPartN, out, s));
            double h[3];
            EF_CUDA(cudaMemcpyAsync(h, out, sizeof(h), cudaMemcpyDeviceToHost, s));
            EF_CUDA(cudaStreamSynchronize(s));
            for (int g = 0; g < 3; ++g) acc[g] += h[g];
        }
        for (int g = 0; g < 3; ++g) {
            const double rms = sqrt(acc[g] / (3.0 * nN * nS));
            c->nnS[g] = rms > 0.0 ? (float)(1.0 / rms) : 1.f;
        }
        c->nnScalesSet = true;
        if (c->nnGraph) {
            cudaGraphExecDestroy(c->nnGraph);
            c->nnGraph = nullptr;
        }
    }
    ef_status st = EF_OK;
    double* lossBuf = dalloc<double>(3 * (size_t)nS, &st);
    if (!lossBuf) return st;
    std::vector<double> hl(3 * (size_t)nS);
    std::vector<int> order(nS);
    const int np = ef_mpnn_nparam();
    for (int ep = 0; ep < std::max(epochs, 1); ++ep) {
        for (int i = 0; i < nS; ++i) order[i] = i;
        std::mt19937_64 g(0x5eed0000ull + (uint64_t)c->nnStep + (uint64_t)ep);
        for (int i = nS - 1; i > 0; --i) std::swap(order[i], order[(int)(g() % (uint64_t)(i + 1))]);
        for (int t = 0; t < nS; ++t) {
            const ef_ctx::NNSample& S = c->nnSamples[valid[order[t]]];
            const ef_ctx::NNSystem& Y = c->nnSystems[S.sys];
            EF_CHECK(ef_mpnn_scale_features((int)nN, S.f, c->nnS[0], c->nnS[1], c->nnS[2], c->nnF, s));
            EF_CHECK(ef_mpnn_forward((int)nN, c->dRowPtr, c->dColIdx, Y.a, c->nnPf, c->nnF, S.base, c->dMask, c->nnSo,
                                     c->nnActs, c->vcOut2, c->nnTensorCores, c->dFlags, s));
            // rho = dL/dz up to the factor scale: d, K d or K (K z - r), d = z - e
            const float* rho = c->nnD;
            double ref = S.ee;
            double* lb = lossBuf + 3 * order[t];
            if (norm == 0) {
                EF_CHECK(ef_launch_sub(n, c->vcOut2, S.e, c->nnD, s));
                EF_CHECK(ef_mpnn_sumsq(n, 1, c->nnD, nullptr, c->dMask, c->nnRed, c->nnPartN, lb, s));
            } else if (norm == 1) {
                EF_CHECK(ef_launch_sub(n, c->vcOut2, S.e, c->nnD, s));
                EF_CHECK(ef_launch_spmv_f32((int)nN, c->dRowPtr, c->dColIdx, Y.K, c->nnD, c->dMask, c->nnKd, s));
                EF_CHECK(ef_mpnn_sumsq(n, 0, c->nnD, c->nnKd, c->dMask, c->nnRed, c->nnPartN, lb, s));
                rho = c->nnKd;
                ref = S.er;
            } else {
                EF_CHECK(ef_launch_spmv_f32((int)nN, c->dRowPtr, c->dColIdx, Y.K, c->vcOut2, c->dMask, c->nnKd, s));
                EF_CHECK(ef_launch_sub(n, c->nnKd, S.r, c->nnKd, s));
                EF_CHECK(ef_mpnn_sumsq(n, 1, c->nnKd, nullptr, c->dMask, c->nnRed, c->nnPartN, lb, s));
                EF_CHECK(ef_launch_spmv_f32((int)nN, c->dRowPtr, c->dColIdx, Y.K, c->nnKd, c->dMask, c->nnD, s));
                rho = c->nnD;
                ref = S.rr;
            }
            if (epochs == 0) continue;
            // gradient of 0.5 * |.|^2 / ref: backward with z := rho, e := 0, scale 1 / ref
            EF_CHECK(ef_launch_gather_f32(c->nBlocks, c->nnTpos, Y.a, c->nnAT, s));
            EF_CHECK(ef_mpnn_backward((int)nN, c->dRowPtr, c->dColIdx, c->nnAT, c->nnPf, c->nnF, c->nnActs, rho,
                                      nullptr, c->dMask, (float)(1.0 / ref), c->nnSo, c->nnG, c->nnWork, c->nnPart,
                                      c->nnPartN, s));
            EF_CHECK(ef_mpnn_adam(np, c->nnP, c->nnG, c->nnM1, c->nnM2, lr, 0.9f, 0.999f, 1e-8f, ++c->nnStep, c->nnPb,
                                  c->nnPf, s));
        }
        EF_CUDA(cudaMemcpyAsync(hl.data(), lossBuf, sizeof(double) * hl.size(), cudaMemcpyDeviceToHost, s));
        EF_CUDA(cudaStreamSynchronize(s));
        double mean = 0.0;
        for (int t = 0; t < nS; ++t) {
            const ef_ctx::NNSample& S = c->nnSamples[valid[t]];
            mean += hl[3 * t] / (norm == 0 ? S.ee : (norm == 1 ? S.er : S.rr));
        }
        mean /= nS;
        if (ep == 0 && lossFirst) *lossFirst = mean;
        if (lossLast) *lossLast = mean;
    }
    cudaFree(lossBuf);
    return EF_OK;
}

// FGMRES(m) on the free DOFs for K x = b (FP32 vectors, FP64 reductions and Hessenberg);
// x starts at 0; stops at ||b - K x|| <= rtol ||b|| (Arnoldi estimate) or maxIter
static ef_status run_fgmres(ef_ctx* c, const float* b, float* x, int maxIter, double rtol, int restart, int* iters,
                            ef_solve_info* prof, cudaStream_t s) {
    const int64_t n = c->nDof;
    const int m = std::max(2, std::min(restart, ef_fgmres_max_basis() - 2));
    ef_status st = EF_OK;
    if (c->fgRestart < m) {
        if (c->fgV) cudaFree(c->fgV);
        if (c->fgZ) cudaFree(c->fgZ);
        c->fgV = dalloc<float>((size_t)(m + 1) * n, &st);
        c->fgZ = dalloc<float>((size_t)m * n, &st);
        if (!c->fgV || !c->fgZ) return st;
        c->fgRestart = m;
    }
    if (!c->fgW) {
        c->fgW = dalloc<float>(n, &st);
        c->fgNPart = 4 * c->nSM;  // 1024 threads per SM
        c->fgPart = dalloc<double>((size_t)c->fgNPart * ef_fgmres_max_basis(), &st);
        c->fgPartN = dalloc<double>((size_t)c->fgNPart, &st);
        c->fgH = dalloc<double>(4 * (size_t)ef_fgmres_max_basis(), &st);
        if (!c->fgW || !c->fgPart || !c->fgPartN || !c->fgH) return st;
        if (const char* e = getenv("EF_FGMRES_ETA")) c->fgEta2 = atof(e) * atof(e);
        bool staged = false;  // measured slower than the unstaged kernel (EF_SPMV_STAGED=1 turns it on)
        if (const char* e = getenv("EF_SPMV_STAGED")) staged = atoi(e) != 0;
        c->spCap = staged ? ef_sp_stage_cap((int)c->nNodes, c->hRowPtr0.data()) : 0;
        if (c->spCap > 2048) c->spCap = 0;  // rows too long for a shared-memory stage
    }
    const int MB = ef_fgmres_max_basis();
    double* hG = c->fgH;            // first-pass coefficients and |w|^2 (the DGKS gate)
    double* hTmp = c->fgH + MB;     // second-pass coefficients
    double* hAcc = c->fgH + 2 * MB; // column of the Hessenberg matrix
    double* dy = c->fgH + 3 * MB;   // solution coefficients
    float* V = c->fgV;
    float* Z = c->fgZ;
    // Results of a column reach the host through mapped pinned memory written by the
    // normalisation kernel: [0, j] coefficients, ldh - 2 re-orthogonalised flag, ldh - 1 |w|^2.
    const int ldh = MB + 2;
    if (!c->fgPin) {
        EF_CUDA(cudaHostAlloc(&c->fgPin, sizeof(double) * 3 * ldh, cudaHostAllocMapped));
        EF_CUDA(cudaHostGetDevicePointer((void**)&c->fgPinDev, c->fgPin, 0));
        for (int k = 0; k < 2; ++k) {
            EF_CUDA(cudaEventCreateWithFlags(&c->fgDone[k], cudaEventDisableTiming));
            for (int e = 0; e < 4; ++e) EF_CUDA(cudaEventCreate(&c->fgEv[k][e]));
        }
    }
    double* pinRestart = c->fgPin + 2 * ldh;
    double* pinRestartDev = c->fgPinDev + 2 * ldh;
    EF_CUDA(cudaMemsetAsync(x, 0, sizeof(float) * n, s));
    // r0 = b (x = 0); v0 = r0 / |r0| (also into the preconditioner's input)
    EF_CUDA(cudaMemcpyAsync(V, b, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
    EF_CHECK(ef_launch_normalize_first(n, V, c->fgPart, c->fgNPart, c->vcIn, pinRestartDev, 0, s));
    c->vcInStale = false;
    EF_CUDA(cudaStreamSynchronize(s));
    const double bnorm = sqrt(pinRestart[0]);
    *iters = 0;
    if (!(bnorm > 0.0)) return EF_OK;
    double beta = bnorm;
    const bool collect = c->nnInit && c->nnEvery > 0 && c->nnMaxPerSolve > 0;
    const bool snap = collect && c->nnKind == 0;
    const bool krylovSamples = collect && c->nnKind == 1;
    int nKrylov = 0;
    c->nnSnapCount = 0;
    if (snap) {  // x_0 = 0
        float* p = nullptr;
        EF_CHECK(nn_snapshot_buffer(c, &p));
        EF_CUDA(cudaMemsetAsync(p, 0, sizeof(float) * n, s));
    }
    std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1);
    // The GPU work of column j+1 is enqueued before the host waits for column j's coefficients
    // (Givens rotations and the convergence test run on the host), so the GPU never idles on the
    // host; a converged cycle computes at most one column it does not use.
    auto enqueue_column = [&](int j) -> ef_status {
        const int sl = j & 1;
        if (prof) EF_CUDA(cudaEventRecord(c->fgEv[sl][0], s));
        const float* pz = nullptr;
        EF_CHECK(fgmres_precond(c, V + (int64_t)j * n, &pz, s));
        if (prof) EF_CUDA(cudaEventRecord(c->fgEv[sl][2], s));
        // w = K z_j straight into the next basis slot; z_j kept in Z
        if (c->sellMode == 1)
            EF_CHECK(ef_launch_sell_spmv3((int)c->nNodes, c->sellSlices, c->dSellOff, c->dSellPerm, c->dSellCol,
                                          c->dSellV9, pz, c->dMask, V + (int64_t)(j + 1) * n, Z + (int64_t)j * n, s));
        else if (c->spCap > 0)
            EF_CHECK(ef_launch_spmv_f32_staged(c->nSM, c->spCap, (int)c->nNodes, c->dRowPtr, c->dColIdx,
                                               (const float*)c->dBsrVals, pz, c->dMask, V + (int64_t)(j + 1) * n,
                                               Z + (int64_t)j * n, s));
        else
            EF_CHECK(ef_launch_spmv_f32_copy((int)c->nNodes, c->dRowPtr, c->dColIdx, (const float*)c->dBsrVals, pz,
                                             c->dMask, V + (int64_t)(j + 1) * n, Z + (int64_t)j * n, s));
        if (prof) EF_CUDA(cudaEventRecord(c->fgEv[sl][3], s));
        EF_CHECK(ef_launch_cgs_column(n, j + 1, V, n, c->fgPart, c->fgPartN, c->fgNPart, hG, hTmp, hAcc, c->fgEta2,
                                      c->vcIn, c->fgPinDev + sl * ldh, ldh - 1, s));
        c->vcInStale = false;
        if (prof) EF_CUDA(cudaEventRecord(c->fgEv[sl][1], s));
        EF_CUDA(cudaEventRecord(c->fgDone[sl], s));
        return EF_OK;
    };
    int total = 0;
    bool converged = false;
    while (total < maxIter && !converged) {
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        int j = 0;
        EF_CHECK(enqueue_column(0));
        for (; j < m && total < maxIter; ++j) {
            if (j + 1 < m && total + 1 < maxIter) EF_CHECK(enqueue_column(j + 1));
            const int sl = j & 1;
            EF_CUDA(cudaEventSynchronize(c->fgDone[sl]));
            const double* hcol = c->fgPin + sl * ldh;
            const double hn2 = hcol[ldh - 1];
            if (prof) {
                float ms = 0.f;
                EF_CUDA(cudaEventElapsedTime(&ms, c->fgEv[sl][0], c->fgEv[sl][1]));
                prof->kernelMs += ms;
                prof->kernelLaunches += 1;
                EF_CUDA(cudaEventElapsedTime(&ms, c->fgEv[sl][2], c->fgEv[sl][3]));
                prof->spmvMs += ms;
                prof->spmvLaunches += 1;
                EF_CUDA(cudaEventElapsedTime(&ms, c->fgEv[sl][0], c->fgEv[sl][2]));
                prof->precondMs += ms;
                EF_CUDA(cudaEventElapsedTime(&ms, c->fgEv[sl][3], c->fgEv[sl][1]));
                prof->orthoMs += ms;
            }
            if (prof && hcol[ldh - 2] != 0.0) prof->reorths += 1;
            ++total;
            double* Hj = &H[(size_t)j * (m + 1)];  // column j
            for (int i = 0; i <= j; ++i) Hj[i] = hcol[i];
            Hj[j + 1] = sqrt(hn2);
            for (int i = 0; i < j; ++i) {  // previous Givens rotations
                const double t0 = cs[i] * Hj[i] + sn[i] * Hj[i + 1];
                Hj[i + 1] = -sn[i] * Hj[i] + cs[i] * Hj[i + 1];
                Hj[i] = t0;
            }
            const double den = hypot(Hj[j], Hj[j + 1]);
            cs[j] = den > 0.0 ? Hj[j] / den : 1.0;
            sn[j] = den > 0.0 ? Hj[j + 1] / den : 0.0;
            Hj[j] = den;
            Hj[j + 1] = 0.0;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            if (!(g[j + 1] == g[j + 1]) || !(den == den)) {
                EF_CUDA(cudaStreamSynchronize(s));
                return EF_NAN;
            }
            if (krylovSamples && total % c->nnEvery == 0 && nKrylov < c->nnMaxPerSolve) {
                EF_CHECK(nn_add_sample(c, V + (int64_t)j * n, nullptr, s));
                ++nKrylov;
            }
            if (snap && total % c->nnEvery == 0 && c->nnSnapCount < c->nnMaxPerSolve && j + 1 < m) {
                // iterate after j + 1 steps: x + Z y, R y = g (current Givens factor)
                std::vector<double> ys(j + 1);
                for (int i = j; i >= 0; --i) {
                    double acc = g[i];
                    for (int k = i + 1; k <= j; ++k) acc -= H[(size_t)k * (m + 1) + i] * ys[k];
                    ys[i] = acc / H[(size_t)i * (m + 1) + i];
                }
                float* p = nullptr;
                EF_CHECK(nn_snapshot_buffer(c, &p));
                EF_CUDA(cudaMemcpyAsync(p, x, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
                EF_CUDA(cudaMemcpyAsync(dy, ys.data(), sizeof(double) * (j + 1), cudaMemcpyHostToDevice, s));
                EF_CHECK(ef_launch_combine(n, j + 1, Z, n, dy, p, s));
            }
            if (fabs(g[j + 1]) <= rtol * bnorm || hn2 <= 0.0) {
                converged = fabs(g[j + 1]) <= rtol * bnorm;
                ++j;
                break;
            }
        }
        // y = R^-1 g, x += Z y
        std::vector<double> y(j);
        for (int i = j - 1; i >= 0; --i) {
            double acc = g[i];
            for (int k = i + 1; k < j; ++k) acc -= H[(size_t)k * (m + 1) + i] * y[k];
            y[i] = acc / H[(size_t)i * (m + 1) + i];
        }
        EF_CUDA(cudaMemcpyAsync(dy, y.data(), sizeof(double) * j, cudaMemcpyHostToDevice, s));
        EF_CHECK(ef_launch_combine(n, j, Z, n, dy, x, s));
        if (converged || total >= maxIter) break;
        // restart: r = b - K x
        EF_CHECK(ef_launch_spmv_f32((int)c->nNodes, c->dRowPtr, c->dColIdx, (const float*)c->dBsrVals, x, c->dMask,
                                    c->fineT, s));
        EF_CHECK(ef_launch_sub(n, b, c->fineT, V, s));
        EF_CHECK(ef_launch_normalize_first(n, V, c->fgPart, c->fgNPart, c->vcIn, pinRestartDev, 0, s));
        c->vcInStale = false;
        EF_CUDA(cudaStreamSynchronize(s));
        beta = sqrt(pinRestart[0]);
        if (beta <= rtol * bnorm) {
            converged = true;
            break;
        }
    }
    *iters = total;
    if (snap && converged) EF_CHECK(nn_collect_snapshots(c, x, s));
    c->nnSnapCount = 0;
    return converged ? EF_OK : EF_NOT_CONVERGED;
}

extern "C" {

ef_status ef_solve(ef_ctx* c, const ef_solve_opts* o, const double* b, double* x, ef_solve_info* info, void* stream) {
    EF_REQUIRE_FINALIZED(c);
    if (!o || !b || !x) return EF_ERR_ARG;
    if (o->method != EF_SOLVE_PCG && o->method != EF_SOLVE_FGMRES) {
        ef_set_error("ef_solve: unknown method");
        return EF_ERR_ARG;
    }
    if (o->method == EF_SOLVE_FGMRES && (c->keFp64 || !o->mixed)) {
        ef_set_error("ef_solve: FGMRES runs as the FP32 inner solver of the mixed-precision refinement");
        return EF_ERR_ARG;
    }
    if (!o->mixed && !c->keFp64) {
        ef_set_error("ef_solve: an all-FP64 solve needs an FP64 system (EF_OPT_KE_FP64)");
        return EF_ERR_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t n = c->nDof;
    double* xd = c->w64[0];
    double* xf = c->w64[1];
    double* r64 = c->w64[2];
    double* tmp = c->w64[3];
    ef_solve_info inf;
    memset(&inf, 0, sizeof(inf));
    inf.status = EF_OK;
    double bb = 0.0;
    EF_CHECK(dot_host(c, b, b, &bb, s));
    // Dirichlet part: x_d = b on Dirichlet DOFs; lifted RHS b~ = b_f - K_fd x_d
    EF_CHECK(ef_launch_masked_copy(n, b, c->dMask, 1, 1.0, xd, 1, s));
    EF_CHECK(residual64(c, xd, b, r64, s));
    EF_CUDA(cudaMemsetAsync(xf, 0, sizeof(double) * n, s));
    if (!(bb > 0.0)) {
        EF_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, s));
        inf.relResidual = 0.0;
        if (info) *info = inf;
        return EF_OK;
    }
    const double bnorm = sqrt(bb);
    double rr = 0.0;
    EF_CHECK(dot_host(c, r64, r64, &rr, s));
    int total = 0;
    ef_status result = EF_OK;
    if (!o->mixed) {
        // all-FP64 PCG to the target tolerance (relative to ||b||)
        EF_CUDA(cudaMemcpyAsync(c->w64k[0], r64, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
        const double rel = rr > 0.0 ? o->rtol * bnorm / sqrt(rr) : 1.0;
        PcgResultHost pr;
        if (rr > 0.0) {
            EF_CHECK(run_pcg(c, 1, c->w64k[0], c->w64k[1], o->maxIter, std::min(rel, 1.0), &pr, o->profile ? &inf : nullptr, s));
            total = pr.iterations;
            if (pr.status == EF_NAN) result = EF_NAN;
            EF_CHECK(ef_launch_axpy(n, 1.0, c->w64k[1], 1, xf, s));
        }
    } else {
        for (int sweep = 0; sweep < o->maxRefine; ++sweep) {
            if (!(rr == rr)) {
                result = EF_NAN;
                break;
            }
            if (sqrt(rr) <= o->rtol * bnorm) break;
            if (total >= o->maxIter) break;
            const double rn = sqrt(rr);
            // inner solve of K d = r / ||r|| in the system's precision (FP32 unless EF_OPT_KE_FP64)
            const int vd = c->keFp64;
            void** wv = vd ? c->w64k : c->w32;
            EF_CHECK(ef_launch_masked_copy(n, r64, c->dMask, 0, 1.0 / rn, wv[0], vd, s));
            const double inner = std::max(o->innerRtol, 0.5 * o->rtol * bnorm / rn);
            PcgResultHost pr;
            if (o->method == EF_SOLVE_FGMRES) {
                const bool timeSetup = o->profile && (c->sellStale || c->amgStale);
                if (timeSetup) EF_CUDA(cudaEventRecord(c->ev[0], s));
                EF_CHECK(sell_refresh(c, s));
                if (c->fgPc == EF_FGMRES_PC_MULTIGRID) {
                    EF_CHECK(amg_build(c));
                    EF_CHECK(amg_refresh(c, s));
                } else {
                    EF_CHECK(amg_workspace(c));
                    EF_CHECK(nn_edge_refresh(c, s));
                }
                if (timeSetup) {
                    EF_CUDA(cudaEventRecord(c->ev[1], s));
                    EF_CUDA(cudaEventSynchronize(c->ev[1]));
                    float ms = 0.f;
                    EF_CUDA(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
                    inf.setupMs += ms;
                }
                int its = 0;
                const ef_status fs = run_fgmres(c, (const float*)wv[0], (float*)wv[1], o->maxIter - total,
                                                std::min(inner, 0.5), o->restart, &its, o->profile ? &inf : nullptr, s);
                if (fs != EF_OK && fs != EF_NOT_CONVERGED && fs != EF_NAN) return fs;
                pr.iterations = its;
                pr.status = fs;
                pr.rr = 0.0;
                pr.bb = 0.0;
            } else {
                EF_CHECK(run_pcg(c, vd, wv[0], wv[1], o->maxIter - total, std::min(inner, 0.5), &pr,
                                 o->profile ? &inf : nullptr, s));
            }
            total += pr.iterations;
            inf.refinements++;
            if (pr.status == EF_NAN) {
                result = EF_NAN;
                break;
            }
            if (pr.iterations == 0) break;  // no progress possible
            EF_CHECK(ef_launch_axpy(n, rn, wv[1], vd, xf, s));
            // r64 = b~ - K x_f  (FP64 accumulation); b~ = b - K x_d on free rows
            EF_CHECK(ef_launch_add(n, xd, xf, tmp, s));
            EF_CHECK(residual64(c, tmp, b, r64, s));
            EF_CHECK(dot_host(c, r64, r64, &rr, s));
        }
    }
    EF_CHECK(ef_launch_add(n, xd, xf, x, s));
    if (c->dTieS) EF_CHECK(ef_launch_tie_fill((int64_t)c->hTieS.size(), c->dTieS, c->dTieA, c->dTieB, x, s));
    // final FP64 residual of the full system (Dirichlet rows are exact)
    EF_CHECK(residual64(c, x, b, r64, s));
    EF_CHECK(dot_host(c, r64, r64, &rr, s));
    inf.iterations = total;
    inf.relResidual = sqrt(rr) / bnorm;
    if (result == EF_OK && !(inf.relResidual <= o->rtol)) result = (rr == rr) ? EF_NOT_CONVERGED : EF_NAN;
    inf.status = result;
    if (info) *info = inf;
    if (o->method == EF_SOLVE_FGMRES && c->nnOn && c->nnTensorCores) {
        // a tensor-core tile that gave up waiting freed its TMEM while its MMA may still have been
        // running: the solve that used the network is discarded and the network continues on
        // the CUDA-core layer for the rest of this context
        int f = 0;
        EF_CUDA(cudaMemcpy(&f, c->dFlags, sizeof(int), cudaMemcpyDeviceToHost));
        if (f & EF_FLAG_TCWAIT) {
            EF_CUDA(cudaMemset(c->dFlags, 0, sizeof(int)));
            c->nnTensorCores = 0;
            if (c->nnGraph) {  // the captured network pass holds the tensor-core layer: capture again
                cudaGraphExecDestroy(c->nnGraph);
                c->nnGraph = nullptr;
            }
            ef_set_error("ef_solve: the learned correction's tensor-core accumulator wait timed out; this solve is "
                         "discarded and the network runs on the CUDA cores from now on");
            if (info) info->status = EF_ERR_DEVICE;
            return EF_ERR_DEVICE;
        }
    }
    return result;
}

ef_status ef_fgmres_set_reuse(ef_ctx* c, int maxReuse) {
    EF_REQUIRE_FINALIZED(c);
    if (maxReuse < 0) {
        ef_set_error("ef_fgmres_set_reuse: maxReuse must be >= 0");
        return EF_ERR_ARG;
    }
    c->amgMaxReuse = maxReuse;
    c->amgReuseLeft = 0;  // the next new system rebuilds the coarse levels
    return EF_OK;
}

ef_status ef_fgmres_set_preconditioner(ef_ctx* c, int kind) {
    EF_REQUIRE_FINALIZED(c);
    if (kind != EF_FGMRES_PC_MULTIGRID && kind != EF_FGMRES_PC_JACOBI) {
        ef_set_error("ef_fgmres_set_preconditioner: unknown kind");
        return EF_ERR_ARG;
    }
    if (kind != c->fgPc && c->nnGraph) {  // the correction's captured graph reads the base output
        cudaGraphExecDestroy(c->nnGraph);
        c->nnGraph = nullptr;
    }
    c->fgPc = kind;
    return EF_OK;
}

ef_status ef_batch_setup(ef_ctx* c, int nProb, const int32_t* nodePtr) {
    EF_REQUIRE_FINALIZED(c);
    if (nProb <= 0 || !nodePtr || nodePtr[0] != 0 || nodePtr[nProb] != (int32_t)c->nNodes) {
        ef_set_error("ef_batch_setup: node ranges must cover [0, nNodes)");
        return EF_ERR_ARG;
    }
    for (int p = 0; p < nProb; ++p)
        if (nodePtr[p + 1] < nodePtr[p]) {
            ef_set_error("ef_batch_setup: node ranges must be increasing");
            return EF_ERR_ARG;
        }
    if (!c->keFp64) {
        ef_set_error("ef_batch_setup: the batched solve runs on the FP64 system (EF_OPT_KE_FP64)");
        return EF_ERR_ARG;
    }
    // every block must couple nodes of one problem (block-diagonal system)
    std::vector<int32_t> prob(c->nNodes);
    for (int p = 0; p < nProb; ++p)
        for (int32_t m = nodePtr[p]; m < nodePtr[p + 1]; ++m) prob[m] = p;
    for (int64_t m = 0; m < c->nNodes; ++m)
        for (int32_t k = c->hRowPtr0[m]; k < c->hRowPtr0[m + 1]; ++k)
            if (prob[c->hColIdx0[k]] != prob[m]) {
                ef_set_error("ef_batch_setup: a block couples two problems");
                return EF_ERR_ARG;
            }
    std::vector<int32_t> order(nProb);
    for (int p = 0; p < nProb; ++p) order[p] = p;
    std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
        return nodePtr[a + 1] - nodePtr[a] > nodePtr[b + 1] - nodePtr[b];
    });
    if (c->dBatchNodePtr) cudaFree(c->dBatchNodePtr);
    if (c->dBatchOrder) cudaFree(c->dBatchOrder);
    ef_status st = EF_OK;
    c->dBatchNodePtr = dalloc<int32_t>(nProb + 1, &st);
    c->dBatchOrder = dalloc<int32_t>(nProb, &st);
    if (st != EF_OK) return st;
    EF_CUDA(cudaMemcpy(c->dBatchNodePtr, nodePtr, sizeof(int32_t) * (nProb + 1), cudaMemcpyHostToDevice));
    EF_CUDA(cudaMemcpy(c->dBatchOrder, order.data(), sizeof(int32_t) * nProb, cudaMemcpyHostToDevice));
    c->batchN = nProb;
    return EF_OK;
}

ef_status ef_batch_set_tile(ef_ctx* c, int tile) {
    EF_REQUIRE_FINALIZED(c);
    if (tile < 0 || tile >= ef_batch_num_tiles()) {
        ef_set_error("ef_batch_set_tile: unknown tile shape");
        return EF_ERR_ARG;
    }
    c->batchTile = tile;
    return EF_OK;
}

int ef_batch_tile_count(void) { return ef_batch_num_tiles(); }

ef_status ef_batch_tile_info(int tile, int* threadsPerCta, int* lanesPerRow) {
    if (tile < 0 || tile >= ef_batch_num_tiles() || !threadsPerCta || !lanesPerRow) return EF_ERR_ARG;
    ef_batch_tile_shape(tile, threadsPerCta, lanesPerRow);
    return EF_OK;
}

static ef_status batch_solve(ef_ctx* c, int tile, double rtol, int maxIter, const double* b, double* x, int* iters,
                             double* relres, cudaStream_t s) {
    const int64_t n = c->nDof;
    double* xd = c->w64[0];
    double* r64 = c->w64[2];
    // Dirichlet DOFs take b; the free part solves K_ff x_f = b_f - K_fd x_d per problem
    EF_CHECK(ef_launch_masked_copy(n, b, c->dMask, 1, 1.0, xd, 1, s));
    EF_CHECK(residual64(c, xd, b, r64, s));
    double* w[5];
    for (int i = 0; i < 5; ++i) w[i] = (double*)c->w64k[1 + i];
    EF_CHECK(ef_launch_batched_pcg(tile, c->nSM, c->batchN, c->dBatchNodePtr, c->dBatchOrder, c->dRowPtr, c->dColIdx,
                                   (const double*)c->dBsrVals, (const double*)c->dBinv, c->dMask, r64, w[0], w[1],
                                   w[2], w[3], w[4], maxIter, rtol * rtol, iters, relres, s));
    return ef_launch_add(n, xd, w[0], x, s);
}

ef_status ef_batch_solve(ef_ctx* c, double rtol, int maxIter, const double* b, double* x, int* iters, double* relres,
                         void* stream) {
    EF_REQUIRE_FINALIZED(c);
    if (c->batchN == 0) {
        ef_set_error("ef_batch_solve: call ef_batch_setup first");
        return EF_ERR_STATE;
    }
    if (!b || !x || !iters || !relres || !(rtol > 0.0) || maxIter < 0) return EF_ERR_ARG;
    return batch_solve(c, c->batchTile, rtol, maxIter, b, x, iters, relres, (cudaStream_t)stream);
}

ef_status ef_batch_autotune(ef_ctx* c, double rtol, int maxIter, const double* b, double* x, int* iters,
                            double* relres, void* stream, int* tileOut, float* msOut) {
    EF_REQUIRE_FINALIZED(c);
    if (c->batchN == 0) {
        ef_set_error("ef_batch_autotune: call ef_batch_setup first");
        return EF_ERR_STATE;
    }
    cudaStream_t s = (cudaStream_t)stream;
    float best = 1e30f;
    int bestT = c->batchTile;
    for (int t = 0; t < ef_batch_num_tiles(); ++t) {
        EF_CHECK(batch_solve(c, t, rtol, maxIter, b, x, iters, relres, s));  // warm-up
        EF_CUDA(cudaEventRecord(c->ev[0], s));
        EF_CHECK(batch_solve(c, t, rtol, maxIter, b, x, iters, relres, s));
        EF_CUDA(cudaEventRecord(c->ev[1], s));
        EF_CUDA(cudaEventSynchronize(c->ev[1]));
        float ms = 0.f;
        EF_CUDA(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
        if (msOut) msOut[t] = ms;
        if (ms < best) {
            best = ms;
            bestT = t;
        }
    }
    c->batchTile = bestT;
    if (tileOut) *tileOut = bestT;
    return EF_OK;
}

ef_status ef_batch_norms(ef_ctx* c, const double* R, const double* F, const double* ddU, double* out, void* stream) {
    EF_REQUIRE_FINALIZED(c);
    if (c->batchN == 0) {
        ef_set_error("ef_batch_norms: call ef_batch_setup first");
        return EF_ERR_STATE;
    }
    if (!R || !F || !out) return EF_ERR_ARG;
    return ef_launch_batch_norms(c->batchN, c->dBatchNodePtr, R, F, ddU, out, (cudaStream_t)stream);
}

ef_status ef_mpnn_dense_eval(int tensorCores, int nNodes, const float* h, const float* agg, const float* W,
                             float* q, float* hout, int* flags, void* stream) {
    if (nNodes <= 0 || !h || !agg || !W || !q || !hout || !flags) return EF_ERR_ARG;
    return ef_mpnn_dense_eval_host(tensorCores ? 1 : 0, nNodes, h, agg, W, q, hout, flags, (cudaStream_t)stream);
}

int64_t ef_kernel_launches(void) { return (int64_t)ef::launches(); }

int ef_mpnn_param_count(void) { return ef_mpnn_nparam(); }

ef_status ef_mpnn_init(ef_ctx* c, uint64_t seed, int maxSamples) {
    EF_REQUIRE_FINALIZED(c);
    if (maxSamples < 0) return EF_ERR_ARG;
    if (c->keFp64) {
        ef_set_error("ef_mpnn_init: the learned correction runs inside the FP32 FGMRES (mixed mode)");
        return EF_ERR_ARG;
    }
    EF_CHECK(ef_mpnn_setup_kernels());
    const int np = ef_mpnn_nparam(), H = ef_mpnn_hidden();
    if (!c->nnInit) {
        ef_status st = EF_OK;
        const int64_t nN = c->nNodes, NH = nN * H;
        c->nnP = dalloc<float>(np, &st);
        c->nnPf = dalloc<float>(np, &st);
        c->nnM1 = dalloc<float>(np, &st);
        c->nnM2 = dalloc<float>(np, &st);
        c->nnG = dalloc<float>(np, &st);
        c->nnPb = dalloc<uint16_t>(np, &st);
        c->nnActs = dalloc<float>(10 * NH, &st);
        c->nnF = dalloc<float>(9 * nN, &st);
        c->nnWork = dalloc<float>(4 * NH, &st);
        c->nnPartN = 2 * c->nSM;
        c->nnPart = dalloc<float>((size_t)c->nnPartN * H * H, &st);
        c->nnA = dalloc<float>(c->nBlocks, &st);
        c->nnAT = dalloc<float>(c->nBlocks, &st);
        c->nnTpos = dalloc<int64_t>(c->nBlocks, &st);
        if (!c->nnRed) c->nnRed = dalloc<double>(3 * (size_t)c->nnPartN + 8, &st);
        c->vcOut2 = dalloc<float>(c->nDof, &st);
        c->nnD = dalloc<float>(c->nDof, &st);
        c->nnKd = dalloc<float>(c->nDof, &st);
        c->nnRho = dalloc<float>(c->nDof, &st);
        c->nnN = dalloc<float>(c->nDof, &st);
        c->nnKN = dalloc<float>(c->nDof, &st);
        if (st != EF_OK) return st;
        std::vector<int64_t> tpos;
        EF_CHECK(nn_transpose_map(c->hRowPtr0, c->hColIdx0, tpos));
        EF_CUDA(cudaMemcpy(c->nnTpos, tpos.data(), sizeof(int64_t) * tpos.size(), cudaMemcpyHostToDevice));
        c->nnInit = true;
        c->amgStale = true;  // edge weights are computed with the next refresh
        c->nnEdgeStale = true;
    }
    // He-scaled normal weights; residual branches damped; output layer zero (z = Mv at start)
    std::mt19937_64 g(seed);
    std::vector<float> hp(np, 0.f);
    nn_normal(g, (float)sqrt(2.0 / 9.0), hp.data(), H * 9);
    for (int l = 0; l < 3; ++l) nn_normal(g, (float)(0.5 * sqrt(2.0 / (2.0 * H))), hp.data() + ef_mpnn_layer_offset(l), 2 * H * H);
    EF_CHECK(nn_upload_params(c, hp.data(), nullptr));
    c->nnScalesSet = false;
    c->nnS[0] = c->nnS[1] = c->nnS[2] = 1.f;
    c->nnSo = 1.f;
    c->nnMaxSamples = maxSamples;
    c->nnMaxSystems = std::min(maxSamples, 16);
    if (c->nnGraph) {
        cudaGraphExecDestroy(c->nnGraph);
        c->nnGraph = nullptr;
    }
    return EF_OK;
}

ef_status ef_mpnn_set_params(ef_ctx* c, const float* params, const float* scales) {
    EF_REQUIRE_FINALIZED(c);
    if (!c->nnInit) {
        ef_set_error("ef_mpnn_set_params: call ef_mpnn_init first");
        return EF_ERR_STATE;
    }
    if (params) EF_CHECK(nn_upload_params(c, params, nullptr));
    if (scales) {
        for (int i = 0; i < 3; ++i) c->nnS[i] = scales[i];
        c->nnSo = scales[3];
        c->nnScalesSet = true;
        if (c->nnGraph) {
            cudaGraphExecDestroy(c->nnGraph);
            c->nnGraph = nullptr;
        }
    }
    return EF_OK;
}

ef_status ef_mpnn_get_params(ef_ctx* c, float* params, float* scales) {
    EF_REQUIRE_FINALIZED(c);
    if (!c->nnInit) {
        ef_set_error("ef_mpnn_get_params: call ef_mpnn_init first");
        return EF_ERR_STATE;
    }
    if (params) EF_CUDA(cudaMemcpy(params, c->nnP, sizeof(float) * ef_mpnn_nparam(), cudaMemcpyDeviceToHost));
    if (scales) {
        for (int i = 0; i < 3; ++i) scales[i] = c->nnS[i];
        scales[3] = c->nnSo;
    }
    return EF_OK;
}

ef_status ef_mpnn_enable(ef_ctx* c, int on) {
    EF_REQUIRE_FINALIZED(c);
    if (on && !c->nnInit) {
        ef_set_error("ef_mpnn_enable: call ef_mpnn_init first");
        return EF_ERR_STATE;
    }
    c->nnOn = on != 0;
    return EF_OK;
}

ef_status ef_mpnn_collect(ef_ctx* c, int every, int maxPerSolve, int kind) {
    EF_REQUIRE_FINALIZED(c);
    if (every < 0 || maxPerSolve < 0 || kind < 0 || kind > 1) return EF_ERR_ARG;
    c->nnKind = kind;
    if ((every > 0 || maxPerSolve > 0) && !c->nnInit) {
        ef_set_error("ef_mpnn_collect: call ef_mpnn_init first");
        return EF_ERR_STATE;
    }
    c->nnEvery = every;
    c->nnMaxPerSolve = maxPerSolve;
    return EF_OK;
}

ef_status ef_mpnn_add_sample(ef_ctx* c, const double* r, const double* e, void* stream) {
    EF_REQUIRE_FINALIZED(c);
    if (!r || !e) return EF_ERR_ARG;
    if (!c->nnInit) {
        ef_set_error("ef_mpnn_add_sample: call ef_mpnn_init first");
        return EF_ERR_STATE;
    }
    if (c->nnMaxSamples == 0) return EF_OK;
    cudaStream_t s = (cudaStream_t)stream;
    if (c->fgPc == EF_FGMRES_PC_MULTIGRID) {
        EF_CHECK(amg_build(c));
        EF_CHECK(amg_refresh(c, s));
    } else {
        EF_CHECK(amg_workspace(c));
        EF_CHECK(nn_edge_refresh(c, s));
    }
    const int64_t n = c->nDof;
    float* rf = (float*)c->w32[5];
    float* ef = (float*)c->w32[6];
    EF_CHECK(ef_launch_masked_copy(n, r, c->dMask, 0, 1.0, rf, 0, s));
    EF_CHECK(ef_launch_masked_copy(n, e, c->dMask, 0, 1.0, ef, 0, s));
    return nn_add_sample(c, rf, ef, s);
}

ef_status ef_mpnn_num_samples(const ef_ctx* c, int* n) {
    if (!c || !n) return EF_ERR_ARG;
    int k = 0;
    for (const auto& S : c->nnSamples) k += S.sys >= 0;
    *n = k;
    return EF_OK;
}

ef_status ef_mpnn_clear_samples(ef_ctx* c) {
    EF_REQUIRE_FINALIZED(c);
    for (auto& S : c->nnSamples) S.sys = -1;
    for (auto& Y : c->nnSystems) Y.version = -1;
    c->nnAdded = 0;
    return EF_OK;
}

ef_status ef_mpnn_train(ef_ctx* c, int epochs, float lr, int norm, double* lossFirst, double* lossLast,
                        void* stream) {
    EF_REQUIRE_FINALIZED(c);
    if (epochs < 0 || !(lr >= 0.f) || norm < 0 || norm > 2) return EF_ERR_ARG;
    if (!c->nnInit) {
        ef_set_error("ef_mpnn_train: call ef_mpnn_init first");
        return EF_ERR_STATE;
    }
    return nn_train(c, epochs, lr, norm, lossFirst, lossLast, (cudaStream_t)stream);
}

ef_status ef_mpnn_eval(int nNodes, const int32_t* rowPtr, const int32_t* colIdx, const float* vals,
                       const float* params, const float* f, const float* base, const float* e, const uint8_t* mask,
                       float so, float scale, float* z, float* grad, double* loss, void* stream) {
    if (nNodes <= 0 || !rowPtr || !colIdx || !vals || !params || !f || !e || !z) return EF_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    EF_CHECK(ef_mpnn_setup_kernels());
    const int64_t nN = nNodes, nb = rowPtr[nNodes], n = 3 * nN, H = ef_mpnn_hidden(), np = ef_mpnn_nparam();
    std::vector<int32_t> hr(rowPtr, rowPtr + nN + 1), hc(colIdx, colIdx + nb);
    for (int64_t m = 0; m < nN; ++m)
        if (hr[m + 1] < hr[m]) return EF_ERR_ARG;
    for (int32_t k : hc)
        if (k < 0 || k >= nNodes) return EF_ERR_ARG;
    std::vector<int64_t> tpos;
    EF_CHECK(nn_transpose_map(hr, hc, tpos));
    int dev = 0, nSM = 1;
    EF_CUDA(cudaGetDevice(&dev));
    EF_CUDA(cudaDeviceGetAttribute(&nSM, cudaDevAttrMultiProcessorCount, dev));
    const int nPart = 2 * nSM;
    ef_status st = EF_OK;
    std::vector<void*> owned;
    auto A = [&](size_t bytes) {
        void* p = nullptr;
        if (cudaMalloc(&p, bytes ? bytes : 1) != cudaSuccess) {
            st = EF_ERR_CUDA;
            return (void*)nullptr;
        }
        owned.push_back(p);
        return p;
    };
    int32_t* dR = (int32_t*)A(sizeof(int32_t) * (nN + 1));
    int32_t* dC = (int32_t*)A(sizeof(int32_t) * nb);
    float* dV = (float*)A(sizeof(float) * 9 * nb);
    float* dA = (float*)A(sizeof(float) * nb);
    float* dAT = (float*)A(sizeof(float) * nb);
    int64_t* dT = (int64_t*)A(sizeof(int64_t) * nb);
    float* dP = (float*)A(sizeof(float) * np);
    float* dF = (float*)A(sizeof(float) * 9 * nN);
    float* dB = base ? (float*)A(sizeof(float) * n) : nullptr;
    float* dE = (float*)A(sizeof(float) * n);
    uint8_t* dM = mask ? (uint8_t*)A(n) : nullptr;
    float* dZ = (float*)A(sizeof(float) * n);
    float* dG = (float*)A(sizeof(float) * np);
    float* acts = (float*)A(sizeof(float) * 10 * nN * H);
    float* work = (float*)A(sizeof(float) * 4 * nN * H);
    float* part = (float*)A(sizeof(float) * (size_t)nPart * H * H);
    double* red = (double*)A(sizeof(double) * (3 * nPart + 8));
    auto finish = [&](ef_status r) {
        for (void* p : owned) cudaFree(p);
        return r;
    };
    if (st != EF_OK) {
        ef_set_error("ef_mpnn_eval: cudaMalloc failed");
        return finish(st);
    }
#define EV_CUDA(x)                                                              \
    do {                                                                        \
        cudaError_t e_ = (x);                                                   \
        if (e_ != cudaSuccess) {                                                \
            ef_set_error(std::string("ef_mpnn_eval: ") + cudaGetErrorString(e_)); \
            return finish(EF_ERR_CUDA);                                         \
        }                                                                       \
    } while (0)
#define EV_CHECK(x)                   \
    do {                              \
        ef_status s_ = (x);           \
        if (s_ != EF_OK) return finish(s_); \
    } while (0)
    EV_CUDA(cudaMemcpyAsync(dR, hr.data(), sizeof(int32_t) * (nN + 1), cudaMemcpyHostToDevice, s));
    EV_CUDA(cudaMemcpyAsync(dC, hc.data(), sizeof(int32_t) * nb, cudaMemcpyHostToDevice, s));
    EV_CUDA(cudaMemcpyAsync(dV, vals, sizeof(float) * 9 * nb, cudaMemcpyHostToDevice, s));
    EV_CUDA(cudaMemcpyAsync(dT, tpos.data(), sizeof(int64_t) * nb, cudaMemcpyHostToDevice, s));
    EV_CUDA(cudaMemcpyAsync(dP, params, sizeof(float) * np, cudaMemcpyHostToDevice, s));
    EV_CUDA(cudaMemcpyAsync(dF, f, sizeof(float) * 9 * nN, cudaMemcpyHostToDevice, s));
    if (dB) EV_CUDA(cudaMemcpyAsync(dB, base, sizeof(float) * n, cudaMemcpyHostToDevice, s));
    EV_CUDA(cudaMemcpyAsync(dE, e, sizeof(float) * n, cudaMemcpyHostToDevice, s));
    if (dM) EV_CUDA(cudaMemcpyAsync(dM, mask, n, cudaMemcpyHostToDevice, s));
    EV_CHECK(ef_launch_edge_weights((int)nN, dR, dC, dV, dA, s));
    EV_CHECK(ef_launch_gather_f32(nb, dT, dA, dAT, s));
    EV_CHECK(ef_mpnn_forward((int)nN, dR, dC, dA, dP, dF, dB, dM, so, acts, dZ, 0, nullptr, s));
    EV_CHECK(ef_mpnn_sumsq(n, 1, dZ, dE, dM, red, nPart, red + 3 * nPart, s));
    if (grad)
        EV_CHECK(ef_mpnn_backward((int)nN, dR, dC, dAT, dP, dF, acts, dZ, dE, dM, scale, so, dG, work, part, nPart, s));
    EV_CUDA(cudaMemcpyAsync(z, dZ, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
    if (grad) EV_CUDA(cudaMemcpyAsync(grad, dG, sizeof(float) * np, cudaMemcpyDeviceToHost, s));
    double l2 = 0.0;
    EV_CUDA(cudaMemcpyAsync(&l2, red + 3 * nPart, sizeof(double), cudaMemcpyDeviceToHost, s));
    EV_CUDA(cudaStreamSynchronize(s));
    if (loss) *loss = 0.5 * (double)scale * l2;
#undef EV_CUDA
#undef EV_CHECK
    return finish(EF_OK);
}

ef_status ef_newton_residual(ef_ctx* c, int mode, const double* P, const double* PExt, const double* dirValues,
                             const double* F, const double* ddU, int iteration, double prevResidual, int nGrew,
                             const ef_newton_opts* o, double* R, ef_newton_check* out, void* stream) {
    EF_REQUIRE_FINALIZED(c);
    if (!P || !R || (mode != 0 && mode != 1) || (mode == 1 && (!F || !o || !out)) ||
        (mode == 0 && c->nDir > 0 && !dirValues)) {
        ef_set_error("ef_newton_residual: bad arguments");
        return EF_ERR_ARG;
    }
    if (!c->dDirMask) {
        ef_set_error("ef_newton_residual: call ef_set_dirichlet first");
        return EF_ERR_STATE;
    }
    cudaStream_t s = (cudaStream_t)stream;
    if (mode == 0) return ef_launch_newton_first(c->nDof, P, PExt, c->nDir, c->dDirIdx, dirValues, R, s);
    if (!c->dNewton) {
        ef_status st = EF_OK;
        c->dNewton = dalloc<double>(16, &st);
        if (!c->dNewton) return st;
    }
    const double q[9] = {o->fluxTol, o->fluxTolAlt, o->corrTol, o->fluxFloor, o->nAccFluxes, prevResidual,
                         (double)iteration, (double)nGrew, ddU ? 1.0 : 0.0};
    EF_CUDA(cudaMemcpyAsync(c->dNewton, q, sizeof(q), cudaMemcpyHostToDevice, s));
    EF_CHECK(ef_launch_newton_check(c->nDof, P, PExt, c->dDirMask, F, ddU, R, c->dPart, c->nPart, c->dNewton,
                                    c->dNewton + 9, s));
    double r[5];
    EF_CUDA(cudaMemcpyAsync(r, c->dNewton + 9, sizeof(r), cudaMemcpyDeviceToHost, s));
    EF_CUDA(cudaStreamSynchronize(s));
    out->converged = r[0] != 0.0;
    out->nGrew = (int)r[1];
    out->fluxResidual = r[2];
    out->fieldCorrection = r[3];
    out->spatialAveragedFlux = r[4];
    return EF_OK;
}

ef_status ef_norms(ef_ctx* c, const double* R, const double* F, const double* ddU, double* out, void* stream) {
    EF_REQUIRE_FINALIZED(c);
    if (!out) return EF_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    EF_CHECK(ef_launch_norms(c->nDof, R, F, ddU, c->dPart, c->nPart, c->dRed, s));
    EF_CUDA(cudaMemcpyAsync(out, c->dRed, 3 * sizeof(double), cudaMemcpyDeviceToHost, s));
    EF_CUDA(cudaStreamSynchronize(s));
    return EF_OK;
}

// ---- element result collectors (utils/elementresultcollector.pyx:38-120) ----------------------

static ResultCollector* result_collector(ef_ctx* c, int id) {
    if (id < 0 || id >= (int)c->results.size() || c->results[id].group < 0) {
        ef_set_error("element result collector: unknown id");
        return nullptr;
    }
    return &c->results[id];
}

ef_status ef_results_create(ef_ctx* c, int groupId, const int32_t* elements, int nEls, const int32_t* qps, int nQps,
                            int first, int count, int* collectorId) {
    EF_REQUIRE_FINALIZED(c);
    if (groupId < 0 || groupId >= (int)c->groups.size() || !collectorId) {
        ef_set_error("ef_results_create: invalid group or output");
        return EF_ERR_ARG;
    }
    const Group& g = c->groups[groupId];
    if (first < 0 || count < 1 || first + count > g.nState) {
        ef_set_error("ef_results_create: state slice outside [0, nState)");
        return EF_ERR_ARG;
    }
    std::vector<int32_t> el, qp;
    if (elements) {
        if (nEls < 1) {
            ef_set_error("ef_results_create: empty element list");
            return EF_ERR_ARG;
        }
        el.assign(elements, elements + nEls);
    } else {
        el.resize(g.nEl);
        for (int e = 0; e < g.nEl; ++e) el[e] = e;
    }
    if (qps) {
        if (nQps < 1) {
            ef_set_error("ef_results_create: empty quadrature point list");
            return EF_ERR_ARG;
        }
        qp.assign(qps, qps + nQps);
    } else {
        qp.resize(g.nQP);
        for (int q = 0; q < g.nQP; ++q) qp[q] = q;
    }
    for (int32_t e : el)
        if (e < 0 || e >= g.nEl) {
            ef_set_error("ef_results_create: element index outside the group");
            return EF_ERR_ARG;
        }
    for (int32_t q : qp)
        if (q < 0 || q >= g.nQP) {
            ef_set_error("ef_results_create: quadrature point outside the element");
            return EF_ERR_ARG;
        }
    ResultCollector r;
    r.nEls = (int)el.size();
    r.nQ = (int)qp.size();
    r.first = first;
    r.count = count;
    ef_status st = upload(&r.dEl, el);
    if (st == EF_OK) st = upload(&r.dQp, qp);
    if (st == EF_OK) r.dTable = dalloc<double>((size_t)r.nEls * r.nQ * count, &st);
    if (st != EF_OK) {
        for (void* p : {(void*)r.dEl, (void*)r.dQp, (void*)r.dTable})
            if (p) cudaFree(p);
        return st;
    }
    r.group = groupId;
    int id = 0;
    while (id < (int)c->results.size() && c->results[id].group >= 0) ++id;
    if (id == (int)c->results.size())
        c->results.push_back(r);
    else
        c->results[id] = r;
    *collectorId = id;
    return EF_OK;
}

ef_status ef_results_update(ef_ctx* c, int collectorId, int trial, double* hostOut, void* stream) {
    EF_REQUIRE_FINALIZED(c);
    const ResultCollector* r = result_collector(c, collectorId);
    if (!r) return EF_ERR_ARG;
    const Group& g = c->groups[r->group];
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t nPts = (int64_t)r->nEls * r->nQ;
    EF_CHECK(ef_launch_results_gather(nPts, r->nQ, g.nQP, (int64_t)g.nEl * g.nQP, r->first, r->count, r->dEl, r->dQp,
                                      g.state[trial ? 1 - g.cur : g.cur], r->dTable, s));
    if (hostOut) {
        EF_CUDA(cudaMemcpyAsync(hostOut, r->dTable, sizeof(double) * nPts * r->count, cudaMemcpyDeviceToHost, s));
        EF_CUDA(cudaStreamSynchronize(s));
    }
    return EF_OK;
}

ef_status ef_results_device(ef_ctx* c, int collectorId, const double** table, int64_t* nValues) {
    EF_REQUIRE_FINALIZED(c);
    const ResultCollector* r = result_collector(c, collectorId);
    if (!r || !table) return EF_ERR_ARG;
    *table = r->dTable;
    if (nValues) *nValues = (int64_t)r->nEls * r->nQ * r->count;
    return EF_OK;
}

ef_status ef_results_destroy(ef_ctx* c, int collectorId) {
    EF_REQUIRE_FINALIZED(c);
    ResultCollector* r = result_collector(c, collectorId);
    if (!r) return EF_ERR_ARG;
    EF_CUDA(cudaFree(r->dEl));
    EF_CUDA(cudaFree(r->dQp));
    EF_CUDA(cudaFree(r->dTable));
    *r = ResultCollector();
    return EF_OK;
}

}  // extern "C"
