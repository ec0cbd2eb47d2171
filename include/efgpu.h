/*
 * efgpu.h -- C ABI of the GB300 (sm_103a) implementation of EdelweissFE's
 * data-parallel hot path: the NISTParallel element loop, the VIJ -> CSR
 * scatter and the Krylov solve that consumes the assembled system.
 *
 * Conventions
 *  - Plain pointers and sizes only.  Vectors named U, dU, P, F, PExt, b, x,
 *    Kvij, csrData are DEVICE pointers owned by the caller; setup arrays
 *    (coordinates, element DOF lists, Dirichlet DOF lists) are HOST pointers
 *    and are copied.  `stream` is a cudaStream_t (NULL = legacy stream).
 *  - All hot-path calls are stream ordered and do not synchronise, except
 *    the ones documented as synchronising (status reads, solve info).
 *  - No exception crosses the ABI: every call returns an ef_status and
 *    ef_last_error() holds a message for the calling thread.
 *  - A context is not re-entrant: one host thread at a time.
 *
 * Reference call sites each entry point replaces are cited (paths relative to
 * the EdelweissFE source tree).
 */
#ifndef EFGPU_H
#define EFGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum ef_status {
    EF_OK = 0,
    EF_CUTBACK = 1,       /* an element requested a smaller increment (utils/exceptions.py:44 CutbackRequest) */
    EF_NAN = 2,           /* NaN in element results or in a solve (solvers/nonlinearimplicitstatic.py:748) */
    EF_NOT_CONVERGED = 3, /* Krylov solve reached its iteration cap without meeting the tolerance */
    EF_ERR_ARG = 10,      /* invalid argument */
    EF_ERR_CUDA = 11,     /* CUDA runtime error (message in ef_last_error) */
    EF_ERR_STATE = 12,    /* call out of order (e.g. before ef_finalize) */
    EF_ERR_DEVICE = 13    /* device-side failure reported by a kernel (e.g. a bounded wait gave up) */
} ef_status;

typedef struct ef_ctx ef_ctx;

/* options of ef_finalize */
#define EF_OPT_KE_FP64 1      /* element stiffness and BSR system in FP64 (default FP32) */
#define EF_OPT_NO_SCALAR_CSR 2 /* do not build the scalar (reference-layout) CSR slot map */

/* solve methods */
#define EF_SOLVE_PCG 0     /* block-Jacobi (3x3 nodal) preconditioned CG */
#define EF_SOLVE_FGMRES 1  /* flexible GMRES(m), right preconditioned by block Jacobi */

typedef struct ef_info {
    int64_t nDof;
    int64_t nNodes;      /* DOF triplets (block rows of the BSR system) */
    int64_t nElements;
    int64_t nVIJ;        /* length of the VIJ value vector (sum of nDofEl^2) */
    int64_t nnz;         /* scalar CSR non-zeros (0 when EF_OPT_NO_SCALAR_CSR) */
    int64_t nBlocks;     /* 3x3 blocks of the BSR system */
    int64_t nPe;         /* length of the element residual buffer (sum of nDofEl) */
    int keFp64;
} ef_info;

typedef struct ef_solve_opts {
    int method;          /* EF_SOLVE_PCG or EF_SOLVE_FGMRES */
    int mixed;           /* 1: FP32 inner iterations + FP64 iterative refinement; 0: all FP64 */
    double rtol;         /* target ||b - A x||_2 / ||b||_2 in FP64 */
    double innerRtol;    /* relative tolerance of one inner solve (mixed mode) */
    int maxIter;         /* cap on the total number of Krylov iterations */
    int restart;         /* FGMRES restart length */
    int maxRefine;       /* cap on refinement sweeps (mixed mode) */
    int profile;         /* 1: time the Krylov kernel launches with CUDA events (ef_solve_info.kernelMs) */
} ef_solve_opts;

typedef struct ef_solve_info {
    int iterations;      /* total Krylov iterations */
    int refinements;     /* outer refinement sweeps */
    double relResidual;  /* final ||b - A x|| / ||b|| computed in FP64 */
    int status;          /* ef_status of the solve */
    double kernelMs;     /* summed duration of the Krylov kernel launches (profile = 1) */
    int kernelLaunches;  /* number of Krylov kernel launches timed */
} ef_solve_info;

int ef_abi_version(void);
const char* ef_last_error(void);

/* ---- model setup: numerics/dofmanager.py:153-218 (DofManager), :522-557 (VIJ pattern),
 *      elements/displacementelement/element.py:194-240 (initializeElement, setMaterial),
 *      numerics/csrgenerator.pyx:47-97 (CSRGenerator.__init__) ---- */

/* nodeCoords: host [nDof]; entry d is the coordinate (component d - first DOF of the
 * node) of the node that owns DOF d, i.e. the node coordinates written into a DofVector. */
ef_status ef_create(int64_t nDof, const double* nodeCoords, ef_ctx** out);
void ef_destroy(ef_ctx* ctx);

/* elType: C3D8, C3D8R, C3D8E, C3D20, C3D20R (small strain) or C3D8TL, C3D20TL (total
 * Lagrange); material: linearelastic [E, nu], vonmises [E, nu, fy0, HLin, dfy, delta],
 * neohookewa [mu, K].  elDofs: host [nEl][3*nNodes] global DOFs of each element in element
 * DOF order (DofManager.idcsOfHigherOrderEntitiesInDofVector); each node's three DOFs must
 * be consecutive.  Groups are appended in the reference's element order. */
ef_status ef_add_group(ef_ctx* ctx, const char* elType, const char* material, const double* props, int nProps,
                       int nEl, const int32_t* elDofs, int* groupId);
ef_status ef_finalize(ef_ctx* ctx, int options);
ef_status ef_get_info(const ef_ctx* ctx, ef_info* out);

/* ---- element loop: solvers/nonlinearimplicitstaticparallelmk2.pyx:111-198 and
 *      solvers/nonlinearimplicitstatic.py:794-849 (computeElements) ---- */

/* Evaluates every element from the committed state: trial state, Pe, Ke (kept on the
 * device), and condenses P[d] = sum Pe, F[d] = sum |Pe| in element order.  U_np, dU, P, F
 * are device [nDof].  time2 is host [stepTime, totalTime]. */
ef_status ef_compute_elements(ef_ctx* ctx, const double* U_np, const double* dU, const double* time2, double dT,
                              double* P, double* F, void* stream);

/* Synchronises `stream` and returns the element status of the last ef_compute_elements:
 * EF_OK, EF_CUTBACK (J2 return map failed; the reference raises CutbackRequest(.., 0.5),
 * materials/vonmises/vonmises.py:231) or EF_NAN.  *pNewDT receives the suggested increment
 * scale (1.0, or 0.5 on cutback).  Resets the flags. */
ef_status ef_element_status(ef_ctx* ctx, void* stream, double* pNewDT);

/* Per-Gauss-point state of a group, host [nEl][nQP][nState] with the reference layout
 * [stress(6), strain(6), material state] (elements/displacementelement/element.py:222-236).
 * ef_set_state writes the committed state (setInitialCondition / restart);
 * ef_get_state reads the committed (trial = 0) or trial (trial = 1) state (getResultArray). */
ef_status ef_get_state_size(const ef_ctx* ctx, int groupId, int* nQP, int* nState);
ef_status ef_set_state(ef_ctx* ctx, int groupId, const double* state);
ef_status ef_get_state(ef_ctx* ctx, int groupId, int trial, double* state);

/* elements/displacementelement/element.py:373-379 acceptLastState for all elements */
ef_status ef_accept_state(ef_ctx* ctx);

/* elements/displacementelement/element.py:348-371 computeBodyForce, added into PExt (device [nDof]) */
ef_status ef_add_body_force(ef_ctx* ctx, int groupId, const double* load3, double* PExt, void* stream);

/* ---- VIJ -> CSR: numerics/dofmanager.py:47-82 (VIJSystemMatrix values) and
 *      numerics/csrgenerator.pyx:100-115 (updateCSR) ---- */

/* Writes the VIJ value vector (device [nVIJ], FP64) in the reference layout: value a*n+b
 * of an element's slice is Ke[a][b]. */
ef_status ef_export_vij(ef_ctx* ctx, double* Kvij, void* stream);
/* Canonical CSR pattern of the (I, J) pairs; host or device buffers [nDof+1], [nnz]. */
ef_status ef_csr_pattern(ef_ctx* ctx, int32_t* indptr, int32_t* indices);
/* data[s] = sum of Kvij[k] over the VIJ pairs k of slot s, added in increasing k from 0.0:
 * bit-identical to the reference's serial loop.  Kvij = NULL uses the context's own element
 * stiffness (exported in FP64 first). */
ef_status ef_update_csr(ef_ctx* ctx, const double* Kvij, double* csrData, void* stream);
/* solvers/nonlinearimplicitstaticparallelmk2.pyx:66-109 applyDirichletK without the final
 * eliminate_zeros: rows (host [nRows]) zeroed, diagonal 1. */
ef_status ef_csr_dirichlet_rows(ef_ctx* ctx, double* csrData, const int64_t* rows, int64_t nRows, void* stream);

/* ---- fast path: 3x3-block (BSR) system assembled from the element blocks without
 *      atomics, Dirichlet DOFs eliminated symmetrically, Krylov solve.
 *      Replaces NIST.assembleStiffnessCSR + applyDirichletK + linearSolve
 *      (solvers/nonlinearimplicitstatic.py:451-454, 559-593, 727-769) ---- */

/* Dirichlet DOFs (host [n]); they are eliminated from the BSR operator and the solution
 * takes b at these DOFs (the reference's rows with diagonal 1 give the same solution). */
ef_status ef_set_dirichlet(ef_ctx* ctx, const int64_t* dofs, int64_t n);
ef_status ef_assemble_bsr(ef_ctx* ctx, void* stream);
/* Solves K x = b for the last assembled BSR system; b, x device [nDof] FP64.  Synchronises
 * `stream` to return the info. */
ef_status ef_solve(ef_ctx* ctx, const ef_solve_opts* opts, const double* b, double* x, ef_solve_info* info,
                   void* stream);
/* y = K x with the Dirichlet elimination applied (FP64 accumulation), device [nDof]. */
ef_status ef_bsr_matvec(ef_ctx* ctx, const double* x, double* y, void* stream);

/* ---- allocation-free solve.  No counterpart in the reference: it exists for callers that
 *      cannot allocate device memory when they solve -- a host framework that has reserved the
 *      device memory for its own pool, or a latency-critical loop that must not take the
 *      device-wide synchronisation cudaMalloc/cudaFree imply. ---- */

/* Largest number of 3x3 block rows ef_pcg_solve_noalloc accepts (its scratch is a fixed 8 MiB
 * device array that every GPU loading the library holds until the process exits). */
int64_t ef_pcg_noalloc_max_nodes(void);
/* Block-Jacobi PCG on a caller-provided FP64 BSR(3x3) system: rowPtr [nNodes+1], colIdx
 * [nBlocks] (block columns), vals [nBlocks][9] row-major blocks, binv [nNodes][9] inverses of
 * the diagonal blocks (identity rows/columns on masked DOFs), mask [3*nNodes] (1 = Dirichlet
 * DOF: its row is masked and b must be 0 there), b, x device [3*nNodes]; x is overwritten.
 * Stops at ||r||/||b|| <= rtol (recurrence residual) or maxIter.  Allocates nothing: the work
 * vectors live in the fixed scratch array.  The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress) and should come before any stream capture.  All calls
 * share the one array and it keeps the last call's contents, so calls that overlap on the GPU
 * (different streams or threads) race; serialise them.  Sizes beyond
 * ef_pcg_noalloc_max_nodes() are rejected with EF_ERR_ARG.  Synchronises `stream`. */
ef_status ef_pcg_solve_noalloc(int64_t nNodes, const int32_t* rowPtr, const int32_t* colIdx, const double* vals,
                               const double* binv, const uint8_t* mask, const double* b, double* x, int maxIter,
                               double rtol, ef_solve_info* info, void* stream);

/* ---- device reductions for the convergence check: solvers/nonlinearimplicitstatic.py:625-725
 *      (checkConvergence), :771-792 (computeSpatialAveragedFluxes) ---- */

/* out (host [3]) = { max_i |R_i|, sum_i |F_i|, max_i |ddU_i| } (ddU may be NULL -> 0).
 * Deterministic; synchronises `stream`. */
ef_status ef_norms(ef_ctx* ctx, const double* R, const double* F, const double* ddU, double* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* EFGPU_H */
