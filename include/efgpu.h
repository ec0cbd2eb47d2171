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
#define EF_SOLVE_FGMRES 1  /* flexible GMRES(m), right preconditioned by an aggregation multigrid cycle */

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
    double innerRtol;    /* relative tolerance of an inner solve (mixed mode); with FGMRES and the
                            multigrid preconditioner the solves after the first of a system stop at
                            max(innerRtol, 1e-2 or EF_REFINE_FLOOR, half the remaining target
                            relative to their right-hand side) */
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
    int kernelLaunches;  /* number of Krylov kernel launches timed (PCG: solves; FGMRES: iterations) */
    double spmvMs;       /* FGMRES: summed duration of its fine-level FP32 SpMV launches (profile = 1) */
    int spmvLaunches;    /* number of those SpMV launches */
    double precondMs;    /* FGMRES: summed duration of the preconditioner applications (profile = 1) */
    double orthoMs;      /* FGMRES: summed duration of the Gram-Schmidt steps (profile = 1) */
    int reorths;         /* FGMRES: columns that the DGKS test re-orthogonalised (profile = 1) */
    double setupMs;      /* FGMRES: duration of the preconditioner set-up for a new system (profile = 1) */
} ef_solve_info;

int ef_abi_version(void);
const char* ef_last_error(void);
/* Kernels this library has launched in this process so far (a CUDA-graph launch counts the
 * kernels in the graph). */
int64_t ef_kernel_launches(void);

/* ---- model setup: numerics/dofmanager.py:153-218 (DofManager), :522-557 (VIJ pattern),
 *      elements/displacementelement/element.py:194-240 (initializeElement, setMaterial),
 *      numerics/csrgenerator.pyx:47-97 (CSRGenerator.__init__) ---- */

/* nodeCoords: host [nDof]; entry d is the coordinate (component d - first DOF of the
 * node) of the node that owns DOF d, i.e. the node coordinates written into a DofVector. */
ef_status ef_create(int64_t nDof, const double* nodeCoords, ef_ctx** out);
void ef_destroy(ef_ctx* ctx);

/* elType (elements/library.py): C3D8, C3D8R, C3D8E, C3D20, C3D20R (small strain) or C3D8TL,
 * C3D8RTL, C3D8ETL, C3D20TL, C3D20RTL (total Lagrange), and the aliases C3D8N, C3D20N, C3D8NTL,
 * C3D20NTL; material: linearelastic [E, nu], vonmises [E, nu, fy0, HLin, dfy, delta],
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
 * EF_OK, EF_CUTBACK (a material update failed: the reference's J2 raises CutbackRequest(.., 0.5),
 * materials/vonmises/vonmises.py:231) or EF_NAN.  *pNewDT receives the suggested increment
 * scale: 1.0, or on cutback the smallest scale any failing element asked for (its group's
 * ef_set_group_cutback value, default 0.5), the min over elements of the Marmot element loop
 * (solvers/nonlinearimplicitstaticparallel.pyx:136-150).  Resets the flags. */
ef_status ef_element_status(ef_ctx* ctx, void* stream, double* pNewDT);

/* Per-Gauss-point state of a group, host [nEl][nQP][nState] with the reference layout
 * [stress(6), strain(6), material state] (elements/displacementelement/element.py:222-236).
 * ef_set_state writes the committed state (setInitialCondition / restart);
 * ef_get_state reads the committed (trial = 0) or trial (trial = 1) state (getResultArray). */
ef_status ef_get_state_size(const ef_ctx* ctx, int groupId, int* nQP, int* nState);
ef_status ef_set_state(ef_ctx* ctx, int groupId, const double* state);
ef_status ef_get_state(ef_ctx* ctx, int groupId, int trial, double* state);

/* Element results (utils/elementresultcollector.pyx:38-120 ElementResultCollector, over
 * elements/displacementelement/element.py:386-409 getResultArray, whose names map to state
 * slices: "stress" [0, 6), "strain" [6, 12), "materialstate" [12, nState), the J2 "kappa" and
 * the NeoHookeWa "energy" [12, 13)).  A collector gathers, for a list of elements of one group
 * (indices within the group; NULL: all, in order) and a list of their quadrature points (NULL:
 * all), the state entries [first, first + count) of every point into one FP64 table
 * [nEls][nQps][count] on the device.  ef_results_create checks and uploads the lists (EF_ERR_ARG
 * for an index outside the group or a slice outside the state).  ef_results_update gathers the
 * committed (trial = 0, what the reference's result views show) or trial (trial = 1) state on
 * `stream` and, with hostOut non-NULL, copies the table there (host [nEls*nQps*count]; the call
 * then synchronises the stream).  ef_results_device returns the device table and its length.
 * Collectors belong to their context: ef_destroy frees those still open. */
ef_status ef_results_create(ef_ctx* ctx, int groupId, const int32_t* elements, int nEls, const int32_t* qps,
                            int nQps, int first, int count, int* collectorId);
ef_status ef_results_update(ef_ctx* ctx, int collectorId, int trial, double* hostOut, void* stream);
ef_status ef_results_device(ef_ctx* ctx, int collectorId, const double** table, int64_t* nValues);
ef_status ef_results_destroy(ef_ctx* ctx, int collectorId);

/* elements/displacementelement/element.py:373-379 acceptLastState for all elements: the trial
 * state is copied into the committed state (device-wide synchronous copy; the state buffers keep
 * their addresses, so element launches captured in a CUDA graph remain valid). */
ef_status ef_accept_state(ef_ctx* ctx);
/* elements/displacementelement/element.py:381-384 resetToLastValidState for all elements: the
 * trial state is set back to the committed one (device-wide synchronous copy).  Every element
 * pass starts from the committed state, so only a caller that reads the trial state
 * (ef_get_state or ef_results_update with trial = 1) sees a difference. */
ef_status ef_reset_state(ef_ctx* ctx);

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

/* Tolerances of the convergence check (config/phenomena.py: 1e-8, 5e-3, 1e-8; the flux floor 1e-7
 * of solvers/nonlinearimplicitstatic.py:680) and the accumulated nodal flux count of the field
 * (numerics/dofmanager.py:354-380, the sum of the elements' DOF counts). */
typedef struct ef_newton_opts {
    double fluxTol;
    double fluxTolAlt;   /* from the 15th iteration on */
    double corrTol;
    double fluxFloor;
    double nAccFluxes;
} ef_newton_opts;

typedef struct ef_newton_check {
    int converged;               /* the increment's Newton iteration converged */
    int nGrew;                   /* residual growth count after this check */
    double fluxResidual;         /* max |R| */
    double fieldCorrection;      /* max |ddU| (0 without ddU) */
    double spatialAveragedFlux;  /* max(1e-10, sum |F| / nAccFluxes) */
} ef_newton_check;

/* The Newton iteration's residual and convergence decision on the device
 * (solvers/nonlinearimplicitstatic.py:418-440 and checkConvergence :625-725), for the
 * displacement field.  R, P, PExt (may be NULL), F, ddU (may be NULL), dirValues: device [nDof]
 * (dirValues [nDir], in the order of the ef_set_dirichlet list).
 * mode 0 (the first iteration of an increment that was not extrapolated): R = P + PExt with the
 * prescribed increments dirValues at the Dirichlet DOFs; no check, out unused, no synchronisation.
 * mode 1: R = P + PExt with 0 at the Dirichlet DOFs, then the reference's test: converged when
 * max |ddU| < corrTol and max |R| <= max(tol * max(1e-10, sum |F| / nAccFluxes), fluxFloor) with
 * tol = fluxTol below iteration 15, else fluxTolAlt; nGrew counts max |R| > prevResidual.  One
 * synchronising read of `out`. */
ef_status ef_newton_residual(ef_ctx* ctx, int mode, const double* P, const double* PExt, const double* dirValues,
                             const double* F, const double* ddU, int iteration, double prevResidual, int nGrew,
                             const ef_newton_opts* opts, double* R, ef_newton_check* out, void* stream);

/* ---- batches of independent small problems ----
 * The reference runs one model per job; a batch is many independent meshes held in one context
 * (one element group may carry a material row per element), each with its own Newton checks.
 * The per-problem solve replaces linearSolve (solvers/nonlinearimplicitstatic.py:727-751) and
 * the per-problem norms the reductions of checkConvergence (:625-725). */

/* Node ties u_slave = (u_masterA + u_masterB) / 2 for all three components (host int64 [n] node
 * indices, before ef_finalize), e.g. the mid-side nodes of 20-node faces on an interface with
 * 8-node elements.  The reference has no such constraint (constraints/ only equates DOFs); the
 * tied DOFs are eliminated: the assembled system is T^T K T, P and F are condensed with T^T, the
 * tied DOFs are masked in the solves and filled from their masters in every solution.  Turns off
 * the scalar reference CSR. */
ef_status ef_set_ties(ef_ctx* ctx, const int64_t* slave, const int64_t* masterA, const int64_t* masterB, int64_t n);

/* Increment scale in (0, 1) that an element of group `groupId` requests when its material update
 * fails (before ef_finalize; default 0.5, the reference's J2, materials/vonmises/vonmises.py:231;
 * a Marmot material sets its own pNewDT, elements/marmotelement/element.pyx:233-239). */
ef_status ef_set_group_cutback(ef_ctx* ctx, int groupId, double scale);

/* Per-element material rows for group `groupId` (before ef_finalize): table host
 * [nRows][nProps] (the material's property order), elemRow host [nEl] (row of each element). */
ef_status ef_set_group_props(ef_ctx* ctx, int groupId, const double* table, int nRows, int nProps,
                             const int32_t* elemRow);
/* Declares the problems: problem p owns the nodes [nodePtr[p], nodePtr[p+1]) (host int32
 * [nProb+1], covering all nodes); no 3x3 block may couple two problems.  Needs EF_OPT_KE_FP64. */
ef_status ef_batch_setup(ef_ctx* ctx, int nProb, const int32_t* nodePtr);
/* Tile shapes of the batched PCG: tile t in [0, ef_batch_tile_count()) runs threadsPerCta threads
 * per problem with lanesPerRow lanes per 3x3 block row in the matrix products. */
int ef_batch_tile_count(void);
ef_status ef_batch_tile_info(int tile, int* threadsPerCta, int* lanesPerRow);
ef_status ef_batch_set_tile(ef_ctx* ctx, int tile);
/* Solves K x = b problem by problem in one persistent launch (block-Jacobi PCG, FP64): Dirichlet
 * DOFs take b, each problem stops at |r| <= rtol |b_p| (its lifted right-hand side) or maxIter.
 * b, x device FP64 [nDof]; iters (device int32 [nProb]) and relres (device FP64 [nProb]) receive
 * each problem's iteration count and final relative residual (NaN on breakdown).  Does not
 * synchronise `stream` (capturable into a CUDA graph). */
ef_status ef_batch_solve(ef_ctx* ctx, double rtol, int maxIter, const double* b, double* x, int* iters,
                         double* relres, void* stream);
/* Times ef_batch_solve on (b, x) for every tile shape and keeps the fastest; tileOut (host)
 * receives it, msOut (host [ef_batch_tile_count()], may be NULL) the times.  Synchronises `stream`. */
ef_status ef_batch_autotune(ef_ctx* ctx, double rtol, int maxIter, const double* b, double* x, int* iters,
                            double* relres, void* stream, int* tileOut, float* msOut);
/* out (device FP64 [nProb][3]) = per problem {max |R|, sum |F|, max |ddU|} (ddU may be NULL).
 * Does not synchronise `stream`. */
ef_status ef_batch_norms(ef_ctx* ctx, const double* R, const double* F, const double* ddU, double* out,
                         void* stream);

/* Base preconditioner of EF_SOLVE_FGMRES (and of the learned correction's inputs):
 * EF_FGMRES_PC_MULTIGRID (default) the aggregation multigrid cycle, EF_FGMRES_PC_JACOBI one
 * block-Jacobi step D^-1. */
#define EF_FGMRES_PC_MULTIGRID 0
#define EF_FGMRES_PC_JACOBI 1
ef_status ef_fgmres_set_preconditioner(ef_ctx* ctx, int kind);

/* Lagged multigrid for the Newton iterations of one increment (inexact Newton-Krylov: the
 * preconditioner may lag the tangent, the FP64 refinement against the exact tangent decides the
 * solution): after this call the next newly assembled system rebuilds the coarse levels
 * (smoothed prolongators, Galerkin operators, damping estimates), and up to maxReuse systems
 * after it reuse them; the fine level (blocks, block inverses, BF16 copy) is always the current
 * system's, and a new Dirichlet set always rebuilds.  With maxReuse > 0 the rebuilds inside the
 * increment also keep the damping estimates (power iterations on D^-1 A) of its first build.
 * maxReuse = 0 (the default) rebuilds everything for every system.  The Newton drivers call it
 * at the start of each increment. */
ef_status ef_fgmres_set_reuse(ef_ctx* ctx, int maxReuse);

/* Diagnostics of the FGMRES solve's fine-level kernels on the last assembled system (after an
 * FGMRES solve with the sliced-ELL fine level): each is launched once, then `reps` times back to
 * back on `stream` between two CUDA events.  ms (host [3]) receives the average duration of one
 * launch of [0] the BF16 fine residual / smoothing sweep as the multigrid cycle runs it, [1] the
 * FP32 product, [2] the fused prolongation + post-smoothing (0 when the cycle does not use it);
 * bytes (host [3]) their algorithmic DRAM bytes per launch (the real blocks' values and column
 * indices, the per-row vectors).  Overwrites the multigrid's fine work vectors.  Synchronises
 * `stream`. */
ef_status ef_fine_kernel_profile(ef_ctx* ctx, int reps, double* ms, double* bytes, void* stream);

/* ---- learned preconditioner correction for the FGMRES solve (EF_SOLVE_FGMRES) ----
 * The reference solves every Newton system with a direct or plain Krylov solver
 * (solvers/nonlinearimplicitstatic.py:547-571, linearSolve; utils/linearsolve.py:35-77); this
 * optional stage replaces nothing there.  With it enabled the FGMRES preconditioner becomes
 * z = Mv + alpha N, N = NN([Mv, rho, D^-1 rho]), rho = v - K Mv: Mv the multigrid cycle, D the
 * 3x3 diagonal blocks, NN a 3-layer message-passing network (hidden width 64, no biases, BF16
 * weights, FP32 accumulation) on the node graph of the block system with edge weights
 * |K_mn|_F / sum_n' |K_mn'|_F, and alpha = rho.KN / |KN|^2 (the step that minimises |v - K z|).
 * It is trained with Adam on pairs (r, e), K e = r, taken from solves with the network disabled. */

/* Number of network weights (W_in [64][9], 3 x (Ws [64][64], Wn [64][64]), W_out [3][64]). */
int ef_mpnn_param_count(void);
/* Allocates the network state (once) and (re)initialises the weights from `seed` (the output
 * layer at zero, so the initial correction is zero); keeps up to maxSamples training pairs. */
ef_status ef_mpnn_init(ef_ctx* ctx, uint64_t seed, int maxSamples);
/* Host FP32 weights [ef_mpnn_param_count()] and scales [4] = {s_Mv, s_v, s_Dv, s_out}; either may
 * be NULL.  Setting weights resets the Adam moments. */
ef_status ef_mpnn_set_params(ef_ctx* ctx, const float* params, const float* scales);
ef_status ef_mpnn_get_params(ef_ctx* ctx, float* params, float* scales);
/* on != 0: FGMRES solves apply the network after the multigrid cycle. */
ef_status ef_mpnn_enable(ef_ctx* ctx, int on);
/* Training pairs from the following FGMRES solves, every `every` iterations and at most
 * maxPerSolve per inner solve.  kind 0: the iterate x_k is kept (plus x_0 = 0) and, when the
 * solve converges to x, (K (x - x_k), x - x_k) becomes a pair; kind 1: the Krylov basis vector
 * v_k becomes an input without correction (usable by the residual-norm loss only).
 * every = 0 switches collection off. */
ef_status ef_mpnn_collect(ef_ctx* ctx, int every, int maxPerSolve, int kind);
/* Adds one training pair from device FP64 vectors [nDof] with K e = r on the free DOFs. */
ef_status ef_mpnn_add_sample(ef_ctx* ctx, const double* r, const double* e, void* stream);
ef_status ef_mpnn_num_samples(const ef_ctx* ctx, int* n);
ef_status ef_mpnn_clear_samples(ef_ctx* ctx);
/* `epochs` passes of Adam (one pair per step, deterministic shuffle) at learning rate lr;
 * epochs = 0 only evaluates.  Loss of a pair with d = z - e on the free DOFs, relative to the
 * same norm of e: norm 0 |d|^2, norm 1 d.K d (energy), norm 2 |K d|^2 (residual), K the system
 * the pair came from (up to 16 systems are kept; the pairs of the oldest are dropped first).
 * lossFirst / lossLast (host, may be NULL) receive the mean over the pairs in the first and the
 * last epoch.  Synchronises `stream`. */
ef_status ef_mpnn_train(ef_ctx* ctx, int epochs, float lr, int norm, double* lossFirst, double* lossLast,
                        void* stream);
/* One forward and backward pass of the network on a caller's graph, all arrays on the HOST:
 * rowPtr [nNodes+1], colIdx [nBlocks] (structurally symmetric, sorted rows), vals [nBlocks][9],
 * params FP32 [ef_mpnn_param_count()], f [nNodes][9] features, base [3 nNodes] (may be NULL),
 * e [3 nNodes] target, mask [3 nNodes] (may be NULL).  z = base + so * W_out h3 (0 on masked),
 * loss = 0.5 * scale * sum_free (z - e)^2, grad = d loss / d params (may be NULL).  For
 * verification against an independent implementation; synchronises `stream`. */
ef_status ef_mpnn_eval(int nNodes, const int32_t* rowPtr, const int32_t* colIdx, const float* vals,
                       const float* params, const float* f, const float* base, const float* e, const uint8_t* mask,
                       float so, float scale, float* z, float* grad, double* loss, void* stream);

/* One dense layer of the network, q = relu(Ws h + Wn agg), hout = h + q, on HOST arrays h, agg
 * [nNodes][64], W [2][64][64] (Ws then Wn, row = output channel), q, hout [nNodes][64]: on the
 * tensor cores (tcgen05, BF16 operands, FP32 accumulation; tensorCores != 0) or the FP32 CUDA
 * cores.  flags (host) receives the kernel's status bits (16: a tile gave up waiting for its
 * accumulator; its TMEM was freed while the MMA may still run, so the results of the call are
 * to be discarded).  For verification; synchronises `stream`.
 * In an FGMRES solve with the network enabled the same event makes ef_solve return
 * EF_ERR_DEVICE: that solve is discarded and the context's network runs on the FP32 CUDA cores
 * from then on. */
ef_status ef_mpnn_dense_eval(int tensorCores, int nNodes, const float* h, const float* agg, const float* W,
                             float* q, float* hout, int* flags, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* EFGPU_H */
