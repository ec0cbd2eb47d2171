"""NISTGPU: the reference's Newton driver with its hot path on the GPU.

Mirrors ``solvers/nonlinearimplicitstatic.py`` (NIST) method by method -- same
names, argument meaning, tolerances and exceptions -- so Newton iteration counts
match the reference:

* ``solveStep`` :110-332 and ``solveIncrement`` :334-458 run on the host;
* ``computeElements`` :794-849 -> ``ef_compute_elements`` (element kernels + condensation),
* ``assembleStiffnessCSR`` :753-769 -> ``ef_assemble_bsr`` (atomic-free 3x3-block scatter),
* ``applyDirichletK`` :559-593 -> Dirichlet mask (symmetric elimination inside the solver),
* ``linearSolve`` :727-751 -> ``ef_solve`` (block-Jacobi PCG, FP32 inner + FP64 refinement),
* ``checkConvergence`` :625-725 -> ``ef_norms`` (device reductions) + the same host logic.

Vectors (U, dU, P, F, R, PExt) live on the GPU as torch float64 tensors; the
host sees three scalars per Newton iteration.
"""

import ctypes
import math
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .exceptions import CutbackRequest, DivergingSolution, ReachedMaxIterations, StepFailed
from .model import Model


@dataclass
class TimeStep:
    number: int
    stepProgressIncrement: float
    stepProgress: float
    timeIncrement: float
    stepTime: float
    totalTime: float


class AdaptiveTimeStepper:
    """timesteppers/adaptivetimestepper.py: generateTimeStep, preventIncrementIncrease,
    reduceNextIncrement, discardAndChangeIncrement (a zero first increment; x1.1 after 3 good ones)."""

    def __init__(self, currentTime, stepLength, startIncrement, maxIncrement, minIncrement, maxNumberIncrements,
                 increaseFactor=1.1):  # fmt: skip
        self.nPassedGoodIncrements = 0
        self.incrementCounter = 0
        self.maxIncrement = maxIncrement
        self.minIncrement = minIncrement
        self.maxNumberIncrements = maxNumberIncrements
        self.finishedStepProgress = 0.0
        self.increment = min(startIncrement, maxIncrement)
        self.allowedToIncreasedNext = True
        self.currentTime = currentTime
        self.stepLength = stepLength
        self.increaseFactor = increaseFactor

    def generateTimeStep(self):
        while self.finishedStepProgress < (1.0 - 1e-15):
            remainder = 1.0 - self.finishedStepProgress
            if remainder < self.increment:
                self.increment = remainder
            inc = self.increment if self.incrementCounter > 0 else 0.0
            self.finishedStepProgress += inc
            t = self.stepLength * self.finishedStepProgress
            yield TimeStep(self.incrementCounter, inc, self.finishedStepProgress, self.stepLength * inc, t,
                           self.currentTime + t)  # fmt: skip
            if self.incrementCounter > self.maxNumberIncrements:
                raise StepFailed("Reached maximum number of increments")
            if self.nPassedGoodIncrements >= 3 and self.allowedToIncreasedNext:
                self.increment = min(self.increment * self.increaseFactor, self.maxIncrement)
            self.allowedToIncreasedNext = True
            self.incrementCounter += 1
            self.nPassedGoodIncrements += 1

    def preventIncrementIncrease(self):
        self.allowedToIncreasedNext = False

    def discardAndChangeIncrement(self, scaleFactor):
        if self.incrementCounter == 0:
            raise StepFailed("Failed zero increment")
        self.finishedStepProgress -= self.increment
        self.incrementCounter -= 1
        self.nPassedGoodIncrements = 0
        if self.increment == self.minIncrement:
            raise StepFailed("Cannot reduce increment size")
        new = self.increment * scaleFactor
        self.increment = self.maxIncrement if new > self.maxIncrement else max(new, self.minIncrement)


@dataclass
class Step:
    """Step parameters with the defaults of steps/adaptivestep.py:56-64."""

    stepLength: float = 1.0
    startInc: float = 1.0
    maxInc: float = 1.0
    minInc: float = 1e-4
    maxNumInc: int = 1000
    maxIter: int = 10
    criticalIter: int = 5
    maxGrowIter: int = 10
    cutbackFactor: float = 0.25
    extrapolation: str = "linear"


@dataclass
class LinSolverOptions:
    method: str = "pcg"  # "pcg" (block-Jacobi CG) or "fgmres"
    mixed: bool = True  # FP32 inner iterations + FP64 refinement (False: all FP64, needs keFp64)
    rtol: float = 1e-10  # FP64 ||b - K x|| / ||b||; tight enough that Newton counts match a direct solver
    innerRtol: float = 1e-4
    maxIter: int = 20000
    restart: int = 40
    maxRefine: int = 30
    profile: bool = False
    # FGMRES: Newton systems of an increment that reuse the coarse multigrid levels built for the one
    # before (1: rebuilt every other system; measured best on the 160k-element J2 box)
    precondReuse: int = 1


class NISTGPU:
    identification = "NISTGPUSolver"

    fieldCorrectionTolerance = 1e-8  # config/phenomena.py displacement
    fluxResidualTolerance = 1e-8
    fluxResidualToleranceAlternative = 5e-3
    acceptableResidual = 1e-6  # largest relative residual of a stalled Krylov solve that is still used

    def __init__(self, model: Model, dirichlets=(), nodeforces=(), bodyforces=(), keFp64=False,
                 linsolver: LinSolverOptions = None, scalarCSR=False, device="cuda"):  # fmt: skip
        if not torch.cuda.is_available():
            raise RuntimeError("NISTGPU needs a CUDA device")
        self.lib = _lib.lib()
        self.model = model
        self.dirichlets = list(dirichlets)
        self.nodeforces = list(nodeforces)
        self.bodyforces = list(bodyforces)
        self.linsolver = linsolver or LinSolverOptions()
        if not self.linsolver.mixed and not keFp64:
            raise ValueError("an all-FP64 linear solve needs keFp64=True")
        self.device = torch.device(device)
        self.nDof = model.nDof
        self.ctx = ctypes.c_void_p()
        X = model.dof_coordinates()
        _lib.check(self.lib.ef_create(self.nDof, X.ctypes.data, ctypes.byref(self.ctx)), "ef_create")
        self.groupIds = []
        for g in model.groups:
            ed = np.ascontiguousarray(model.element_dofs(g))
            props = np.ascontiguousarray(np.asarray(g.props, dtype=float))
            gid = ctypes.c_int()
            _lib.check(
                self.lib.ef_add_group(self.ctx, g.elType.encode(), g.material.encode(), props.ctypes.data, props.size,
                                      ed.shape[0], ed.ctypes.data, ctypes.byref(gid)),
                "ef_add_group",
            )  # fmt: skip
            self.groupIds.append(gid.value)
            if g.cutback is not None:
                _lib.check(self.lib.ef_set_group_cutback(self.ctx, gid.value, float(g.cutback)), "ef_set_group_cutback")
            if g.propsTable is not None:
                tab = np.ascontiguousarray(np.asarray(g.propsTable, dtype=float))
                rows = np.ascontiguousarray(np.asarray(g.elemRow, dtype=np.int32))
                _lib.check(self.lib.ef_set_group_props(self.ctx, gid.value, tab.ctypes.data, tab.shape[0], tab.shape[1],
                                                       rows.ctypes.data), "ef_set_group_props")  # fmt: skip
        if model.ties is not None and len(model.ties[0]):
            ts, ta, tb = (np.ascontiguousarray(np.asarray(v, dtype=np.int64)) for v in model.ties)
            _lib.check(self.lib.ef_set_ties(self.ctx, ts.ctypes.data, ta.ctypes.data, tb.ctypes.data, ts.size),
                       "ef_set_ties")  # fmt: skip
        opts = (_lib.EF_OPT_KE_FP64 if keFp64 else 0) | (0 if scalarCSR else _lib.EF_OPT_NO_SCALAR_CSR)
        _lib.check(self.lib.ef_finalize(self.ctx, opts), "ef_finalize")
        self.info = _lib.EfInfo()
        _lib.check(self.lib.ef_get_info(self.ctx, ctypes.byref(self.info)), "ef_get_info")
        self.nAccumulatedFluxes = model.n_accumulated_fluxes()
        dirDofs = [d.dofs for d in self.dirichlets]
        self.dirIdxHost = np.concatenate(dirDofs).astype(np.int64) if dirDofs else np.zeros(0, np.int64)
        self.dirIdx = torch.as_tensor(self.dirIdxHost, device=self.device)
        _lib.check(self.lib.ef_set_dirichlet(self.ctx, self.dirIdxHost.ctypes.data, self.dirIdxHost.size),
                   "ef_set_dirichlet")  # fmt: skip
        self.newtonOpts = _lib.EfNewtonOpts(self.fluxResidualTolerance, self.fluxResidualToleranceAlternative,
                                            self.fieldCorrectionTolerance, 1e-7, float(self.nAccumulatedFluxes))
        self.computationTimes = {}
        self.iterationHistory = []  # (increment number, Newton iterations) per converged increment
        self.krylovIterations = []  # per linear solve
        self.lastSolveInfo = None

    def __del__(self):
        try:
            if getattr(self, "ctx", None) and self.ctx.value:
                self.lib.ef_destroy(self.ctx)
                self.ctx = None
        except Exception:
            pass

    # -- helpers ------------------------------------------------------------------
    def _stream(self):
        return torch.cuda.current_stream(self.device).cuda_stream

    def _vec(self):
        return torch.zeros(self.nDof, dtype=torch.float64, device=self.device)

    def _dirichletDelta(self, timeStep):
        if not self.dirichlets:
            return None
        d = np.concatenate([bc.getDelta(timeStep) for bc in self.dirichlets])
        return torch.as_tensor(d, device=self.device)

    def _externalLoads(self, timeStep):
        PExt = self._vec()
        if self.nodeforces:
            loads = torch.zeros(self.nDof, dtype=torch.float64)
            for nf in self.nodeforces:
                loads.index_add_(0, torch.as_tensor(nf.dofs), torch.as_tensor(nf.getCurrentLoad(timeStep)))
            PExt += loads.to(self.device)
        for bf in self.bodyforces:
            load = np.ascontiguousarray(bf.getCurrentLoad(timeStep))
            _lib.check(
                self.lib.ef_add_body_force(self.ctx, self.groupIds[bf.groupId], load.ctypes.data, PExt.data_ptr(),
                                           self._stream()),
                "ef_add_body_force",
            )  # fmt: skip
        return PExt

    # -- the hot path ---------------------------------------------------------------
    def computeElements(self, U_np, dU, P, F, timeStep):
        """Element loop: P = sum Pe, F = sum |Pe| (element order); K stays on the device."""
        t = np.array([timeStep.stepTime, timeStep.totalTime], dtype=float)
        _lib.check(
            self.lib.ef_compute_elements(self.ctx, U_np.data_ptr(), dU.data_ptr(), t.ctypes.data,
                                         timeStep.timeIncrement, P.data_ptr(), F.data_ptr(), self._stream()),
            "ef_compute_elements",
        )  # fmt: skip
        pNewDT = ctypes.c_double(1.0)
        st = self.lib.ef_element_status(self.ctx, self._stream(), ctypes.byref(pNewDT))
        if st == _lib.EF_CUTBACK:
            raise CutbackRequest("Von Mises Newton failed.", pNewDT.value)
        if st == _lib.EF_NAN:
            raise DivergingSolution("Obtained NaN in element evaluation")
        _lib.check(st, "ef_element_status")
        return P, F

    def assembleStiffnessCSR(self):
        _lib.check(self.lib.ef_assemble_bsr(self.ctx, self._stream()), "ef_assemble_bsr")

    def applyDirichletK(self):
        """The Dirichlet DOFs are eliminated inside the solver (mask set once per step)."""

    def linearSolve(self, R):
        o = self.linsolver
        opts = _lib.EfSolveOpts(
            _lib.EF_SOLVE_FGMRES if o.method == "fgmres" else _lib.EF_SOLVE_PCG,
            1 if o.mixed else 0, o.rtol, o.innerRtol, o.maxIter, o.restart, o.maxRefine, 1 if o.profile else 0,
        )  # fmt: skip
        info = _lib.EfSolveInfo()
        ddU = self._vec()
        st = self.lib.ef_solve(self.ctx, ctypes.byref(opts), R.data_ptr(), ddU.data_ptr(), ctypes.byref(info),
                               self._stream())  # fmt: skip
        self.lastSolveInfo = info
        self.krylovIterations.append(info.iterations)
        if st == _lib.EF_NAN:
            raise DivergingSolution("Obtained NaN in linear solve")
        if st == _lib.EF_NOT_CONVERGED:
            # an inexact Newton step is kept while the Krylov solve got close to its target (very
            # ill-conditioned systems stagnate above rtol in FP64); Newton's own convergence test decides
            if not (info.relResidual <= self.acceptableResidual):
                raise DivergingSolution(f"Krylov solve stalled at relative residual {info.relResidual:.2e}")
            return ddU
        _lib.check(st, "ef_solve")
        return ddU

    # ---- element results ---------------------------------------------------------------------------

    def getResultArray(self, groupId: int, element: int, result: str, quadraturePoint: int, trial: bool = False):
        """One element's result at one quadrature point (elements/displacementelement/element.py:386-409),
        as a copy of the committed state (trial=True: the current iteration's state)."""
        from .results import ElementResultCollector

        c = ElementResultCollector(self, groupId, [element], [quadraturePoint], result, trial=trial)
        try:
            return c.getCurrentResults()[0].copy()
        finally:
            c.close()

    def resultCollector(self, groupId: int, elements, quadraturePoints, result: str, trial: bool = False):
        """An ElementResultCollector over elements (indices within the group, None: all) and
        quadrature points of one group (utils/elementresultcollector.pyx)."""
        from .results import ElementResultCollector

        return ElementResultCollector(self, groupId, elements, quadraturePoints, result, trial=trial)

    # ---- learned preconditioner correction (FGMRES only) ----------------------------------------

    FGMRES_PRECONDITIONERS = {"multigrid": 0, "jacobi": 1}

    def setFgmresPreconditioner(self, kind="multigrid"):
        """Base preconditioner of the FGMRES solves (and of the learned correction's inputs):
        "multigrid" (aggregation cycle) or "jacobi" (one block-Jacobi step)."""
        _lib.check(self.lib.ef_fgmres_set_preconditioner(self.ctx, self.FGMRES_PRECONDITIONERS[kind]),
                   "ef_fgmres_set_preconditioner")  # fmt: skip

    def initLearnedPreconditioner(self, seed=0, maxSamples=64):
        """Allocates the message-passing correction applied after the multigrid cycle and sets
        its initial weights (zero output layer: no correction until trained)."""
        _lib.check(self.lib.ef_mpnn_init(self.ctx, seed, maxSamples), "ef_mpnn_init")

    def collectTrainingPairs(self, every=25, maxPerSolve=10, kind="iterates"):
        """Keep training pairs from the following FGMRES solves (every = 0: stop): "iterates"
        (K e_k, e_k) with e_k the error of the k-th iterate, or "krylov" basis vectors (inputs
        without a correction, for the residual-norm loss)."""
        k = {"iterates": 0, "krylov": 1}[kind]
        _lib.check(self.lib.ef_mpnn_collect(self.ctx, every, maxPerSolve, k), "ef_mpnn_collect")

    def addTrainingPair(self, r, e):
        """One pair of device FP64 vectors with K e = r on the free DOFs."""
        _lib.check(self.lib.ef_mpnn_add_sample(self.ctx, r.data_ptr(), e.data_ptr(), self._stream()),
                   "ef_mpnn_add_sample")  # fmt: skip

    def clearTrainingPairs(self):
        _lib.check(self.lib.ef_mpnn_clear_samples(self.ctx), "ef_mpnn_clear_samples")

    def numTrainingPairs(self):
        n = ctypes.c_int()
        _lib.check(self.lib.ef_mpnn_num_samples(self.ctx, ctypes.byref(n)), "ef_mpnn_num_samples")
        return n.value

    LOSS_NORMS = {"error": 0, "energy": 1, "residual": 2}

    def trainLearnedPreconditioner(self, epochs=20, lr=1e-3, norm="energy"):
        """Adam over the stored pairs; returns the mean relative loss of the first and the last
        epoch (epochs = 0: evaluation only).  norm: "error" |z - e|^2, "energy" (z - e).K(z - e)
        or "residual" |K(z - e)|^2, each relative to the same norm of e."""
        first, last = ctypes.c_double(), ctypes.c_double()
        _lib.check(self.lib.ef_mpnn_train(self.ctx, epochs, lr, self.LOSS_NORMS[norm], ctypes.byref(first),
                                          ctypes.byref(last), self._stream()), "ef_mpnn_train")  # fmt: skip
        return first.value, last.value

    def enableLearnedPreconditioner(self, on=True):
        _lib.check(self.lib.ef_mpnn_enable(self.ctx, 1 if on else 0), "ef_mpnn_enable")

    def learnedParameters(self):
        p = np.zeros(self.lib.ef_mpnn_param_count(), np.float32)
        sc = np.zeros(4, np.float32)
        _lib.check(self.lib.ef_mpnn_get_params(self.ctx, p.ctypes.data, sc.ctypes.data), "ef_mpnn_get_params")
        return p, sc

    def setLearnedParameters(self, params=None, scales=None):
        p = None if params is None else np.ascontiguousarray(params, np.float32)
        sc = None if scales is None else np.ascontiguousarray(scales, np.float32)
        _lib.check(self.lib.ef_mpnn_set_params(self.ctx, None if p is None else p.ctypes.data,
                                               None if sc is None else sc.ctypes.data), "ef_mpnn_set_params")  # fmt: skip

    def checkConvergence(self, R, ddU, F, iterationCounter, residualHistory):
        out = np.zeros(3)
        _lib.check(
            self.lib.ef_norms(self.ctx, R.data_ptr(), F.data_ptr(), None if ddU is None else ddU.data_ptr(),
                              out.ctypes.data, self._stream()),
            "ef_norms",
        )  # fmt: skip
        fluxResidual, sumF, corr = out
        spatialAveragedFlux = max(1e-10, sumF / self.nAccumulatedFluxes)
        tol = self.fluxResidualTolerance if iterationCounter < 15 else self.fluxResidualToleranceAlternative
        fieldCorrection = corr if ddU is not None else 0.0
        convergedCorrection = fieldCorrection < self.fieldCorrectionTolerance
        convergedFlux = fluxResidual <= max(tol * spatialAveragedFlux, 1e-7)
        prev, nGrew = residualHistory["displacement"]
        if fluxResidual > prev:
            nGrew += 1
        residualHistory["displacement"] = (fluxResidual, nGrew)
        return convergedCorrection and convergedFlux

    def newtonResidual(self, first, P, PExt, R, F, ddU, iterationCounter, residualHistory, timeStep):
        """R = P + PExt with the Dirichlet rows of solvers/nonlinearimplicitstatic.py:418-436 and,
        unless `first` (the first iteration of an increment that was not extrapolated: the
        prescribed increments go into R, nothing is checked), checkConvergence (:625-725) decided on
        the device (ef_newton_residual: one read per Newton iteration).  Returns converged."""
        if first:
            vals = self._dirichletDelta(timeStep)
            _lib.check(self.lib.ef_newton_residual(self.ctx, 0, P.data_ptr(), PExt.data_ptr(), vals.data_ptr(), None,
                                                   None, 0, 0.0, 0, None, R.data_ptr(), None, self._stream()),
                       "ef_newton_residual")  # fmt: skip
            return False
        prev, nGrew = residualHistory["displacement"]
        out = _lib.EfNewtonCheck()
        _lib.check(self.lib.ef_newton_residual(self.ctx, 1, P.data_ptr(), PExt.data_ptr(), None, F.data_ptr(),
                                               None if ddU is None else ddU.data_ptr(), iterationCounter, prev, nGrew,
                                               ctypes.byref(self.newtonOpts), R.data_ptr(), ctypes.byref(out),
                                               self._stream()), "ef_newton_residual")  # fmt: skip
        residualHistory["displacement"] = (out.fluxResidual, out.nGrew)
        return bool(out.converged)

    # -- Newton loop (same control flow as NIST.solveIncrement) ------------------------
    def extrapolateLastIncrement(self, extrapolation, timeStep, dU, prevTimeStep):
        if extrapolation == "linear" and prevTimeStep is not None and prevTimeStep.timeIncrement:
            dU *= timeStep.stepProgressIncrement / prevTimeStep.stepProgressIncrement
            if self.dirichlets:
                dU[self.dirIdx] = self._dirichletDelta(timeStep)
            return dU, True
        dU.zero_()
        return dU, False

    def solveIncrement(self, U_n, dU, P, timeStep, prevTimeStep, step: Step):
        iterationCounter = 0
        residualHistory = {"displacement": (0.0, 0)}
        R = self._vec()
        F = self._vec()
        U_np = self._vec()
        ddU = None
        dU, isExtrapolated = self.extrapolateLastIncrement(step.extrapolation, timeStep, dU, prevTimeStep)
        PExt = self._externalLoads(timeStep)
        if self.linsolver.method == "fgmres":
            _lib.check(self.lib.ef_fgmres_set_reuse(self.ctx, self.linsolver.precondReuse), "ef_fgmres_set_reuse")
        while True:
            torch.add(U_n, dU, out=U_np)
            P, F = self.computeElements(U_np, dU, P, F, timeStep)
            first = iterationCounter == 0 and not isExtrapolated and bool(self.dirichlets)
            converged = self.newtonResidual(first, P, PExt, R, F, ddU, iterationCounter, residualHistory, timeStep)
            if not first:
                if converged:
                    break
                if residualHistory["displacement"][1] > step.maxGrowIter:
                    raise DivergingSolution(f"Residual grew {step.maxGrowIter} times, cutting back")
                if iterationCounter == step.maxIter:
                    raise ReachedMaxIterations("Reached max. iterations in current increment, cutting back")
            self.assembleStiffnessCSR()
            self.applyDirichletK()
            ddU = self.linearSolve(R)
            dU += ddU
            iterationCounter += 1
        return U_np, dU, P, iterationCounter

    def solveStep(self, step: Step, maxIncrements=None, callback=None):
        """Runs the adaptive increment loop of the step; returns (U, P) as device tensors."""
        _lib.check(self.lib.ef_set_dirichlet(self.ctx, self.dirIdxHost.ctypes.data, self.dirIdxHost.size),
                   "ef_set_dirichlet")  # fmt: skip
        U = self._vec()
        dU = self._vec()
        P = self._vec()
        prevTimeStep = None
        stepper = AdaptiveTimeStepper(0.0, step.stepLength, step.startInc, step.maxInc, step.minInc, step.maxNumInc)
        done = 0
        for timeStep in stepper.generateTimeStep():
            try:
                U_np, dU, P, iters = self.solveIncrement(U, dU, P, timeStep, prevTimeStep, step)
            except CutbackRequest as e:
                stepper.discardAndChangeIncrement(max(e.cutbackSize, step.cutbackFactor))
                prevTimeStep = None
                self.iterationHistory.append((timeStep.number, math.inf))
                continue
            except (ReachedMaxIterations, DivergingSolution):
                stepper.discardAndChangeIncrement(step.cutbackFactor)
                prevTimeStep = None
                self.iterationHistory.append((timeStep.number, math.inf))
                continue
            U = U_np
            prevTimeStep = timeStep
            if iters >= step.criticalIter:
                stepper.preventIncrementIncrease()
            _lib.check(self.lib.ef_accept_state(self.ctx), "ef_accept_state")
            self.iterationHistory.append((timeStep.number, iters))
            if callback is not None:
                callback(timeStep, iters, U)
            done += 1
            if maxIncrements is not None and done >= maxIncrements:
                break
        return U, P


class IndirectControl:
    """Indirect displacement control for the arc-length driver (stepactions/indirectcontrol.py:29-44):
    the load-factor correction ddLambda that makes c . dU over the controlled DOFs (node 1's
    components, then node 2's) grow by stepProgressIncrement * L in the increment."""

    def __init__(self, dofs1, cVector1, dofs2, cVector2, L: float):
        self.idcs = np.concatenate([np.asarray(dofs1, np.int64), np.asarray(dofs2, np.int64)])
        self.c = np.concatenate([np.asarray(cVector1, float), np.asarray(cVector2, float)])
        self.L = float(L)

    def computeDDLambda(self, dU, ddU_0, ddU_f, timeStep):
        """dU, ddU_0, ddU_f: host arrays of the controlled DOFs."""
        dL = timeStep.stepProgressIncrement * self.L
        return (dL - self.c.dot(dU + ddU_0)) / self.c.dot(ddU_f)


class NISTGPUArcLength(NISTGPU):
    """The arc-length driver of solvers/nonlinearimplicitstaticparallelarclength.py:120-320 over the
    same GPU hot path.  Each Newton iteration evaluates the elements once, forms
    R_0 = P_0 + (Lambda + dLambda) P_f + P from the dead loads P_0, the reference loads P_f (the
    node and body forces at step progress 1 minus those at 0) and the internal forces P, and
    solves the one assembled system twice (K ddU_0 = R_0, K ddU_f = P_f; the preconditioner set-up
    is shared).  The controller gives ddLambda from the controlled DOFs (one small device-to-host
    read) and ddU = ddU_0 + ddLambda ddU_f.  Dirichlet rows take the prescribed values scaled like
    the load: zero in the first iteration of an extrapolated increment, else the increment over
    [Lambda, Lambda + dLambda] in R_0 and the full value in P_f.  The convergence test runs on R_0
    from the second iteration on, or from the first after an extrapolation, and the load factor
    is extrapolated with the displacements (:355-368).  Without a controller the increments are
    the plain Newton increments of NISTGPU, as in the reference."""

    identification = "NISTGPUArcLength"

    def __init__(self, *args, arcLengthController: IndirectControl = None, **kw):
        super().__init__(*args, **kw)
        self.arcLengthController = arcLengthController
        self.Lambda = 0.0
        self.dLambda = 0.0
        self.lambdaHistory = []  # Lambda after each converged increment

    def _dirichletAt(self, number, progressIncrement, progress):
        return self._dirichletDelta(TimeStep(number, progressIncrement, progress, 0.0, 0.0, 0.0))

    def solveIncrement(self, U_n, dU, P, timeStep, prevTimeStep, step: Step):
        ctl = self.arcLengthController
        if ctl is None:
            return super().solveIncrement(U_n, dU, P, timeStep, prevTimeStep, step)
        iterationCounter = 0
        residualHistory = {"displacement": (0.0, 0)}
        F = self._vec()
        U_np = self._vec()
        ddU = None
        Lambda, dLambda = self.Lambda, self.dLambda
        if step.extrapolation == "linear" and prevTimeStep is not None and prevTimeStep.stepProgressIncrement:
            ratio = timeStep.stepProgressIncrement / prevTimeStep.stepProgressIncrement
            dLambda = dLambda * ratio
            dU *= ratio
            isExtrapolated = True
        else:
            dLambda = 0.0
            dU.zero_()
            isExtrapolated = False
        P_0 = self._externalLoads(TimeStep(timeStep.number, 0.0, 0.0, 0.0, 0.0, 0.0))
        P_f = self._externalLoads(TimeStep(timeStep.number, 1.0, 1.0, 0.0, 0.0, 0.0)) - P_0
        R_f = P_f.clone()
        if self.dirichlets:
            R_f[self.dirIdx] = self._dirichletAt(timeStep.number, 1.0, 1.0)
        idx = torch.as_tensor(ctl.idcs, device=self.device)
        while True:
            torch.add(U_n, dU, out=U_np)
            P, F = self.computeElements(U_np, dU, P, F, timeStep)
            R_0 = P_0 + (Lambda + dLambda) * P_f + P
            if self.dirichlets:
                if isExtrapolated and iterationCounter == 0:
                    R_0[self.dirIdx] = self._dirichletAt(timeStep.number, 0.0, 0.0)
                else:
                    R_0[self.dirIdx] = self._dirichletAt(timeStep.number, dLambda, Lambda + dLambda)
            if iterationCounter > 0 or isExtrapolated:
                if self.checkConvergence(R_0, ddU, F, iterationCounter, residualHistory):
                    break
                if residualHistory["displacement"][1] > step.maxGrowIter:
                    raise DivergingSolution(f"Residual grew {step.maxGrowIter} times, cutting back")
                if iterationCounter == step.maxIter:
                    raise ReachedMaxIterations("Reached max. iterations in current increment, cutting back")
            self.assembleStiffnessCSR()
            self.applyDirichletK()
            ddU_0 = self.linearSolve(R_0)
            ddU_f = self.linearSolve(R_f)
            ctlValues = torch.stack([dU[idx], ddU_0[idx], ddU_f[idx]]).cpu().numpy()
            ddLambda = float(ctl.computeDDLambda(ctlValues[0], ctlValues[1], ctlValues[2], timeStep))
            ddU = ddU_0 + ddLambda * ddU_f
            dU += ddU
            dLambda += ddLambda
            iterationCounter += 1
        self.Lambda += dLambda
        self.dLambda = dLambda
        self.lambdaHistory.append(self.Lambda)
        return U_np, dU, P, iterationCounter
