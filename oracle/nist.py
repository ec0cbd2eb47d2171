"""Newton-Raphson load-step driver of the oracle (serial NIST semantics).

Follows ``solvers/nonlinearimplicitstatic.py``:

* ``solveStep`` :110-332 -- increment loop, cutback handling (:247-279), commit of
  element states after a converged increment (:296), critical-iteration rule;
* ``solveIncrement`` :334-458 -- U_np = U_n + dU, element loop, loads, first
  iteration with prescribed Dirichlet increments, convergence check from the
  second residual on, CSR assembly, Dirichlet rows, linear solve, dU += ddU;
* ``checkConvergence`` :625-725 with ``computeSpatialAveragedFluxes`` :771-792
  (tolerances of ``config/phenomena.py``: correction 1e-8, flux 1e-8,
  alternative flux 5e-3 from the 15th iteration, absolute floor 1e-7);
* ``extrapolateLastIncrement`` :964-1000 (linear extrapolation, default on);
* ``timesteppers/adaptivetimestepper.py`` ``generateTimeStep`` (a zero first
  increment, x1.1 growth after 3 good increments), ``discardAndChangeIncrement``
  and ``reduceNextIncrement``;
* step defaults of ``steps/adaptivestep.py:56-64``.
"""

from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from .materials import ReturnMapFailed
from .system import condense, csr_slot_map, csr_update, dirichlet_rows, vij_pattern


class ReachedMaxIterations(Exception):
    pass


class DivergingSolution(Exception):
    pass


class StepFailed(Exception):
    pass


@dataclass
class TimeStep:
    number: int
    stepProgressIncrement: float
    stepProgress: float
    timeIncrement: float
    stepTime: float
    totalTime: float


class AdaptiveTimeStepper:
    def __init__(self, currentTime, stepLength, startInc, maxInc, minInc, maxNumInc, increaseFactor=1.1):
        self.nPassedGoodIncrements = 0
        self.incrementCounter = 0
        self.maxIncrement = maxInc
        self.minIncrement = minInc
        self.maxNumberIncrements = maxNumInc
        self.finishedStepProgress = 0.0
        self.increment = min(startInc, maxInc)
        self.allowedToIncreasedNext = True
        self.currentTime = currentTime
        self.stepLength = stepLength
        self.increaseFactor = increaseFactor

    def generate(self):
        while self.finishedStepProgress < (1.0 - 1e-15):
            remainder = 1.0 - self.finishedStepProgress
            if remainder < self.increment:
                self.increment = remainder
            inc = self.increment if self.incrementCounter > 0 else 0.0
            dT = self.stepLength * inc
            self.finishedStepProgress += inc
            tStep = self.stepLength * self.finishedStepProgress
            yield TimeStep(self.incrementCounter, inc, self.finishedStepProgress, dT, tStep, self.currentTime + tStep)
            if self.incrementCounter > self.maxNumberIncrements:
                raise StepFailed("Reached maximum number of increments")
            if self.nPassedGoodIncrements >= 3 and self.allowedToIncreasedNext:
                self.increment *= self.increaseFactor
                if self.increment > self.maxIncrement:
                    self.increment = self.maxIncrement
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
        self.increment = self.maxIncrement if new > self.maxIncrement else (self.minIncrement if new < self.minIncrement else new)


@dataclass
class Step:
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
class Model:
    """Element groups with their DOF maps plus linearly ramped loads/BCs (amplitude f(t) = t)."""

    nDof: int
    groups: list  # of (elements object, elDofs [nEl, n])
    dirichlet: list = field(default_factory=list)  # of (dof indices, prescribed total value per dof)
    nodeforces: list = field(default_factory=list)  # of (dof indices, load per dof)
    bodyforces: list = field(default_factory=list)  # of (group index, load vector (3,))
    # node ties u_s = (u_a + u_b) / 2 (all components) as (slave, masterA, masterB) node arrays; the
    # reference has no such constraint, the oracle eliminates the slaves: K^ = T^T K T, R^ = T^T R,
    # F^ = T^T F, ddU = T ddU^ (slave rows of K^ are identity rows with zero right-hand side)
    ties: tuple = None


def tie_matrix(nDof, ties):
    """T [nDof, nDof]: identity except slave DOF rows (1/2 at both masters, 0 on the diagonal)."""
    s, a, b = (np.asarray(v, dtype=np.int64) for v in ties)
    rows, cols, vals = [], [], []
    slaveDof = (3 * s[:, None] + np.arange(3)).ravel()
    keep = np.setdiff1d(np.arange(nDof), slaveDof)
    rows.append(keep), cols.append(keep), vals.append(np.ones(keep.size))
    for m in (a, b):
        rows.append(slaveDof)
        cols.append((3 * m[:, None] + np.arange(3)).ravel())
        vals.append(np.full(slaveDof.size, 0.5))
    T = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(nDof, nDof))
    return T, slaveDof


def spsolve_direct(A, b):
    return spla.spsolve(A, b, use_umfpack=False)


class NIST:
    fieldCorrectionTolerance = 1e-8
    fluxResidualTolerance = 1e-8
    fluxResidualToleranceAlt = 5e-3

    def __init__(self, model: Model, linsolve=spsolve_direct):
        self.model = model
        self.linsolve = linsolve
        elDofsAll = [g[1] for g in model.groups]
        I = np.concatenate([vij_pattern(d)[0] for d in elDofsAll])
        J = np.concatenate([vij_pattern(d)[1] for d in elDofsAll])
        self.I, self.J = I, J
        self.indptr, self.indices, self.x = csr_slot_map(I, J, model.nDof)
        self.nAccFlux = sum(d.size for d in elDofsAll)
        self.dirIdx = np.concatenate([d for d, _ in model.dirichlet]) if model.dirichlet else np.array([], dtype=np.int64)
        self.history = []  # (increment number, iterations) of converged increments
        self.iterationLog = []  # per Newton iteration (flux residual, correction)
        self.T = None
        if model.ties is not None and len(model.ties[0]):
            self.T, self.slaveDof = tie_matrix(model.nDof, model.ties)
            self.Tt = self.T.T.tocsr()

    # -- the four hot-path methods -------------------------------------------------
    def computeElements(self, U_np, dU):
        nDof = self.model.nDof
        P = np.zeros(nDof)
        F = np.zeros(nDof)
        Vs = []
        for els, elDofs in self.model.groups:
            Ke, Pe = els.compute_yourself(U_np[elDofs], dU[elDofs])
            Vs.append(Ke.reshape(Ke.shape[0], -1).ravel())
            p, f = condense(Pe, elDofs, nDof)
            P += p
            F += f
        if self.T is not None:
            P, F = self.Tt @ P, self.Tt @ F
        return P, np.concatenate(Vs), F

    def assembleStiffnessCSR(self, V):
        return csr_update(V, self.x, len(self.indices))

    def applyDirichletK(self, data):
        if self.T is None:
            return dirichlet_rows(self.indptr, self.indices, data, self.dirIdx)
        n = self.model.nDof
        A = sp.csr_matrix((data, self.indices, self.indptr), shape=(n, n))
        A = (self.Tt @ A @ self.T).tocsr()
        A = (A + sp.csr_matrix((np.ones(self.slaveDof.size), (self.slaveDof, self.slaveDof)), shape=(n, n))).tocsr()
        A.sum_duplicates()
        A.sort_indices()
        return dirichlet_rows(A.indptr, A.indices, A.data, self.dirIdx)

    def linearSolve(self, A, b):
        ddU = self.linsolve(A, b)
        if self.T is not None:
            ddU = self.T @ ddU
        if np.isnan(ddU).any():
            raise DivergingSolution("Obtained NaN in linear solve")
        return ddU

    # -- Newton loop -----------------------------------------------------------------
    def _dirichletDelta(self, ts):
        # stepactions/dirichlet.py getDelta: delta * (f(t) - f(t - dt)), f(t) = t
        a = ts.stepProgress
        return np.concatenate([v * (a - (a - ts.stepProgressIncrement)) for _, v in self.model.dirichlet])

    def _externalLoads(self, ts):
        PExt = np.zeros(self.model.nDof)
        for dofs, load in self.model.nodeforces:
            PExt[dofs] += load * ts.stepProgress
        for gi, load in self.model.bodyforces:
            els, elDofs = self.model.groups[gi]
            Pe = els.body_force(np.asarray(load) * ts.stepProgress)
            for e in range(elDofs.shape[0]):
                PExt[elDofs[e]] += Pe[e]
        return PExt

    def checkConvergence(self, R, ddU, F, it, hist):
        avgFlux = max(1e-10, np.linalg.norm(F, 1) / self.nAccFlux)
        tol = self.fluxResidualTolerance if it < 15 else self.fluxResidualToleranceAlt
        flux = np.max(np.abs(R))
        corr = np.linalg.norm(ddU, np.inf) if ddU is not None else 0.0
        ok = (corr < self.fieldCorrectionTolerance) and (flux <= max(tol * avgFlux, 1e-7))
        prev, nGrew = hist[0]
        if flux > prev:
            nGrew += 1
        hist[0] = (flux, nGrew)
        self.iterationLog.append((flux, corr))
        return ok

    def solveIncrement(self, U_n, dU, ts, prevTs, step):
        it = 0
        hist = [(0.0, 0)]
        ddU = None
        if step.extrapolation == "linear" and prevTs is not None and prevTs.timeIncrement:
            dU = dU * (ts.stepProgressIncrement / prevTs.stepProgressIncrement)
            if self.dirIdx.size:
                dU[self.dirIdx] = self._dirichletDelta(ts)
            extrap = True
        else:
            dU = np.zeros_like(dU)
            extrap = False
        PExt = self._externalLoads(ts)
        while True:
            U_np = U_n + dU
            P, V, F = self.computeElements(U_np, dU)
            R = P + PExt
            if it == 0 and not extrap and self.dirIdx.size:
                R[self.dirIdx] = self._dirichletDelta(ts)
            else:
                R[self.dirIdx] = 0.0
                if self.checkConvergence(R, ddU, F, it, hist):
                    break
                if hist[0][1] > step.maxGrowIter:
                    raise DivergingSolution("Residual grew too often")
                if it == step.maxIter:
                    raise ReachedMaxIterations("Reached max. iterations")
            A = self.applyDirichletK(self.assembleStiffnessCSR(V))
            ddU = self.linearSolve(A, R)
            dU = dU + ddU
            it += 1
        return U_np, dU, P, it

    def solveStep(self, step: Step, maxIncrements=None, callback=None):
        """The increment loop of solveStep (solvers/nonlinearimplicitstatic.py:185-316); callback(ts,
        iterations, U) after every converged increment."""
        nDof = self.model.nDof
        U = np.zeros(nDof)
        dU = np.zeros(nDof)
        P = np.zeros(nDof)
        prevTs = None
        stepper = AdaptiveTimeStepper(0.0, step.stepLength, step.startInc, step.maxInc, step.minInc, step.maxNumInc)
        nDone = 0
        for ts in stepper.generate():
            try:
                Un, dUn, Pn, it = self.solveIncrement(U, dU, ts, prevTs, step)
            except ReturnMapFailed as e:
                stepper.discardAndChangeIncrement(max(e.cutbackSize, step.cutbackFactor))
                prevTs = None
                self.history.append((ts.number, -1))
                continue
            except (ReachedMaxIterations, DivergingSolution):
                stepper.discardAndChangeIncrement(step.cutbackFactor)
                prevTs = None
                self.history.append((ts.number, -1))
                continue
            U, dU, P = Un, dUn, Pn
            prevTs = ts
            if it >= step.criticalIter:
                stepper.preventIncrementIncrease()
            for els, _ in self.model.groups:
                els.accept_last_state()
            self.history.append((ts.number, it))
            if callback is not None:
                callback(ts, it, U)
            nDone += 1
            if maxIncrements is not None and nDone >= maxIncrements:
                break
        return U, P


@dataclass
class IndirectControl:
    """Indirect displacement control of the arc-length driver (stepactions/indirectcontrol.py:29-44,
    ``computeDDLambda``): the load-factor correction that makes c . dU over the controlled DOFs
    (node 1's then node 2's displacement components) grow by stepProgressIncrement * L."""

    idcs: np.ndarray
    c: np.ndarray
    L: float

    def computeDDLambda(self, dU, ddU_0, ddU_f, ts):
        dL = ts.stepProgressIncrement * self.L
        return (dL - self.c.dot(dU[self.idcs] + ddU_0[self.idcs])) / self.c.dot(ddU_f[self.idcs])


class NISTArcLength(NIST):
    """Arc-length increment of ``solvers/nonlinearimplicitstaticparallelarclength.py:120-320``: per
    Newton iteration the residual R_0 = P_0 + (Lambda + dLambda) P_f + P of the dead loads P_0, the
    reference loads P_f (the loads at step progress 1 minus those at 0) and the internal forces,
    two solves K ddU_0 = R_0 and K ddU_f = P_f, the controller's ddLambda, and
    ddU = ddU_0 + ddLambda ddU_f.  Dirichlet rows take the prescribed values scaled like the load
    (a zero increment in the first iteration of an extrapolated increment); the convergence test
    runs on R_0 from the second iteration on, or from the first after an extrapolation; the load
    factor and the displacement increment are extrapolated together (:355-368)."""

    def __init__(self, model: Model, controller: IndirectControl, linsolve=spsolve_direct):
        super().__init__(model, linsolve)
        self.controller = controller
        self.Lambda = 0.0
        self.dLambda = 0.0
        self.lambdaHistory = []  # Lambda after each converged increment

    def _dirichletAt(self, number, progressIncrement, progress):
        return self._dirichletDelta(TimeStep(number, progressIncrement, progress, 0.0, 0.0, 0.0))

    def solveIncrement(self, U_n, dU, ts, prevTs, step):
        it = 0
        hist = [(0.0, 0)]
        ddU = None
        Lambda, dLambda = self.Lambda, self.dLambda
        if step.extrapolation == "linear" and prevTs is not None and prevTs.stepProgressIncrement:
            dLambda = dLambda * (ts.stepProgressIncrement / prevTs.stepProgressIncrement)
            dU = dU * (ts.stepProgressIncrement / prevTs.stepProgressIncrement)
            extrap = True
        else:
            dLambda = 0.0
            dU = np.zeros_like(dU)
            extrap = False
        P_0 = self._externalLoads(TimeStep(ts.number, 0.0, 0.0, 0.0, 0.0, 0.0))
        P_f = self._externalLoads(TimeStep(ts.number, 1.0, 1.0, 0.0, 0.0, 0.0)) - P_0
        while True:
            U_np = U_n + dU
            P, V, F = self.computeElements(U_np, dU)
            R_0 = P_0 + (Lambda + dLambda) * P_f + P
            R_f = P_f.copy()
            if self.dirIdx.size:
                if extrap and it == 0:
                    R_0[self.dirIdx] = self._dirichletAt(ts.number, 0.0, 0.0)
                else:
                    R_0[self.dirIdx] = self._dirichletAt(ts.number, dLambda, Lambda + dLambda)
                R_f[self.dirIdx] = self._dirichletAt(ts.number, 1.0, 1.0)
            if it > 0 or extrap:
                if self.checkConvergence(R_0, ddU, F, it, hist):
                    break
                if hist[0][1] > step.maxGrowIter:
                    raise DivergingSolution("Residual grew too often")
                if it == step.maxIter:
                    raise ReachedMaxIterations("Reached max. iterations")
            A = self.applyDirichletK(self.assembleStiffnessCSR(V))
            ddU_0 = self.linearSolve(A, R_0)
            ddU_f = self.linearSolve(A, R_f)
            ddLambda = self.controller.computeDDLambda(dU, ddU_0, ddU_f, ts)
            ddU = ddU_0 + ddLambda * ddU_f
            dU = dU + ddU
            dLambda += ddLambda
            it += 1
        self.Lambda += dLambda
        self.dLambda = dLambda
        self.lambdaHistory.append(self.Lambda)
        return U_np, dU, P, it
