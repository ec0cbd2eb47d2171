"""Many independent small problems solved as one batch (uneven hex8 J2 cubes).

The reference runs one model per job (solvers/nonlinearimplicitstatic.py:334-458).  Here a batch
of independent meshes lives in one library context: one element pass and one assembly cover all
of them, one persistent launch solves every problem's system (``ef_batch_solve``: one CTA per
problem at a time, block-Jacobi PCG with CTA-wide reductions), and the Newton decisions of the
reference's driver (``checkConvergence`` :625-725, growth and iteration limits :451-456) are taken
per problem from per-problem norms (``ef_batch_norms``).  A problem that has converged keeps its
increment: its residual is masked out of the following solves, so its correction is zero and its
element results repeat bit for bit.  The Newton iteration body from one solve to the next
convergence check is captured once as a CUDA graph and replayed.
"""

import ctypes

import numpy as np
import torch

from . import _lib
from .exceptions import CutbackRequest, DivergingSolution, ReachedMaxIterations
from .mesh import box_mesh
from .model import DirichletDofs, ElementGroup, Model
from .solver import AdaptiveTimeStepper, LinSolverOptions, NISTGPU, Step


def cube_batch_spec(nProb, seed, nMin=4, nMax=16, E=210000.0):
    """Per problem: edge n ~ U{nMin..nMax} elements, sigma_y ~ U[150, 350], H ~ U[200, 2000],
    nu ~ U[0.2, 0.4], drawn from numpy.random.default_rng(seed) in that order."""
    rng = np.random.default_rng(seed)
    n = rng.integers(nMin, nMax + 1, nProb)
    fy = rng.uniform(150.0, 350.0, nProb)
    H = rng.uniform(200.0, 2000.0, nProb)
    nu = rng.uniform(0.2, 0.4, nProb)
    return [dict(n=int(n[p]), props=[E, float(nu[p]), float(fy[p]), float(H[p]), 0.0, 0.0]) for p in range(nProb)]


def cube_mesh(n, h=0.1, strain=0.01, bc="clamped"):
    """One cube of n^3 C3D8 elements with edge L = n*h strained by `strain` along z.

    bc "clamped": z = 0 face fully fixed, z = L face pulled to u_z = strain*L (lateral motion free;
    the clamped base makes the field non-homogeneous).  bc "confined": uniaxial strain, u_x = 0 on
    x = 0 and x = L, u_y = 0 on y = 0 and y = L, u_z = 0 on z = 0, u_z = strain*L on z = L (exact
    solution u = (0, 0, strain*z)).  Returns (mesh dict, Dirichlet DOFs, their step totals)."""
    L = n * h
    m = box_mesh(n, n, n, L, L, L)
    s = m["nodeSets"]
    if bc == "clamped":
        bcs = [("gen_back", 0, 0.0), ("gen_back", 1, 0.0), ("gen_back", 2, 0.0), ("gen_front", 2, strain * L)]
    elif bc == "confined":
        bcs = [("gen_left", 0, 0.0), ("gen_right", 0, 0.0), ("gen_bottom", 1, 0.0), ("gen_top", 1, 0.0),
               ("gen_back", 2, 0.0), ("gen_front", 2, strain * L)]  # fmt: skip
    else:
        raise ValueError(bc)
    dofs, vals = [], []
    for name, comp, v in bcs:
        nodes = np.asarray(s[name], dtype=np.int64)
        dofs.append(3 * nodes + comp)
        vals.append(np.full(nodes.size, v))
    return m, np.concatenate(dofs), np.concatenate(vals)


class BatchNISTGPU(NISTGPU):
    """Newton driver over a batch of independent cubes strained by 1 % along z in 10 increments."""

    def __init__(self, spec, h=0.1, strain=0.01, bc="clamped", device="cuda", tile=None, rtol=1e-10, maxKrylov=20000,
                 graph=True):  # fmt: skip
        coords, elements, rows, dofs, vals, nodePtr, nEl = [], [], [], [], [], [0], []
        base = 0
        for p, prob in enumerate(spec):
            m, d, v = cube_mesh(prob["n"], h, strain, bc)
            coords.append(m["coords"])
            elements.append(m["elements"] + base)
            rows.append(np.full(m["elements"].shape[0], p, np.int32))
            dofs.append(d + 3 * base)
            vals.append(v)
            base += m["coords"].shape[0]
            nodePtr.append(base)
            nEl.append(m["elements"].shape[0])
        table = np.array([prob["props"] for prob in spec], dtype=float)
        group = ElementGroup("C3D8", np.concatenate(elements), "vonmises", table[0], table, np.concatenate(rows))
        model = Model(np.concatenate(coords), [group])
        dir_ = DirichletDofs(np.concatenate(dofs), np.concatenate(vals))
        super().__init__(model, [dir_], keFp64=True, linsolver=LinSolverOptions(mixed=False), device=device)
        self.nProb = len(spec)
        self.nodePtr = np.asarray(nodePtr, dtype=np.int32)
        self.nElProb = np.asarray(nEl)
        self.nAccProb = 24.0 * self.nElProb  # sum of element DOF counts per problem
        _lib.check(self.lib.ef_batch_setup(self.ctx, self.nProb, self.nodePtr.ctypes.data), "ef_batch_setup")
        self.rtol = rtol
        self.maxKrylov = maxKrylov
        self.useGraph = graph
        self.profile = False  # eager mode only: CUDA-event time of every batched solve in solveMs
        self.solveMs = []
        self.tile = None
        self.tuning = None
        if tile is not None:
            _lib.check(self.lib.ef_batch_set_tile(self.ctx, tile), "ef_batch_set_tile")
            self.tile = tile
        dofOwner = np.repeat(np.arange(self.nProb), 3 * np.diff(self.nodePtr))
        self.dofOwner = torch.as_tensor(dofOwner, device=self.device)
        # static buffers of the captured iteration body
        z = self._vec
        self.U_n, self.dU, self.U_np, self.P, self.F, self.R, self.PExt, self.ddU = (z() for _ in range(8))
        self.activeDof = z()
        self.freeDof = torch.ones(self.nDof, dtype=torch.float64, device=self.device)
        self.freeDof[self.dirIdx] = 0.0
        self.norms = torch.zeros(self.nProb, 3, dtype=torch.float64, device=self.device)
        self.kIters = torch.zeros(self.nProb, dtype=torch.int32, device=self.device)
        self.kRel = torch.zeros(self.nProb, dtype=torch.float64, device=self.device)
        self._graph = None
        self._warm = False
        self._time2 = np.zeros(2)
        self._dT = 0.0
        self.problemHistory = []  # per converged increment: Newton iterations per problem
        self.krylovPerProblem = np.zeros(self.nProb, dtype=np.int64)

    # -- device pieces --------------------------------------------------------------------------
    def _elements(self):
        s = self._stream()
        _lib.check(self.lib.ef_compute_elements(self.ctx, self.U_np.data_ptr(), self.dU.data_ptr(),
                                                self._time2.ctypes.data, self._dT, self.P.data_ptr(),
                                                self.F.data_ptr(), s), "ef_compute_elements")  # fmt: skip

    def _norms(self, withCorrection):
        _lib.check(self.lib.ef_batch_norms(self.ctx, self.R.data_ptr(), self.F.data_ptr(),
                                           self.ddU.data_ptr() if withCorrection else None, self.norms.data_ptr(),
                                           self._stream()), "ef_batch_norms")  # fmt: skip

    def _solve_update(self):
        """Iteration body: assemble, solve the active problems, update, elements, residual, norms."""
        _lib.check(self.lib.ef_assemble_bsr(self.ctx, self._stream()), "ef_assemble_bsr")
        self.R.mul_(self.activeDof)
        if self.profile:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
        _lib.check(self.lib.ef_batch_solve(self.ctx, self.rtol, self.maxKrylov, self.R.data_ptr(), self.ddU.data_ptr(),
                                           self.kIters.data_ptr(), self.kRel.data_ptr(), self._stream()),
                   "ef_batch_solve")  # fmt: skip
        if self.profile:
            e1.record()
            e1.synchronize()
            self.solveMs.append(e0.elapsed_time(e1))
        self.dU.add_(self.ddU)
        torch.add(self.U_n, self.dU, out=self.U_np)
        self._elements()
        torch.add(self.P, self.PExt, out=self.R)
        self.R.mul_(self.freeDof)  # Dirichlet rows of the residual are zero
        self._norms(True)

    def _run_body(self):
        """The first run is eager (all lazy setup in the library happens there); the second one
        captures the body as a CUDA graph (capture records, it does not execute), then replays."""
        if self.useGraph and self._graph is None and self._warm:
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, capture_error_mode="thread_local"):
                self._solve_update()
            self._graph = g
        if self._graph is not None:
            self._graph.replay()
        else:
            self._solve_update()
            self._warm = True

    def tile_shapes(self):
        out = []
        for t in range(self.lib.ef_batch_tile_count()):
            a, b = ctypes.c_int(), ctypes.c_int()
            _lib.check(self.lib.ef_batch_tile_info(t, ctypes.byref(a), ctypes.byref(b)), "ef_batch_tile_info")
            out.append((a.value, b.value))
        return out

    def autotune(self):
        """Picks the batched-PCG tile shape (threads per problem, lanes per block row) by timing
        every shape on the current system (ef_batch_autotune)."""
        _lib.check(self.lib.ef_assemble_bsr(self.ctx, self._stream()), "ef_assemble_bsr")
        tile = ctypes.c_int()
        ms = np.zeros(self.lib.ef_batch_tile_count(), np.float32)
        x = self._vec()
        _lib.check(self.lib.ef_batch_autotune(self.ctx, self.rtol, self.maxKrylov, self.R.data_ptr(), x.data_ptr(),
                                              self.kIters.data_ptr(), self.kRel.data_ptr(), self._stream(),
                                              ctypes.byref(tile), ms.ctypes.data), "ef_batch_autotune")  # fmt: skip
        self.tile = tile.value
        self.tuning = {f"{a}x{b}": float(t) for (a, b), t in zip(self.tile_shapes(), ms)}
        return self.tile, self.tuning

    # -- Newton loop over all problems --------------------------------------------------------------
    def solveIncrementBatch(self, timeStep, prevTimeStep, step: Step, tune=False):
        self._time2[:] = [timeStep.stepTime, timeStep.totalTime]
        self._dT = timeStep.timeIncrement
        dU, isExtrapolated = self.extrapolateLastIncrement(step.extrapolation, timeStep, self.dU, prevTimeStep)
        self.PExt.copy_(self._externalLoads(timeStep))
        nP = self.nProb
        active = np.ones(nP, bool)
        iters = np.zeros(nP, np.int64)
        prevRes = np.zeros(nP)
        nGrew = np.zeros(nP, np.int64)
        self.activeDof.fill_(1.0)
        # iteration 0: elements at the extrapolated (or zero) increment, Dirichlet deltas as residual
        torch.add(self.U_n, self.dU, out=self.U_np)
        self._elements()
        torch.add(self.P, self.PExt, out=self.R)
        if not isExtrapolated:
            self.R[self.dirIdx] = self._dirichletDelta(timeStep)
            if tune and self.tile is None and timeStep.stepProgressIncrement > 0:
                self.autotune()  # on the first system with a load
            self._status()
            self._run_body()
            k = 1
        else:
            self.R.mul_(self.freeDof)
            self._norms(False)
            k = 0
        while True:
            self._status()
            nrm = self.norms.cpu().numpy()
            if k > 0:
                self.krylovPerProblem += np.where(active, self.kIters.cpu().numpy(), 0)
                rel = self.kRel.cpu().numpy()
                bad = active & ~(rel <= self.acceptableResidual)
                if bad.any():
                    raise DivergingSolution(f"batched Krylov solve failed for {int(bad.sum())} problems")
            flux, sumF, corr = nrm[:, 0], nrm[:, 1], nrm[:, 2]
            avg = np.maximum(1e-10, sumF / self.nAccProb)
            tol = self.fluxResidualTolerance if k < 15 else self.fluxResidualToleranceAlternative
            fieldCorr = corr if k > 0 else np.zeros(nP)
            conv = (fieldCorr < self.fieldCorrectionTolerance) & (flux <= np.maximum(tol * avg, 1e-7))
            nGrew += (flux > prevRes) & active
            prevRes = np.where(active, flux, prevRes)
            newly = active & conv
            iters[newly] = k
            active &= ~conv
            if not active.any():
                break
            if (nGrew[active] > step.maxGrowIter).any():
                raise DivergingSolution(f"Residual grew {step.maxGrowIter} times, cutting back")
            if k == step.maxIter:
                raise ReachedMaxIterations("Reached max. iterations in current increment, cutting back")
            if newly.any():
                self.activeDof.mul_((torch.as_tensor(active, device=self.device)[self.dofOwner]).to(torch.float64))
            self._run_body()
            k += 1
        return iters

    def _status(self):
        newDT = ctypes.c_double()
        st = self.lib.ef_element_status(self.ctx, self._stream(), ctypes.byref(newDT))
        if st == _lib.EF_CUTBACK:
            raise CutbackRequest("Von Mises Newton failed.", newDT.value)
        if st == _lib.EF_NAN:
            raise DivergingSolution("NaN in the element results")
        _lib.check(st, "ef_element_status")

    def solveStepBatch(self, step: Step, maxIncrements=None, tune=True):
        """Fixed sequence of increments for all problems; returns U (device) and per-increment
        Newton iterations per problem."""
        _lib.check(self.lib.ef_set_dirichlet(self.ctx, self.dirIdxHost.ctypes.data, self.dirIdxHost.size),
                   "ef_set_dirichlet")  # fmt: skip
        self.U_n.zero_()
        self.dU.zero_()
        prev = None
        stepper = AdaptiveTimeStepper(0.0, step.stepLength, step.startInc, step.maxInc, step.minInc, step.maxNumInc)
        done = 0
        for ts in stepper.generateTimeStep():
            iters = self.solveIncrementBatch(ts, prev, step, tune=tune)
            self.U_n.add_(self.dU)
            prev = ts
            if iters.max() >= step.criticalIter:
                stepper.preventIncrementIncrease()
            _lib.check(self.lib.ef_accept_state(self.ctx), "ef_accept_state")
            self.problemHistory.append((ts.number, iters.copy()))
            done += 1
            if maxIncrements is not None and done >= maxIncrements:
                break
        return self.U_n.clone()

    def problem_dofs(self, p):
        return slice(3 * int(self.nodePtr[p]), 3 * int(self.nodePtr[p + 1]))
