"""Host logic of the GPU solver's drivers on the CPU: the NISTGPU / NISTGPUArcLength increment
loops (edelweissfe_gb300/solver.py) run on CPU tensors with the four hot-path methods and the
norms of the C ABI answered by the oracle, so that their control flow -- extrapolation, Dirichlet
rows, the two right-hand sides and the controller of the arc-length increment, convergence -- is
checked against the reference's own runs without a GPU."""

import ctypes

import numpy as np
import torch

from conftest import golden
from oracle.element import make_elements
from oracle.mesh import BoxMesh
from oracle.nist import NIST
from oracle.nist import Model as OracleModel
from oracle.system import element_dofs


class _OracleLib:
    """The few C-ABI calls that the drivers make themselves, on host memory."""

    def __init__(self, nDof, elements):
        self.nDof = nDof
        self.elements = elements
        self.dirIdx = np.zeros(0, np.int64)

    def _arr(self, ptr):
        return np.ctypeslib.as_array((ctypes.c_double * self.nDof).from_address(ptr))

    def ef_norms(self, ctx, R, F, ddU, out, stream):
        o = np.ctypeslib.as_array((ctypes.c_double * 3).from_address(out))
        o[0] = np.max(np.abs(self._arr(R)))
        o[1] = np.sum(np.abs(self._arr(F)))
        o[2] = np.max(np.abs(self._arr(ddU))) if ddU is not None else 0.0
        return 0

    def ef_set_dirichlet(self, ctx, dofs, n):
        self.dirIdx = np.ctypeslib.as_array((ctypes.c_int64 * n).from_address(dofs)).copy() if n else np.zeros(0, int)
        return 0

    def ef_newton_residual(self, ctx, mode, P, PExt, dirValues, F, ddU, iteration, prev, nGrew, opts, R, out, stream):
        """The device check's arithmetic (solvers/nonlinearimplicitstatic.py:418-436, :625-725) on host memory."""
        r = self._arr(R)
        r[:] = self._arr(P) + (self._arr(PExt) if PExt else 0.0)
        if mode == 0:
            r[self.dirIdx] = np.ctypeslib.as_array((ctypes.c_double * self.dirIdx.size).from_address(dirValues))
            return 0
        r[self.dirIdx] = 0.0
        o, res = opts._obj, out._obj
        flux = np.max(np.abs(r))
        avg = max(1e-10, np.sum(np.abs(self._arr(F))) / o.nAccFluxes)
        corr = np.max(np.abs(self._arr(ddU))) if ddU else 0.0
        tol = o.fluxTol if iteration < 15 else o.fluxTolAlt
        res.converged = int(corr < o.corrTol and flux <= max(tol * avg, o.fluxFloor))
        res.nGrew = nGrew + (1 if flux > prev else 0)
        res.fluxResidual, res.fieldCorrection, res.spatialAveragedFlux = flux, corr, avg
        return 0

    def ef_accept_state(self, ctx):
        self.elements.accept_last_state()
        return 0


def _oracle_backed(cls, model, dirichlets, nodeforces, elements, elDofs, **kw):
    """An instance of the driver class whose element loop, assembly and linear solve are the
    oracle's (scipy direct solve), on CPU tensors."""
    nDof = model.nDof
    oracle = NIST(OracleModel(nDof, [(elements, elDofs)], [(d.dofs, d.delta) for d in dirichlets], []))

    class Driver(cls):
        def _stream(self):
            return None

        def computeElements(self, U_np, dU, P, F, timeStep):
            p, V, f = oracle.computeElements(U_np.numpy(), dU.numpy())
            self._V = V
            P.copy_(torch.from_numpy(p))
            F.copy_(torch.from_numpy(f))
            return P, F

        def assembleStiffnessCSR(self):
            self._A = oracle.applyDirichletK(oracle.assembleStiffnessCSR(self._V))

        def applyDirichletK(self):
            pass

        def linearSolve(self, R):
            self.krylovIterations.append(0)
            return torch.from_numpy(oracle.linearSolve(self._A, R.numpy()))

    s = Driver.__new__(Driver)
    s.lib = _OracleLib(nDof, elements)
    s.ctx = None
    s.model = model
    s.dirichlets = list(dirichlets)
    s.nodeforces = list(nodeforces)
    s.bodyforces = []
    s.device = torch.device("cpu")
    s.nDof = nDof
    s.nAccumulatedFluxes = model.n_accumulated_fluxes()
    from edelweissfe_gb300 import _lib

    s.newtonOpts = _lib.EfNewtonOpts(s.fluxResidualTolerance, s.fluxResidualToleranceAlternative,
                                     s.fieldCorrectionTolerance, 1e-7, float(s.nAccumulatedFluxes))
    s.dirIdxHost = np.concatenate([d.dofs for d in s.dirichlets]).astype(np.int64)
    s.dirIdx = torch.as_tensor(s.dirIdxHost)
    s.computationTimes = {}
    s.iterationHistory = []
    s.krylovIterations = []
    s.lastSolveInfo = None
    from edelweissfe_gb300.solver import LinSolverOptions

    s.linsolver = LinSolverOptions()
    for k, v in kw.items():
        setattr(s, k, v)
    return s


def test_arclength_driver_host_logic_matches_reference():
    """NISTGPUArcLength's increment loop with the oracle's element loop and direct solves: the
    reference arc-length run's Newton iteration counts, load factors and displacements."""
    from edelweissfe_gb300.mesh import box_mesh
    from edelweissfe_gb300.model import DirichletBC, ElementGroup, Model, NodeForces
    from edelweissfe_gb300.solver import IndirectControl, NISTGPUArcLength, Step

    g = golden("nist_arclength_j2_10x2x2.npz")
    dims = [int(g[k]) for k in ("nX", "nY", "nZ")] + [float(g[k]) for k in ("lX", "lY", "lZ")]
    m = box_mesh(*dims)
    props = [210000.0, 0.3, 250.0, 1000.0, 0.0, 0.0]
    model = Model(m["coords"], [ElementGroup("C3D8", m["elements"], "vonmises", np.array(props))])
    mesh = BoxMesh(*dims)
    assert np.array_equal(mesh.elements, m["elements"])
    elements = make_elements("C3D8", mesh.coords[mesh.elements], "vonmises", props)
    n1, n2 = (int(np.argmin(np.linalg.norm(m["coords"] - [float(g[k]), 0.0, 0.0], axis=1))) for k in ("x1", "x2"))
    ctl = IndirectControl(3 * n1 + np.arange(3), [-1.0, 0.0, 0.0], 3 * n2 + np.arange(3), [1.0, 0.0, 0.0], float(g["L"]))
    s = _oracle_backed(NISTGPUArcLength, model, [DirichletBC(m["nodeSets"]["gen_left"], {0: 0.0, 1: 0.0, 2: 0.0})],
                       [NodeForces(m["nodeSets"]["gen_right"], [float(g["f"]), 0.0, 0.0])], elements,
                       element_dofs(mesh.elements), arcLengthController=ctl, Lambda=0.0, dLambda=0.0,
                       lambdaHistory=[])  # fmt: skip
    inc = float(g["maxInc"])
    U, _ = s.solveStep(Step(startInc=inc, maxInc=inc, minInc=1e-6, maxIter=25))
    assert [it for _, it in s.iterationHistory] == list(g["iters"])
    assert np.max(np.abs(np.array(s.lambdaHistory) - g["Lambda"])) <= 1e-12 * np.max(g["Lambda"])
    assert np.max(np.abs(U.numpy() - g["U"])) <= 1e-10 * np.max(np.abs(g["U"]))
    # two solves per Newton iteration
    assert len(s.krylovIterations) == 2 * sum(g["iters"])


def test_newton_driver_host_logic_matches_reference():
    """NISTGPU's increment loop the same way: the reference NIST run of the 3D J2 box."""
    from edelweissfe_gb300.mesh import box_mesh
    from edelweissfe_gb300.model import DirichletBC, ElementGroup, Model
    from edelweissfe_gb300.solver import NISTGPU, Step

    g = golden("nist_j2_box_10x4x4.npz")
    dims = [int(g[k]) for k in ("nX", "nY", "nZ")] + [float(g[k]) for k in ("lX", "lY", "lZ")]
    m = box_mesh(*dims)
    props = [210000.0, 0.3, 250.0, 1000.0, 0.0, 0.0]
    model = Model(m["coords"], [ElementGroup("C3D8", m["elements"], "vonmises", np.array(props))])
    mesh = BoxMesh(*dims)
    elements = make_elements("C3D8", mesh.coords[mesh.elements], "vonmises", props)
    dirs = [DirichletBC(m["nodeSets"]["gen_left"], {0: 0.0, 1: 0.0, 2: 0.0}),
            DirichletBC(m["nodeSets"]["gen_right"], {0: float(g["ux"])})]  # fmt: skip
    s = _oracle_backed(NISTGPU, model, dirs, [], elements, element_dofs(mesh.elements))
    U, _ = s.solveStep(Step(maxInc=float(g["maxInc"]), minInc=1e-6, maxIter=25))
    assert [it for _, it in s.iterationHistory] == list(g["iters"])
    assert np.max(np.abs(U.numpy() - g["U"])) <= 1e-10 * np.max(np.abs(g["U"]))


_NAN_DOF = 3 * ((2 * 3 + 1) * 3 + 1)  # x of the node (2, 1, 1) of a 4 x 2 x 2 box: a free DOF


class _ElementLib(_OracleLib):
    """ef_compute_elements / ef_element_status answered by the oracle's element loop, with a
    return-map failure or a NaN injected at chosen element-loop calls (1-based), so that the
    solver's own status mapping and cutback handling run."""

    def __init__(self, nDof, elements, oracle, inject):
        super().__init__(nDof, elements)
        self.oracle = oracle
        self.inject = inject
        self.calls = 0
        self.status = 0
        self.V = None

    def ef_compute_elements(self, ctx, U_np, dU, time2, dT, P, F, stream):
        from oracle.materials import ReturnMapFailed

        self.calls += 1
        kind = self.inject.get(self.calls)
        try:
            if kind == "returnmap":
                raise ReturnMapFailed("Von Mises Newton failed.")
            p, self.V, f = self.oracle.computeElements(self._arr(U_np).copy(), self._arr(dU).copy())
        except ReturnMapFailed:
            self.status = 1  # EF_CUTBACK
            return 0
        if kind == "nan":
            p = p.copy()
            p[_NAN_DOF] = np.nan
        self._arr(P)[:] = p
        self._arr(F)[:] = f
        self.status = 2 if np.isnan(p).any() else 0  # EF_NAN
        return 0

    def ef_element_status(self, ctx, stream, pNewDT):
        st, self.status = self.status, 0
        if pNewDT is not None:
            pNewDT._obj.value = 0.5 if st == 1 else 1.0
        return st


def test_newton_driver_cutbacks_match_oracle():
    """Failure handling of NISTGPU (solvers/nonlinearimplicitstatic.py:247-279): a return-map
    failure reported by the element status (CutbackRequest, increment x max(0.5, cutbackFactor)),
    a NaN in the element results (DivergingSolution, x cutbackFactor) and too many iterations
    (ReachedMaxIterations), injected at the same element-loop calls of the oracle's NIST, give the
    same increment sequence, iteration counts and displacements."""
    import math

    from edelweissfe_gb300.mesh import box_mesh
    from edelweissfe_gb300.model import DirichletBC, ElementGroup, Model
    from edelweissfe_gb300.solver import NISTGPU, Step
    from oracle.materials import ReturnMapFailed
    from oracle.nist import Step as OracleStep

    props = [210000.0, 0.3, 250.0, 1000.0, 0.0, 0.0]
    dims = (4, 2, 2, 1.0, 0.5, 0.5)
    inject = {12: "returnmap", 20: "nan"}
    results = {}
    for side in ("oracle", "gpu-host"):
        m = box_mesh(*dims)
        mesh = BoxMesh(*dims)
        elements = make_elements("C3D8", mesh.coords[mesh.elements], "vonmises", props)
        dirs = [DirichletBC(m["nodeSets"]["gen_left"], {0: 0.0, 1: 0.0, 2: 0.0}),
                DirichletBC(m["nodeSets"]["gen_right"], {0: 0.01})]  # fmt: skip
        oracle = NIST(OracleModel(3 * mesh.nNodes, [(elements, element_dofs(mesh.elements))],
                                  [(d.dofs, d.delta) for d in dirs], []))  # fmt: skip
        if side == "oracle":
            calls = [0]
            base = oracle.computeElements

            def computeElements(U_np, dU, base=base, calls=calls):
                calls[0] += 1
                kind = inject.get(calls[0])
                if kind == "returnmap":
                    raise ReturnMapFailed("Von Mises Newton failed.")
                P, V, F = base(U_np, dU)
                if kind == "nan":
                    P = P.copy()
                    P[_NAN_DOF] = np.nan
                return P, V, F

            oracle.computeElements = computeElements
            with np.errstate(invalid="ignore"):
                U, _ = oracle.solveStep(OracleStep(maxInc=0.5, minInc=1e-4, maxIter=4))
            results[side] = ([(n, it if it >= 0 else math.inf) for n, it in oracle.history], U)
        else:
            model = Model(m["coords"], [ElementGroup("C3D8", m["elements"], "vonmises", np.array(props))])
            s = _oracle_backed(NISTGPU, model, dirs, [], elements, element_dofs(mesh.elements))
            lib = _ElementLib(3 * mesh.nNodes, elements, oracle, inject)
            s.lib = lib
            type(s).computeElements = NISTGPU.computeElements  # the solver's own status mapping
            type(s).assembleStiffnessCSR = lambda self: setattr(self, "_A", oracle.applyDirichletK(
                oracle.assembleStiffnessCSR(lib.V)))  # fmt: skip
            with np.errstate(invalid="ignore"):
                U, _ = s.solveStep(Step(maxInc=0.5, minInc=1e-4, maxIter=4))
            results[side] = (list(s.iterationHistory), U.numpy())
    (ho, Uo), (hg, Ug) = results["oracle"], results["gpu-host"]
    assert hg == ho, (hg, ho)
    assert sum(1 for _, it in ho if it == math.inf) >= 3  # the iteration limit and both injections
    assert np.max(np.abs(Ug - Uo)) <= 1e-12 * np.max(np.abs(Uo))
