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

    def _arr(self, ptr):
        return np.ctypeslib.as_array((ctypes.c_double * self.nDof).from_address(ptr))

    def ef_norms(self, ctx, R, F, ddU, out, stream):
        o = np.ctypeslib.as_array((ctypes.c_double * 3).from_address(out))
        o[0] = np.max(np.abs(self._arr(R)))
        o[1] = np.sum(np.abs(self._arr(F)))
        o[2] = np.max(np.abs(self._arr(ddU))) if ddU is not None else 0.0
        return 0

    def ef_set_dirichlet(self, ctx, dofs, n):
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
    s.dirIdxHost = np.concatenate([d.dofs for d in s.dirichlets]).astype(np.int64)
    s.dirIdx = torch.as_tensor(s.dirIdxHost)
    s.computationTimes = {}
    s.iterationHistory = []
    s.krylovIterations = []
    s.lastSolveInfo = None
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
