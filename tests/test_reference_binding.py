"""The drop-in boundary: the GPU methods inside a Newton driver that keeps its vectors on the host.

* CPU: the reference's own ``finiteElementSimulation`` runs the reference's own input file
  ``testfiles/TensionBarHexa8/test.inp`` with ``*solver, solver=NISTGPU`` (the subclass of the
  reference's NIST from ``edelweissfe_gb300.reference_nist``, registered in the reference's solver
  library) and reproduces the reference's golden ``U.ref``; the backend under the four hot-path
  methods is answered by the oracle on host arrays (no GPU here), so the test checks the binding
  itself: element types, materials and DOF maps read from the reference's objects, signatures,
  Dirichlet indices, state commits and the exceptions of the reference.  Needs the reference's
  sources (``EF_REFERENCE``, default /root/reference); skipped where they are absent.
* GPU: ``HostArrayBackend`` (the GPU backend of that binding, numpy arrays in and out) under the
  oracle's restatement of the reference's Newton loop reproduces the reference's J2 box run
  (Newton counts identical, displacements within 1e-6).
"""

import os
import sys

import numpy as np
import pytest

from conftest import ROOT, golden
from oracle.element import make_elements
from oracle.system import condense

REF = os.environ.get("EF_REFERENCE", "/root/reference")


class OracleBackend:
    """The calls NISTGPU makes on its backend, answered by the oracle on host arrays."""

    def __init__(self, nDof, X, groups, keFp64, linsolver):
        import scipy.sparse  # noqa: F401

        self.nDof = nDof
        self.groupIds = list(range(len(groups)))
        self.groups = []
        for g in groups:
            ed = np.asarray(g["elDofs"], dtype=np.int64)
            coords = X[ed].reshape(ed.shape[0], -1, 3)
            els = make_elements(g["elType"], coords, g["material"], g["props"])
            els.stateRef[:] = g["state"]
            self.groups.append((els, ed))
        self.dirichlet = np.zeros(0, np.int64)
        self.calls = {"compute": 0, "assemble": 0, "solve": 0, "accept": 0}

    def compute_elements(self, U, dU, time2, dT):
        self.calls["compute"] += 1
        P = np.zeros(self.nDof)
        F = np.zeros(self.nDof)
        self._K = []
        for els, ed in self.groups:
            Ke, Pe = els.compute_yourself(U[ed], dU[ed])
            p, f = condense(Pe, ed, self.nDof)
            P += p
            F += f
            self._K.append((Ke, ed))
        return P, F

    def assemble(self):
        import scipy.sparse as sp

        self.calls["assemble"] += 1
        rows = np.concatenate([np.repeat(ed, ed.shape[1], axis=1).ravel() for _, ed in self._K])
        cols = np.concatenate([np.tile(ed, (1, ed.shape[1])).ravel() for _, ed in self._K])
        vals = np.concatenate([Ke.ravel() for Ke, _ in self._K])
        self._A = sp.csr_matrix((vals, (rows, cols)), shape=(self.nDof, self.nDof))

    def set_dirichlet(self, dofs):
        self.dirichlet = np.asarray(dofs, dtype=np.int64)

    def solve(self, b):
        import scipy.sparse as sp
        import scipy.sparse.linalg as spla

        self.calls["solve"] += 1
        keep = np.ones(self.nDof)
        keep[self.dirichlet] = 0.0
        D = sp.diags(keep)
        A = (D @ self._A + sp.diags(1.0 - keep)).tocsc()
        return spla.spsolve(A, np.asarray(b, dtype=float))

    def accept_state(self):
        self.calls["accept"] += 1
        for els, _ in self.groups:
            els.accept_last_state()

    def get_state(self, gid, nEl, trial=False):
        els = self.groups[gid][0]
        return (els.stateTemp if trial else els.stateRef).copy()

    def close(self):
        pass


@pytest.fixture(scope="module")
def reference(tmp_path_factory):
    if not os.path.isdir(os.path.join(REF, "edelweissfe")):
        pytest.skip("the reference's sources are not present")
    import torch  # noqa: F401  (before the harness stubs matplotlib, which torch's import inspects)

    import edelweissfe_gb300.solver  # noqa: F401

    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_golden

    scratch = str(tmp_path_factory.mktemp("efref"))
    make_golden.prepare_reference(scratch, modules=["numerics/csrgenerator", "utils/elementresultcollector"])
    return scratch


def test_reference_driver_runs_the_gpu_methods_and_matches_uref(reference, tmp_path, monkeypatch):
    from edelweissfe.config import solvers
    from edelweissfe.drivers.inputfiledrivensimulation import finiteElementSimulation
    from edelweissfe.solvers.nonlinearimplicitstatic import NIST
    from edelweissfe.utils.inputfileparser import parseInputFile

    from edelweissfe_gb300 import reference_nist

    made = []

    def factory(*a, **k):
        made.append(OracleBackend(*a, **k))
        return made[-1]

    cls = reference_nist.nist_gpu_class(backendFactory=factory)
    assert issubclass(cls, NIST)
    # the four hot-path methods are overridden; the Newton iteration's control (solveIncrement only
    # gains the device-state commit after the reference's own loop), the convergence test, the
    # Dirichlet rows of R, the loads and the extrapolation are the reference's
    for name in ("computeElements", "assembleStiffnessCSR", "applyDirichletK", "linearSolve"):
        assert name in cls.__dict__
    for name in ("checkConvergence", "applyDirichlet", "assembleLoads", "extrapolateLastIncrement"):
        assert name not in cls.__dict__
    monkeypatch.setitem(sys.modules, "edelweissfe.solvers.nonlinearimplicitstaticgpu",
                        type(sys)("edelweissfe.solvers.nonlinearimplicitstaticgpu"))  # fmt: skip
    sys.modules["edelweissfe.solvers.nonlinearimplicitstaticgpu"].NISTGPU = cls
    monkeypatch.setitem(solvers.solverLibrary, "NISTGPU", "nonlinearimplicitstaticgpu")

    with open(os.path.join(REF, "testfiles", "TensionBarHexa8", "test.inp")) as f:
        text = f.read()
    assert "solver=NIST," in text
    monkeypatch.chdir(tmp_path)
    with open("test.inp", "w") as f:
        f.write(text.replace("solver=NIST,", "solver=NISTGPU,"))
    model, _ = finiteElementSimulation(parseInputFile("test.inp"), verbose=False, suppressPlots=True)
    U = np.hstack([fl["U"].flatten() for fl in model.nodeFields.values()])
    ref = np.loadtxt(os.path.join(REF, "testfiles", "TensionBarHexa8", "U.ref"))
    # the reference runner's tolerance (_cli/_run_tests_edelweissfe.py:105)
    assert np.max(np.abs(U - ref)) < 1e-6
    assert np.max(np.abs(U - ref)) <= 1e-9 * np.max(np.abs(ref))
    (b,) = made
    # the zero increment (1 Newton iteration) and the load increment (2): an element pass per
    # iteration plus the converged one, a solve per iteration, a commit per increment
    assert b.calls == {"compute": 5, "assemble": 3, "solve": 3, "accept": 2}, b.calls
    # the committed state came back into the reference's element objects (stress of a linear bar)
    els = list(model.elements.values())
    assert max(np.abs(np.asarray(el._stateVarsRef)[:, 2]).max() for el in els) > 0.0


def test_binding_rejects_models_it_cannot_run(reference):
    from edelweissfe.elements.displacementelement.element import DisplacementElement

    from edelweissfe_gb300 import reference_nist

    el = DisplacementElement("CPE4", 1)
    with pytest.raises(NotImplementedError):
        reference_nist.element_type_of(el)
    with pytest.raises(NotImplementedError):
        reference_nist.material_of(object())


@pytest.mark.gpu
def test_host_array_backend_under_the_oracle_newton_loop(gpu_lib):
    """HostArrayBackend (host vectors in and out) under the oracle's restatement of the
    reference's Newton loop: the reference's J2 box run (Newton counts, displacements)."""
    from oracle.mesh import BoxMesh
    from oracle.nist import NIST, Model, Step
    from oracle.system import element_dofs

    from edelweissfe_gb300.hostbackend import HostArrayBackend
    from edelweissfe_gb300.solver import LinSolverOptions

    g = golden("nist_j2_box_10x4x4.npz")
    dims = [int(g[k]) for k in ("nX", "nY", "nZ")] + [float(g[k]) for k in ("lX", "lY", "lZ")]
    m = BoxMesh(*dims)
    props = [210000.0, 0.3, 250.0, 1000.0, 0.0, 0.0]
    ed = element_dofs(m.elements)
    els = make_elements("C3D8", m.coords[m.elements], "vonmises", props)
    left, right = m.nodeSets["gen_left"], m.nodeSets["gen_right"]
    dirs = [((3 * left[:, None] + np.arange(3)).ravel(), np.zeros(3 * left.size)),
            (3 * right, np.full(right.size, float(g["ux"])))]  # fmt: skip
    nDof = 3 * m.nNodes
    backend = HostArrayBackend(nDof, m.coords.reshape(-1),
                               [{"elType": "C3D8", "material": "vonmises", "props": props, "elDofs": ed}],
                               linsolver=LinSolverOptions(method="fgmres", rtol=1e-10))  # fmt: skip

    class Driver(NIST):
        def computeElements(self, U_np, dU):
            P, F = backend.compute_elements(U_np, dU, np.zeros(2), 0.0)
            return P, None, F

        def assembleStiffnessCSR(self, V):
            backend.assemble()
            return None

        def applyDirichletK(self, data):
            backend.set_dirichlet(self.dirIdx)
            return backend

        def linearSolve(self, A, b):
            return A.solve(b)

    s = Driver(Model(nDof, [(els, ed)], dirs))
    accept = els.accept_last_state  # the oracle driver commits the group's state; the device state with it
    els.accept_last_state = lambda: (accept(), backend.accept_state())
    U, _ = s.solveStep(Step(maxInc=float(g["maxInc"]), minInc=1e-6, maxIter=25))
    assert [it for _, it in s.history] == list(g["iters"])
    assert np.max(np.abs(U - g["U"])) <= 1e-6 * np.max(np.abs(g["U"]))
    backend.close()
