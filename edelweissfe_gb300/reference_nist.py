"""The GPU hot path inside the reference's own Newton driver.

``nist_gpu_class()`` returns a subclass of EdelweissFE's ``NIST``
(``solvers/nonlinearimplicitstatic.py:60``) that keeps every method of the reference but the four
that the Newton iteration calls on its hot path (``solveIncrement``, :412-456):

* ``computeElements(elements, U_np, dU, P, K, F, timeStep)`` (:794-849) -- the element loop and the
  ``P += Pe``, ``F += |Pe|`` condensation run on the GPU; ``K`` (the host ``VIJSystemMatrix``) is
  passed through untouched, the element stiffness stays on the device;
* ``assembleStiffnessCSR(K)`` (:753-769) -- the 3x3-block system is scattered on the device; the
  return value is a handle to it, not a ``csr_matrix``;
* ``applyDirichletK(K_, dirichlets)`` (:559-593) -- the constrained DOFs of
  ``findDirichletIndices`` are eliminated inside the device solve (their rows take the
  right-hand side, the solution the reference's rows with diagonal 1 give);
* ``linearSolve(A, b)`` (:727-751) -- block-Jacobi PCG or FGMRES + multigrid on the device; a NaN
  raises the reference's ``DivergingSolution``.

``solveStep``, ``solveIncrement``, ``checkConvergence``, the Dirichlet and load step actions, the
increment control and the output managers are the reference's own.  The element objects keep their
role as the model's description: type, nodes and material are read from them when the first
element pass of a step builds the GPU context, and their committed state is uploaded then.  After
every converged increment the device state is written into each element's ``_stateVarsTemp``, so
that the reference's own ``model.advanceToTime`` -> ``acceptLastState`` commits it and result
output sees it (option ``gpuSyncStates=0`` skips this for large models; the state is then written
into the elements once, when the step ends).

Options (``*solver`` or ``options, category=NISTSolver``; the reference's ``_updateOptions``):
``gpuSolver`` ("pcg" or "fgmres"), ``gpuMixed`` (1: FP32 inner iterations + FP64 refinement),
``gpuRtol`` (FP64 relative residual of each solve), ``gpuKeFp64`` (1: FP64 element stiffness),
``gpuSyncStates``, ``gpuPrecondReuse`` (Newton systems of an increment that reuse the coarse
multigrid levels built for its first one).

Supported entities: ``DisplacementElement`` and ``DisplacementTLElement`` of the 3D hexahedra
(C3D8, C3D8R, C3D8E, C3D20, C3D20R and their TL forms) with ``LinearElasticMaterial``,
``VonMisesMaterial`` or ``NeoHookeanWaMaterial``; a model with other elements or with constraints
raises ``NotImplementedError`` when the step starts.
"""

from time import time as getCurrentTime

import numpy as np

# (element class, nodes, integration points) -> elements/library.py type name
_ELEMENT_TYPES = {
    ("DisplacementElement", 8, 8): "C3D8",
    ("DisplacementElement", 8, 1): "C3D8R",
    ("DisplacementElement", 8, 27): "C3D8E",
    ("DisplacementElement", 20, 27): "C3D20",
    ("DisplacementElement", 20, 8): "C3D20R",
    ("DisplacementTLElement", 8, 8): "C3D8TL",
    ("DisplacementTLElement", 8, 1): "C3D8RTL",
    ("DisplacementTLElement", 8, 27): "C3D8ETL",
    ("DisplacementTLElement", 20, 27): "C3D20TL",
    ("DisplacementTLElement", 20, 8): "C3D20RTL",
}


def material_of(mat):
    """(library material name, property vector) of a reference material instance
    (materials/linearelastic/linearelastic.py:58-62, materials/vonmises/vonmises.py:76-95,
    materials/neohooke/neohookepencegouformulationa.py:64-70)."""
    name = type(mat).__name__
    if name == "VonMisesMaterial":
        return "vonmises", [mat._E, mat._v, mat.yieldStress, mat.HLin, mat.deltaYieldStress, mat.delta]
    if name == "LinearElasticMaterial":
        return "linearelastic", [mat._E, mat._v]
    if name == "NeoHookeanWaMaterial":
        return "neohookewa", [mat._mu, mat._K]
    raise NotImplementedError(f"material {name} has no GPU kernel")


def element_type_of(el):
    key = (type(el).__name__, int(el._nNodes), int(el._nInt))
    if key not in _ELEMENT_TYPES or getattr(el, "nSpatialDimensions", 3) != 3:
        raise NotImplementedError(f"element {key} has no GPU kernel")
    return _ELEMENT_TYPES[key]


def groups_from_elements(elements, idcsOfElements, nDof):
    """Element groups of the GPU context from the reference's element objects, in the model's
    element order (consecutive elements of one type and material form one group; the
    condensation then sums P and F in the reference's order), and the DOF coordinates.
    Returns (groups, dofCoordinates, members) with members[g] the element objects of group g."""
    X = np.zeros(nDof)
    groups, members = [], []
    for el in elements.values():
        elType = element_type_of(el)
        material, props = material_of(el.material)
        dofs = np.asarray(idcsOfElements[el], dtype=np.int64)
        nn = int(el._nNodes)
        if dofs.size != 3 * nn or np.any(np.diff(dofs.reshape(nn, 3), axis=1) != 1):
            raise NotImplementedError("the GPU kernels need each node's three displacement DOFs consecutive")
        X[dofs] = np.array([n.coordinates for n in el.nodes], dtype=float).reshape(-1)
        key = (elType, material, tuple(float(p) for p in props))
        if not groups or groups[-1]["key"] != key:
            groups.append({"key": key, "elType": elType, "material": material, "props": list(key[2]), "elDofs": []})
            members.append([])
        groups[-1]["elDofs"].append(dofs)
        members[-1].append(el)
    for g, mem in zip(groups, members):
        g["elDofs"] = np.array(g["elDofs"], dtype=np.int32)
        g["state"] = np.array([np.asarray(el._stateVarsRef) for el in mem])
        del g["key"]
    return groups, X, members


class DeviceSystem:
    """Handle to the assembled system on the device (what assembleStiffnessCSR returns)."""

    def __init__(self, backend):
        self.backend = backend
        self.shape = (backend.nDof, backend.nDof)


def nist_gpu_class(NIST=None, exceptions=None, backendFactory=None):
    """The GPU subclass of the reference's NIST.  NIST and the reference's exceptions module
    default to ``edelweissfe.solvers.nonlinearimplicitstatic.NIST`` and
    ``edelweissfe.utils.exceptions``; backendFactory(nDof, dofCoordinates, groups, keFp64,
    linsolver) defaults to ``HostArrayBackend``."""
    if NIST is None:
        from edelweissfe.solvers.nonlinearimplicitstatic import NIST
    if exceptions is None:
        from edelweissfe.utils import exceptions
    if backendFactory is None:
        from .hostbackend import HostArrayBackend as backendFactory
    from . import exceptions as own
    from .solver import LinSolverOptions

    class NISTGPU(NIST):
        identification = "NISTGPUSolver"

        NISTOptions = dict(NIST.NISTOptions, linsolver="superlu", gpuSolver="fgmres", gpuMixed=1, gpuRtol=1e-10,
                           gpuKeFp64=0, gpuSyncStates=1, gpuPrecondReuse=0)  # fmt: skip

        def solveStep(self, step, model, fieldOutputController, outputmanagers):
            self._gpu = None
            self._gpuMembers = None
            if getattr(model, "constraints", None):
                raise NotImplementedError("constraints are not assembled on the GPU")
            try:
                return super().solveStep(step, model, fieldOutputController, outputmanagers)
            finally:
                if self._gpu is not None:
                    self._writeStates(committed=True)
                    self._gpu.close()
                    self._gpu = None

        # ---- context -------------------------------------------------------------------------
        def _backend(self, elements):
            if self._gpu is None:
                groups, X, members = groups_from_elements(elements, self.theDofManager.idcsOfElementsInDofVector,
                                                          self.theDofManager.nDof)  # fmt: skip
                o = self.options
                ls = LinSolverOptions(method=o["gpuSolver"], mixed=bool(o["gpuMixed"]), rtol=o["gpuRtol"],
                                      restart=64 if o["gpuSolver"] == "fgmres" else 40,
                                      precondReuse=int(o["gpuPrecondReuse"]))  # fmt: skip
                self._gpu = backendFactory(self.theDofManager.nDof, X, groups, bool(o["gpuKeFp64"]), ls)
                self._gpuMembers = members
            return self._gpu

        def _writeStates(self, committed):
            """Device state -> the element objects: into _stateVarsTemp after an increment (the
            reference's acceptLastState then commits it), into _stateVarsRef at the end."""
            b = self._gpu
            for gid, mem in zip(b.groupIds, self._gpuMembers):
                st = b.get_state(gid, len(mem))
                for el, s in zip(mem, st):
                    (el._stateVarsRef if committed else el._stateVarsTemp)[:] = s

        # ---- the Newton iteration's hot path ---------------------------------------------------
        def solveIncrement(self, *args, **kwargs):
            if self._gpu is not None and hasattr(self._gpu, "begin_increment"):
                self._gpu.begin_increment()
            out = super().solveIncrement(*args, **kwargs)
            self._gpu.accept_state()
            if self.options["gpuSyncStates"]:
                self._writeStates(committed=False)
            return out

        def computeElements(self, elements, U_np, dU, P, K, F, timeStep):
            tic = getCurrentTime()
            b = self._backend(elements)
            time = np.array([timeStep.stepTime, timeStep.totalTime])
            try:
                Pd, Fd = b.compute_elements(np.asarray(U_np), np.asarray(dU), time, timeStep.timeIncrement)
            except own.CutbackRequest as e:
                raise exceptions.CutbackRequest(str(e), e.cutbackSize)
            except own.DivergingSolution as e:
                raise exceptions.DivergingSolution(str(e))
            P += Pd
            F += Fd
            self.computationTimes["elements"] += getCurrentTime() - tic
            return P, K, F

        def assembleStiffnessCSR(self, K):
            tic = getCurrentTime()
            self._gpu.assemble()
            self.computationTimes["CSR generation"] += getCurrentTime() - tic
            return DeviceSystem(self._gpu)

        def applyDirichletK(self, K, dirichlets):
            tic = getCurrentTime()
            idx = [self.findDirichletIndices(d) for d in dirichlets]
            self._gpu.set_dirichlet(np.concatenate(idx) if idx else np.zeros(0, np.int64))
            self.computationTimes["dirichlet K"] += getCurrentTime() - tic
            return K

        def linearSolve(self, A, b):
            if not isinstance(A, DeviceSystem):
                raise TypeError("NISTGPU.linearSolve solves the system assembled on the device")
            tic = getCurrentTime()
            try:
                ddU = A.backend.solve(np.asarray(b))
            except own.DivergingSolution as e:
                raise exceptions.DivergingSolution(str(e))
            self.computationTimes["linear solve"] += getCurrentTime() - tic
            if np.isnan(ddU).any():
                raise exceptions.DivergingSolution("Obtained NaN in linear solve")
            return ddU

    return NISTGPU


def register(name="NISTGPU"):
    """Makes the GPU solver selectable as ``*solver, solver=NISTGPU`` in the reference's input
    files: adds it to ``config/solvers.py``'s solverLibrary through a module object
    ``edelweissfe.solvers.nonlinearimplicitstaticgpu`` (what a maintainer adds as a file)."""
    import sys
    import types

    from edelweissfe.config import solvers

    modname = "nonlinearimplicitstaticgpu"
    mod = types.ModuleType("edelweissfe.solvers." + modname)
    setattr(mod, name, nist_gpu_class())
    sys.modules[mod.__name__] = mod
    solvers.solverLibrary[name] = modname
    return getattr(mod, name)
