"""The GPU hot path behind host (numpy) vectors.

The reference's Newton driver keeps its vectors as numpy ``DofVector`` objects on the host
(``numerics/dofmanager.py:98-120``) and calls four methods per Newton iteration
(``solvers/nonlinearimplicitstatic.py:451-454``): ``computeElements``, ``assembleStiffnessCSR``,
``applyDirichletK`` and ``linearSolve``.  ``HostArrayBackend`` answers those calls through the C ABI
of ``libefgpu.so``: host inputs are staged through pinned buffers into device vectors, the element
loop, the 3x3-block assembly and the Krylov solve run on the GPU, and the results come back into
host arrays.  The element stiffness and the assembled system never leave the device.

Per Newton iteration the host <-> device traffic is U_np and dU up, P and F down (element loop),
b up and x down (solve): 6 nDof doubles.
"""

import ctypes

import numpy as np
import torch

from . import _lib
from .exceptions import CutbackRequest, DivergingSolution


class HostArrayBackend:
    """One context of the GPU library over host arrays.

    groups: list of dicts with keys ``elType`` (elements/library.py name), ``material``
    (linearelastic, vonmises, neohookewa), ``props`` (the material's property vector),
    ``elDofs`` (int [nEl][3 nNodes], DofVector index of each element DOF in element DOF order),
    optional ``propsTable``/``elemRow`` (a material row per element) and ``state``
    ([nEl][nQP][nState] committed state to start from, the reference layout of
    ``elements/displacementelement/element.py:222-236``).  The DofVector of the caller has nDof
    entries; ``dofCoordinates[d]`` is the coordinate of DOF d's node in DOF d's direction.
    """

    def __init__(self, nDof, dofCoordinates, groups, keFp64=False, linsolver=None, device="cuda"):
        from .solver import LinSolverOptions

        if not torch.cuda.is_available():
            raise RuntimeError("the GPU backend needs a CUDA device")
        self.lib = _lib.lib()
        self.device = torch.device(device)
        self.nDof = int(nDof)
        self.linsolver = linsolver or LinSolverOptions()
        if not self.linsolver.mixed and not keFp64:
            raise ValueError("an all-FP64 linear solve needs keFp64=True")
        self.ctx = ctypes.c_void_p()
        X = np.ascontiguousarray(np.asarray(dofCoordinates, dtype=float))
        if X.shape != (self.nDof,):
            raise ValueError("dofCoordinates must have nDof entries")
        _lib.check(self.lib.ef_create(self.nDof, X.ctypes.data, ctypes.byref(self.ctx)), "ef_create")
        self.groupIds = []
        states = []
        for g in groups:
            ed = np.ascontiguousarray(np.asarray(g["elDofs"], dtype=np.int32))
            props = np.ascontiguousarray(np.asarray(g["props"], dtype=float))
            gid = ctypes.c_int()
            _lib.check(self.lib.ef_add_group(self.ctx, g["elType"].encode(), g["material"].encode(), props.ctypes.data,
                                             props.size, ed.shape[0], ed.ctypes.data, ctypes.byref(gid)),
                       "ef_add_group")  # fmt: skip
            self.groupIds.append(gid.value)
            if g.get("propsTable") is not None:
                tab = np.ascontiguousarray(np.asarray(g["propsTable"], dtype=float))
                rows = np.ascontiguousarray(np.asarray(g["elemRow"], dtype=np.int32))
                _lib.check(self.lib.ef_set_group_props(self.ctx, gid.value, tab.ctypes.data, tab.shape[0], tab.shape[1],
                                                       rows.ctypes.data), "ef_set_group_props")  # fmt: skip
            states.append(g.get("state"))
        opts = (_lib.EF_OPT_KE_FP64 if keFp64 else 0) | _lib.EF_OPT_NO_SCALAR_CSR
        _lib.check(self.lib.ef_finalize(self.ctx, opts), "ef_finalize")
        for gid, st in zip(self.groupIds, states):
            if st is not None:
                self.set_state(gid, st)
        self.info = _lib.EfInfo()
        _lib.check(self.lib.ef_get_info(self.ctx, ctypes.byref(self.info)), "ef_get_info")
        z = dict(dtype=torch.float64, device=self.device)
        self._U, self._dU, self._P, self._F, self._b, self._x = (torch.zeros(self.nDof, **z) for _ in range(6))
        self._hIn = [torch.zeros(self.nDof, dtype=torch.float64).pin_memory() for _ in range(2)]
        self._hOut = [torch.zeros(self.nDof, dtype=torch.float64).pin_memory() for _ in range(2)]
        self._dirichlet = None
        self.lastSolveInfo = None
        self.krylovIterations = []

    # ---- helpers -----------------------------------------------------------------------------
    def _stream(self):
        return torch.cuda.current_stream(self.device).cuda_stream

    def _up(self, host, slot, dev):
        """host numpy [nDof] -> pinned staging -> device vector (stream ordered)."""
        h = self._hIn[slot]
        h.numpy()[:] = host
        dev.copy_(h, non_blocking=True)

    def _down(self, dev, slot):
        h = self._hOut[slot]
        h.copy_(dev, non_blocking=True)
        return h

    # ---- the hot path ------------------------------------------------------------------------
    def compute_elements(self, U_np, dU, time2, dT):
        """Element loop from the committed state: returns host copies (P, F) of the condensed
        element residuals P = sum Pe and fluxes F = sum |Pe| (element order).  Raises CutbackRequest
        (return map failed, materials/vonmises/vonmises.py:231) or DivergingSolution (NaN)."""
        self._up(U_np, 0, self._U)
        self._up(dU, 1, self._dU)
        t = np.ascontiguousarray(np.asarray(time2, dtype=float))
        _lib.check(self.lib.ef_compute_elements(self.ctx, self._U.data_ptr(), self._dU.data_ptr(), t.ctypes.data,
                                                float(dT), self._P.data_ptr(), self._F.data_ptr(), self._stream()),
                   "ef_compute_elements")  # fmt: skip
        hp = self._down(self._P, 0)
        hf = self._down(self._F, 1)
        pNewDT = ctypes.c_double(1.0)
        st = self.lib.ef_element_status(self.ctx, self._stream(), ctypes.byref(pNewDT))  # synchronises the stream
        if st == _lib.EF_CUTBACK:
            raise CutbackRequest("Von Mises Newton failed.", pNewDT.value)
        if st == _lib.EF_NAN:
            raise DivergingSolution("Obtained NaN in element evaluation")
        _lib.check(st, "ef_element_status")
        return hp.numpy().copy(), hf.numpy().copy()

    def assemble(self):
        """The element stiffness scattered into the 3x3-block system, on the device."""
        _lib.check(self.lib.ef_assemble_bsr(self.ctx, self._stream()), "ef_assemble_bsr")

    def set_dirichlet(self, dofs):
        """Constrained DOFs (their rows take the right-hand side, as the reference's rows with
        diagonal 1 do); uploaded only when the set changes."""
        d = np.ascontiguousarray(np.asarray(dofs, dtype=np.int64))
        if self._dirichlet is not None and np.array_equal(d, self._dirichlet):
            return
        _lib.check(self.lib.ef_set_dirichlet(self.ctx, d.ctypes.data, d.size), "ef_set_dirichlet")
        self._dirichlet = d

    def solve(self, b):
        """x with K x = b for the last assembled system; host arrays in and out.  A NaN raises
        DivergingSolution (solvers/nonlinearimplicitstatic.py:748-749); a stalled Krylov solve is
        kept below a relative residual of 1e-6, else DivergingSolution."""
        o = self.linsolver
        opts = _lib.EfSolveOpts(_lib.EF_SOLVE_FGMRES if o.method == "fgmres" else _lib.EF_SOLVE_PCG,
                                1 if o.mixed else 0, o.rtol, o.innerRtol, o.maxIter, o.restart, o.maxRefine,
                                1 if o.profile else 0)  # fmt: skip
        self._up(b, 0, self._b)
        info = _lib.EfSolveInfo()
        st = self.lib.ef_solve(self.ctx, ctypes.byref(opts), self._b.data_ptr(), self._x.data_ptr(), ctypes.byref(info),
                               self._stream())  # fmt: skip
        self.lastSolveInfo = info
        self.krylovIterations.append(info.iterations)
        if st == _lib.EF_NAN:
            raise DivergingSolution("Obtained NaN in linear solve")
        if st == _lib.EF_NOT_CONVERGED and not (info.relResidual <= 1e-6):
            raise DivergingSolution(f"Krylov solve stalled at relative residual {info.relResidual:.2e}")
        if st not in (_lib.EF_OK, _lib.EF_NOT_CONVERGED):
            _lib.check(st, "ef_solve")
        h = self._down(self._x, 0)
        torch.cuda.current_stream(self.device).synchronize()
        return h.numpy().copy()

    def begin_increment(self):
        """A new increment: its first new system rebuilds the FGMRES multigrid's coarse levels, the
        following ones reuse them (LinSolverOptions.precondReuse; ef_fgmres_set_reuse)."""
        if self.linsolver.method == "fgmres":
            _lib.check(self.lib.ef_fgmres_set_reuse(self.ctx, self.linsolver.precondReuse), "ef_fgmres_set_reuse")

    def accept_state(self):
        """acceptLastState for every element (trial -> committed state, on the device)."""
        _lib.check(self.lib.ef_accept_state(self.ctx), "ef_accept_state")

    # ---- element state -----------------------------------------------------------------------
    def state_shape(self, groupId):
        nQP, nState = ctypes.c_int(), ctypes.c_int()
        _lib.check(self.lib.ef_get_state_size(self.ctx, groupId, ctypes.byref(nQP), ctypes.byref(nState)),
                   "ef_get_state_size")  # fmt: skip
        return nQP.value, nState.value

    def set_state(self, groupId, state):
        nQP, nState = self.state_shape(groupId)
        s = np.ascontiguousarray(np.asarray(state, dtype=float))
        if s.shape[1:] != (nQP, nState):
            raise ValueError(f"state of group {groupId} must be [nEl][{nQP}][{nState}], got {s.shape}")
        _lib.check(self.lib.ef_set_state(self.ctx, groupId, s.ctypes.data), "ef_set_state")

    def get_state(self, groupId, nEl, trial=False):
        nQP, nState = self.state_shape(groupId)
        out = np.zeros((nEl, nQP, nState))
        _lib.check(self.lib.ef_get_state(self.ctx, groupId, 1 if trial else 0, out.ctypes.data), "ef_get_state")
        return out

    def close(self):
        if getattr(self, "ctx", None) is not None and self.ctx.value:
            self.lib.ef_destroy(self.ctx)
        self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
