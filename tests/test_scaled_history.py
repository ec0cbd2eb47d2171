"""The benchmark's J2 box at a quarter of its edge counts (25x10x10 C3D8 on 2.5x1x1, the same
element size, material, boundary conditions and 20-increment load history as the 160k-element
100x40x40 box), pinned to the reference's own NIST run increment by increment
(tests/golden/nist_j2_box_25x10x10_history.npz, made by tests/golden/make_golden.py headline).

* CPU: the oracle reproduces the reference's Newton iteration count and displacements of every
  increment and the final Gauss-point stresses.
* GPU (through the C ABI): the all-FP64 path, the mixed-precision block-Jacobi PCG path and the
  benchmark's own solver (FGMRES(64) + multigrid, FP32 inner iterations to 1e-5, FP64 refinement
  to 1e-8) give the reference's Newton iteration count in every increment and displacements
  within 1e-6 of the reference's (relative to the increment's largest displacement), and the
  final stresses within 1e-6 of the largest stress.
"""

import ctypes

import numpy as np
import pytest

from cases import build_gpu_solver, j2_box_spec
from conftest import golden

CASE = "nist_j2_box_25x10x10_history.npz"


def _dims(g):
    return [int(g[k]) for k in ("nX", "nY", "nZ")] + [float(g[k]) for k in ("lX", "lY", "lZ")]


def _check_history(g, iters, Us, stress):
    assert list(iters) == list(g["iters"]), (list(iters), list(g["iters"]))
    U_inc = g["U_inc"]
    assert len(Us) == U_inc.shape[0]
    for k, (u, ref) in enumerate(zip(Us, U_inc)):
        err = np.max(np.abs(u - ref))
        assert err <= 1e-6 * np.max(np.abs(ref)) + 1e-15, (k, err, np.max(np.abs(ref)))
    sref = g["stress"]
    assert np.max(np.abs(stress - sref)) <= 1e-6 * np.max(np.abs(sref))


def test_oracle_matches_reference_scaled_benchmark_history():
    from oracle.element import SmallStrainElements
    from oracle.mesh import BoxMesh
    from oracle.nist import NIST, Model, Step
    from oracle.system import element_dofs

    g = golden(CASE)
    m = BoxMesh(*_dims(g))
    els = SmallStrainElements("C3D8", m.coords[m.elements], "vonmises", [210000.0, 0.3, 250.0, 1000.0, 0.0, 0.0])
    left, right = m.nodeSets["gen_left"], m.nodeSets["gen_right"]
    dirs = [((3 * left[:, None] + np.arange(3)).ravel(), np.zeros(3 * left.size)),
            (3 * right, np.full(right.size, float(g["ux"])))]  # fmt: skip
    s = NIST(Model(3 * m.nNodes, [(els, element_dofs(m.elements))], dirs))
    Us = []
    s.solveStep(Step(maxInc=float(g["maxInc"]), minInc=1e-6, maxIter=25), callback=lambda ts, it, U: Us.append(U.copy()))
    _check_history(g, [it for _, it in s.history], Us, els.stateRef[:, :, 0:6])


MODES = {
    "fp64": dict(keFp64=True, linsolver=dict(mixed=False)),
    "mixed_pcg": dict(keFp64=False, linsolver=dict()),
    "headline_fgmres": dict(keFp64=False, linsolver=dict(method="fgmres", rtol=1e-8, restart=64, innerRtol=1e-5)),
}


@pytest.mark.gpu
@pytest.mark.parametrize("mode", sorted(MODES))
def test_gpu_matches_reference_scaled_benchmark_history(gpu_lib, mode):
    from edelweissfe_gb300 import _lib
    from edelweissfe_gb300.solver import LinSolverOptions, Step

    g = golden(CASE)
    spec = j2_box_spec(*_dims(g), ux=float(g["ux"]))
    cfg = MODES[mode]
    s = build_gpu_solver(spec, keFp64=cfg["keFp64"], linsolver=LinSolverOptions(**cfg["linsolver"]))
    Us = []
    s.solveStep(Step(maxInc=float(g["maxInc"]), minInc=1e-6, maxIter=25),
                callback=lambda ts, it, U: Us.append(U.cpu().numpy()))  # fmt: skip
    nQP, nState = ctypes.c_int(), ctypes.c_int()
    _lib.check(gpu_lib.ef_get_state_size(s.ctx, 0, ctypes.byref(nQP), ctypes.byref(nState)), "size")
    st = np.zeros((g["stress"].shape[0], nQP.value, nState.value))
    _lib.check(gpu_lib.ef_get_state(s.ctx, 0, 0, st.ctypes.data), "ef_get_state")
    _check_history(g, [it for _, it in s.iterationHistory], Us, st[:, :, 0:6])
