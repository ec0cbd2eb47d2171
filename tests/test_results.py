"""Element result readback (getResultArray / ElementResultCollector of the reference) from the
device state: the result names and their state slices on the CPU; on the GPU, the collector's
gathered tables against the reference's element fixtures and the full state readback, bit for bit."""

import ctypes

import numpy as np
import pytest

from conftest import golden


def test_result_names_map_to_the_reference_state_slices():
    """stress / strain / materialstate views (elements/displacementelement/element.py:222-236,
    case-insensitive) and the material results kappa (J2) and energy (NeoHookeWa)."""
    from edelweissfe_gb300.results import result_slice

    assert result_slice("vonmises", "stress", 13) == (0, 6)
    assert result_slice("linearelastic", "STRAIN", 12) == (6, 6)
    assert result_slice("vonmises", "materialstate", 13) == (12, 1)
    assert result_slice("linearelastic", "materialState", 12) == (12, 0)
    assert result_slice("vonmises", "kappa", 13) == (12, 1)
    assert result_slice("neohookewa", "energy", 13) == (12, 1)
    for mat, name in [("linearelastic", "kappa"), ("vonmises", "energy"), ("vonmises", "nonsense")]:
        with pytest.raises(Exception, match="doesn't exist for the current material"):
            result_slice(mat, name, 13)
    # the reference's fixtures have this layout: the strain slice moves by the increment (but at
    # the points of elements without one), the J2 kappa (13th entry) never decreases
    g = golden("elem_C3D8_vonmises.npz")
    s0, s1 = g["state0"], g["state1"]
    assert s1.shape[-1] == 13 and np.all(s1[..., 12] >= s0[..., 12]) and np.any(s1[..., 12] > s0[..., 12])
    assert np.any(s1[..., 6:12] != s0[..., 6:12])


@pytest.mark.gpu
@pytest.mark.parametrize("elType,mat,name", [("C3D8", "vonmises", "kappa"), ("C3D8TL", "neohookewa", "energy")])
def test_result_collector_gathers_the_state(gpu_lib, elType, mat, name):
    import torch

    from edelweissfe_gb300 import _lib
    from edelweissfe_gb300.results import result_slice
    from test_gpu_parity import _ctx_for_elements

    g = golden(f"elem_{elType}_{mat}.npz")
    ctx, nDof = _ctx_for_elements(gpu_lib, elType, mat, g["props"], g["coords"], False)
    try:
        nEl, nQP, nState = g["state0"].shape
        state0 = np.ascontiguousarray(g["state0"])
        _lib.check(gpu_lib.ef_set_state(ctx, 0, state0.ctypes.data), "ef_set_state")
        dev = torch.device("cuda")
        U = torch.as_tensor(g["U"].reshape(-1), device=dev)
        dU = torch.as_tensor(g["dU"].reshape(-1), device=dev)
        P = torch.zeros(nDof, dtype=torch.float64, device=dev)
        F = torch.zeros_like(P)
        t = np.array([0.5, 0.5])
        _lib.check(gpu_lib.ef_compute_elements(ctx, U.data_ptr(), dU.data_ptr(), t.ctypes.data, 0.1, P.data_ptr(),
                                               F.data_ptr(), None), "ef_compute_elements")  # fmt: skip
        assert gpu_lib.ef_element_status(ctx, None, None) == _lib.EF_OK
        trial = np.zeros_like(g["state1"])
        _lib.check(gpu_lib.ef_get_state(ctx, 0, 1, trial.ctypes.data), "ef_get_state")

        def collect(els, qps, first, count, which):
            cid = ctypes.c_int()
            e = None if els is None else np.ascontiguousarray(els, dtype=np.int32)
            q = None if qps is None else np.ascontiguousarray(qps, dtype=np.int32)
            _lib.check(gpu_lib.ef_results_create(ctx, 0, None if e is None else e.ctypes.data, 0 if e is None else e.size,
                                                 None if q is None else q.ctypes.data, 0 if q is None else q.size,
                                                 first, count, ctypes.byref(cid)), "ef_results_create")  # fmt: skip
            nE = nEl if e is None else e.size
            nQ = nQP if q is None else q.size
            out = np.full((nE, nQ, count), np.nan)
            _lib.check(gpu_lib.ef_results_update(ctx, cid.value, which, out.ctypes.data, None), "ef_results_update")
            return cid.value, out

        # every element and point, the stress of the committed state: the state that was set
        cAll, stress = collect(None, None, 0, 6, 0)
        assert np.array_equal(stress, state0[..., 0:6])
        # repeated, unordered elements and points, the material result of the trial state
        els, qps = [5, 0, nEl - 1, 5], [nQP - 1, 2]
        first, count = result_slice(mat, name, nState)
        cSome, kap = collect(els, qps, first, count, 1)
        assert np.array_equal(kap, trial[els][:, qps][..., first:first + count])
        ref = g["state1"][els][:, qps][..., first:first + count]
        assert np.max(np.abs(kap - ref)) <= 1e-11 * (np.max(np.abs(ref)) + 1e-30)
        # the whole state vector of one point
        cOne, full = collect([3], [1], 0, nState, 1)
        assert np.array_equal(full[0, 0], trial[3, 1])
        # resetToLastValidState: the trial state is the committed one again; a new pass restores it
        _lib.check(gpu_lib.ef_reset_state(ctx), "ef_reset_state")
        back = np.zeros_like(trial)
        _lib.check(gpu_lib.ef_get_state(ctx, 0, 1, back.ctypes.data), "ef_get_state")
        assert np.array_equal(back, state0)
        _lib.check(gpu_lib.ef_compute_elements(ctx, U.data_ptr(), dU.data_ptr(), t.ctypes.data, 0.1, P.data_ptr(),
                                               F.data_ptr(), None), "ef_compute_elements")  # fmt: skip
        assert gpu_lib.ef_element_status(ctx, None, None) == _lib.EF_OK
        # acceptLastState: the committed stress is the accepted trial stress
        _lib.check(gpu_lib.ef_accept_state(ctx), "ef_accept_state")
        out = np.full((nEl, nQP, 6), np.nan)
        _lib.check(gpu_lib.ef_results_update(ctx, cAll, 0, out.ctypes.data, None), "ef_results_update")
        assert np.array_equal(out, trial[..., 0:6])
        # the device table
        ptr, n = ctypes.c_void_p(), ctypes.c_int64()
        _lib.check(gpu_lib.ef_results_device(ctx, cAll, ctypes.byref(ptr), ctypes.byref(n)), "ef_results_device")
        assert ptr.value and n.value == nEl * nQP * 6
        # argument checks: indices outside the group, a slice outside the state, unknown ids
        cid = ctypes.c_int()
        bad = np.array([nEl], np.int32)
        q0 = np.array([0], np.int32)
        badQ = np.array([nQP], np.int32)
        assert gpu_lib.ef_results_create(ctx, 0, bad.ctypes.data, 1, None, 0, 0, 6, ctypes.byref(cid)) == _lib.EF_ERR_ARG
        assert gpu_lib.ef_results_create(ctx, 0, None, 0, badQ.ctypes.data, 1, 0, 6, ctypes.byref(cid)) == _lib.EF_ERR_ARG
        assert gpu_lib.ef_results_create(ctx, 0, None, 0, q0.ctypes.data, 1, nState - 1, 2,
                                         ctypes.byref(cid)) == _lib.EF_ERR_ARG  # fmt: skip
        assert gpu_lib.ef_results_create(ctx, 1, None, 0, None, 0, 0, 6, ctypes.byref(cid)) == _lib.EF_ERR_ARG
        for c in (cAll, cSome, cOne):
            assert gpu_lib.ef_results_destroy(ctx, c) == _lib.EF_OK
        assert gpu_lib.ef_results_destroy(ctx, cAll) == _lib.EF_ERR_ARG
        assert gpu_lib.ef_results_update(ctx, cAll, 0, out.ctypes.data, None) == _lib.EF_ERR_ARG
    finally:
        gpu_lib.ef_destroy(ctx)


@pytest.mark.gpu
def test_solver_result_arrays_after_a_plastic_increment(gpu_lib):
    """NISTGPU.getResultArray and resultCollector after a J2 step: the committed state of the
    accepted increment, as the reference's result views show it, against the oracle's committed
    state (same Newton iteration counts; 1e-6 relative, the displacement tolerance)."""
    from cases import build_gpu_solver, j2_box_spec
    from edelweissfe_gb300 import _lib
    from edelweissfe_gb300.solver import LinSolverOptions, Step
    from oracle.mesh import BoxMesh
    from oracle.nist import NIST
    from oracle.nist import Step as OracleStep
    from test_oracle import _box_model

    props = [210000.0, 0.3, 250.0, 1000.0, 0.0, 0.0]
    mesh = BoxMesh(4, 2, 2, 1.0, 0.5, 0.5)
    model = _box_model(mesh, "C3D8", "vonmises", props, [("gen_left", [0, 1, 2]), ("gen_right", [0])],
                       dir_values={"gen_right": [0.01]})  # fmt: skip
    o = NIST(model)
    o.solveStep(OracleStep(maxInc=0.5, minInc=1e-6, maxIter=25))
    oState = model.groups[0][0].stateRef

    s = build_gpu_solver(j2_box_spec(4, 2, 2, 1.0, 0.5, 0.5, ux=0.01), keFp64=True,
                         linsolver=LinSolverOptions(mixed=False))  # fmt: skip
    s.solveStep(Step(maxInc=0.5, minInc=1e-6, maxIter=25))
    assert [it for _, it in s.iterationHistory] == [it for _, it in o.history]
    nEl = 16
    state = np.zeros((nEl, 8, 13))
    _lib.check(s.lib.ef_get_state(s.ctx, 0, 0, state.ctypes.data), "ef_get_state")
    assert np.min(state[..., 12]) > 0.0  # every point plastic
    for sl in (slice(0, 6), slice(6, 12), slice(12, 13)):
        assert np.max(np.abs(state[..., sl] - oState[..., sl])) <= 1e-6 * np.max(np.abs(oState[..., sl]))
    kap = s.resultCollector(0, None, range(8), "kappa").getCurrentResults()
    assert kap.shape == (nEl, 8, 1) and np.array_equal(kap[..., 0], state[..., 12])
    st = s.resultCollector(0, [2, 7], [3], "Stress").getCurrentResults()
    assert st.shape == (2, 6) and np.array_equal(st, state[[2, 7], 3, 0:6])
    assert np.array_equal(s.getResultArray(0, 5, "strain", 6), state[5, 6, 6:12])
    with pytest.raises(Exception, match="doesn't exist"):
        s.getResultArray(0, 0, "energy", 0)
