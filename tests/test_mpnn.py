"""Learned preconditioner correction: the float64 oracle against finite differences (CPU), the
CUDA forward/backward against the oracle, the tensor-core layer against the CUDA-core one, and
the iteration gain of the network trained on the GPU (GPU)."""

import ctypes

import numpy as np
import pytest

from oracle import mpnn as om
from oracle.mesh import BoxMesh


def _graph(nX=4, nY=3, nZ=3):
    m = BoxMesh(nX, nY, nZ)
    return om.node_pattern(m.elements, m.nNodes)


def test_oracle_edge_weights_are_row_normalised():
    rowPtr, colIdx = _graph()
    case = om.random_case(rowPtr, colIdx, seed=1)
    a = om.edge_weights(rowPtr, colIdx, case["vals"])
    rows = np.repeat(np.arange(len(rowPtr) - 1), np.diff(rowPtr))
    assert np.all(a[colIdx == rows] == 0.0)
    np.testing.assert_allclose(np.bincount(rows, weights=a), 1.0, rtol=1e-12)
    # symmetric block magnitudes: a_mn * tot_m = a_nm * tot_n
    assert np.all(a >= 0.0)


def test_oracle_gradient_matches_finite_differences():
    rowPtr, colIdx = _graph(3, 2, 2)
    c = om.random_case(rowPtr, colIdx, seed=2)
    P = c["P"].astype(np.float64)
    args = (rowPtr, colIdx, c["vals"])
    rest = (c["f"], c["base"], c["e"], c["mask"], 0.7, 0.5)
    _, loss, g = om.loss_and_grad(*args, P, *rest)
    rng = np.random.default_rng(0)
    # a few parameters of every block (input, each layer's Ws / Wn, output) and one random direction
    idx = np.concatenate([rng.integers(lo, hi, 6) for lo, hi in [
        (om.OFF_WIN, om.OFF_L0), (om.OFF_L0, om.OFF_L0 + om.H * om.H), (om.OFF_L0 + om.H * om.H, om.OFF_L0 + om.PER_LAYER),
        (om.OFF_L0 + 2 * om.PER_LAYER, om.OFF_WOUT), (om.OFF_WOUT, om.NPARAM)]])  # fmt: skip
    h = 1e-6
    for i in idx:
        Pp, Pm = P.copy(), P.copy()
        Pp[i] += h
        Pm[i] -= h
        fd = (om.loss_and_grad(*args, Pp, *rest)[1] - om.loss_and_grad(*args, Pm, *rest)[1]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, fd, g[i])
    d = rng.normal(size=P.size)
    fd = (om.loss_and_grad(*args, P + h * d, *rest)[1] - om.loss_and_grad(*args, P - h * d, *rest)[1]) / (2 * h)
    assert abs(fd - g @ d) <= 1e-6 * max(1.0, abs(g @ d))
    assert loss > 0.0


def test_oracle_network_is_positively_homogeneous():
    rowPtr, colIdx = _graph()
    c = om.random_case(rowPtr, colIdx, seed=3)
    a = om.edge_weights(rowPtr, colIdx, c["vals"])
    f, base = c["f"].astype(np.float64), c["base"].astype(np.float64)
    z1, _ = om.forward(rowPtr, colIdx, a, c["P"], f, base, c["mask"], 1.0)
    z2, _ = om.forward(rowPtr, colIdx, a, c["P"], 3.5 * f, 3.5 * base, c["mask"], 1.0)
    np.testing.assert_allclose(z2, 3.5 * z1, rtol=1e-12, atol=1e-12)


def _eval_gpu(lib, rowPtr, colIdx, c, so, scale, with_grad=True):
    nN = len(rowPtr) - 1
    z = np.zeros(3 * nN, np.float32)
    g = np.zeros(om.NPARAM, np.float32)
    loss = ctypes.c_double()
    arrs = dict(r=np.ascontiguousarray(rowPtr, np.int32), c=np.ascontiguousarray(colIdx, np.int32),
                v=np.ascontiguousarray(c["vals"], np.float32), p=np.ascontiguousarray(c["P"], np.float32),
                f=np.ascontiguousarray(c["f"], np.float32), b=np.ascontiguousarray(c["base"], np.float32),
                e=np.ascontiguousarray(c["e"], np.float32), m=np.ascontiguousarray(c["mask"], np.uint8))  # fmt: skip
    st = lib.ef_mpnn_eval(nN, arrs["r"].ctypes.data, arrs["c"].ctypes.data, arrs["v"].ctypes.data,
                          arrs["p"].ctypes.data, arrs["f"].ctypes.data, arrs["b"].ctypes.data, arrs["e"].ctypes.data,
                          arrs["m"].ctypes.data, so, scale, z.ctypes.data, g.ctypes.data if with_grad else None,
                          ctypes.byref(loss), None)  # fmt: skip
    assert st == 0, lib.ef_last_error().decode()
    return z, g, loss.value


@pytest.mark.gpu
@pytest.mark.parametrize("dims", [(4, 3, 3), (12, 7, 5)])
def test_gpu_network_forward_backward_match_oracle(gpu_lib, dims):
    """FP32 CUDA forward/backward against the float64 oracle: z to 1e-5 and every gradient block
    to 1e-4 of its largest entry (FP32 accumulation over the nodes)."""
    rowPtr, colIdx = _graph(*dims)
    c = om.random_case(rowPtr, colIdx, seed=7)
    so, scale = 0.8, 1.0 / (3 * (len(rowPtr) - 1))
    z, g, loss = _eval_gpu(gpu_lib, rowPtr, colIdx, c, so, scale)
    zo, lo, go = om.loss_and_grad(rowPtr, colIdx, c["vals"], c["P"].astype(np.float64), c["f"], c["base"], c["e"],
                                  c["mask"], so, scale)  # fmt: skip
    assert np.max(np.abs(z - zo)) <= 1e-5 * np.max(np.abs(zo))
    assert abs(loss - lo) <= 1e-5 * lo
    blocks = [(om.OFF_WIN, om.OFF_L0)] + [
        (om.OFF_L0 + l * om.PER_LAYER + k * om.H * om.H, om.OFF_L0 + l * om.PER_LAYER + (k + 1) * om.H * om.H)
        for l in range(om.NL) for k in range(2)] + [(om.OFF_WOUT, om.NPARAM)]  # fmt: skip
    for lo_, hi_ in blocks:
        ref = go[lo_:hi_]
        assert np.max(np.abs(g[lo_:hi_] - ref)) <= 1e-4 * np.max(np.abs(ref)), (lo_, hi_)


def _bf16_round(a):
    """Round float32 values to the nearest BF16 (ties to even), returned as float32."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


@pytest.mark.gpu
@pytest.mark.parametrize("nN", [128, 1000])
def test_gpu_dense_layer_tensor_cores_match_cuda_cores(gpu_lib, nN):
    """q = relu(Ws h + Wn agg) on the tensor cores (tcgen05, BF16 operands, FP32 accumulation)
    against the FP32 CUDA-core kernel: within the BF16 rounding of h and agg (1e-2 of max |q|),
    residual output hout = h + q likewise, and no tile gave up waiting."""
    rng = np.random.default_rng(5)
    h = rng.normal(size=(nN, om.H)).astype(np.float32)
    agg = rng.normal(size=(nN, om.H)).astype(np.float32)
    W = _bf16_round(rng.normal(scale=0.1, size=(2, om.H, om.H)).astype(np.float32))
    out = {}
    for tc in (0, 1):
        q = np.zeros((nN, om.H), np.float32)
        ho = np.zeros((nN, om.H), np.float32)
        fl = ctypes.c_int()
        st = gpu_lib.ef_mpnn_dense_eval(tc, nN, h.ctypes.data, agg.ctypes.data, W.ctypes.data, q.ctypes.data,
                                        ho.ctypes.data, ctypes.byref(fl), None)  # fmt: skip
        assert st == 0, gpu_lib.ef_last_error().decode()
        assert fl.value == 0
        out[tc] = (q, ho)
    qr = np.maximum(h.astype(np.float64) @ W[0].T.astype(np.float64) + agg @ W[1].T.astype(np.float64), 0.0)
    assert np.max(np.abs(out[0][0] - qr)) <= 1e-5 * np.max(np.abs(qr))
    assert np.max(np.abs(out[1][0] - out[0][0])) <= 1e-2 * np.max(np.abs(out[0][0]))
    assert np.max(np.abs(out[1][1] - out[0][1])) <= 1e-2 * np.max(np.abs(out[0][1]))


@pytest.mark.gpu
def test_gpu_trained_network_cuts_fgmres_iterations(gpu_lib):
    """The network trained on the GPU (own forward, backward and Adam kernels) on (residual,
    correction) pairs that the plain FGMRES + block-Jacobi solver produces, then used as the
    correction of that preconditioner: at least 40 % fewer FGMRES iterations to 1e-8 on new
    right-hand sides of the same system than the same solver without it (measured on GB300:
    about 2.7x fewer), and a lower training loss at the end than at the start."""
    import torch
    from cases import build_gpu_solver, j2_box_spec
    from edelweissfe_gb300 import _lib
    from edelweissfe_gb300.solver import TimeStep

    s = build_gpu_solver(j2_box_spec(16, 8, 8, 1.6, 0.8, 0.8))
    _lib.check(s.lib.ef_set_dirichlet(s.ctx, s.dirIdxHost.ctypes.data, s.dirIdxHost.size), "dir")
    dU = torch.zeros(s.nDof, dtype=torch.float64, device="cuda")
    P, F = s._vec(), s._vec()
    s.computeElements(dU, dU, P, F, TimeStep(1, 0.1, 0.1, 0.1, 0.1, 0.1))
    s.assembleStiffnessCSR()
    s.linsolver.method = "fgmres"
    s.linsolver.rtol = 1e-8
    s.linsolver.innerRtol = 1e-6
    s.linsolver.restart = 40
    s.setFgmresPreconditioner("jacobi")

    def rhs(seed):
        b = np.random.default_rng(seed).normal(size=s.nDof)
        b[s.dirIdxHost] = 0.0
        return torch.as_tensor(b, device="cuda")

    def iterations(seeds):
        out = []
        for k in seeds:
            s.linearSolve(rhs(k))
            assert s.lastSolveInfo.relResidual <= 1e-8
            out.append(s.lastSolveInfo.iterations)
        return np.array(out)

    off = iterations([100, 101, 102])
    s.initLearnedPreconditioner(seed=0, maxSamples=48)
    s.collectTrainingPairs(every=5, maxPerSolve=8, kind="iterates")
    iterations(range(6))  # the plain solver's own iterates give the pairs
    s.collectTrainingPairs(every=0)
    assert s.numTrainingPairs() == 48
    first, last = s.trainLearnedPreconditioner(epochs=100, lr=1e-3, norm="energy")
    assert last < first
    s.enableLearnedPreconditioner(True)
    on = iterations([100, 101, 102])
    s.enableLearnedPreconditioner(False)
    assert on.mean() <= 0.6 * off.mean(), (off, on)


@pytest.mark.gpu
def test_gpu_network_trained_across_seeds_cuts_iterations_on_unseen_seeds(gpu_lib):
    """The seeded J2 family (per seed sigma_y ~ U[150,350], H ~ U[200,2000], nu ~ U[0.2,0.4]):
    pairs from the Newton iterations of four seeds' load histories (one context, one box per
    seed), GPU training, then the load history of two unseen seeds with FGMRES + block Jacobi
    with and without the trained network: the same Newton iteration counts and displacements
    (1e-6), and fewer Krylov iterations with the network."""
    from edelweissfe_gb300.learned import evaluate_on_seeds, train_across_seeds

    dims = (12, 6, 6)
    params, scales, rec = train_across_seeds([0, 1, 2, 3], dims, increments=14, base="jacobi", epochs=100)
    assert rec["pairs"] > 16 and rec["loss_last"] < rec["loss_first"], rec
    ev = evaluate_on_seeds([4, 5], dims, increments=14, params=params, scales=scales, base="jacobi")
    assert ev["newton_on"] == ev["newton_off"], ev
    assert ev["max_rel_dU"] <= 1e-6, ev
    assert ev["krylov_on"] <= 0.8 * ev["krylov_off"], ev
