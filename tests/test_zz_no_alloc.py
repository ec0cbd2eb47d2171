"""The allocation-free PCG entry point (ef_pcg_solve_noalloc) against the context solver.

Callers that cannot allocate device memory at solve time (a host framework that reserved the
device memory for its own pool, or a latency-critical loop that must not take the device-wide
synchronisation of cudaMalloc/cudaFree) use ef_pcg_solve_noalloc, whose work vectors live in a
fixed 8 MiB device array.  This test feeds it the same FP64 system as ef_solve's all-FP64 PCG and
checks the two solutions agree, on two calls in a row (the shared array keeps the previous call's
contents, which must not leak into the next result).
"""

import ctypes

import numpy as np
import pytest
import torch

from cases import build_gpu_solver, j2_box_spec

pytestmark = pytest.mark.gpu


def _bsr_from_csr(indptr, indices, data, nNodes):
    """3x3 block rows of a scalar CSR whose rows/columns come in node triplets."""
    rowPtr = [0]
    cols, vals = [], []
    for m in range(nNodes):
        blocks = {}
        for i in range(3):
            r = 3 * m + i
            for k in range(indptr[r], indptr[r + 1]):
                c = indices[k]
                blk = blocks.setdefault(c // 3, np.zeros((3, 3)))
                blk[i, c % 3] = data[k]
        for n in sorted(blocks):
            cols.append(n)
            vals.append(blocks[n].ravel())
        rowPtr.append(len(cols))
    return np.array(rowPtr, np.int32), np.array(cols, np.int32), np.array(vals, float)


def test_noalloc_pcg_matches_context_solver_twice(gpu_lib):
    from edelweissfe_gb300 import _lib
    from edelweissfe_gb300.solver import LinSolverOptions, TimeStep

    s = build_gpu_solver(j2_box_spec(8, 4, 4, 0.8, 0.4, 0.4), keFp64=True, scalarCSR=True,
                         linsolver=LinSolverOptions(mixed=False, rtol=1e-9))  # fmt: skip
    _lib.check(s.lib.ef_set_dirichlet(s.ctx, s.dirIdxHost.ctypes.data, s.dirIdxHost.size), "dir")
    ts = TimeStep(1, 0.1, 0.1, 0.1, 0.1, 0.1)
    dU = torch.zeros(s.nDof, dtype=torch.float64, device="cuda")
    P, F = s._vec(), s._vec()
    s.computeElements(dU, dU, P, F, ts)
    s.assembleStiffnessCSR()
    nDof = s.nDof
    nNodes = nDof // 3
    assert nNodes <= gpu_lib.ef_pcg_noalloc_max_nodes()
    # the same FP64 system as a BSR built on the host from the reference-layout CSR
    indptr = np.zeros(nDof + 1, np.int32)
    indices = np.zeros(s.info.nnz, np.int32)
    _lib.check(gpu_lib.ef_csr_pattern(s.ctx, indptr.ctypes.data, indices.ctypes.data), "pattern")
    data = torch.zeros(s.info.nnz, dtype=torch.float64, device="cuda")
    _lib.check(gpu_lib.ef_update_csr(s.ctx, None, data.data_ptr(), None), "update")
    rowPtr, colIdx, vals = _bsr_from_csr(indptr, indices, data.cpu().numpy(), nNodes)
    mask = np.zeros(nDof, np.uint8)
    mask[s.dirIdxHost] = 1
    binv = np.zeros((nNodes, 9))
    for m in range(nNodes):
        k = rowPtr[m] + np.nonzero(colIdx[rowPtr[m]:rowPtr[m + 1]] == m)[0][0]
        D = vals[k].reshape(3, 3).copy()
        for i in range(3):
            if mask[3 * m + i]:
                D[i, :] = 0.0
                D[:, i] = 0.0
                D[i, i] = 1.0
        binv[m] = np.linalg.inv(D).ravel()
    dev = torch.device("cuda")
    t = {k: torch.as_tensor(v, device=dev) for k, v in dict(rowPtr=rowPtr, colIdx=colIdx, vals=vals.ravel(),
                                                              binv=binv.ravel(), mask=mask).items()}  # fmt: skip
    rng = np.random.default_rng(7)
    for call in range(2):
        b = rng.normal(size=nDof)
        b[s.dirIdxHost] = 0.0
        bt = torch.as_tensor(b, device=dev)
        x_ref = s.linearSolve(bt)
        x = torch.full((nDof,), float("nan"), dtype=torch.float64, device=dev)
        info = _lib.EfSolveInfo()
        st = gpu_lib.ef_pcg_solve_noalloc(nNodes, t["rowPtr"].data_ptr(), t["colIdx"].data_ptr(), t["vals"].data_ptr(),
                                          t["binv"].data_ptr(), t["mask"].data_ptr(), bt.data_ptr(), x.data_ptr(),
                                          20000, 1e-9, ctypes.byref(info), None)  # fmt: skip
        assert st == _lib.EF_OK, gpu_lib.ef_last_error()
        assert info.iterations > 0
        # both are block-Jacobi PCG runs on the same FP64 system to 1e-9: agree well inside the
        # 1e-6 relative displacement tolerance of the parity tests
        xr = x_ref.cpu().numpy()
        assert np.max(np.abs(x.cpu().numpy() - xr)) <= 1e-6 * np.max(np.abs(xr))
    # sizes beyond the fixed capacity are rejected without touching the device
    too_big = gpu_lib.ef_pcg_noalloc_max_nodes() + 1
    st = gpu_lib.ef_pcg_solve_noalloc(too_big, t["rowPtr"].data_ptr(), t["colIdx"].data_ptr(), t["vals"].data_ptr(),
                                      t["binv"].data_ptr(), t["mask"].data_ptr(), bt.data_ptr(), x.data_ptr(),
                                      10, 1e-9, ctypes.byref(info), None)  # fmt: skip
    assert st == _lib.EF_ERR_ARG and b"capacity" in gpu_lib.ef_last_error()
