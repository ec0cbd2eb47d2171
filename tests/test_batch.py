"""Batches of independent J2 cubes (uneven sizes, random material per cube, 1 % axial strain in
10 increments): the batched GPU driver against the oracle NIST run cube by cube (base clamped,
non-homogeneous), and the size-independent homogeneous solution of uniaxial strain (laterally
confined) at the full 1024-cube size."""

import numpy as np
import pytest

from edelweissfe_gb300.batch import cube_batch_spec, cube_mesh
from oracle.element import SmallStrainElements
from oracle.nist import NIST, Model, Step
from oracle.system import element_dofs


def oracle_cube(n, props, h=0.1, strain=0.01, nInc=10, bc="clamped"):
    m, dofs, vals = cube_mesh(n, h, strain, bc)
    els = SmallStrainElements("C3D8", m["coords"][m["elements"]], "vonmises", props)
    model = Model(3 * m["coords"].shape[0], [(els, element_dofs(m["elements"]))], [(dofs, vals)])
    s = NIST(model)
    U, _ = s.solveStep(Step(maxInc=1.0 / nInc, minInc=1e-6, maxIter=25))
    return U, [it for _, it in s.history], m


def test_cube_batch_spec_is_seeded_and_in_range():
    a = cube_batch_spec(1024, 7)
    b = cube_batch_spec(1024, 7)
    assert a == b
    n = np.array([p["n"] for p in a])
    props = np.array([p["props"] for p in a])
    assert n.min() >= 4 and n.max() <= 16 and len(set(n.tolist())) == 13
    assert (150 <= props[:, 2]).all() and (props[:, 2] <= 350).all()
    assert (200 <= props[:, 3]).all() and (props[:, 3] <= 2000).all()
    assert (0.2 <= props[:, 1]).all() and (props[:, 1] <= 0.4).all()


def test_oracle_uniaxial_strain_cube_is_homogeneous():
    """The exact solution of uniaxial strain is u = (0, 0, eps z); the oracle reproduces it."""
    U, iters, m = oracle_cube(3, [210000.0, 0.3, 250.0, 1000.0, 0.0, 0.0], bc="confined")
    u = U.reshape(-1, 3)
    z = m["coords"][:, 2]
    assert np.max(np.abs(u[:, 2] - 0.01 * z)) <= 1e-9 * 0.01 * z.max()
    assert np.max(np.abs(u[:, :2])) <= 1e-12
    assert len(iters) == 11 and iters[0] == 1  # zero first increment, then 10 of 0.1


@pytest.mark.gpu
def test_gpu_batch_matches_oracle_per_cube(gpu_lib):
    """24 cubes of 4..6 elements per edge with random J2 properties, base clamped and top pulled:
    per increment the same Newton iteration counts as the oracle run cube by cube, displacements
    within 1e-6."""
    from edelweissfe_gb300.batch import BatchNISTGPU

    spec = cube_batch_spec(24, 3, nMin=4, nMax=6)
    b = BatchNISTGPU(spec)
    U = b.solveStepBatch(Step(maxInc=0.1, minInc=1e-6, maxIter=25)).cpu().numpy()
    hist = np.array([it for _, it in b.problemHistory])  # [increments, problems]
    for p in range(0, 24, 4):
        Uo, iters, _ = oracle_cube(spec[p]["n"], spec[p]["props"])
        assert list(hist[:, p]) == iters, (p, hist[:, p], iters)
        Ug = U[b.problem_dofs(p)]
        assert np.max(np.abs(Ug - Uo)) <= 1e-6 * np.max(np.abs(Uo))


@pytest.mark.gpu
def test_gpu_batch_1024_cubes_uniaxial_strain_is_homogeneous(gpu_lib):
    """The full batch (1024 cubes, n ~ U{4..16}): every cube converges in every increment and
    ends at the exact homogeneous field u = (0, 0, 0.01 z) within 1e-6."""
    from edelweissfe_gb300.batch import BatchNISTGPU

    spec = cube_batch_spec(1024, 0)
    b = BatchNISTGPU(spec, bc="confined")
    U = b.solveStepBatch(Step(maxInc=0.1, minInc=1e-6, maxIter=25)).cpu().numpy().reshape(-1, 3)
    z = b.model.coords[:, 2]
    assert np.max(np.abs(U[:, 2] - 0.01 * z)) <= 1e-6 * 0.01 * z.max()
    assert np.max(np.abs(U[:, :2])) <= 1e-6 * 0.01 * z.max()
    assert len(b.problemHistory) == 11
    assert b.tile in range(len(b.tile_shapes()))
