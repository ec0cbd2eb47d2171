"""The oracle pinned against the reference: its own golden U.ref files and fixtures produced by running it."""

import numpy as np
import pytest

from conftest import golden
from oracle.element import SmallStrainElements, TLElements, make_elements
from oracle.mesh import BoxMesh
from oracle.nist import NIST, IndirectControl, Model, NISTArcLength, Step
from oracle.system import csr_slot_map, csr_update, element_dofs, vij_pattern


def _box_model(mesh, elType, material, props, dir_sets, nodeforces=(), bodyforce=None, dir_values=None):
    els = make_elements(elType, mesh.coords[mesh.elements], material, props)
    ed = element_dofs(mesh.elements)
    dirs = []
    for s, comps in dir_sets:
        nodes = mesh.nodeSets[s]
        d = (3 * nodes[:, None] + np.asarray(comps)[None]).ravel()
        vals = np.tile(np.asarray(dir_values[s] if dir_values and s in dir_values else np.zeros(len(comps))), nodes.size)
        dirs.append((d, vals))
    nfs = []
    for s, comp in nodeforces:
        nodes = mesh.nodeSets[s]
        nfs.append(((3 * nodes[:, None] + np.arange(3)[None]).ravel(), np.tile(comp, nodes.size)))
    return Model(3 * mesh.nNodes, [(els, ed)], dirs, nfs, [(0, bodyforce)] if bodyforce is not None else [])


UREF_CASES = {
    # name: (nX, nY, nZ, lX, lY, lZ, elType, E, nu, dirichlet sets, node forces, body force)
    "TensionBarHexa8": (4, 4, 30, 5, 5, 500, "C3D8", 1.8e4, 0.22, ["gen_front"], [("gen_back", [0, 0, -4.0])], None),
    "SimpleBeamHexa8": (200, 2, 2, 2500, 50, 50, "C3D8", 210000, 0.22, ["gen_leftBack", "gen_rightBack"], [("gen_front", [0, 0, -4.16])], None),
    "WallShearHexa8": (20, 20, 2, 1000, 1000, 5, "C3D8", 2.1e4, 0.22, ["gen_bottom"], [("gen_top", [1.0, 0, 0])], [0, -0.000077, 0]),
    "WallShearHexa20": (10, 10, 1, 1000, 1000, 5, "C3D20", 2.1e4, 0.22, ["gen_bottom"], [("gen_top", [1.18868, 0, 0])], [0, -0.000077, 0]),
}  # fmt: skip


@pytest.mark.parametrize("name", sorted(UREF_CASES))
def test_oracle_matches_reference_uref(name):
    nX, nY, nZ, lX, lY, lZ, elType, E, nu, dsets, nf, bf = UREF_CASES[name]
    mesh = BoxMesh(nX, nY, nZ, lX, lY, lZ, nNodesPerElement=20 if "20" in elType else 8)
    model = _box_model(mesh, elType, "linearelastic", [E, nu], [(s, [0, 1, 2]) for s in dsets], nf, None if bf is None else np.array(bf, float))
    s = NIST(model)
    U, _ = s.solveStep(Step(maxInc=1.0, minInc=1e-9, maxIter=25, extrapolation="off"))
    ref = golden(f"uref_{name}.npz")["U"]
    # the reference runner's own tolerance is 1e-6 (_cli/_run_tests_edelweissfe.py:105)
    assert np.max(np.abs(U - ref)) < 1e-12


ELEM_FIXTURES = [
    ("C3D8", "linearelastic"),
    ("C3D8", "vonmises"),
    ("C3D8", "vonmisesexp"),
    ("C3D20", "linearelastic"),
    ("C3D20", "vonmises"),
    ("C3D8R", "vonmises"),
    ("C3D8E", "vonmises"),
    ("C3D20R", "vonmises"),
]


@pytest.mark.parametrize("elType,mat", ELEM_FIXTURES)
def test_oracle_element_matches_reference(elType, mat):
    g = golden(f"elem_{elType}_{mat}.npz")
    els = SmallStrainElements(elType, g["coords"], "vonmises" if mat.startswith("vonmises") else mat, g["props"])
    els.stateRef[:] = g["state0"]
    Ke, Pe = els.compute_yourself(g["U"], g["dU"])
    n = els.nDof
    Kref = g["Kvij"].reshape(-1, n, n)
    assert np.max(np.abs(Ke - Kref)) <= 1e-12 * np.max(np.abs(Kref))
    assert np.max(np.abs(Pe - g["Pe"])) <= 1e-12 * np.max(np.abs(g["Pe"]))
    s1 = g["state1"]
    scale = np.max(np.abs(s1), axis=(0, 1)) + 1e-30
    assert np.max(np.abs(els.stateTemp - s1) / scale) < 1e-12


def test_oracle_csr_matches_reference_bitwise():
    g = golden("csr_small.npz")
    I, J = vij_pattern(element_dofs(g["elements"]))
    assert np.array_equal(I, g["I"]) and np.array_equal(J, g["J"])
    indptr, indices, x = csr_slot_map(I, J, int(g["nDof"]))
    assert np.array_equal(indptr, g["indptr"]) and np.array_equal(indices, g["indices"])
    data = csr_update(g["V"], x, len(indices))
    assert np.array_equal(data.view(np.uint64), g["data"].view(np.uint64))


def test_oracle_nist_cantilever_matches_reference():
    g = golden("nist_cantilever_20x4x4.npz")
    mesh = BoxMesh(20, 4, 4, 10, 2, 2)
    nf = [("gen_right", [0, 0, -0.25])]
    nf += [(s, [0, 0, 0.125]) for s in ["gen_rightFront", "gen_rightBack", "gen_bottomRight", "gen_topRight"]]
    nf += [(s, [0, 0, -0.0625]) for s in ["gen_bottomRightFront", "gen_bottomRightBack", "gen_topRightFront", "gen_topRightBack"]]
    model = _box_model(mesh, "C3D8", "linearelastic", [210000.0, 0.3], [("gen_left", [0, 1, 2])], nf)
    s = NIST(model)
    U, _ = s.solveStep(Step(maxInc=1.0, minInc=1e-6, maxIter=25))
    assert np.max(np.abs(U - g["U"])) < 1e-12
    assert [it for _, it in s.history] == list(g["iters"])
    assert abs(U.min() - (-4.65324e-3)) < 1e-8


def arclength_case(g):
    """The J2 bar of the arc-length fixture: x = 0 clamped, reference node forces on the x = lX face,
    indirect control of the x displacement of the nodes closest to (x1, 0, 0) and (x2, 0, 0)."""
    mesh = BoxMesh(int(g["nX"]), int(g["nY"]), int(g["nZ"]), float(g["lX"]), float(g["lY"]), float(g["lZ"]))
    n1, n2 = (int(np.argmin(np.linalg.norm(mesh.coords - [float(g[k]), 0.0, 0.0], axis=1))) for k in ("x1", "x2"))
    idcs = np.concatenate([3 * n1 + np.arange(3), 3 * n2 + np.arange(3)])
    return mesh, idcs, np.array([-1.0, 0.0, 0.0, 1.0, 0.0, 0.0])


def test_oracle_arclength_indirect_control_matches_reference():
    """solvers/nonlinearimplicitstaticparallelarclength.py with stepactions/indirectcontrol.py: the
    reference's displacements, Newton iteration counts and load factors."""
    g = golden("nist_arclength_j2_10x2x2.npz")
    mesh, idcs, c = arclength_case(g)
    model = _box_model(mesh, "C3D8", "vonmises", [210000.0, 0.3, 250.0, 1000.0, 0.0, 0.0], [("gen_left", [0, 1, 2])],
                       nodeforces=[("gen_right", [float(g["f"]), 0.0, 0.0])])  # fmt: skip
    s = NISTArcLength(model, IndirectControl(idcs, c, float(g["L"])))
    U, _ = s.solveStep(Step(startInc=float(g["maxInc"]), maxInc=float(g["maxInc"]), minInc=1e-6, maxIter=25))
    assert [it for _, it in s.history] == list(g["iters"])
    assert np.max(np.abs(np.array(s.lambdaHistory) - g["Lambda"])) <= 1e-12 * np.max(g["Lambda"])
    assert np.max(np.abs(U - g["U"])) <= 1e-10 * np.max(np.abs(g["U"]))
    # the control: c . U over the controlled DOFs reaches L at the end of the step
    assert abs(c.dot(U[idcs]) - float(g["L"])) <= 1e-12


@pytest.mark.parametrize("case", ["j2_box_10x4x4", "j2_box_6x3x3_c3d20", "j2_box_4x2x2_c3d20r", "j2_box_8x3x3_c3d8e"])
def test_oracle_nist_j2_matches_reference(case):
    g = golden(f"nist_{case}.npz")
    elType = str(g["elType"])
    mesh = BoxMesh(int(g["nX"]), int(g["nY"]), int(g["nZ"]), float(g["lX"]), float(g["lY"]), float(g["lZ"]), nNodesPerElement=20 if "20" in elType else 8)
    model = _box_model(
        mesh, elType, "vonmises", [210000.0, 0.3, 250.0, 1000.0, 0.0, 0.0],
        [("gen_left", [0, 1, 2]), ("gen_right", [0])], dir_values={"gen_right": [float(g["ux"])]},
    )  # fmt: skip
    s = NIST(model)
    U, _ = s.solveStep(Step(maxInc=float(g["maxInc"]), minInc=1e-6, maxIter=25))
    assert [it for _, it in s.history] == list(g["iters"])
    assert np.max(np.abs(U - g["U"])) <= 1e-10 * np.max(np.abs(g["U"]))


@pytest.mark.parametrize("elType", ["C3D8TL", "C3D20TL", "C3D8RTL", "C3D8ETL", "C3D20RTL"])
def test_oracle_tl_element_matches_reference(elType):
    g = golden(f"elem_{elType}_neohookewa.npz")
    els = TLElements(elType, g["coords"], "neohookewa", g["props"])
    els.stateRef[:] = g["state0"]
    Ke, Pe = els.compute_yourself(g["U"], g["dU"])
    n = els.nDof
    Kref = g["Kvij"].reshape(-1, n, n)
    assert np.max(np.abs(Ke - Kref)) <= 1e-12 * np.max(np.abs(Kref))
    assert np.max(np.abs(Pe - g["Pe"])) <= 1e-12 * np.max(np.abs(g["Pe"]))
    s1 = g["state1"]
    scale = np.max(np.abs(s1), axis=(0, 1)) + 1e-30
    assert np.max(np.abs(els.stateTemp - s1) / scale) < 1e-12


@pytest.mark.parametrize("case", ["tl_box_6x3x3_c3d8tl", "tl_box_3x2x2_c3d20tl", "tl_box_3x2x2_c3d20rtl",
                                  "tl_box_4x2x2_c3d8etl"])
def test_oracle_nist_tl_matches_reference(case):
    g = golden(f"nist_{case}.npz")
    elType = str(g["elType"])
    mesh = BoxMesh(int(g["nX"]), int(g["nY"]), int(g["nZ"]), float(g["lX"]), float(g["lY"]), float(g["lZ"]),
                   nNodesPerElement=20 if "20" in elType else 8)  # fmt: skip
    model = _box_model(mesh, elType, "neohookewa", [80.0, 200.0], [("gen_left", [0, 1, 2]), ("gen_right", [0])],
                       dir_values={"gen_right": [float(g["ux"])]})  # fmt: skip
    s = NIST(model)
    U, _ = s.solveStep(Step(maxInc=float(g["maxInc"]), minInc=1e-6, maxIter=25))
    assert [it for _, it in s.history] == list(g["iters"])
    assert np.max(np.abs(U - g["U"])) <= 1e-10 * np.max(np.abs(g["U"]))


def _tied_model(m, matQ, matL, propsQ, propsL, elQ, elL, dirs):
    from oracle.element import make_elements

    c = m["coords"]
    gq = make_elements(elQ, c[m["elements20"]], matQ, propsQ)
    gl = make_elements(elL, c[m["elements8"]], matL, propsL)
    return Model(3 * c.shape[0], [(gq, element_dofs(m["elements20"])), (gl, element_dofs(m["elements8"]))], dirs,
                 ties=m["ties"])  # fmt: skip


def test_oracle_tied_interface_passes_the_patch_test():
    """Hex20 | hex8 box with the tied interface under uniaxial stress (symmetry planes, end
    displacement): the linear exact field u = eps (x, -nu y, -nu z) is reproduced."""
    from edelweissfe_gb300.mesh import tied_box_mesh

    m = tied_box_mesh(2, 3, 2, 2, 0.4, 0.6, 0.3, 0.3)
    s = m["nodeSets"]
    c = m["coords"]
    eps, nu = 1e-3, 0.3
    y0 = np.flatnonzero(np.abs(c[:, 1]) < 1e-12)
    z0 = np.flatnonzero(np.abs(c[:, 2]) < 1e-12)
    dirs = [(3 * s["gen_left"], np.zeros(s["gen_left"].size)), (3 * s["gen_right"], np.full(s["gen_right"].size, eps)),
            (3 * y0 + 1, np.zeros(y0.size)), (3 * z0 + 2, np.zeros(z0.size))]  # fmt: skip
    model = _tied_model(m, "linearelastic", "linearelastic", [210000.0, nu], [210000.0, nu], "C3D20", "C3D8", dirs)
    U, _ = NIST(model).solveStep(Step(maxInc=1.0, minInc=1e-6, maxIter=25, extrapolation="off"))
    u = U.reshape(-1, 3)
    exact = eps / 1.0 * np.stack([c[:, 0], -nu * c[:, 1], -nu * c[:, 2]], axis=1)
    assert np.max(np.abs(u - exact)) <= 1e-9 * eps
