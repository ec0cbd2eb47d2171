"""Model specifications shared by the oracle tests and the GPU parity tests.

The golden cases restate the inputs of the reference's testfiles/*/test.inp
(boxGen meshes, linear elastic material, Dirichlet sets, node forces, body
forces) and of the fixtures produced by tests/golden/make_golden.py.
"""

import numpy as np

UREF_CASES = {
    # name: (nX, nY, nZ, lX, lY, lZ, elType, E, nu, dirichlet sets, node forces, body force)
    "TensionBarHexa8": (4, 4, 30, 5, 5, 500, "C3D8", 1.8e4, 0.22, ["gen_front"], [("gen_back", [0, 0, -4.0])], None),
    "SimpleBeamHexa8": (200, 2, 2, 2500, 50, 50, "C3D8", 210000, 0.22, ["gen_leftBack", "gen_rightBack"], [("gen_front", [0, 0, -4.16])], None),
    "WallShearHexa8": (20, 20, 2, 1000, 1000, 5, "C3D8", 2.1e4, 0.22, ["gen_bottom"], [("gen_top", [1.0, 0, 0])], [0, -0.000077, 0]),
    "WallShearHexa20": (10, 10, 1, 1000, 1000, 5, "C3D20", 2.1e4, 0.22, ["gen_bottom"], [("gen_top", [1.18868, 0, 0])], [0, -0.000077, 0]),
}  # fmt: skip

CANTILEVER_NODEFORCES = (
    [("gen_right", [0, 0, -0.25])]
    + [(s, [0, 0, 0.125]) for s in ["gen_rightFront", "gen_rightBack", "gen_bottomRight", "gen_topRight"]]
    + [(s, [0, 0, -0.0625]) for s in ["gen_bottomRightFront", "gen_bottomRightBack", "gen_topRightFront", "gen_topRightBack"]]
)

J2_PROPS = [210000.0, 0.3, 250.0, 1000.0, 0.0, 0.0]


def j2_box_spec(nX, nY, nZ, lX, lY, lZ, elType="C3D8", ux=None, props=J2_PROPS):
    """x = 0 face clamped, x = lX face pulled by ux (default: 0.2 % strain)."""
    return dict(
        nX=nX, nY=nY, nZ=nZ, lX=lX, lY=lY, lZ=lZ, elType=elType, material="vonmises", props=list(props),
        dirichlet=[("gen_left", {0: 0.0, 1: 0.0, 2: 0.0}), ("gen_right", {0: 0.002 * lX if ux is None else ux})],
        nodeforces=[], bodyforce=None,
    )  # fmt: skip


def tl_box_spec(nX, nY, nZ, lX, lY, lZ, elType, ux, props=(80.0, 200.0)):
    """Total-Lagrange NeoHookeWa box: x = 0 face clamped, x = lX face displaced by ux."""
    return dict(
        nX=nX, nY=nY, nZ=nZ, lX=lX, lY=lY, lZ=lZ, elType=elType, material="neohookewa", props=list(props),
        dirichlet=[("gen_left", {0: 0.0, 1: 0.0, 2: 0.0}), ("gen_right", {0: ux})], nodeforces=[], bodyforce=None,
    )  # fmt: skip


def uref_spec(name):
    nX, nY, nZ, lX, lY, lZ, elType, E, nu, dsets, nf, bf = UREF_CASES[name]
    return dict(
        nX=nX, nY=nY, nZ=nZ, lX=lX, lY=lY, lZ=lZ, elType=elType, material="linearelastic", props=[E, nu],
        dirichlet=[(s, {0: 0.0, 1: 0.0, 2: 0.0}) for s in dsets], nodeforces=nf,
        bodyforce=None if bf is None else np.array(bf, float),
    )  # fmt: skip


def cantilever_spec():
    return dict(
        nX=20, nY=4, nZ=4, lX=10.0, lY=2.0, lZ=2.0, elType="C3D8", material="linearelastic", props=[210000.0, 0.3],
        dirichlet=[("gen_left", {0: 0.0, 1: 0.0, 2: 0.0})], nodeforces=CANTILEVER_NODEFORCES, bodyforce=None,
    )  # fmt: skip


def build_gpu_solver(spec, **kw):
    from edelweissfe_gb300.mesh import box_mesh
    from edelweissfe_gb300.model import BodyForce, DirichletBC, ElementGroup, Model, NodeForces
    from edelweissfe_gb300.solver import NISTGPU

    m = box_mesh(spec["nX"], spec["nY"], spec["nZ"], spec["lX"], spec["lY"], spec["lZ"],
                 nNodesPerElement=20 if "20" in spec["elType"] else 8)  # fmt: skip
    model = Model(m["coords"], [ElementGroup(spec["elType"], m["elements"], spec["material"], np.array(spec["props"]))])
    dirs = [DirichletBC(m["nodeSets"][s], comps) for s, comps in spec["dirichlet"]]
    nfs = [NodeForces(m["nodeSets"][s], v) for s, v in spec["nodeforces"]]
    bfs = [BodyForce(0, spec["bodyforce"])] if spec.get("bodyforce") is not None else []
    return NISTGPU(model, dirs, nfs, bfs, **kw)


def tied_tl_spec(nXq, nXl, nY, nZ, h=0.1, compression=0.15, props=(80.0, 200.0)):
    """Hex20 (C3D20TL) | hex8 (C3D8TL) NeoHookeWa box with the tied interface, x = 0 face clamped,
    x = L face displaced by -compression * L."""
    from edelweissfe_gb300.mesh import tied_box_mesh

    m = tied_box_mesh(nXq, nXl, nY, nZ, nXq * h, nXl * h, nY * h, nZ * h)
    return dict(mesh=m, props=list(props), ux=-compression * (nXq + nXl) * h)


def build_gpu_tied(spec, **kw):
    from edelweissfe_gb300.model import DirichletBC, ElementGroup, Model
    from edelweissfe_gb300.solver import NISTGPU

    m = spec["mesh"]
    p = np.array(spec["props"])
    model = Model(m["coords"], [ElementGroup("C3D20TL", m["elements20"], "neohookewa", p),
                                ElementGroup("C3D8TL", m["elements8"], "neohookewa", p)], ties=m["ties"])  # fmt: skip
    dirs = [DirichletBC(m["nodeSets"]["gen_left"], {0: 0.0, 1: 0.0, 2: 0.0}),
            DirichletBC(m["nodeSets"]["gen_right"], {0: spec["ux"]})]  # fmt: skip
    return NISTGPU(model, dirs, **kw)


def oracle_tied(spec):
    from oracle.element import TLElements
    from oracle.nist import Model as OModel
    from oracle.system import element_dofs

    m = spec["mesh"]
    c = m["coords"]
    gq = TLElements("C3D20TL", c[m["elements20"]], "neohookewa", spec["props"])
    gl = TLElements("C3D8TL", c[m["elements8"]], "neohookewa", spec["props"])
    left, right = m["nodeSets"]["gen_left"], m["nodeSets"]["gen_right"]
    dirs = [((3 * left[:, None] + np.arange(3)).ravel(), np.zeros(3 * left.size)),
            (3 * right, np.full(right.size, spec["ux"]))]  # fmt: skip
    return OModel(3 * c.shape[0], [(gq, element_dofs(m["elements20"])), (gl, element_dofs(m["elements8"]))], dirs,
                  ties=m["ties"])  # fmt: skip
