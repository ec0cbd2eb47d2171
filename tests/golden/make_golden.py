"""Generate the golden fixtures of this directory from the EdelweissFE reference.

Run in a container where the reference sources are available (default
``/root/reference``; override with ``EF_REFERENCE``):

    python tests/golden/make_golden.py        # all fixtures
    python tests/golden/make_golden.py tl     # only the total-Lagrange ones
    python tests/golden/make_golden.py arclength   # only the arc-length one
    python tests/golden/make_golden.py variants    # only the other integration rules
    python tests/golden/make_golden.py headline    # only the scaled benchmark box history

What it does:

1. copies the reference's own golden solutions ``testfiles/<name>/U.ref`` of the
   boxGen-built small-strain tests into ``uref_<name>.npz``;
2. copies the reference package to a scratch directory, builds its Cython
   modules there (``numerics/csrgenerator.pyx``,
   ``solvers/nonlinearimplicitstaticparallelmk2.pyx``,
   ``utils/elementresultcollector.pyx``), stubs the optional packages that are
   absent here (h5py, matplotlib, prettytable, the Marmot wrappers, MKL PARDISO
   -> SciPy SuperLU, which is the reference's own fallback in
   ``config/linsolve.py``) and imports it;
3. runs the reference's own objects on seeded inputs and stores
   * ``elem_<type>_<material>.npz``: per-element Ke, Pe and trial state from
     ``DisplacementElement.computeYourself`` (distorted geometry, random prior
     state, random increments),
   * ``csr_small.npz``: the CSR pattern and a scatter result of ``CSRGenerator``,
   * ``nist_<case>.npz``: final displacements and Newton iteration counts of
     the reference NIST driver on 3D J2 / elastic boxes,
   * ``nist_arclength_j2_10x2x2.npz``: the same of the reference arc-length
     driver with indirect displacement control, plus its load factors,
   * ``nist_j2_box_25x10x10_history.npz``: the benchmark's J2 box at a quarter
     of its edge counts, displacements after every increment and the final
     stresses.

Nothing here is needed at test time; the tests only read the ``.npz`` files.
"""

import os
import shutil
import subprocess
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("EF_REFERENCE", "/root/reference")

UREF_TESTS = ["TensionBarHexa8", "SimpleBeamHexa8", "WallShearHexa8", "WallShearHexa20"]


def copy_uref():
    for name in UREF_TESTS:
        U = np.loadtxt(os.path.join(REF, "testfiles", name, "U.ref"))
        np.savez_compressed(os.path.join(HERE, f"uref_{name}.npz"), U=U)


CYTHON_MODULES = ["numerics/csrgenerator", "solvers/nonlinearimplicitstaticparallelmk2", "utils/elementresultcollector"]


def prepare_reference(scratch, modules=None):
    """Copies the reference package into `scratch`, builds its Cython modules there (all of
    CYTHON_MODULES, or `modules`), installs the stubs and puts it first on sys.path."""
    shutil.copytree(os.path.join(REF, "edelweissfe"), os.path.join(scratch, "edelweissfe"))
    build = os.path.join(scratch, "build_ext.py")
    with open(build, "w") as f:
        f.write(
            "from setuptools import setup, Extension\n"
            "from Cython.Build import cythonize\n"
            "import numpy as np\n"
            f"mods = {list(modules or CYTHON_MODULES)!r}\n"
            "exts = [Extension('edelweissfe.' + m.replace('/', '.'), ['edelweissfe/' + m + '.pyx'],\n"
            "        include_dirs=[np.get_include()], language='c++', extra_compile_args=['-fopenmp'], extra_link_args=['-fopenmp'])\n"
            "        for m in mods]\n"
            "setup(name='efref', ext_modules=cythonize(exts, language_level=3, quiet=True), script_args=['build_ext', '--inplace'])\n"
        )
    subprocess.run([sys.executable, build], cwd=scratch, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    install_stubs()
    sys.path.insert(0, scratch)


def install_stubs():
    h5 = types.ModuleType("h5py")
    h5.File = None
    sys.modules["h5py"] = h5
    pt = types.ModuleType("prettytable")

    class PrettyTable:
        def __init__(self, *a, **k):
            self.field_names = []

        def add_row(self, r):
            pass

        def __str__(self):
            return ""

    pt.PrettyTable = PrettyTable
    sys.modules["prettytable"] = pt

    class _Any(types.ModuleType):
        def __getattr__(self, n):
            return _Any(n)

        def __call__(self, *a, **k):
            return _Any("x")

    mpl = _Any("matplotlib")
    mpl.use = lambda *a, **k: None
    sys.modules["matplotlib"] = mpl
    for sub in ["pyplot", "tri", "colors", "axes", "cm", "collections", "patches", "ticker", "lines", "figure"]:
        sys.modules["matplotlib." + sub] = _Any("matplotlib." + sub)
    for name, cls in [
        ("edelweissfe.elements.marmotelement.element", "MarmotElementWrapper"),
        (
            "edelweissfe.elements.marmotsingleqpelement.marmotmaterialgradientenhancedhypoelasticwrapper",
            "MarmotMaterialGradientEnhancedHypoElasticWrapper",
        ),
        ("edelweissfe.elements.marmotsingleqpelement.marmotmaterialhypoelasticwrapper", "MarmotMaterialHypoElasticWrapper"),
        ("edelweissfe.elements.marmotsingleqpelement.marmot", "MarmotMaterialWrapper"),
    ]:
        m = types.ModuleType(name)
        setattr(m, cls, type(cls, (), {}))
        sys.modules[name] = m
    import scipy.sparse.linalg as spla

    p = types.ModuleType("edelweissfe.linsolve.pardiso.pardiso")
    p.pardisoSolve = lambda A, b: spla.spsolve(A, b, use_umfpack=False)
    sys.modules["edelweissfe.linsolve.pardiso.pardiso"] = p


def distorted_hex_coords(rng, nNodes, nEl, h=0.1, distortion=0.15):
    """Random distorted hexahedra: unit-cube node table scaled by h, perturbed by up to distortion*h."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from oracle.hexlib import HEX8_NODES, HEX20_NODES

    base = (HEX8_NODES if nNodes == 8 else HEX20_NODES) * (h / 2)
    c = base[None] + rng.uniform(-distortion * h / 2, distortion * h / 2, (nEl, nNodes, 3))
    return c + rng.uniform(-1, 1, (nEl, 1, 3))


def element_fixture(elType, matName, props, nEl, seed, plastic=False):
    from edelweissfe.elements.displacementelement.element import DisplacementElement
    from edelweissfe.materials.linearelastic.linearelastic import LinearElasticMaterial
    from edelweissfe.materials.vonmises.vonmises import VonMisesMaterial
    from edelweissfe.points.node import Node

    rng = np.random.default_rng(seed)
    nNodes = 20 if "20" in elType else 8
    coords = distorted_hex_coords(rng, nNodes, nEl)
    nDof = 3 * nNodes
    Ks, Ps, states0, states1, Us, dUs = [], [], [], [], [], []
    for e in range(nEl):
        el = DisplacementElement(elType, e + 1)
        el.setNodes([Node(i + 1, coords[e, i]) for i in range(nNodes)])
        el.initializeElement()
        mat = (VonMisesMaterial if matName.startswith("vonmises") else LinearElasticMaterial)(np.array(props, dtype=float))
        el.setMaterial(mat)
        st = el._stateVarsRef
        if plastic:
            st[:, 0:6] = rng.normal(0.0, 120.0, (st.shape[0], 6))
            st[:, 6:12] = rng.normal(0.0, 1e-3, (st.shape[0], 6))
            st[:, 12] = rng.uniform(0.0, 0.01, st.shape[0])
        states0.append(st.copy())
        scale = 4e-4 if plastic else 1e-4
        U = rng.normal(0.0, scale, nDof)
        dU = rng.normal(0.0, scale, nDof)
        if plastic and e % 4 == 0:
            dU[:] = 0.0  # exercises the zero-increment shortcut (vonmises.py:211-213)
        K = np.zeros(nDof * nDof)
        P = np.zeros(nDof)
        el.computeYourself(K, P, U, dU, np.array([0.5, 0.5]), 0.1)
        Ks.append(K.copy())
        Ps.append(P.copy())
        states1.append(np.array(el._stateVarsTemp))
        Us.append(U)
        dUs.append(dU)
    np.savez_compressed(
        os.path.join(HERE, f"elem_{elType}_{matName}.npz"),
        coords=coords,
        props=np.array(props, dtype=float),
        U=np.array(Us),
        dU=np.array(dUs),
        state0=np.array(states0),
        Kvij=np.array(Ks),
        Pe=np.array(Ps),
        state1=np.array(states1),
    )


def element_fixture_tl(elType, props, nEl, seed, scale=0.008):
    """Ke, Pe and trial state of the reference's DisplacementTLElement with NeoHookeWa on random
    distorted hexahedra under random total displacements of about `scale` (element size 0.1)."""
    from edelweissfe.elements.displacementtlelement.element import DisplacementTLElement
    from edelweissfe.materials.neohooke.neohookepencegouformulationa import NeoHookeanWaMaterial
    from edelweissfe.points.node import Node

    rng = np.random.default_rng(seed)
    nNodes = 20 if "20" in elType else 8
    coords = distorted_hex_coords(rng, nNodes, nEl)
    nDof = 3 * nNodes
    Ks, Ps, states0, states1, Us, dUs = [], [], [], [], [], []
    for e in range(nEl):
        el = DisplacementTLElement(elType, e + 1)
        el.setNodes([Node(i + 1, coords[e, i]) for i in range(nNodes)])
        el.initializeElement()
        el.setMaterial(NeoHookeanWaMaterial(np.array(props, dtype=float)))
        states0.append(el._stateVarsRef.copy())
        U = rng.normal(0.0, scale, nDof)
        dU = rng.normal(0.0, scale / 4, nDof)
        K = np.zeros(nDof * nDof)
        P = np.zeros(nDof)
        el.computeYourself(K, P, U, dU, np.array([0.5, 0.5]), 0.1)
        Ks.append(K.copy())
        Ps.append(P.copy())
        states1.append(np.array(el._stateVarsTemp))
        Us.append(U)
        dUs.append(dU)
    np.savez_compressed(
        os.path.join(HERE, f"elem_{elType}_neohookewa.npz"),
        coords=coords,
        props=np.array(props, dtype=float),
        U=np.array(Us),
        dU=np.array(dUs),
        state0=np.array(states0),
        Kvij=np.array(Ks),
        Pe=np.array(Ps),
        state1=np.array(states1),
    )


def csr_fixture(seed=3):
    from edelweissfe.numerics.csrgenerator import CSRGenerator
    from edelweissfe.numerics.dofmanager import VIJSystemMatrix

    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from oracle.mesh import BoxMesh
    from oracle.system import element_dofs, vij_pattern

    m = BoxMesh(3, 2, 2, 1.0, 1.0, 1.0)
    ed = element_dofs(m.elements)
    I, J = vij_pattern(ed)
    nDof = 3 * m.nNodes
    K = VIJSystemMatrix(nDof, I, J, {})
    gen = CSRGenerator(K)
    V = np.random.default_rng(seed).normal(size=I.size)
    A = gen.updateCSR(V)
    np.savez_compressed(
        os.path.join(HERE, "csr_small.npz"),
        elements=m.elements,
        I=I,
        J=J,
        V=V,
        indptr=A.indptr,
        indices=A.indices,
        data=A.data,
        nDof=nDof,
    )


BOX_J2_INP = """*material, name=vonmises, id=mat, provider=edelweiss
{E}, {nu}, {fy}, {H}, 0.0, 0.0
*job, name=job, domain=3d
*solver, solver=NIST, name=theSolver
*modelGenerator, generator=boxGen, name=gen
nX ={nX}
nY ={nY}
nZ ={nZ}
lX ={lX}
lY ={lY}
lZ ={lZ}
elProvider =edelweiss
elType ={elType}
*section, name=section1, material=mat, type=solid
all
*step, solver=theSolver, maxInc={maxInc}, minInc=1e-6, maxNumInc=1000, maxIter=25, stepLength=1
dirichlet, name=left, nSet=gen_left, field=displacement, 1=0.0, 2=0.0, 3=0.0
dirichlet, name=right, nSet=gen_right, field=displacement, 1={ux}
"""

CANTILEVER_INP = """*material, name=linearelastic, id=mat, provider=edelweiss
210000.0, 0.3
*job, name=job, domain=3d
*solver, solver=NIST, name=theSolver
*modelGenerator, generator=boxGen, name=gen
nX =20
nY =4
nZ =4
lX =10
lY =2
lZ =2
elProvider =edelweiss
elType =C3D8
*section, name=section1, material=mat, type=solid
all
*step, solver=theSolver, maxInc=1, minInc=1e-6, maxNumInc=1000, maxIter=25, stepLength=1
dirichlet, name=left, nSet=gen_left, field=displacement, 1=0.0, 2=0.0, 3=0.0
nodeforces, name=face, nSet=gen_right, components='0, 0, -0.25', field=displacement
nodeforces, name=e1, nSet=gen_rightFront, components='0, 0, 0.125', field=displacement
nodeforces, name=e2, nSet=gen_rightBack, components='0, 0, 0.125', field=displacement
nodeforces, name=e3, nSet=gen_bottomRight, components='0, 0, 0.125', field=displacement
nodeforces, name=e4, nSet=gen_topRight, components='0, 0, 0.125', field=displacement
nodeforces, name=v1, nSet=gen_bottomRightFront, components='0, 0, -0.0625', field=displacement
nodeforces, name=v2, nSet=gen_bottomRightBack, components='0, 0, -0.0625', field=displacement
nodeforces, name=v3, nSet=gen_topRightFront, components='0, 0, -0.0625', field=displacement
nodeforces, name=v4, nSet=gen_topRightBack, components='0, 0, -0.0625', field=displacement
"""


BOX_TL_INP = """*material, name=neohookewa, id=mat, provider=edelweiss
{mu}, {K}
*job, name=job, domain=3d
*solver, solver=NIST, name=theSolver
*modelGenerator, generator=boxGen, name=gen
nX ={nX}
nY ={nY}
nZ ={nZ}
lX ={lX}
lY ={lY}
lZ ={lZ}
elProvider =edelweiss
elType ={elType}
*section, name=section1, material=mat, type=solid
all
*step, solver=theSolver, maxInc={maxInc}, minInc=1e-6, maxNumInc=1000, maxIter=25, stepLength=1
dirichlet, name=left, nSet=gen_left, field=displacement, 1=0.0, 2=0.0, 3=0.0
dirichlet, name=right, nSet=gen_right, field=displacement, 1={ux}
"""


def run_inp(text, scratch, name):
    from edelweissfe.drivers.inputfiledrivensimulation import finiteElementSimulation
    from edelweissfe.utils.inputfileparser import parseInputFile

    d = os.path.join(scratch, "run_" + name)
    os.makedirs(d, exist_ok=True)
    cwd = os.getcwd()
    os.chdir(d)
    with open("test.inp", "w") as f:
        f.write(text)
    iters = []
    from edelweissfe.solvers.nonlinearimplicitstatic import NIST

    orig = NIST.solveIncrement

    def wrapped(self, *a, **k):
        out = orig(self, *a, **k)
        iters.append(out[3])
        return out

    NIST.solveIncrement = wrapped
    try:
        model, _ = finiteElementSimulation(parseInputFile("test.inp"), verbose=False, suppressPlots=True)
    finally:
        NIST.solveIncrement = orig
        os.chdir(cwd)
    U = np.hstack([f["U"].flatten() for f in model.nodeFields.values()])
    return U, np.array(iters)


NIST_VARIANT_CASES = {
    "j2_box_4x2x2_c3d20r": dict(nX=4, nY=2, nZ=2, lX=0.4, lY=0.2, lZ=0.2, elType="C3D20R", maxInc=0.1, ux=0.0015),
    "j2_box_8x3x3_c3d8e": dict(nX=8, nY=3, nZ=3, lX=0.8, lY=0.3, lZ=0.3, elType="C3D8E", maxInc=0.1, ux=0.0016),
}


def nist_variant_fixtures(scratch):
    """NIST runs of J2 boxes with the 2x2x2 rule on the 20-node and the 3x3x3 rule on the 8-node
    hexahedron (C3D20R, C3D8E), and of NeoHookeWa boxes with the total-Lagrange counterparts
    (C3D20RTL, C3D8ETL)."""
    for name, c in NIST_VARIANT_CASES.items():
        text = BOX_J2_INP.format(E=210000.0, nu=0.3, fy=250.0, H=1000.0, **c)
        U, it = run_inp(text, scratch, name)
        np.savez_compressed(os.path.join(HERE, f"nist_{name}.npz"), U=U, iters=it, **{k: np.array(v) for k, v in c.items()})
    for name, c in TL_VARIANT_CASES.items():
        U, it = run_inp(BOX_TL_INP.format(mu=80.0, K=200.0, **c), scratch, name)
        np.savez_compressed(os.path.join(HERE, f"nist_{name}.npz"), U=U, iters=it, **{k: np.array(v) for k, v in c.items()})


def nist_fixtures(scratch):
    U, it = run_inp(CANTILEVER_INP, scratch, "cantilever")
    np.savez_compressed(os.path.join(HERE, "nist_cantilever_20x4x4.npz"), U=U, iters=it)
    cases = {
        "j2_box_10x4x4": dict(nX=10, nY=4, nZ=4, lX=1.0, lY=0.4, lZ=0.4, elType="C3D8", maxInc=0.05, ux=0.002),
        "j2_box_6x3x3_c3d20": dict(nX=6, nY=3, nZ=3, lX=0.6, lY=0.3, lZ=0.3, elType="C3D20", maxInc=0.1, ux=0.0015),
    }
    for name, c in cases.items():
        text = BOX_J2_INP.format(E=210000.0, nu=0.3, fy=250.0, H=1000.0, **c)
        U, it = run_inp(text, scratch, name)
        np.savez_compressed(os.path.join(HERE, f"nist_{name}.npz"), U=U, iters=it, **{k: np.array(v) for k, v in c.items()})


TL_CASES = {
    "tl_box_6x3x3_c3d8tl": dict(nX=6, nY=3, nZ=3, lX=0.6, lY=0.3, lZ=0.3, elType="C3D8TL", maxInc=0.25, ux=-0.09),
    "tl_box_3x2x2_c3d20tl": dict(nX=3, nY=2, nZ=2, lX=0.3, lY=0.2, lZ=0.2, elType="C3D20TL", maxInc=0.5, ux=-0.045),
}
TL_VARIANT_CASES = {
    "tl_box_3x2x2_c3d20rtl": dict(nX=3, nY=2, nZ=2, lX=0.3, lY=0.2, lZ=0.2, elType="C3D20RTL", maxInc=0.5, ux=-0.045),
    "tl_box_4x2x2_c3d8etl": dict(nX=4, nY=2, nZ=2, lX=0.4, lY=0.2, lZ=0.2, elType="C3D8ETL", maxInc=0.25, ux=-0.06),
}


def tl_fixtures(scratch):
    """Total-Lagrange NeoHookeWa [80, 200] elements and boxes compressed by 15 % (x = 0 clamped)."""
    element_fixture_tl("C3D8TL", [80.0, 200.0], 24, seed=11)
    element_fixture_tl("C3D20TL", [80.0, 200.0], 8, seed=12)
    for name, c in TL_CASES.items():
        U, it = run_inp(BOX_TL_INP.format(mu=80.0, K=200.0, **c), scratch, name)
        np.savez_compressed(os.path.join(HERE, f"nist_{name}.npz"), U=U, iters=it, **{k: np.array(v) for k, v in c.items()})


ARC_INP = """*material, name=vonmises, id=mat, provider=edelweiss
{E}, {nu}, {fy}, {H}, 0.0, 0.0
*job, name=job, domain=3d
*solver, solver=NISTPArcLength, name=theSolver
*modelGenerator, generator=boxGen, name=gen
nX ={nX}
nY ={nY}
nZ ={nZ}
lX ={lX}
lY ={lY}
lZ ={lZ}
elProvider =edelweiss
elType =C3D8
*section, name=section1, material=mat, type=solid
all
*modelGenerator, generator=findClosestNode, name=closestN1, executeAfterManualGeneration=True
location='{x1}, 0, 0'
storeIn=IDC1
*modelGenerator, generator=findClosestNode, name=closestN2, executeAfterManualGeneration=True
location='{x2}, 0, 0'
storeIn=IDC2
*step, solver=theSolver, maxInc={maxInc}, startInc={maxInc}, minInc=1e-6, maxNumInc=1000, maxIter=25, stepLength=1
options, category=NISTArcLength, arcLengthController=indirectcontrol
indirectcontrol, dof1='model.nodeSets["IDC1"][0].fields["displacement"]', cVector1='[-1,0,0]', dof2='model.nodeSets["IDC2"][0].fields["displacement"]', cVector2='[1,0,0]', L={L},
dirichlet, name=left, nSet=gen_left, field=displacement, 1=0.0, 2=0.0, 3=0.0
nodeforces, name=pull, nSet=gen_right, components='{f}, 0, 0', field=displacement
"""

ARC_CASE = dict(nX=10, nY=2, nZ=2, lX=1.0, lY=0.2, lZ=0.2, x1=0.3, x2=0.7, L=0.0016, f=10.0, maxInc=0.25)


def arclength_fixtures(scratch):
    """The reference's arc-length driver (solvers/nonlinearimplicitstaticparallelarclength.py) with
    indirect displacement control (stepactions/indirectcontrol.py) on a J2 bar: the relative x
    displacement of the nodes at x1 and x2 grows to L over the step while the load factor of the
    node forces on the x = lX face follows.  The driver derives from NISTParallel, whose module
    also holds the Marmot element loop (not buildable here); it is stubbed with the serial NIST,
    whose element loop gives the same results as NISTParallel's at one thread.  Stores U, the
    Newton iterations and the load factor Lambda after every increment."""
    from edelweissfe.solvers.nonlinearimplicitstatic import NIST

    stub = types.ModuleType("edelweissfe.solvers.nonlinearimplicitstaticparallel")
    stub.NISTParallel = NIST
    sys.modules["edelweissfe.solvers.nonlinearimplicitstaticparallel"] = stub
    from edelweissfe.solvers.nonlinearimplicitstaticparallelarclength import NISTPArcLength

    rec = []
    orig = NISTPArcLength.solveIncrement

    def wrapped(self, *a, **k):
        out = orig(self, *a, **k)
        rec.append((out[3], self.Lambda))
        return out

    NISTPArcLength.solveIncrement = wrapped
    try:
        text = ARC_INP.format(E=210000.0, nu=0.3, fy=250.0, H=1000.0, **ARC_CASE)
        U, _ = run_inp(text, scratch, "arclength")
    finally:
        NISTPArcLength.solveIncrement = orig
    np.savez_compressed(os.path.join(HERE, "nist_arclength_j2_10x2x2.npz"), U=U, iters=np.array([r[0] for r in rec]),
                        Lambda=np.array([r[1] for r in rec]), **{k: np.array(v) for k, v in ARC_CASE.items()})


J2 = [210000.0, 0.3, 250.0, 1000.0, 0.0, 0.0]

# The 160k-element J2 box of the benchmark (100x40x40 on 10x4x4, u_x = 0.002 lX over 20 increments
# of at most 0.05) at a quarter of its edge counts with the same element size: 2500 C3D8, 9,438 DOFs.
HEADLINE_SCALED_CASE = dict(nX=25, nY=10, nZ=10, lX=2.5, lY=1.0, lZ=1.0, elType="C3D8", maxInc=0.05, ux=0.005)


def headline_scaled_fixture(scratch):
    """The reference's NIST on the scaled benchmark box through its whole load history: the
    displacements after every converged increment (rows of U_inc), the Newton iteration count of
    each, and the committed stress of every Gauss point at the end (stress [nEl][8][6], element
    label order)."""
    from edelweissfe.solvers.nonlinearimplicitstatic import NIST

    c = HEADLINE_SCALED_CASE
    rec = []
    orig = NIST.solveIncrement

    def wrapped(self, *a, **k):
        out = orig(self, *a, **k)
        rec.append(np.array(out[0], dtype=float, copy=True))
        return out

    NIST.solveIncrement = wrapped
    holder = {}
    from edelweissfe.drivers import inputfiledrivensimulation as ifs

    orig_sim = ifs.finiteElementSimulation

    def keep_model(*a, **k):
        model, fo = orig_sim(*a, **k)
        holder["model"] = model
        return model, fo

    ifs.finiteElementSimulation = keep_model
    try:
        text = BOX_J2_INP.format(E=210000.0, nu=0.3, fy=250.0, H=1000.0, **c)
        U, it = run_inp(text, scratch, "headline_scaled")
    finally:
        NIST.solveIncrement = orig
        ifs.finiteElementSimulation = orig_sim
    model = holder["model"]
    labels = sorted(model.elements)
    stress = np.array([np.asarray(model.elements[e]._stateVarsRef)[:, 0:6] for e in labels])
    U_inc = np.array(rec)
    assert np.max(np.abs(U_inc[-1] - U)) == 0.0, "DofVector and node-field orders differ"
    np.savez_compressed(os.path.join(HERE, "nist_j2_box_25x10x10_history.npz"), U=U, U_inc=U_inc, iters=it,
                        stress=stress, **{k: np.array(v) for k, v in c.items()})


def variant_fixtures():
    """The other integration rules of elements/library.py: one point (C3D8R, C3D8RTL), 2x2x2 on
    the 20-node hexahedron (C3D20R, C3D20RTL) and 3x3x3 on the 8-node one (C3D8E, C3D8ETL)."""
    element_fixture("C3D8R", "vonmises", J2, 16, seed=21, plastic=True)
    element_fixture("C3D8E", "vonmises", J2, 8, seed=22, plastic=True)
    element_fixture("C3D20R", "vonmises", J2, 8, seed=23, plastic=True)
    element_fixture_tl("C3D8RTL", [80.0, 200.0], 16, seed=24)
    element_fixture_tl("C3D8ETL", [80.0, 200.0], 8, seed=25)
    element_fixture_tl("C3D20RTL", [80.0, 200.0], 8, seed=26)


def main():
    scratch = tempfile.mkdtemp(prefix="efref_")
    prepare_reference(scratch)
    if sys.argv[1:] == ["tl"]:  # only the total-Lagrange fixtures
        tl_fixtures(scratch)
        shutil.rmtree(scratch, ignore_errors=True)
        return
    if sys.argv[1:] == ["arclength"]:  # only the arc-length fixture
        arclength_fixtures(scratch)
        shutil.rmtree(scratch, ignore_errors=True)
        return
    if sys.argv[1:] == ["variants"]:  # only the reduced / enhanced integration element types
        variant_fixtures()
        nist_variant_fixtures(scratch)
        shutil.rmtree(scratch, ignore_errors=True)
        return
    if sys.argv[1:] == ["headline"]:  # only the scaled benchmark box history
        headline_scaled_fixture(scratch)
        shutil.rmtree(scratch, ignore_errors=True)
        return
    copy_uref()
    element_fixture("C3D8", "linearelastic", [210000.0, 0.3], 24, seed=1)
    element_fixture("C3D8", "vonmises", [210000.0, 0.3, 250.0, 1000.0, 0.0, 0.0], 48, seed=2, plastic=True)
    element_fixture("C3D8", "vonmisesexp", [210000.0, 0.3, 250.0, 1000.0, 80.0, 30.0], 16, seed=5, plastic=True)
    element_fixture("C3D20", "linearelastic", [210000.0, 0.22], 8, seed=4)
    element_fixture("C3D20", "vonmises", [210000.0, 0.3, 250.0, 1000.0, 0.0, 0.0], 8, seed=6, plastic=True)
    csr_fixture()
    nist_fixtures(scratch)
    tl_fixtures(scratch)
    arclength_fixtures(scratch)
    variant_fixtures()
    nist_variant_fixtures(scratch)
    headline_scaled_fixture(scratch)
    shutil.rmtree(scratch, ignore_errors=True)


if __name__ == "__main__":
    main()
