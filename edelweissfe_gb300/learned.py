"""The learned FGMRES correction trained across seeded J2 boxes and used on unseen ones.

The family: J2 boxes whose material is drawn per seed, sigma_y ~ U[150, 350], H ~ U[200, 2000],
nu ~ U[0.2, 0.4] (numpy.random.default_rng(seed), in that order; E = 210000), x = 0 clamped and the
x = lX face pulled to 0.2 % strain over 20 increments.  Several seeds are held in one context as
disjoint boxes, each with its own material row (``ef_set_group_props``), so that one Newton history
produces (residual, correction) pairs from every seed's systems.  The network is trained on those
pairs on the GPU (``ef_mpnn_train``), its weights are moved into a second context holding unseen
seeds, and that context's load history is solved with and without the network.

The reference has no counterpart: its linear solves are direct (PARDISO) or pyamg-preconditioned
GMRES (``linsolve/gmres/gmres.py:87-88``); this stage replaces nothing there.
"""

import numpy as np
import torch

from .mesh import box_mesh
from .model import DirichletBC, ElementGroup, Model
from .solver import LinSolverOptions, NISTGPU, Step


def seeded_j2_props(seed, E=210000.0):
    """[E, nu, sigma_y, H, 0, 0] of one seed (the draws of the cube batch, in the same order)."""
    rng = np.random.default_rng(seed)
    fy = rng.uniform(150.0, 350.0)
    H = rng.uniform(200.0, 2000.0)
    nu = rng.uniform(0.2, 0.4)
    return [E, float(nu), float(fy), float(H), 0.0, 0.0]


def seeded_boxes(seeds, nX, nY, nZ, h=0.1, strain=0.002, linsolver=None):
    """One NISTGPU context with one nX x nY x nZ C3D8 box (element size h) per seed, the boxes
    side by side in y with disjoint nodes."""
    lX, lY, lZ = nX * h, nY * h, nZ * h
    m = box_mesh(nX, nY, nZ, lX, lY, lZ)
    nn = m["coords"].shape[0]
    nEl = m["elements"].shape[0]
    coords, elements, dirs = [], [], []
    for k in range(len(seeds)):
        c = m["coords"].copy()
        c[:, 1] += k * (lY + 2 * h)
        coords.append(c)
        elements.append(m["elements"] + k * nn)
        dirs.append(DirichletBC(m["nodeSets"]["gen_left"] + k * nn, {0: 0.0, 1: 0.0, 2: 0.0}))
        dirs.append(DirichletBC(m["nodeSets"]["gen_right"] + k * nn, {0: strain * lX}))
    table = np.array([seeded_j2_props(s) for s in seeds])
    rows = np.repeat(np.arange(len(seeds), dtype=np.int32), nEl)
    group = ElementGroup("C3D8", np.concatenate(elements), "vonmises", table[0], propsTable=table, elemRow=rows)
    return NISTGPU(Model(np.concatenate(coords), [group]), dirs, linsolver=linsolver or LinSolverOptions())


def solve_history(s, increments, maxInc=0.05):
    """Solves the first `increments` load increments; returns (Newton iterations per increment,
    Krylov iterations of the whole history, final displacements on the host)."""
    s.krylovIterations.clear()
    s.iterationHistory.clear()
    U, _ = s.solveStep(Step(maxInc=maxInc, minInc=1e-6, maxIter=25), maxIncrements=increments)
    torch.cuda.synchronize()
    return [it for _, it in s.iterationHistory], int(sum(s.krylovIterations)), U.cpu().numpy()


def fgmres_options(restart=40):
    return LinSolverOptions(method="fgmres", rtol=1e-8, innerRtol=1e-6, restart=restart, maxIter=20000)


def train_across_seeds(seeds, dims, increments, base="jacobi", epochs=60, lr=1e-3, every=5, maxPerSolve=4,
                       maxSamples=64, netSeed=0):
    """Pairs from the FGMRES solves (preconditioned by `base`) of the first `increments` load
    increments of one context holding every training seed, then Adam on the GPU.  Returns
    (params, scales, record)."""
    import time

    s = seeded_boxes(seeds, *dims, linsolver=fgmres_options())
    s.setFgmresPreconditioner(base)
    s.initLearnedPreconditioner(seed=netSeed, maxSamples=maxSamples)
    s.collectTrainingPairs(every=every, maxPerSolve=maxPerSolve, kind="iterates")
    newton, krylov, _ = solve_history(s, increments)
    s.collectTrainingPairs(0, 0)
    torch.cuda.synchronize()
    t0 = time.time()
    first, last = s.trainLearnedPreconditioner(epochs=epochs, lr=lr, norm="energy")
    torch.cuda.synchronize()
    params, scales = s.learnedParameters()
    rec = {"seeds": list(seeds), "base": base, "pairs": s.numTrainingPairs(), "epochs": epochs, "lr": lr,
           "loss_first": first, "loss_last": last, "train_s": time.time() - t0, "newton": newton,
           "krylov": krylov}  # fmt: skip
    del s
    return params, scales, rec


def evaluate_on_seeds(seeds, dims, increments, params, scales, base="jacobi"):
    """The first `increments` load increments of a context holding the (unseen) `seeds`, solved
    with FGMRES preconditioned by `base` without and then with the trained network (each in a
    fresh context, so both start from the same state): Newton and Krylov iterations and
    load-history seconds of both, and the largest displacement difference relative to the largest
    displacement."""
    import time

    out = {}
    for on in (False, True):
        s = seeded_boxes(seeds, *dims, linsolver=fgmres_options())
        s.setFgmresPreconditioner(base)
        s.initLearnedPreconditioner(seed=0, maxSamples=0)
        s.setLearnedParameters(params, scales)
        s.enableLearnedPreconditioner(on)
        torch.cuda.synchronize()
        t0 = time.time()
        newton, krylov, U = solve_history(s, increments)
        out[on] = (newton, krylov, time.time() - t0, U)
        del s
    (n0, k0, t0, U0), (n1, k1, t1, U1) = out[False], out[True]
    return {"seeds": list(seeds), "base": base, "newton_off": n0, "newton_on": n1, "krylov_off": k0, "krylov_on": k1,
            "history_s_off": t0, "history_s_on": t1, "krylov_ratio": k0 / max(k1, 1),
            "max_rel_dU": float(np.max(np.abs(U1 - U0)) / max(np.max(np.abs(U0)), 1e-300))}  # fmt: skip
