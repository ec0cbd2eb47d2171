"""Constitutive updates of the oracle, batched over quadrature points.

* ``linear_elastic`` follows ``materials/linearelastic/linearelastic.py:95-125`` (3D
  elasticity matrix) and ``:185-210`` (computeStress).
* ``von_mises`` follows ``materials/vonmises/vonmises.py:35-56`` (IDev,
  IDevHalfShear, maxIter=15, tol=1e-12), ``:105-124`` (hardening law),
  ``:126-146`` (elasticity matrix) and ``:186-254`` (computeStress: zero-increment
  shortcut, elastic predictor, Newton on the consistency condition, consistent
  tangent, CutbackRequest after 15 iterations).

Stress/strain are 6-vectors in the reference's small-strain Voigt order
[11, 22, 33, 12, 13, 23] with engineering shear strains.
"""

import numpy as np

IDEV = np.array(
    [
        [2 / 3, -1 / 3, -1 / 3, 0, 0, 0],
        [-1 / 3, 2 / 3, -1 / 3, 0, 0, 0],
        [-1 / 3, -1 / 3, 2 / 3, 0, 0, 0],
        [0, 0, 0, 1, 0, 0],
        [0, 0, 0, 0, 1, 0],
        [0, 0, 0, 0, 0, 1],
    ]
)
IDEV_HALF_SHEAR = np.array(
    [
        [2 / 3, -1 / 3, -1 / 3, 0, 0, 0],
        [-1 / 3, 2 / 3, -1 / 3, 0, 0, 0],
        [-1 / 3, -1 / 3, 2 / 3, 0, 0, 0],
        [0, 0, 0, 0.5, 0, 0],
        [0, 0, 0, 0, 0.5, 0],
        [0, 0, 0, 0, 0, 0.5],
    ]
)
VM_MAX_ITER = 15
VM_TOL = 1e-12


class ReturnMapFailed(Exception):
    """Raised where the reference raises ``CutbackRequest("Von Mises Newton failed.", 0.5)``."""

    cutbackSize = 0.5


def elasticity_matrix(E: float, nu: float) -> np.ndarray:
    f = E / ((1 + nu) * (1 - 2 * nu))
    return f * np.array(
        [
            [1 - nu, nu, nu, 0, 0, 0],
            [nu, 1 - nu, nu, 0, 0, 0],
            [nu, nu, 1 - nu, 0, 0, 0],
            [0, 0, 0, (1 - 2 * nu) / 2, 0, 0],
            [0, 0, 0, 0, (1 - 2 * nu) / 2, 0],
            [0, 0, 0, 0, 0, (1 - 2 * nu) / 2],
        ]
    )


def linear_elastic(props, stress, matstate, dStrain):
    """Returns (new stress [Q,6], new matstate [Q,0], tangent [Q,6,6])."""
    Ei = elasticity_matrix(props[0], props[1])
    newStress = stress + dStrain @ Ei.T
    C = np.broadcast_to(Ei, (stress.shape[0], 6, 6)).copy()
    return newStress, matstate.copy(), C


def von_mises(props, stress, matstate, dStrain):
    """J2 radial return; props = [E, nu, fy0, HLin, dfy, delta]; matstate [Q,1] = kappa.

    Returns (new stress, new matstate, tangent); raises ReturnMapFailed where the
    reference raises CutbackRequest."""
    E, nu, fy0, HLin, dfy, delta = [float(p) for p in props[:6]]
    G = E / (2 * (1.0 + nu))
    Ei = elasticity_matrix(E, nu)

    def fy(k):
        return fy0 + HLin * k + dfy * (1.0 - np.exp(-delta * k))

    def dfy_dk(k):
        return HLin + dfy * delta * np.exp(-delta * k)

    Q = stress.shape[0]
    kappa = matstate[:, 0].copy()
    newStress = stress.copy()
    C = np.broadcast_to(Ei, (Q, 6, 6)).copy()

    zero = np.linalg.norm(dStrain, axis=1) < 1e-14
    trial = stress + dStrain @ Ei  # dStrain @ Ei (vonmises.py:216); Ei is symmetric
    dev = trial @ IDEV.T
    devNorm = np.sqrt(np.sum(dev[:, 0:3] ** 2, axis=1) + 2 * np.sum(dev[:, 3:6] ** 2, axis=1))
    f = devNorm - np.sqrt(2 / 3) * fy(kappa)
    plastic = (f > 0.0) & ~zero
    elastic = ~plastic & ~zero
    newStress[elastic] = trial[elastic]

    idx = np.nonzero(plastic)[0]
    if idx.size:
        dn = devNorm[idx]
        k0 = kappa[idx]

        def R(dk):
            return dn - np.sqrt(6) * G * dk - np.sqrt(2 / 3) * fy(k0 + dk)

        dk = np.zeros(idx.size)
        counter = np.zeros(idx.size, dtype=int)
        active = np.abs(R(dk)) > VM_TOL
        while active.any():
            if np.any(counter[active] == VM_MAX_ITER):
                raise ReturnMapFailed("Von Mises Newton failed.")
            a = np.nonzero(active)[0]
            dR = -np.sqrt(6) * G - np.sqrt(2 / 3) * dfy_dk(k0[a] + dk[a])
            dk[a] -= R(dk)[a] / dR
            counter[a] += 1
            active = np.abs(R(dk)) > VM_TOL
        n = dev[idx] / dn[:, None]
        dLambda = np.sqrt(3 / 2) * dk
        kNew = k0 + dk
        kappa[idx] = kNew
        newStress[idx] = trial[idx] - (2.0 * G * dLambda)[:, None] * n
        c1 = 2.0 * G * (1.0 / (1.0 + dfy_dk(kNew) / (3.0 * G)) - 2.0 * G * dLambda / dn)
        c2 = 4.0 * G**2 * dLambda / dn
        C[idx] = Ei[None] - c1[:, None, None] * np.einsum("qi,qj->qij", n, n) - c2[:, None, None] * IDEV_HALF_SHEAR[None]
    return newStress, kappa[:, None], C


MATERIALS = {
    "linearelastic": (linear_elastic, 0),
    "vonmises": (von_mises, 1),
}


def neo_hooke_wa(props, F):
    """Kirchhoff stress, its derivative w.r.t. F and the energy density of the compressible
    neo-Hookean W_a (materials/neohooke/neohookepencegouformulationa.py:107-141); props = [mu, K].

    F [Q,3,3] -> tau [Q,3,3], dtau/dF [Q,3,3,3,3] (index order ijkl of the reference),
    W [Q] = mu/2 (I1 - 3) + (K/2 - mu/3)(J - 1)^2 - mu ln J (the material's state variable)."""
    mu, K = float(props[0]), float(props[1])
    invF = np.linalg.inv(F)
    B = F @ np.swapaxes(F, 1, 2)
    J = np.linalg.det(F)
    lamBar = (K - 2 / 3 * mu) * (J**2 - J) - mu
    muBar = (K - 2 / 3 * mu) * (2 * J**2 - J)
    I = np.eye(3)
    tau = mu * B + lamBar[:, None, None] * I
    D = mu * (np.einsum("ik,qjl->qijkl", I, F) + np.einsum("qil,jk->qijkl", F, I)) + muBar[
        :, None, None, None, None
    ] * np.einsum("ij,qlk->qijkl", I, invF)
    I1 = np.trace(B, axis1=1, axis2=2)
    W = mu / 2 * (I1 - 3) + (K / 2 - mu / 3) * (J - 1) ** 2 - mu * np.log(J)
    return tau, D, W
