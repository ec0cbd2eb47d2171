"""Small-strain displacement element (C3D8/C3D20 family) of the oracle, batched over elements.

Follows ``elements/displacementelement/element.py``:

* ``initializeElement`` :194-205 -- Jacobian and B operator per Gauss point
  (``_elementcomputationmatrices.py`` ``_J3D8`` :306-366, ``_B3D8`` :679-817,
  ``_J3D20`` :369+, ``_B3D20`` :820+; the conventions are restated in
  ``oracle/hexlib.py``),
* ``setMaterial`` :207-240 -- state layout per Gauss point
  ``[stress(6), strain(6), material state(k)]``,
* ``computeYourself`` :290-346 -- trial state copied from the committed state,
  ``dStrain = B @ dU``, material update per Gauss point,
  ``K += B^T C B detJ w``, ``P -= B^T stress detJ w``, ``strain += dStrain``,
* ``computeBodyForce`` :348-371 -- ``P += N (x) load * detJ * w``,
* ``acceptLastState`` :373-379.

``K`` is returned as ``Ke[e, a, b]``; the reference writes it through a C-order
reshape of its VIJ slice, so VIJ value index ``a*n + b`` holds ``Ke[a, b]``.
"""

import numpy as np

from .hexlib import element_tables
from .materials import MATERIALS, neo_hooke_wa


def voigt_B(dNdx: np.ndarray) -> np.ndarray:
    """B operator [..., 6, 3n] from dN/dx [..., 3, n] (rows 11, 22, 33, 12, 13, 23)."""
    shp = dNdx.shape[:-2]
    n = dNdx.shape[-1]
    B = np.zeros(shp + (6, 3 * n))
    gx, gy, gz = dNdx[..., 0, :], dNdx[..., 1, :], dNdx[..., 2, :]
    B[..., 0, 0::3] = gx
    B[..., 1, 1::3] = gy
    B[..., 2, 2::3] = gz
    B[..., 3, 0::3] = gy
    B[..., 3, 1::3] = gx
    B[..., 4, 0::3] = gz
    B[..., 4, 2::3] = gx
    B[..., 5, 1::3] = gz
    B[..., 5, 2::3] = gy
    return B


class SmallStrainElements:
    """A homogeneous batch of small-strain elements sharing one element type and one material."""

    def __init__(self, elType: str, coords: np.ndarray, material: str, props):
        """coords: [nEl, nNodes, 3] nodal coordinates (element node order)."""
        self.elType = elType
        self.tab = element_tables(elType)
        assert not self.tab["totalLagrange"]
        self.coords = np.asarray(coords, dtype=float)
        self.nEl = self.coords.shape[0]
        self.nNodes = self.tab["nNodes"]
        self.nQP = self.tab["nQP"]
        self.nDof = 3 * self.nNodes
        self.material, nMatState = MATERIALS[material.lower()]
        self.props = np.asarray(props, dtype=float)
        self.nState = 12 + nMatState
        # initializeElement: J[e,q] = dNdS[q] @ X[e]; B = a.b(invJ).c(dNdS)
        J = np.einsum("qra,eac->eqrc", self.tab["dNdS"], self.coords)
        if self.tab["jacobianQuirk"] is not None:
            from .hexlib import HEX20_S2S3_ROW

            a5 = np.einsum("a,eac->ec", HEX20_S2S3_ROW, self.coords)
            J[:, :, 2, :] += self.tab["jacobianQuirk"][None, :, None] * a5[:, None, :]
        self.detJ = np.linalg.det(J)
        self.dNdx = np.einsum("eqrs,qsa->eqra", np.linalg.inv(J), self.tab["dNdS"])
        self.B = voigt_B(self.dNdx)
        self.stateRef = np.zeros((self.nEl, self.nQP, self.nState))
        self.stateTemp = self.stateRef.copy()

    def compute_yourself(self, U: np.ndarray, dU: np.ndarray):
        """Element loop body. U, dU: [nEl, nDof]. Returns (Ke [nEl,n,n], Pe [nEl,n]); sets stateTemp."""
        w = self.tab["w"]
        st = self.stateRef.copy()
        dStrain = np.einsum("eqij,ej->eqi", self.B, dU)
        Ke = np.zeros((self.nEl, self.nDof, self.nDof))
        Pe = np.zeros((self.nEl, self.nDof))
        for q in range(self.nQP):
            stress, mstate, C = self.material(self.props, st[:, q, 0:6], st[:, q, 12:], dStrain[:, q])
            st[:, q, 0:6] = stress
            st[:, q, 12:] = mstate
            B = self.B[:, q]
            f = self.detJ[:, q] * w[q]
            Ke += np.matmul(B.transpose(0, 2, 1), np.matmul(C, B)) * f[:, None, None]  # B^T (C B) per element
            Pe -= np.einsum("eia,ei->ea", B, stress) * f[:, None]
            st[:, q, 6:12] += dStrain[:, q]
        self.stateTemp = st
        return Ke, Pe

    def body_force(self, load: np.ndarray) -> np.ndarray:
        """Consistent nodal body force [nEl, nDof] for a constant load vector (3,)."""
        w = self.tab["w"]
        N = self.tab["N"]
        Pe = np.zeros((self.nEl, self.nDof))
        for q in range(self.nQP):
            Pe += np.outer(np.ones(self.nEl), np.outer(N[q], load).ravel()) * (self.detJ[:, q] * w[q])[:, None]
        return Pe

    def accept_last_state(self):
        self.stateRef[:] = self.stateTemp


def _voigt_stress_tl(T):
    """doVoigtStress(3, .) of utils/voigtnotation.py:72-90: [11, 22, 33, 12, 23, 13]."""
    return np.stack([T[:, 0, 0], T[:, 1, 1], T[:, 2, 2], T[:, 0, 1], T[:, 1, 2], T[:, 0, 2]], axis=1)


def _voigt_strain_tl(E):
    """doVoigtStrain(3, .) of utils/voigtnotation.py:30-48: [11, 22, 33, 2*12, 2*23, 2*13]."""
    return np.stack([E[:, 0, 0], E[:, 1, 1], E[:, 2, 2], 2 * E[:, 0, 1], 2 * E[:, 1, 2], 2 * E[:, 0, 2]], axis=1)


class TLElements:
    """A homogeneous batch of total-Lagrange hyperelastic elements (C3D8TL / C3D20TL family).

    Follows ``elements/displacementtlelement/element.py``:

    * ``initializeElement`` :282-292 -- J and nablaN = dN/dX per Gauss point
      (``_elementcomputationmatrices.py`` ``computeJacobian`` :33-67, ``computeNablaN`` :247-281),
    * ``setMaterial`` :294-330 -- state per Gauss point ``[stress(6), strain(6), energy(1)]``
      (the material writes its strain-energy density into the last entry),
    * ``computeYourself`` :346-427, hyperelastic branch -- ``F = I + sum_a U_a (x) nablaN_a``
      (``computeDeformationGradient`` :70-106), Green-Lagrange strain into the state, Kirchhoff
      stress ``tau`` and ``dtau/dF`` from the material, ``PK1 = inv(F) tau`` (as coded),
      ``K += makeH2D(einsum(NAi, dtau/dF, nablaN) - einsum(NAi, NAi, tau)) detJ w`` with
      ``NAi = nablaN^T inv(F)`` and ``P -= (nablaN^T PK1) detJ w``.
    """

    def __init__(self, elType: str, coords: np.ndarray, material: str, props):
        self.elType = elType
        self.tab = element_tables(elType)
        assert self.tab["totalLagrange"]
        assert material.lower() == "neohookewa"
        self.coords = np.asarray(coords, dtype=float)
        self.nEl = self.coords.shape[0]
        self.nNodes = self.tab["nNodes"]
        self.nQP = self.tab["nQP"]
        self.nDof = 3 * self.nNodes
        self.props = np.asarray(props, dtype=float)
        self.nState = 13
        J = np.einsum("qra,eac->eqrc", self.tab["dNdS"], self.coords)
        if self.tab["jacobianQuirk"] is not None:
            from .hexlib import HEX20_S2S3_ROW

            a5 = np.einsum("a,eac->ec", HEX20_S2S3_ROW, self.coords)
            J[:, :, 2, :] += self.tab["jacobianQuirk"][None, :, None] * a5[:, None, :]
        self.detJ = np.linalg.det(J)
        self.nablaN = np.einsum("eqrs,qsa->eqra", np.linalg.inv(J), self.tab["dNdS"])  # [e,q,3,n]
        self.stateRef = np.zeros((self.nEl, self.nQP, self.nState))
        self.stateTemp = self.stateRef.copy()

    def compute_yourself(self, U: np.ndarray, dU: np.ndarray):
        """U: [nEl, nDof] total displacements (dU unused by the hyperelastic branch)."""
        w = self.tab["w"]
        n = self.nNodes
        st = self.stateRef.copy()
        Ue = np.asarray(U, dtype=float).reshape(self.nEl, n, 3)
        Ke = np.zeros((self.nEl, self.nDof, self.nDof))
        Pe = np.zeros((self.nEl, self.nDof))
        I = np.eye(3)
        for q in range(self.nQP):
            nab = self.nablaN[:, q]  # [e,3,n]
            H = np.einsum("eai,eja->eij", Ue, nab)
            F = I + H
            E = 0.5 * (H + np.swapaxes(H, 1, 2) + np.swapaxes(H, 1, 2) @ H)
            invF = np.linalg.inv(F)
            tau, D, W = neo_hooke_wa(self.props, F)
            NAi = np.swapaxes(nab, 1, 2) @ invF  # [e,n,3]
            Hk = np.einsum("eai,eijkl,ebl->eajbk", NAi, D, np.swapaxes(nab, 1, 2)) - np.einsum(
                "eak,ebi,eij->eajbk", NAi, NAi, tau
            )
            f = self.detJ[:, q] * w[q]
            Ke += Hk.reshape(self.nEl, self.nDof, self.nDof) * f[:, None, None]
            PK1 = invF @ tau
            Pe -= (np.swapaxes(nab, 1, 2) @ PK1).reshape(self.nEl, -1) * f[:, None]
            st[:, q, 0:6] = _voigt_stress_tl(tau)
            st[:, q, 6:12] = _voigt_strain_tl(E)
            st[:, q, 12] = W
        self.stateTemp = st
        return Ke, Pe

    def body_force(self, load: np.ndarray) -> np.ndarray:
        w = self.tab["w"]
        N = self.tab["N"]
        Pe = np.zeros((self.nEl, self.nDof))
        for q in range(self.nQP):
            Pe += np.outer(np.ones(self.nEl), np.outer(N[q], load).ravel()) * (self.detJ[:, q] * w[q])[:, None]
        return Pe

    def accept_last_state(self):
        self.stateRef[:] = self.stateTemp


def make_elements(elType: str, coords: np.ndarray, material: str, props):
    """The oracle element batch of a type: small-strain or total-Lagrange."""
    if element_tables(elType)["totalLagrange"]:
        return TLElements(elType, coords, material, props)
    return SmallStrainElements(elType, coords, material, props)
