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
from .materials import MATERIALS


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
            Ke += np.einsum("eia,eij,ejb->eab", B, C, B) * f[:, None, None]
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
