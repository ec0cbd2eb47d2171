"""Hexahedral element library of the oracle: node tables, Gauss rules, shape functions.

Follows ``elements/library.py`` (C3D8 :212-227, C3D8R :228-242, C3D8E :244-259, C3D20 :260-275,
C3D20R :276-291, C3D8TL :453-467, C3D8RTL :469-484, C3D8ETL :485-500, C3D20TL :501-515,
C3D20RTL :517-532) and the
shape-function conventions of
``elements/displacementelement/_elementcomputationmatrices.py``:

* ``_J3D8`` :306-366 / ``_J3D20`` :369+ fit ``x(S1,S2,S3)`` with a polynomial whose
  node table (the rows of their ``A`` matrices) gives the parametric node
  coordinates below; the Jacobian row r is dx/dS_r.
* ``_B3D8`` :679-817 / ``_B3D20`` :820+ evaluate the shape-function derivatives
  at ``S = (eta[q], xi[q], zeta[q])`` of the library's Gauss arrays (row 0 of
  their ``h`` matrix depends on ``xi`` and ``zeta`` only, i.e. it is d/dS1 with
  S2 = xi, S3 = zeta).
* The total-Lagrange element (``elements/displacementtlelement/_elementcomputationmatrices.py``)
  uses the same conventions: ``_J3D8`` :592-652 / ``_J3D20`` :655+ (with the same row-2 term)
  and ``computeNablaN`` :247-281 with ``_Ndiff3D`` :370-498 evaluated at ``(xi, eta, zeta)``,
  whose row 0 is d/dS1 at S1 = eta -- the same point as the small-strain B operator.
* ``computeNOperator`` :106-213 (used for body forces) evaluates the shape
  functions at ``S = (xi[q], eta[q], zeta[q])`` -- note the swapped first two
  coordinates relative to the B operator; this is reproduced as is.
"""

import numpy as np

# parametric node coordinates (S1, S2, S3); S1 runs along the box generator's x
# index, S2 along y, S3 along z (generators/boxgen.py:200-330 node lists)
HEX8_NODES = np.array(
    [
        [-1, -1, -1],
        [-1, -1, 1],
        [1, -1, 1],
        [1, -1, -1],
        [-1, 1, -1],
        [-1, 1, 1],
        [1, 1, 1],
        [1, 1, -1],
    ],
    dtype=float,
)

HEX20_NODES = np.array(
    [
        [-1, -1, -1],
        [-1, -1, 1],
        [1, -1, 1],
        [1, -1, -1],
        [-1, 1, -1],
        [-1, 1, 1],
        [1, 1, 1],
        [1, 1, -1],
        [-1, -1, 0],
        [0, -1, 1],
        [1, -1, 0],
        [0, -1, -1],
        [-1, 1, 0],
        [0, 1, 1],
        [1, 1, 0],
        [0, 1, -1],
        [-1, 0, -1],
        [-1, 0, 1],
        [1, 0, 1],
        [1, 0, -1],
    ],
    dtype=float,
)

_g = 1.0 / np.sqrt(3.0)
_s8 = _g * np.array([-1, 1, 1, -1])
_t8 = _g * np.array([-1, -1, 1, 1])
_s20 = np.array([-1.0, 0.0, 1.0])
_t20 = np.array([-1.0, -1, -1, 0, 0, 0, 1, 1, 1])
_w1H = (5 / 9) ** 3
_w2H = (5 / 9) ** 2 * (8 / 9)
_w3H = (5 / 9) * (8 / 9) ** 2
_w4H = (8 / 9) ** 3
_wI = np.array([_w1H, _w2H, _w1H])
_wII = np.array([_w2H, _w3H, _w2H])


def _rule_2x2x2():
    xi = _g * np.hstack([-np.ones(4), np.ones(4)])
    eta = np.hstack([_t8, _t8])
    zeta = np.hstack([_s8, _s8])
    return xi, eta, zeta, np.ones(8)


def _rule_3x3x3():
    r = np.sqrt(0.6)
    xi = r * np.hstack([-np.ones(9), np.zeros(9), np.ones(9)])
    eta = r * np.hstack([_t20, _t20, _t20])
    zeta = r * np.hstack([_s20 for _ in range(9)])
    w = np.hstack([_wI, _wII, _wI, _wII, np.array([_w3H, _w4H, _w3H]), _wII, _wI, _wII, _wI])
    return xi, eta, zeta, w


def _rule_1():
    return np.zeros(1), np.zeros(1), np.zeros(1), np.array([8.0])


# element type -> (node table, Gauss rule, total Lagrange?)
ELEMENT_TYPES = {
    "C3D8": (HEX8_NODES, _rule_2x2x2, False),
    "C3D8R": (HEX8_NODES, _rule_1, False),
    "C3D8E": (HEX8_NODES, _rule_3x3x3, False),
    "C3D20": (HEX20_NODES, _rule_3x3x3, False),
    "C3D20R": (HEX20_NODES, _rule_2x2x2, False),
    "C3D8TL": (HEX8_NODES, _rule_2x2x2, True),
    "C3D8RTL": (HEX8_NODES, _rule_1, True),
    "C3D8ETL": (HEX8_NODES, _rule_3x3x3, True),
    "C3D20TL": (HEX20_NODES, _rule_3x3x3, True),
    "C3D20RTL": (HEX20_NODES, _rule_2x2x2, True),
}


def shape_functions(nodes: np.ndarray, S: np.ndarray) -> np.ndarray:
    """Trilinear (8 nodes) or serendipity (20 nodes) shape functions at points S [nP,3] -> [nP,nNodes]."""
    S = np.atleast_2d(S)
    out = np.zeros((S.shape[0], nodes.shape[0]))
    for a, sa in enumerate(nodes):
        f = [(1 + sa[k] * S[:, k]) if sa[k] != 0 else (1 - S[:, k] ** 2) for k in range(3)]
        if nodes.shape[0] == 8:
            out[:, a] = f[0] * f[1] * f[2] / 8
        elif np.all(sa != 0):
            out[:, a] = f[0] * f[1] * f[2] * (sa[0] * S[:, 0] + sa[1] * S[:, 1] + sa[2] * S[:, 2] - 2) / 8
        else:
            out[:, a] = f[0] * f[1] * f[2] / 4
    return out


def shape_derivatives(nodes: np.ndarray, S: np.ndarray) -> np.ndarray:
    """dN_a/dS_r at points S [nP,3] -> [nP, 3, nNodes]."""
    S = np.atleast_2d(S)
    nP = S.shape[0]
    out = np.zeros((nP, 3, nodes.shape[0]))
    for a, sa in enumerate(nodes):
        f = [(1 + sa[k] * S[:, k]) if sa[k] != 0 else (1 - S[:, k] ** 2) for k in range(3)]
        df = [sa[k] * np.ones(nP) if sa[k] != 0 else -2 * S[:, k] for k in range(3)]
        for r in range(3):
            o = [k for k in range(3) if k != r]
            if nodes.shape[0] == 8:
                out[:, r, a] = df[r] * f[o[0]] * f[o[1]] / 8
            elif np.all(sa != 0):
                lin = sa[0] * S[:, 0] + sa[1] * S[:, 1] + sa[2] * S[:, 2] - 2
                out[:, r, a] = (df[r] * f[o[0]] * f[o[1]] * lin + f[0] * f[1] * f[2] * sa[r]) / 8
            else:
                out[:, r, a] = df[r] * f[o[0]] * f[o[1]] / 4
    return out


# Coefficient of the S2*S3 monomial of the 20-node polynomial fit, as a row acting
# on the nodal coordinates (row 5 of inv(A) in _J3D20).  The reference's _J3D20
# (_elementcomputationmatrices.py:481-495) writes this term of dx/dS3 as
# ``a5 * zeta`` instead of ``a5 * xi``; for the C3D20 family of the small-strain
# element the Jacobian is therefore J_true + (zeta - xi) * a5 in row 2.  The term
# vanishes on undistorted (parallelepiped) elements.
HEX20_S2S3_ROW = np.zeros(20)
HEX20_S2S3_ROW[[9, 11, 13, 15]] = np.array([-0.25, 0.25, 0.25, -0.25])


def element_tables(elType: str):
    """Constant per-type tables.

    Returns dict with nodes, nNodes, nQP, w [nQP], dNdS [nQP,3,nNodes] (B/J
    evaluation points) and N [nQP,nNodes] (body-force evaluation points)."""
    nodes, rule, tl = ELEMENT_TYPES[elType]
    xi, eta, zeta, w = rule()
    S_b = np.stack([eta, xi, zeta], axis=1)
    S_n = np.stack([xi, eta, zeta], axis=1)
    return dict(
        nodes=nodes,
        nNodes=nodes.shape[0],
        nQP=len(w),
        w=np.asarray(w, dtype=float),
        dNdS=shape_derivatives(nodes, S_b),
        N=shape_functions(nodes, S_n),
        totalLagrange=tl,
        # per Gauss point: row-2 Jacobian quirk factor (zeta - xi) of the B/J evaluation point; the
        # total-Lagrange family shares _J3D20 (displacementtlelement/_elementcomputationmatrices.py:655+)
        jacobianQuirk=(zeta - xi) if nodes.shape[0] == 20 else None,
    )
