"""Structured box meshes (the reference's ``boxGen`` model generator).

Same node numbering, element node lists and set names as
``generators/boxgen.py:91-400`` so that DOF vectors line up with the
reference's: grid points x-major, then y, then z; hex20 meshes use a doubled
grid without points that have two or more odd grid indices.
"""

import numpy as np

# element node offsets on the grid: hex8 in element steps, hex20 in half-element steps
_HEX8 = ((0, 0, 0), (0, 0, 1), (1, 0, 1), (1, 0, 0), (0, 1, 0), (0, 1, 1), (1, 1, 1), (1, 1, 0))
_HEX20 = tuple((2 * a, 2 * b, 2 * c) for a, b, c in _HEX8) + (
    (0, 0, 1), (1, 0, 2), (2, 0, 1), (1, 0, 0), (0, 2, 1), (1, 2, 2), (2, 2, 1), (1, 2, 0),
    (0, 1, 0), (0, 1, 2), (2, 1, 2), (2, 1, 0))  # fmt: skip


def box_mesh(nX, nY, nZ, lX=1.0, lY=1.0, lZ=1.0, x0=0.0, y0=0.0, z0=0.0, nNodesPerElement=8, name="gen"):
    """Returns dict(coords [nNodes,3], elements [nEl,nNodesPerElement], nodeSets {name: node indices})."""
    if nNodesPerElement not in (8, 20):
        raise ValueError("boxGen supports 8- and 20-node hexahedra")
    h = 2 if nNodesPerElement == 20 else 1
    shape = (h * nX + 1, h * nY + 1, h * nZ + 1)
    gi = np.indices(shape).reshape(3, -1).T  # x-major, z fastest
    keep = (gi % 2).sum(axis=1) < 2 if h == 2 else np.ones(len(gi), bool)
    node_of = np.full(len(gi), -1, dtype=np.int64)
    node_of[keep] = np.arange(int(keep.sum()))
    node_of = node_of.reshape(shape)
    axes = [np.linspace(o, o + l, n) for o, l, n in zip((x0, y0, z0), (lX, lY, lZ), shape)]
    g = gi[keep]
    coords = np.stack([axes[k][g[:, k]] for k in range(3)], axis=1)
    corner = h * np.indices((nX, nY, nZ)).reshape(3, -1).T
    offs = np.array(_HEX20 if h == 2 else _HEX8)
    p = corner[:, None, :] + offs[None]
    elements = node_of[p[..., 0], p[..., 1], p[..., 2]]
    keepg = keep.reshape(shape)

    def sel(s):
        n = np.atleast_1d(node_of[s])
        k = np.atleast_1d(keepg[s])
        return n[k].ravel()

    S = np.s_
    faces = {
        "top": S[:, -1, :], "bottom": S[:, 0, :], "right": S[-1, :, :], "left": S[0, :, :],
        "front": S[:, :, -1], "back": S[:, :, 0],
        "bottomRight": S[-1, 0, :], "bottomLeft": S[0, 0, :], "bottomFront": S[:, 0, -1], "bottomBack": S[:, 0, 0],
        "topRight": S[-1, -1, :], "topLeft": S[0, -1, :], "topFront": S[:, -1, -1], "topBack": S[:, -1, 0],
        "rightBack": S[-1, :, 0], "rightFront": S[-1, :, -1], "leftBack": S[0, :, 0], "leftFront": S[0, :, -1],
        "bottomRightFront": S[-1, 0, -1], "bottomRightBack": S[-1, 0, 0],
        "bottomLeftFront": S[0, 0, -1], "bottomLeftBack": S[0, 0, 0],
        "topRightFront": S[-1, -1, -1], "topRightBack": S[-1, -1, 0],
        "topLeftFront": S[0, -1, -1], "topLeftBack": S[0, -1, 0],
    }  # fmt: skip
    sets = {f"{name}_{k}": sel(v) for k, v in faces.items()}
    sets[f"{name}_all"] = np.arange(coords.shape[0])
    return dict(coords=coords, elements=elements, nodeSets=sets)


def tied_box_mesh(nXq, nXl, nY, nZ, lXq, lXl, lY=1.0, lZ=1.0, name="gen"):
    """A box of two structured halves: x in [0, lXq] meshed with nXq x nY x nZ 20-node hexahedra,
    x in [lXq, lXq + lXl] with nXl x nY x nZ 8-node hexahedra.  The 8-node half's nodes on the
    interface are the 20-node half's corner nodes there; the 20-node half's mid-side nodes on the
    interface are tied to the two corner nodes of their edge (u_mid = (u_a + u_b) / 2), which
    makes the interface conforming.  The reference has no generator and no constraint for this
    (its box generator makes one element type, constraints/ only equates DOFs).

    Returns dict(coords, elements20, elements8, nodeSets (left = x = 0, right = x = lXq + lXl,
    all), ties = (slave, masterA, masterB) node index arrays)."""
    q = box_mesh(nXq, nY, nZ, lXq, lY, lZ, nNodesPerElement=20, name=name)
    lin = box_mesh(nXl, nY, nZ, lXl, lY, lZ, x0=lXq, nNodesPerElement=8, name=name)
    dy, dz = lY / nY, lZ / nZ
    nq = q["coords"].shape[0]

    def half_index(c):
        return np.rint(c[:, 1] / (dy / 2)).astype(np.int64), np.rint(c[:, 2] / (dz / 2)).astype(np.int64)

    face_q = np.asarray(q["nodeSets"][f"{name}_right"])
    iy, iz = half_index(q["coords"][face_q])
    key_q = {(a, b): n for a, b, n in zip(iy.tolist(), iz.tolist(), face_q.tolist())}
    # renumber the 8-node half: interface nodes -> the matching 20-node corner nodes
    face_l = np.asarray(lin["nodeSets"][f"{name}_left"])
    ly, lz = half_index(lin["coords"][face_l])
    new_of = np.full(lin["coords"].shape[0], -1, dtype=np.int64)
    new_of[face_l] = [key_q[(a, b)] for a, b in zip(ly.tolist(), lz.tolist())]
    rest = np.flatnonzero(new_of < 0)
    new_of[rest] = nq + np.arange(rest.size)
    coords = np.concatenate([q["coords"], lin["coords"][rest]])
    # ties: interface mid-side nodes (exactly one odd half-index) -> their edge's corner nodes
    slave, ma, mb = [], [], []
    for (a, b), n in key_q.items():
        if a % 2 == 1:
            slave.append(n)
            ma.append(key_q[(a - 1, b)])
            mb.append(key_q[(a + 1, b)])
        elif b % 2 == 1:
            slave.append(n)
            ma.append(key_q[(a, b - 1)])
            mb.append(key_q[(a, b + 1)])
    order = np.argsort(slave)
    sets = {f"{name}_left": np.asarray(q["nodeSets"][f"{name}_left"]),
            f"{name}_right": new_of[np.asarray(lin["nodeSets"][f"{name}_right"])],
            f"{name}_all": np.arange(coords.shape[0])}  # fmt: skip
    for side in ("top", "bottom", "front", "back"):
        s = np.union1d(q["nodeSets"][f"{name}_{side}"], new_of[np.asarray(lin["nodeSets"][f"{name}_{side}"])])
        sets[f"{name}_{side}"] = s
    return dict(coords=coords, elements20=q["elements"], elements8=new_of[lin["elements"]], nodeSets=sets,
                ties=(np.asarray(slave)[order], np.asarray(ma)[order], np.asarray(mb)[order]))  # fmt: skip
