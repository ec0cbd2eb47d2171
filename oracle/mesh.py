"""Structured box mesh generator of the oracle.

Follows ``generators/boxgen.py:91-400``: nodes on an (nNodesX, nNodesY, nNodesZ)
grid numbered x-major, then y, then z (z fastest); hex20 meshes use the doubled
grid and drop grid points with two or more odd indices; element node lists as
in :151-330; node sets are grid slices (:336-386) and element sets (:388-400).
"""

import numpy as np

# (dx, dy, dz) in grid steps of each element node; hex20 in half-element steps
_HEX8_OFFS = [(0, 0, 0), (0, 0, 1), (1, 0, 1), (1, 0, 0), (0, 1, 0), (0, 1, 1), (1, 1, 1), (1, 1, 0)]
_HEX20_OFFS = [
    (0, 0, 0), (0, 0, 2), (2, 0, 2), (2, 0, 0), (0, 2, 0), (0, 2, 2), (2, 2, 2), (2, 2, 0),
    (0, 0, 1), (1, 0, 2), (2, 0, 1), (1, 0, 0), (0, 2, 1), (1, 2, 2), (2, 2, 1), (1, 2, 0),
    (0, 1, 0), (0, 1, 2), (2, 1, 2), (2, 1, 0),
]  # fmt: skip


class BoxMesh:
    def __init__(self, nX, nY, nZ, lX=1.0, lY=1.0, lZ=1.0, x0=0.0, y0=0.0, z0=0.0, nNodesPerElement=8, name="gen"):
        self.nX, self.nY, self.nZ = nX, nY, nZ
        quad = nNodesPerElement == 20
        m = 2 if quad else 1
        nx, ny, nz = m * nX + 1, m * nY + 1, m * nZ + 1
        self.gridShape = (nx, ny, nz)
        xs = np.linspace(x0, x0 + lX, nx)
        ys = np.linspace(y0, y0 + lY, ny)
        zs = np.linspace(z0, z0 + lZ, nz)
        ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
        if quad:
            keep = (ix % 2 + iy % 2 + iz % 2) < 2
        else:
            keep = np.ones(ix.shape, dtype=bool)
        gridToNode = -np.ones(ix.shape, dtype=np.int64)
        gridToNode[keep] = np.arange(int(keep.sum()))
        self.gridToNode = gridToNode
        self.keep = keep
        self.coords = np.stack([xs[ix[keep]], ys[iy[keep]], zs[iz[keep]]], axis=1)
        self.nNodes = self.coords.shape[0]
        offs = np.array(_HEX20_OFFS if quad else _HEX8_OFFS)
        ex, ey, ez = np.meshgrid(np.arange(nX), np.arange(nY), np.arange(nZ), indexing="ij")
        base = np.stack([m * ex.ravel(), m * ey.ravel(), m * ez.ravel()], axis=1)
        g = base[:, None, :] + offs[None, :, :]
        self.elements = gridToNode[g[..., 0], g[..., 1], g[..., 2]]
        assert (self.elements >= 0).all()
        self.nEl = self.elements.shape[0]
        self.name = name
        self.nodeSets = self._node_sets()
        self.elementSets = {f"{name}_all": np.arange(self.nEl)}

    def _sel(self, s):
        g = np.atleast_1d(self.gridToNode[s])
        k = np.atleast_1d(self.keep[s])
        return g[k].ravel()

    def _node_sets(self):
        n = self.name
        nx, ny, nz = self.gridShape
        S = np.s_
        defs = {
            "top": S[:, -1, :], "bottom": S[:, 0, :], "right": S[-1, :, :], "left": S[0, :, :],
            "front": S[:, :, -1], "back": S[:, :, 0],
            "bottomRight": S[-1, 0, :], "bottomLeft": S[0, 0, :], "bottomFront": S[:, 0, -1], "bottomBack": S[:, 0, 0],
            "topRight": S[-1, -1, :], "topLeft": S[0, -1, :], "topFront": S[:, -1, -1], "topBack": S[:, -1, 0],
            "rightBack": S[-1, :, 0], "rightFront": S[-1, :, -1], "leftBack": S[0, :, 0], "leftFront": S[0, :, -1],
            "centerX": S[int(nx / 2), :, :], "centerY": S[:, int(ny / 2), :], "centerZ": S[:, :, int(nz / 2)],
            "bottomRightFront": S[-1, 0, -1], "bottomRightBack": S[-1, 0, 0],
            "bottomLeftFront": S[0, 0, -1], "bottomLeftBack": S[0, 0, 0],
            "topRightFront": S[-1, -1, -1], "topRightBack": S[-1, -1, 0],
            "topLeftFront": S[0, -1, -1], "topLeftBack": S[0, -1, 0],
        }  # fmt: skip
        sets = {f"{n}_{k}": self._sel(v) for k, v in defs.items()}
        sets[f"{n}_all"] = np.arange(self.nNodes)
        sets["all"] = np.arange(self.nNodes)
        return sets
