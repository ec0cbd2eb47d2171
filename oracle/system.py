"""Equation-system bookkeeping of the oracle: DOF numbering, VIJ pattern, CSR slot map and scatter.

* DOF numbering follows ``numerics/dofmanager.py:254-298``
  (``_reserveSpaceForNodeFields``): node-major, the field's components contiguous.
* The VIJ pattern follows ``numerics/dofmanager.py:522-557``
  (``_initializeVIJPattern``): for an entity with DOF list ``d`` of length ``n``
  the value at offset ``p`` maps to row ``d[p % n]`` and column ``d[p // n]``.
* The CSR pattern and slot map follow ``numerics/csrgenerator.pyx:47-97``
  (SciPy canonical CSR of the (I, J) pairs, then the position of each pair in
  its row), and the scatter follows ``updateCSR`` :100-115
  (``data[:] = 0; data[x[k]] += V[k]`` for increasing k).
* ``dirichlet_rows`` follows ``solvers/nonlinearimplicitstaticparallelmk2.pyx:66-109``
  (constrained rows zeroed, diagonal 1, then ``eliminate_zeros``).
"""

import numpy as np
import scipy.sparse as sp


def element_dofs(elements: np.ndarray, nodeDofBase: np.ndarray = None, dim: int = 3) -> np.ndarray:
    """[nEl, nNodes] node indices -> [nEl, dim*nNodes] global DOF indices."""
    base = dim * elements if nodeDofBase is None else nodeDofBase[elements]
    return (base[:, :, None] + np.arange(dim)[None, None, :]).reshape(elements.shape[0], -1)


def vij_pattern(elDofs: np.ndarray):
    """I, J (int64) of the VIJ system matrix for equally sized entities stored in order."""
    nEl, n = elDofs.shape
    I = np.tile(elDofs, (1, n)).reshape(-1)  # value p -> d[p % n]
    J = np.repeat(elDofs, n, axis=1).reshape(-1)  # value p -> d[p // n]
    return I.astype(np.int64), J.astype(np.int64)


def csr_slot_map(I: np.ndarray, J: np.ndarray, nDof: int):
    """Canonical CSR pattern (indptr, indices as int32) and slot x[k] of every VIJ pair."""
    key = I.astype(np.int64) * nDof + J.astype(np.int64)
    uniq, inv = np.unique(key, return_inverse=True)
    rows = uniq // nDof
    indices = (uniq % nDof).astype(np.int32)
    indptr = np.zeros(nDof + 1, dtype=np.int64)
    np.add.at(indptr, rows + 1, 1)
    indptr = np.cumsum(indptr).astype(np.int32)
    return indptr, indices, inv.astype(np.int32)


def csr_update(V: np.ndarray, x: np.ndarray, nnz: int) -> np.ndarray:
    """Serial scatter ``data[x[k]] += V[k]`` for increasing k (ufunc.at is unbuffered, in order)."""
    data = np.zeros(nnz)
    np.add.at(data, x, V)
    return data


def dirichlet_rows(indptr, indices, data, rows):
    """Zero constrained rows, set their diagonal to 1, drop explicit zeros -> scipy csr_matrix."""
    data = data.copy()
    for i in rows:
        s, e = indptr[i], indptr[i + 1]
        data[s:e] = np.where(indices[s:e] == i, 1.0, 0.0)
    n = len(indptr) - 1
    A = sp.csr_matrix((data, indices.copy(), indptr.copy()), shape=(n, n))
    A.eliminate_zeros()
    return A


def condense(Pe: np.ndarray, elDofs: np.ndarray, nDof: int):
    """P[d] += Pe, F[d] += |Pe| over elements in order (nonlinearimplicitstaticparallelmk2.pyx:186-193)."""
    P = np.zeros(nDof)
    F = np.zeros(nDof)
    np.add.at(P, elDofs.ravel(), Pe.ravel())
    np.add.at(F, elDofs.ravel(), np.abs(Pe).ravel())
    return P, F
