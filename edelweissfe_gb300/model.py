"""Model description consumed by the GPU solver: element groups, nodal DOFs, boundary conditions.

This is the batched counterpart of the reference's model tree for the hot path:

* ``ElementGroup`` bundles elements of one type and one material -- what
  ``sections/solid.py`` does per element with ``initializeElement`` and
  ``setMaterial`` (elements/displacementelement/element.py:194-240);
* ``Model`` numbers DOFs node-major with three displacement components per node
  (numerics/dofmanager.py:254-298);
* ``DirichletBC``, ``NodeForces`` and ``BodyForce`` follow the step actions
  ``stepactions/dirichlet.py`` (getDelta), ``stepactions/nodeforces.py``
  (getCurrentLoad) and ``stepactions/bodyforce.py`` (getCurrentLoad) with the
  default amplitude f(t) = t.
"""

from dataclasses import dataclass

import numpy as np


@dataclass
class ElementGroup:
    elType: str
    elements: np.ndarray  # [nEl, nNodes] node indices, element node order of the reference
    material: str
    props: np.ndarray
    propsTable: np.ndarray = None  # optional per-element material rows [nRows, nProps]
    elemRow: np.ndarray = None  # element -> row of propsTable
    cutback: float = None  # increment scale requested when the material fails (None: the library's 0.5)


class Model:
    def __init__(self, coords: np.ndarray, groups, nodeSets=None, ties=None):
        self.coords = np.asarray(coords, dtype=float)
        self.nNodes = self.coords.shape[0]
        self.nDof = 3 * self.nNodes
        self.groups = list(groups)
        self.nodeSets = dict(nodeSets or {})
        # node ties u_s = (u_a + u_b) / 2: (slave, masterA, masterB) node index arrays, or None
        self.ties = ties

    def element_dofs(self, g: ElementGroup) -> np.ndarray:
        e = np.asarray(g.elements, dtype=np.int64)
        return (3 * e[:, :, None] + np.arange(3)[None, None, :]).reshape(e.shape[0], -1).astype(np.int32)

    def dof_coordinates(self) -> np.ndarray:
        """Node coordinates written into a DOF vector (entry 3n+c = coordinate c of node n)."""
        return self.coords.reshape(-1).copy()

    def n_accumulated_fluxes(self) -> int:
        """sum over elements of their DOF count (numerics/dofmanager.py:381-420)."""
        return int(sum(3 * np.asarray(g.elements).size for g in self.groups))


class DirichletBC:
    """Prescribed displacement components on a node set; values are the step totals."""

    def __init__(self, nodes, components: dict):
        nodes = np.asarray(nodes, dtype=np.int64)
        comps = sorted(components)
        # findDirichletIndices (solvers/nonlinearimplicitstatic.py:1077-1084): node-major, selected components
        self.dofs = (3 * nodes[:, None] + np.asarray(comps)[None, :]).reshape(-1)
        self.delta = np.tile(np.array([float(components[c]) for c in comps]), nodes.size)

    def getDelta(self, timeStep):
        a = timeStep.stepProgress
        return self.delta * (a - (a - timeStep.stepProgressIncrement))


class DirichletDofs:
    """Prescribed step totals on explicit DOFs (many node sets with different values at once)."""

    def __init__(self, dofs, totals):
        self.dofs = np.asarray(dofs, dtype=np.int64)
        self.delta = np.asarray(totals, dtype=float)

    def getDelta(self, timeStep):
        a = timeStep.stepProgress
        return self.delta * (a - (a - timeStep.stepProgressIncrement))


class NodeForces:
    def __init__(self, nodes, vector):
        nodes = np.asarray(nodes, dtype=np.int64)
        self.dofs = (3 * nodes[:, None] + np.arange(3)[None, :]).reshape(-1)
        self.load = np.tile(np.asarray(vector, dtype=float), nodes.size)

    def getCurrentLoad(self, timeStep):
        return self.load * timeStep.stepProgress


class BodyForce:
    def __init__(self, groupId: int, vector):
        self.groupId = groupId
        self.vector = np.asarray(vector, dtype=float)

    def getCurrentLoad(self, timeStep):
        return self.vector * timeStep.stepProgress
