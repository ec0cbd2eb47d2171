"""Element results read back from the device state.

The reference reads results per element and quadrature point through
``BaseElement.getResultArray(result, quadraturePoint, getPersistentView)``
(elements/displacementelement/element.py:386-409): ``"stress"``, ``"strain"`` and
``"materialstate"`` are views of the point's state vector [stress(6), strain(6), material state]
(:222-236, names case-insensitive), and any other name is asked of the material
(``"kappa"`` of J2, materials/vonmises/vonmises.py:281-299; ``"energy"`` of NeoHookeWa,
materials/neohooke/neohookepencegouformulationa.py:168-186), which raises for names it does not
know.  ``ElementResultCollector`` (utils/elementresultcollector.pyx:38-120) gathers one result
of many elements and points into a table [elements, points, size] (2-D for a single point).

Here the state lives on the device in structure-of-arrays layout, so a collector is a device
gather (``ef_results_*`` of the C ABI) of the result's state slice into a table that one copy
brings into pinned host memory.  Results show the committed state, as the reference's views
do; ``trial=True`` reads the state of the current Newton iteration instead.
"""

import ctypes

import numpy as np
import torch

from . import _lib

_ELEMENT_RESULTS = {"stress": (0, 6), "strain": (6, 6)}
_MATERIAL_RESULTS = {"linearelastic": {}, "vonmises": {"kappa": (12, 1)}, "neohookewa": {"energy": (12, 1)}}


def result_slice(material: str, result: str, nState: int):
    """(first, count) of ``result`` in the per-point state vector of ``material`` (length nState)."""
    r = result.lower()
    if r in _ELEMENT_RESULTS:
        return _ELEMENT_RESULTS[r]
    if r == "materialstate":
        return 12, nState - 12
    sl = _MATERIAL_RESULTS.get(material.lower(), {}).get(r)
    if sl is None:
        raise Exception("This result doesn't exist for the current material.")
    return sl


class ElementResultCollector:
    """One result of a list of elements of one group at a list of quadrature points.

    ``elements``: indices within the group (None: all, in order); ``quadraturePoints``: an
    iterable of point numbers.  ``update()`` refreshes ``resultsTable`` ([elements, points,
    size], or [elements, size] for one point); ``getCurrentResults()`` updates and returns it.
    The table is overwritten by every update: copy it to keep a result.
    """

    def __init__(self, solver, groupId: int, elements, quadraturePoints, result: str, trial: bool = False):
        self.solver = solver
        self.lib = solver.lib
        self.trial = bool(trial)
        group = solver.model.groups[groupId]
        nQP, nState = ctypes.c_int(), ctypes.c_int()
        _lib.check(self.lib.ef_get_state_size(solver.ctx, solver.groupIds[groupId], ctypes.byref(nQP),
                                              ctypes.byref(nState)), "ef_get_state_size")  # fmt: skip
        first, count = result_slice(group.material, result, nState.value)
        qps = np.ascontiguousarray(np.asarray(list(quadraturePoints), dtype=np.int32))
        if elements is None:
            els, nEls = None, len(group.elements)
        else:
            els = np.ascontiguousarray(np.asarray(elements, dtype=np.int32).reshape(-1))
            nEls = els.size
        self.nEls, self.nGauss, self.nSize = nEls, qps.size, count
        self._pinned = torch.empty((nEls, qps.size, count), dtype=torch.float64, pin_memory=True)
        table = self._pinned.numpy()
        self.resultsTable = table.reshape(nEls, -1) if qps.size == 1 else table
        self.id = None
        if count == 0:  # e.g. the empty material state of a linear elastic material
            return
        cid = ctypes.c_int()
        _lib.check(self.lib.ef_results_create(solver.ctx, solver.groupIds[groupId],
                                              None if els is None else els.ctypes.data, nEls, qps.ctypes.data,
                                              qps.size, first, count, ctypes.byref(cid)), "ef_results_create")  # fmt: skip
        self.id = cid.value

    def update(self):
        if self.id is not None:
            _lib.check(self.lib.ef_results_update(self.solver.ctx, self.id, int(self.trial), self._pinned.data_ptr(),
                                                  self.solver._stream()), "ef_results_update")  # fmt: skip

    def getCurrentResults(self) -> np.ndarray:
        self.update()
        return self.resultsTable

    def close(self):
        if self.id is not None and getattr(self.solver, "ctx", None):
            self.lib.ef_results_destroy(self.solver.ctx, self.id)
        self.id = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
