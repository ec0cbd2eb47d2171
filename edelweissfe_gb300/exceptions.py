"""Exceptions with the meaning of the reference's ``utils/exceptions.py``.

The Newton driver maps the C ABI's status codes onto them exactly where the
reference raises its own: EF_CUTBACK -> CutbackRequest (materials/vonmises/vonmises.py:231,
solvers/nonlinearimplicitstaticparallel.pyx:148-150), EF_NAN -> DivergingSolution
(solvers/nonlinearimplicitstatic.py:748-749).
"""


class CutbackRequest(Exception):
    """The evaluation of the residual failed due to a too large time increment."""

    def __init__(self, message, cutbackSize):
        super().__init__(message)
        self.cutbackSize = float(cutbackSize)


class ReachedMaxIterations(Exception):
    """The maximum number of nonlinear iterations was attained."""


class DivergingSolution(Exception):
    """The nonlinear solution diverges (growing residual or NaN)."""


class ReachedMaxIncrements(Exception):
    pass


class ReachedMinIncrementSize(Exception):
    pass


class StepFailed(Exception):
    pass
