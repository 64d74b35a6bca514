"""Exceptions of the engine (names follow ``pycc/exceptions.py:12-50``)."""


class PyCCError(Exception):
    """Base class of the engine's errors."""


class InvalidKeywordError(PyCCError, ValueError):
    """A keyword argument has a value outside its allowed set (``pycc/exceptions.py:27-50``)."""

    def __init__(self, keyword, value, allowed):
        self.keyword, self.value, self.allowed = keyword, value, list(allowed)
        super().__init__("Invalid value %r for keyword %r; allowed: %s" % (value, keyword, self.allowed))


class ConvergenceError(PyCCError, RuntimeError):
    """The amplitude iteration exhausted ``maxiter`` (the reference silently returns None)."""

    def __init__(self, what, maxiter, ediff, rms):
        self.maxiter, self.ediff, self.rms = maxiter, ediff, rms
        super().__init__("%s did not converge in %d iterations (last dE = %.3e, rms = %.3e)"
                         % (what, maxiter, ediff, rms))


class NumericalError(PyCCError, FloatingPointError):
    """A residual norm or energy became NaN/Inf during the iteration."""
