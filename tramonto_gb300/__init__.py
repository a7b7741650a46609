"""GB300-native nonlocal-density path of Tramonto (FMT + WCA fill and Schur operator)."""
from .problem import Problem, from_golden  # noqa: F401
