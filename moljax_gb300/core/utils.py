"""Status codes and small helpers (moljax/core/utils.py)."""

from __future__ import annotations


class StatusCode:
    """moljax/core/utils.py:265-272."""
    SUCCESS = 0
    RUNNING = 1
    MAX_STEPS_REACHED = 2
    DT_TOO_SMALL = 3
    NON_FINITE_VALUES = 4
    NK_FAILED = 5


def get_interior(field, grid):
    """Interior view of a padded field (moljax/core/utils.py:24-40)."""
    return field[grid.interior_slice]
