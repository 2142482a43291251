"""Access descriptors (same enum values as pyop2/types/access.py:4-10)."""
import enum


class Access(enum.IntEnum):
    READ = 1
    WRITE = 2
    RW = 3
    INC = 4
    MIN = 5
    MAX = 6


READ = Access.READ
"""The data is only read."""

WRITE = Access.WRITE
"""The data is only written; write conflicts are the user's concern."""

RW = Access.RW
"""The data is read and written; write conflicts are the user's concern."""

INC = Access.INC
"""The kernel computes increments summed onto the data; the framework resolves
the write conflicts (atomics, warp aggregation or colouring)."""

MIN = Access.MIN
"""The kernel contributes to a ``min`` reduction."""

MAX = Access.MAX
"""The kernel contributes to a ``max`` reduction."""


class IterationRegion(enum.IntEnum):
    """Extruded iteration regions (pyop2/types/__init__.py:14-18)."""
    BOTTOM = 1
    TOP = 2
    INTERIOR_FACETS = 3
    ALL = 4


ON_BOTTOM = IterationRegion.BOTTOM
ON_TOP = IterationRegion.TOP
ON_INTERIOR_FACETS = IterationRegion.INTERIOR_FACETS
ALL = IterationRegion.ALL
