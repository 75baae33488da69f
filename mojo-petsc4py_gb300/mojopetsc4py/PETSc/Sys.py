"""System information, mirroring the reference's `Sys` (python/mojopetsc4py/PETSc/Sys.py)."""

from __future__ import annotations

import platform
import sys

PETSC_VERSION = (3, 25, 5)
PETSC_VERSION_MAJOR, PETSC_VERSION_MINOR, PETSC_VERSION_SUBMINOR = PETSC_VERSION
PETSC_VERSION_STRING = ".".join(str(v) for v in PETSC_VERSION)

Scalar = float
Real = float
Int = int
Bool = bool

__version__ = PETSC_VERSION_STRING


def getVersion():
    """The PETSc release whose API and numerics are mirrored."""
    return PETSC_VERSION


def getVersionInfo() -> str:
    return (f"PETSc {PETSC_VERSION_STRING} interface (mojopetsc4py, GB300 CUDA) on"
            f" Python {sys.version.split()[0]} {platform.machine()}")


def getMachine() -> str:
    return platform.machine()


def hasThreads() -> bool:
    return False
