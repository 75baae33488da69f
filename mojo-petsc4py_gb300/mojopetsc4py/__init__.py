"""GB300 implementation of lee101/mojo-petsc4py's sequential Krylov path.

`from mojopetsc4py import PETSc` gives the same Vec / Mat / PC / KSP classes,
method names, argument order and defaults as the reference; the kernels run
on the GPU through libgpetsc.so (include/gpetsc.h).
"""

from . import PETSc  # noqa: F401
from ._lib import get_arithmetic, set_arithmetic  # noqa: F401

__version__ = "0.1.0"
__upstream__ = "petsc4py 3.25.5"

__all__ = ["PETSc", "get_arithmetic", "set_arithmetic"]
