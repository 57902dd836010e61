"""
Test-only stand-in for ``tad-mctc`` (not installed in this container).

It exists so that tad-dftd4's own modules can be imported and run to produce
golden fixtures.  It provides the generic helpers tad-dftd4 imports, written
from their documented behaviour, and an independent restatement of the D4 and
EEQ coordination numbers.  Element tables come from the product's table file,
so the reference code sees exactly the inputs the kernels see.
"""

from . import batch, convert, data, math, ncoord, storch, typing  # noqa: F401
