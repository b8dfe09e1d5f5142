"""hbtg - GB300-native iterative gravitational unbinding for HBT-HERONS.

Product modules: ``gpu`` (ctypes binding of libhbtg.so), ``abi`` (the C ABI
structs), ``build`` (in-tree nvcc build), ``config`` (reference parameter
files).  ``synthetic`` generates seeded benchmark inputs.  ``oracle`` loads
the CPU oracle and is imported only by tests and measurement code.
"""
from . import abi  # noqa: F401
