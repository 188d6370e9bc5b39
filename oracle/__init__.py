"""ORACLE (test infrastructure only).

CPU restatements of the MCTomo forward-modelling hot path, loaded through
ctypes. Only tests/, ``__graft_entry__.smoke()`` and the CPU legs of
``bench.py`` may import this package: it is the checker, never the product.
"""
from .lib import load, load_reference, build, build_reference  # noqa: F401
