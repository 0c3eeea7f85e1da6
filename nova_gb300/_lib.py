"""Loader for libnova.so, the nova-gb300 C-ABI library.

The library is built in-tree (nova_gb300/build.py) into nova_gb300/lib/. This
module loads it once and fails loudly if it is missing: there is no
pure-Python or CPU fallback for any solver.
"""
import ctypes as ct
import os

LIB_PATH = os.path.join(os.path.dirname(os.path.realpath(__file__)), "lib", "libnova.so")

_nova = None


def load():
    global _nova
    if _nova is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("nova-gb300: %s is missing; build it with `python -m nova_gb300.build` "
                              "(or __graft_entry__.build())" % LIB_PATH)
        _nova = ct.CDLL(LIB_PATH)
    return _nova
