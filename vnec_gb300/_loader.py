"""Locate and load the in-tree shared libraries built by ``vnec_gb300.build``."""
from __future__ import annotations

import ctypes
import os

LIB_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib")
_cache: dict[str, ctypes.CDLL] = {}


class LibraryMissing(RuntimeError):
    """Raised when a native library has not been built (no silent fallback)."""


def path(name: str) -> str:
    return os.path.join(LIB_DIR, f"lib{name}.so")


def load(name: str) -> ctypes.CDLL:
    lib = _cache.get(name)
    if lib is None:
        p = path(name)
        if not os.path.exists(p):
            raise LibraryMissing(f"{p} is not built; run `python -c 'import __graft_entry__ as g; g.build()'`")
        lib = ctypes.CDLL(p)
        _cache[name] = lib
    return lib


def load_path(p: str) -> ctypes.CDLL:
    """Loads a library by file path (cached like `load`)."""
    lib = _cache.get(p)
    if lib is None:
        if not os.path.exists(p):
            raise LibraryMissing(f"{p} is not built")
        lib = ctypes.CDLL(p)
        _cache[p] = lib
    return lib
