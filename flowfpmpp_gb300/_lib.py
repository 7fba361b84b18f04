"""Loads the in-tree CUDA library libfpm_gb300.so through ctypes.

There is no CPU fallback: if the library is missing or cannot be loaded the
import of any solver entry point raises.  Call ``flowfpmpp_gb300.build.build()``
(or ``__graft_entry__.build()``) first.
"""
from __future__ import annotations

import ctypes
import os
import re

from .build import LIB_PATH, INCLUDE

_lib = None

STATUS = {
    0: "FPM_OK",
    1: "FPM_E_METHOD",
    2: "FPM_E_SIZE",
    3: "FPM_E_ISOLATED",
    4: "FPM_E_NO_OUTER_FACE",
    5: "FPM_E_ARG",
    6: "FPM_E_CUDA",
    7: "FPM_E_NO_DEVICE",
    8: "FPM_E_LIMIT",
    9: "FPM_E_TIMEOUT",
}


class FpmError(RuntimeError):
    """A nonzero status from the C ABI; the reference stops with error stop here."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{STATUS.get(code, code)}: {message}")
        self.code = code
        self.message = message


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is not built; run flowfpmpp_gb300.build.build()")
        _lib = ctypes.CDLL(LIB_PATH)
        _lib.fpm_last_error.restype = ctypes.c_char_p
        _lib.fpm_host_alloc.restype = ctypes.c_void_p
        _lib.fpm_host_alloc.argtypes = [ctypes.c_size_t]
        _lib.fpm_host_free.argtypes = [ctypes.c_void_p]
    return _lib


def check(code: int) -> None:
    if code != 0:
        msg = lib().fpm_last_error().decode(errors="replace")
        raise FpmError(code, msg)


def declared_symbols() -> list[str]:
    """Every function name declared in include/*.h (for the export check)."""
    names = []
    for fn in sorted(os.listdir(INCLUDE)):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(INCLUDE, fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(fpm_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))
