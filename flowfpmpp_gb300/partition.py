"""Host-side mirror of the reference module ``fpm_partition_2d`` over the C ABI
(src/fpm_partition_2d.f90:35-154)."""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import check, lib
from .stairstep import _need, _ptr

_D, _I = ctypes.c_double, ctypes.c_int


def fpm_partition_terms_2d(phi, g, u, v, solid, xf, yf, kin, ring, dt, nu, nx=None, ny=None, slip_body=False):
    """Returns (terms[4] = [F_KINE, F_VIF, F_VIS, F_BOUND], vif_density, omega).
    ``solid`` is any boolean-like (nx, ny) array (the reference's logical)."""
    if nx is None or ny is None:
        nx, ny = np.asarray(u).shape
    f64 = np.float64
    _need(phi, (nx, ny), f64, "phi")
    _need(u, (nx, ny), f64, "u")
    _need(v, (nx, ny), f64, "v")
    s8 = np.asfortranarray(np.asarray(solid) != 0, dtype=np.uint8)
    if s8.shape != (nx, ny):
        raise ValueError("solid must be (nx, ny)")
    xf = _need(np.asarray(xf, dtype=f64), (nx + 1,), f64, "xf")
    yf = _need(np.asarray(yf, dtype=f64), (ny + 1,), f64, "yf")
    _need(ring, (2 * nx + 2 * ny, 2, 2), f64, "ring")
    gg = np.ascontiguousarray(g, dtype=f64)
    kk = np.ascontiguousarray(kin, dtype=f64)
    if gg.shape != (2,) or kk.shape != (6,):
        raise ValueError("g has 2 entries and kin 6")
    terms = np.zeros(4)
    vif = np.empty((nx, ny), order="F")
    omega = np.empty((nx, ny), order="F")
    check(lib().fpm_partition_terms_2d(_ptr(phi), _ptr(gg), _ptr(u), _ptr(v), _ptr(s8), _ptr(xf), _ptr(yf),
                                       _ptr(kk), _ptr(ring), _D(dt), _D(nu), _I(nx), _I(ny), _ptr(terms),
                                       _ptr(vif), _ptr(omega), _I(int(bool(slip_body)))))
    return terms, vif, omega
