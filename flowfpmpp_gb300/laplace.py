"""Host-side mirror of the reference modules ``fpm_laplace_3d`` and
``fpm_terms_3d`` (no body), over the C ABI.

Same procedure names and argument order as src/fpm_laplace_3d.f90 and
src/fpm_terms_3d.f90.  numpy arrays in Fortran layout: the uniform solver's
``phi`` is ``(nx+2, ny+2, nz+2)`` (full ghost layer), the non-uniform
solver's ``phi`` is ``(nx, ny, nz)``; the non-uniform axes carry no halo.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import check, lib
from .stairstep import _need, _ptr

_D, _I = ctypes.c_double, ctypes.c_int


def _faces(nx, ny, nz, faces, writable=False):
    names = ("xlo", "xhi", "ylo", "yhi", "zlo", "zhi")
    shapes = ((ny, nz), (ny, nz), (nx, nz), (nx, nz), (nx, ny), (nx, ny))
    return [_need(f, s, np.float64, n, writable) for f, s, n in zip(faces, shapes, names)]


def enforce_neumann_compatibility_3d(rhs, xlo, xhi, ylo, yhi, zlo, zhi, nx, ny, nz, dx, dy, dz):
    """src/fpm_laplace_3d.f90:9-53; shifts the faces in place, returns (correction, imbalance)."""
    _need(rhs, (nx, ny, nz), np.float64, "rhs")
    f = _faces(nx, ny, nz, (xlo, xhi, ylo, yhi, zlo, zhi), True)
    c, m = _D(), _D()
    check(lib().fpm_enforce_neumann_compatibility_3d(_ptr(rhs), *[_ptr(a) for a in f], _I(nx), _I(ny), _I(nz),
                                                     _D(dx), _D(dy), _D(dz), ctypes.byref(c), ctypes.byref(m)))
    return c.value, m.value


def solve_neumann_poisson_3d(phi, rhs, xlo, xhi, ylo, yhi, zlo, zhi, nx, ny, nz, dx, dy, dz, tolerance,
                             max_iterations, check_interval):
    """src/fpm_laplace_3d.f90:55-107; in place, returns (iterations, final_residual)."""
    _need(phi, (nx + 2, ny + 2, nz + 2), np.float64, "phi", True)
    _need(rhs, (nx, ny, nz), np.float64, "rhs")
    f = _faces(nx, ny, nz, (xlo, xhi, ylo, yhi, zlo, zhi))
    it, res = _I(), _D()
    check(lib().fpm_solve_neumann_poisson_3d(_ptr(phi), _ptr(rhs), *[_ptr(a) for a in f], _I(nx), _I(ny), _I(nz),
                                             _D(dx), _D(dy), _D(dz), _D(tolerance), _I(max_iterations),
                                             _I(check_interval), ctypes.byref(it), ctypes.byref(res)))
    return it.value, res.value


def enforce_neumann_compatibility_nonuniform_3d(rhs, xlo, xhi, ylo, yhi, zlo, zhi, dx, dy, dz, nx, ny, nz):
    """src/fpm_laplace_3d.f90:150-217."""
    _need(rhs, (nx, ny, nz), np.float64, "rhs")
    f = _faces(nx, ny, nz, (xlo, xhi, ylo, yhi, zlo, zhi), True)
    ax = [_need(np.asarray(a), (n,), np.float64, nm) for a, n, nm in ((dx, nx, "dx"), (dy, ny, "dy"), (dz, nz, "dz"))]
    c, m = _D(), _D()
    check(lib().fpm_enforce_neumann_compatibility_nonuniform_3d(_ptr(rhs), *[_ptr(a) for a in f],
                                                                *[_ptr(a) for a in ax], _I(nx), _I(ny), _I(nz),
                                                                ctypes.byref(c), ctypes.byref(m)))
    return c.value, m.value


def solve_neumann_poisson_nonuniform_3d(phi, rhs, xlo, xhi, ylo, yhi, zlo, zhi, xc, yc, zc, dx, dy, dz, nx, ny, nz,
                                        tolerance, max_iterations, check_interval):
    """src/fpm_laplace_3d.f90:219-293; in place, returns (iterations, final_residual)."""
    _need(phi, (nx, ny, nz), np.float64, "phi", True)
    _need(rhs, (nx, ny, nz), np.float64, "rhs")
    f = _faces(nx, ny, nz, (xlo, xhi, ylo, yhi, zlo, zhi))
    ax = [_need(np.asarray(a), (n,), np.float64, nm) for a, n, nm in
          ((xc, nx, "xc"), (yc, ny, "yc"), (zc, nz, "zc"), (dx, nx, "dx"), (dy, ny, "dy"), (dz, nz, "dz"))]
    it, res = _I(), _D()
    check(lib().fpm_solve_neumann_poisson_nonuniform_3d(_ptr(phi), _ptr(rhs), *[_ptr(a) for a in f],
                                                        *[_ptr(a) for a in ax], _I(nx), _I(ny), _I(nz),
                                                        _D(tolerance), _I(max_iterations), _I(check_interval),
                                                        ctypes.byref(it), ctypes.byref(res)))
    return it.value, res.value


def _flow(nx, ny, nz, arrays):
    names = ("u", "v", "w", "ox", "oy", "oz", "ax", "ay", "az")
    return [_need(a, (nx, ny, nz), np.float64, n) for a, n in zip(arrays, names)]


def compute_fpm_terms_uniform_3d(phi, u, v, w, ox, oy, oz, ax, ay, az, fluid, nx, ny, nz, dx, dy, dz):
    """src/fpm_terms_3d.f90:8-37; returns (gx, gy, gz, vortex, advection, totals)."""
    _need(phi, (nx + 2, ny + 2, nz + 2), np.float64, "phi")
    fl = _flow(nx, ny, nz, (u, v, w, ox, oy, oz, ax, ay, az))
    _need(fluid, (nx, ny, nz), np.int32, "fluid")
    outs = [np.empty((nx, ny, nz), order="F") for _ in range(5)]
    totals = np.zeros(2)
    check(lib().fpm_compute_fpm_terms_uniform_3d(_ptr(phi), *[_ptr(a) for a in fl], _ptr(fluid),
                                                 *[_ptr(o) for o in outs], _ptr(totals), _I(nx), _I(ny), _I(nz),
                                                 _D(dx), _D(dy), _D(dz)))
    return (*outs, totals)


def compute_fpm_terms_nonuniform_3d(phi, u, v, w, ox, oy, oz, ax, ay, az, fluid, xc, yc, zc, dx, dy, dz, xlo, xhi,
                                    ylo, yhi, zlo, zhi, bounds, nx, ny, nz):
    """src/fpm_terms_3d.f90:39-88; returns (gx, gy, gz, vortex, advection, totals)."""
    _need(phi, (nx, ny, nz), np.float64, "phi")
    fl = _flow(nx, ny, nz, (u, v, w, ox, oy, oz, ax, ay, az))
    _need(fluid, (nx, ny, nz), np.int32, "fluid")
    axs = [_need(np.asarray(a), (n,), np.float64, nm) for a, n, nm in
           ((xc, nx, "xc"), (yc, ny, "yc"), (zc, nz, "zc"), (dx, nx, "dx"), (dy, ny, "dy"), (dz, nz, "dz"))]
    f = _faces(nx, ny, nz, (xlo, xhi, ylo, yhi, zlo, zhi))
    bd = np.ascontiguousarray(bounds, dtype=np.float64)
    outs = [np.empty((nx, ny, nz), order="F") for _ in range(5)]
    totals = np.zeros(2)
    check(lib().fpm_compute_fpm_terms_nonuniform_3d(_ptr(phi), *[_ptr(a) for a in fl], _ptr(fluid),
                                                    *[_ptr(a) for a in axs], *[_ptr(a) for a in f], _ptr(bd),
                                                    *[_ptr(o) for o in outs], _ptr(totals), _I(nx), _I(ny), _I(nz)))
    return (*outs, totals)
