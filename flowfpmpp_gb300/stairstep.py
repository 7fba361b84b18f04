"""Host-side mirror of the reference module ``fpm_stairstep_mpi_3d``.

Same procedure names, argument order and meaning as
src/fpm_stairstep_mpi_3d.f90, for one rank on one GPU (no west/east/south/north
or comm arguments: every side is a physical boundary).  Arrays are numpy
arrays in the reference's Fortran layout (``order='F'`` with the Fortran
shapes): ``phi`` and ``solid`` are ``(nx+2, ny+2, nz)``, interior fields
``(nx, ny, nz)``, ``xlo`` ``(ny, nz)``, ``ylo`` ``(nx, nz)``, ``zlo``
``(nx, ny)``, ``xc`` ``(nx+2,)``, ``zc`` ``(nz,)``.  Arguments updated in
place by the reference (``phi``, the face arrays in compatibility, the solid
halo) are updated in place here.  Errors raise :class:`FpmError` where the
reference stops with ``error stop``.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import check, lib

METHODS = {"pcg": 0, "jacobi": 1, "jacobi_df": 2, "pcg_mixed": 3, "pcg_mg": 4, "fcg_learned": 5, "jacobi_fma": 6, "jacobi_tf": 7}

_D = ctypes.c_double
_I = ctypes.c_int


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _need(a, shape, dtype, name, writable=False):
    if not isinstance(a, np.ndarray):
        raise TypeError(f"{name} must be a numpy array")
    if a.dtype != dtype:
        raise TypeError(f"{name} must be {np.dtype(dtype).name}, got {a.dtype}")
    if tuple(a.shape) != tuple(shape):
        raise ValueError(f"{name} has shape {a.shape}, expected {tuple(shape)}")
    if not a.flags.f_contiguous:
        raise ValueError(f"{name} must be Fortran-contiguous (order='F')")
    if writable and not a.flags.writeable:
        raise ValueError(f"{name} must be writable")
    return a


def _bg(body_grad):
    b = np.ascontiguousarray(body_grad, dtype=np.float64)
    if b.shape != (3,):
        raise ValueError("body_grad must have 3 entries")
    return b


def _faces(nx, ny, nz, xlo, xhi, ylo, yhi, zlo, zhi, writable=False):
    f64 = np.float64
    return [_need(xlo, (ny, nz), f64, "xlo", writable), _need(xhi, (ny, nz), f64, "xhi", writable),
            _need(ylo, (nx, nz), f64, "ylo", writable), _need(yhi, (nx, nz), f64, "yhi", writable),
            _need(zlo, (nx, ny), f64, "zlo", writable), _need(zhi, (nx, ny), f64, "zhi", writable)]


def _axes(nx, ny, nz, xc, yc, zc, dx, dy, dz):
    f64 = np.float64
    return [_need(np.asarray(xc), (nx + 2,), f64, "xc"), _need(np.asarray(yc), (ny + 2,), f64, "yc"),
            _need(np.asarray(zc), (nz,), f64, "zc"), _need(np.asarray(dx), (nx,), f64, "dx"),
            _need(np.asarray(dy), (ny,), f64, "dy"), _need(np.asarray(dz), (nz,), f64, "dz")]


def exchange_solid_halo_3d(solid):
    """src/fpm_stairstep_mpi_3d.f90:25-36: zero the physical halo of ``solid``."""
    nx, ny, nz = solid.shape[0] - 2, solid.shape[1] - 2, solid.shape[2]
    _need(solid, (nx + 2, ny + 2, nz), np.int32, "solid", True)
    check(lib().fpm_exchange_solid_halo_3d(_ptr(solid), _I(nx), _I(ny), _I(nz)))


def enforce_stairstep_compatibility_3d(rhs, solid, body_grad, xlo, xhi, ylo, yhi, zlo, zhi, dx, dy, dz):
    """src/fpm_stairstep_mpi_3d.f90:41-92.  Shifts the face arrays in place and
    returns ``(correction, imbalance)``."""
    nx, ny, nz = rhs.shape
    _need(rhs, (nx, ny, nz), np.float64, "rhs")
    _need(solid, (nx + 2, ny + 2, nz), np.int32, "solid")
    faces = _faces(nx, ny, nz, xlo, xhi, ylo, yhi, zlo, zhi, True)
    ax = [_need(np.asarray(dx), (nx,), np.float64, "dx"), _need(np.asarray(dy), (ny,), np.float64, "dy"),
          _need(np.asarray(dz), (nz,), np.float64, "dz")]
    bg = _bg(body_grad)
    c, m = _D(), _D()
    check(lib().fpm_enforce_stairstep_compatibility_3d(
        _ptr(rhs), _ptr(solid), _ptr(bg), *[_ptr(f) for f in faces], *[_ptr(a) for a in ax],
        _I(nx), _I(ny), _I(nz), ctypes.byref(c), ctypes.byref(m)))
    return c.value, m.value


def solve_stairstep_poisson_3d(phi, rhs, solid, body_grad, xlo, xhi, ylo, yhi, zlo, zhi, xc, yc, zc, dx, dy, dz,
                               tolerance, max_sweeps, check_interval, method="pcg"):
    """src/fpm_stairstep_mpi_3d.f90:106-330.  Solves in place (``phi`` is the
    initial guess) and returns ``(sweeps, residual)``.  ``method`` is 'pcg'
    (default), 'jacobi', 'jacobi_fma' (the same weighted Jacobi in FP64 with
    fused multiply-adds), 'jacobi_tf' (FP64 storage, triple-float arithmetic),
    'jacobi_df' (in double-float arithmetic),
    'pcg_mixed' (FP32 PCG inside FP64 iterative refinement) or 'pcg_mg' (the
    refinement with a multigrid-preconditioned FP32 PCG)."""
    nx, ny, nz = rhs.shape
    _need(phi, (nx + 2, ny + 2, nz), np.float64, "phi", True)
    _need(rhs, (nx, ny, nz), np.float64, "rhs")
    _need(solid, (nx + 2, ny + 2, nz), np.int32, "solid")
    faces = _faces(nx, ny, nz, xlo, xhi, ylo, yhi, zlo, zhi)
    axes = _axes(nx, ny, nz, xc, yc, zc, dx, dy, dz)
    bg = _bg(body_grad)
    meth = METHODS.get(method, -1)
    sw, res = _I(), _D()
    check(lib().fpm_solve_stairstep_poisson_3d(
        _ptr(phi), _ptr(rhs), _ptr(solid), _ptr(bg), *[_ptr(f) for f in faces], *[_ptr(a) for a in axes],
        _I(nx), _I(ny), _I(nz), _D(tolerance), _I(max_sweeps), _I(check_interval), _I(meth),
        ctypes.byref(sw), ctypes.byref(res)))
    return sw.value, res.value


def stairstep_residual_3d(phi, rhs, solid, body_grad, xlo, xhi, ylo, yhi, zlo, zhi, xc, yc, zc, dx, dy, dz):
    """src/fpm_stairstep_mpi_3d.f90:403-419: independent max-norm residual."""
    nx, ny, nz = rhs.shape
    _need(phi, (nx + 2, ny + 2, nz), np.float64, "phi")
    _need(rhs, (nx, ny, nz), np.float64, "rhs")
    _need(solid, (nx + 2, ny + 2, nz), np.int32, "solid")
    faces = _faces(nx, ny, nz, xlo, xhi, ylo, yhi, zlo, zhi)
    axes = _axes(nx, ny, nz, xc, yc, zc, dx, dy, dz)
    bg = _bg(body_grad)
    v = _D()
    check(lib().fpm_stairstep_residual_3d(
        _ptr(phi), _ptr(rhs), _ptr(solid), _ptr(bg), *[_ptr(f) for f in faces], *[_ptr(a) for a in axes],
        _I(nx), _I(ny), _I(nz), ctypes.byref(v)))
    return v.value


def compute_stairstep_fpm_terms_3d(phi, u, v, w, ox, oy, oz, ax, ay, az, solid, body_grad, xc, yc, zc, dx, dy, dz,
                                   xlo, xhi, ylo, yhi, zlo, zhi, bounds):
    """src/fpm_stairstep_mpi_3d.f90:426-469.  Returns
    ``(gx, gy, gz, vortex, advection, totals)``."""
    nx, ny, nz = u.shape
    f64 = np.float64
    _need(phi, (nx + 2, ny + 2, nz), f64, "phi")
    flow = [_need(a, (nx, ny, nz), f64, n) for a, n in
            zip((u, v, w, ox, oy, oz, ax, ay, az), ("u", "v", "w", "ox", "oy", "oz", "ax", "ay", "az"))]
    _need(solid, (nx + 2, ny + 2, nz), np.int32, "solid")
    axes = _axes(nx, ny, nz, xc, yc, zc, dx, dy, dz)
    faces = _faces(nx, ny, nz, xlo, xhi, ylo, yhi, zlo, zhi)
    bg = _bg(body_grad)
    bd = np.ascontiguousarray(bounds, dtype=f64)
    if bd.shape != (6,):
        raise ValueError("bounds must have 6 entries")
    outs = [np.empty((nx, ny, nz), order="F") for _ in range(5)]
    totals = np.zeros(2)
    check(lib().fpm_compute_stairstep_fpm_terms_3d(
        _ptr(phi), *[_ptr(a) for a in flow], _ptr(solid), _ptr(bg), *[_ptr(a) for a in axes],
        *[_ptr(f) for f in faces], _ptr(bd), *[_ptr(o) for o in outs], _ptr(totals), _I(nx), _I(ny), _I(nz)))
    return (*outs, totals)
