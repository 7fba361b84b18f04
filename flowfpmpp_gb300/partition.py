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


def partition_frames_2d(frames, tolerance=1e-10, max_sweeps=2000000, check_interval=50, return_phi=False):
    """Batched uneven 2-D frames: for each frame (dict with nx, ny, xf, yf, u,
    v, solid, ring, kin, dt and a shared nu) the reference foil example's
    phi_x, phi_y solve (examples/flapping_foil_fpm.f90:61-81) and
    fpm_partition_terms_2d for both directions, all frames together on the GPU.
    Returns (terms (nframes, 2, 4), sweeps (nframes, 2), residual (nframes, 2)
    [, phi list of (2, nx, ny) arrays])."""
    nf = len(frames)
    VP = ctypes.c_void_p
    keep = []

    def arr(a, dtype):
        a = np.asfortranarray(a, dtype=dtype)
        keep.append(a)
        return a.ctypes.data

    nx = np.array([f["nx"] for f in frames], dtype=np.int32)
    ny = np.array([f["ny"] for f in frames], dtype=np.int32)
    xf = (VP * nf)(*[arr(f["xf"], np.float64) for f in frames])
    yf = (VP * nf)(*[arr(f["yf"], np.float64) for f in frames])
    u = (VP * nf)(*[arr(f["u"], np.float64) for f in frames])
    v = (VP * nf)(*[arr(f["v"], np.float64) for f in frames])
    solid = (VP * nf)(*[arr(np.asarray(f["solid"]) != 0, np.uint8) for f in frames])
    ring = (VP * nf)(*[arr(f["ring"], np.float64) for f in frames])
    kin = np.ascontiguousarray(np.concatenate([np.asarray(f["kin"], dtype=np.float64) for f in frames]))
    dt = np.ascontiguousarray([float(f["dt"]) for f in frames])
    nu = float(frames[0]["nu"])
    terms = np.zeros((nf, 2, 4))
    sweeps = np.zeros((nf, 2), dtype=np.int32)
    res = np.zeros((nf, 2))
    phis = None
    phi_ptrs = None
    if return_phi:
        phis = [np.zeros((2, f["ny"], f["nx"])) for f in frames]
        phi_ptrs = (VP * nf)(*[p.ctypes.data for p in phis])
    check(lib().fpm_partition_frames_2d(_I(nf), _ptr(nx), _ptr(ny), xf, yf, u, v, solid, ring, _ptr(kin), _ptr(dt),
                                        _D(nu), _D(tolerance), _I(max_sweeps), _I(check_interval), _ptr(terms),
                                        _ptr(sweeps), _ptr(res), phi_ptrs))
    if return_phi:
        # (2, ny, nx) C-order buffers hold (nx, ny) Fortran-order planes
        phis = [np.stack([np.asfortranarray(p[r].T) for r in range(2)]) for p in phis]
        return terms, sweeps, res, phis
    return terms, sweeps, res


def fpm_partition_terms_3d(phi, g, u, v, w, solid, xf, yf, zf, kin, shell=None, dt=1.0, nu=0.0, slip_body=False):
    """3-D four-term partition (the 2-D scheme of src/fpm_partition_2d.f90 on
    six faces).  Returns (terms[4], vif_density (nx,ny,nz), omega (3,nx,ny,nz))."""
    nx, ny, nz = np.asarray(u).shape
    f64 = np.float64
    arrs = [_need(a, (nx, ny, nz), f64, n) for a, n in ((phi, "phi"), (u, "u"), (v, "v"), (w, "w"))]
    s8 = np.asfortranarray(np.asarray(solid) != 0, dtype=np.uint8)
    faces = [np.ascontiguousarray(a, dtype=f64) for a in (xf, yf, zf)]
    gg = np.ascontiguousarray(g, dtype=f64)
    kk = np.ascontiguousarray(kin, dtype=f64)
    if gg.shape != (3,) or kk.shape != (12,):
        raise ValueError("g has 3 entries and kin 12")
    sh = None if shell is None else np.asfortranarray(shell, dtype=f64)
    terms = np.zeros(4)
    vif = np.empty((nx, ny, nz), order="F")
    om = np.empty(3 * nx * ny * nz)
    check(lib().fpm_partition_terms_3d(*[_ptr(a) for a in (arrs[0], gg, arrs[1], arrs[2], arrs[3], s8, *faces, kk)],
                                       _ptr(sh) if sh is not None else None, _D(dt), _D(nu), _I(nx), _I(ny), _I(nz),
                                       _ptr(terms), _ptr(vif), _ptr(om), _I(int(bool(slip_body)))))
    omega = np.stack([om[a * nx * ny * nz:(a + 1) * nx * ny * nz].reshape((nx, ny, nz), order="F") for a in range(3)])
    return terms, vif, omega
