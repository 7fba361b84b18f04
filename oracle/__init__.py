"""ctypes bindings for the CPU oracle (``fpm_oracle.c``).

Test infrastructure only: tests, ``__graft_entry__.smoke()`` and ``bench.py``'s
CPU-baseline leg use this package to check and time results.  The product library
(``flowfpmpp_gb300``) never imports it.

Arrays follow the reference's Fortran layout, held in numpy arrays with
``order='F'`` and the Fortran shapes, e.g. ``phi`` is ``(nx+2, ny+2, nz)`` for
the stair-step solver (``phi[i, j, k-1]`` is Fortran ``phi(i,j,k)``), ``rhs``
is ``(nx, ny, nz)``, ``xlo`` is ``(ny, nz)``, ``xc`` is ``(nx+2,)``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liborc_fpm.so")
_lib = None

ERRORS = {
    1: "stair-step method must be pcg or jacobi",
    2: "stair-step solve needs nz>=2 and nonempty ranks",
    3: "stair-step fluid cell has no fluid neighbour",
    4: "stair-step compatibility needs at least one fluid outer face",
    5: "allocation failed",
}


class OracleError(RuntimeError):
    pass


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc -O2 -ffp-contract=off)."""
    src = os.path.join(_HERE, "fpm_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE, "-B" if force else "liborc_fpm.so"], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(_LIB_PATH)
        _lib.orc_operator_residual.restype = ctypes.c_double
        _lib.orc_stairstep_residual_3d.restype = ctypes.c_double
        _lib.orc_residual_norm_uniform.restype = ctypes.c_double
        _lib.orc_residual_nonuniform.restype = ctypes.c_double
    return _lib


def _p(a):
    """Pointer to a contiguous Fortran-ordered float64/int32/uint8 array."""
    if a is None:
        return None
    assert a.flags.f_contiguous, "oracle arrays must be Fortran-contiguous"
    return a.ctypes.data_as(ctypes.c_void_p)


def _f64(a):
    return np.asfortranarray(a, dtype=np.float64)


def _i32(a):
    return np.asfortranarray(a, dtype=np.int32)


def _check(code):
    if code != 0:
        raise OracleError(ERRORS.get(code, f"oracle error {code}"))


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def max_threads() -> int:
    return int(lib().orc_get_max_threads())


D = ctypes.c_double
I = ctypes.c_int


# ---------------------------------------------------------------- stair-step
def exchange_solid_halo_3d(solid):
    nx, ny, nz = solid.shape[0] - 2, solid.shape[1] - 2, solid.shape[2]
    lib().orc_exchange_solid_halo_3d(_p(solid), I(nx), I(ny), I(nz))


def enforce_stairstep_compatibility_3d(rhs, solid, body_grad, xlo, xhi, ylo, yhi, zlo, zhi, dx, dy, dz):
    """Shifts the six face arrays in place; returns (correction, imbalance)."""
    nx, ny, nz = rhs.shape
    c, m = D(), D()
    bg = _f64(body_grad)
    _check(lib().orc_enforce_stairstep_compatibility_3d(
        _p(rhs), _p(solid), _p(bg), _p(xlo), _p(xhi), _p(ylo), _p(yhi), _p(zlo), _p(zhi),
        _p(dx), _p(dy), _p(dz), I(nx), I(ny), I(nz), ctypes.byref(c), ctypes.byref(m)))
    return c.value, m.value


def solve_stairstep_poisson_3d(phi, rhs, solid, body_grad, xlo, xhi, ylo, yhi, zlo, zhi, xc, yc, zc, dx, dy, dz,
                               tolerance, max_sweeps, check_interval, method="pcg"):
    """Solves in place (phi is the initial guess); returns (sweeps, residual)."""
    nx, ny, nz = rhs.shape
    meth = {"pcg": 0, "jacobi": 1}.get(method, 99)
    sw, res = I(), D()
    bg = _f64(body_grad)
    _check(lib().orc_solve_stairstep_poisson_3d(
        _p(phi), _p(rhs), _p(solid), _p(bg), _p(xlo), _p(xhi), _p(ylo), _p(yhi), _p(zlo), _p(zhi),
        _p(xc), _p(yc), _p(zc), _p(dx), _p(dy), _p(dz), I(nx), I(ny), I(nz), D(tolerance), I(max_sweeps),
        I(check_interval), I(meth), ctypes.byref(sw), ctypes.byref(res)))
    return sw.value, res.value


def stairstep_residual_3d(phi, rhs, solid, body_grad, xlo, xhi, ylo, yhi, zlo, zhi, xc, yc, zc, dx, dy, dz):
    nx, ny, nz = rhs.shape
    bg = _f64(body_grad)
    return lib().orc_stairstep_residual_3d(
        _p(phi), _p(rhs), _p(solid), _p(bg), _p(xlo), _p(xhi), _p(ylo), _p(yhi), _p(zlo), _p(zhi),
        _p(xc), _p(yc), _p(zc), _p(dx), _p(dy), _p(dz), I(nx), I(ny), I(nz))


def compute_stairstep_fpm_terms_3d(phi, u, v, w, ox, oy, oz, ax, ay, az, solid, body_grad, xc, yc, zc, dx, dy, dz,
                                   xlo, xhi, ylo, yhi, zlo, zhi, bounds):
    """Returns (gx, gy, gz, vortex, advection, totals)."""
    nx, ny, nz = u.shape
    outs = [np.zeros((nx, ny, nz), order="F") for _ in range(5)]
    totals = np.zeros(2)
    bg, bd = _f64(body_grad), _f64(bounds)
    lib().orc_compute_stairstep_fpm_terms_3d(
        _p(phi), _p(u), _p(v), _p(w), _p(ox), _p(oy), _p(oz), _p(ax), _p(ay), _p(az), _p(solid), _p(bg),
        _p(xc), _p(yc), _p(zc), _p(dx), _p(dy), _p(dz), _p(xlo), _p(xhi), _p(ylo), _p(yhi), _p(zlo), _p(zhi),
        _p(bd), *[_p(o) for o in outs], _p(totals), I(nx), I(ny), I(nz))
    return (*outs, totals)


def stairstep_coefficients(xc, yc, zc, dx, dy, dz):
    nx, ny, nz = dx.size, dy.size, dz.size
    out = [np.zeros(n) for n in (nx, nx, ny, ny, nz, nz)]
    lib().orc_stairstep_coefficients(_p(xc), _p(yc), _p(zc), _p(dx), _p(dy), _p(dz), I(nx), I(ny), I(nz),
                                     *[_p(o) for o in out])
    return out


def build_operator(rhs, solid, body_grad, xlo, xhi, ylo, yhi, zlo, zhi, coefs, dx, dy, dz, for_pcg):
    """Returns (src, diag, rdiag, isolated)."""
    nx, ny, nz = rhs.shape
    src, diag, rdiag = (np.zeros((nx, ny, nz), order="F") for _ in range(3))
    bg = _f64(body_grad)
    iso = lib().orc_build_operator(_p(rhs), _p(solid), _p(bg), _p(xlo), _p(xhi), _p(ylo), _p(yhi), _p(zlo),
                                   _p(zhi), *[_p(c) for c in coefs], _p(dx), _p(dy), _p(dz), I(nx), I(ny), I(nz),
                                   I(int(for_pcg)), _p(src), _p(diag), _p(rdiag))
    return src, diag, rdiag, iso


def jacobi_sweep(a, b, src, rdiag, coefs):
    nx, ny, nz = src.shape
    lib().orc_jacobi_sweep(_p(a), _p(b), _p(src), _p(rdiag), *[_p(c) for c in coefs], I(nx), I(ny), I(nz))


def operator_residual(phi, src, diag, coefs):
    nx, ny, nz = src.shape
    return lib().orc_operator_residual(_p(phi), _p(src), _p(diag), *[_p(c) for c in coefs], I(nx), I(ny), I(nz))


# ---------------------------------------------------------------- fpm_laplace_3d / fpm_terms_3d
def enforce_neumann_compatibility_3d(rhs, xlo, xhi, ylo, yhi, zlo, zhi, dx, dy, dz):
    nx, ny, nz = rhs.shape
    c, m = D(), D()
    lib().orc_enforce_neumann_compatibility_3d(_p(rhs), _p(xlo), _p(xhi), _p(ylo), _p(yhi), _p(zlo), _p(zhi),
                                               I(nx), I(ny), I(nz), D(dx), D(dy), D(dz), ctypes.byref(c),
                                               ctypes.byref(m))
    return c.value, m.value


def solve_neumann_poisson_3d(phi, rhs, xlo, xhi, ylo, yhi, zlo, zhi, dx, dy, dz, tolerance, max_iterations,
                             check_interval):
    nx, ny, nz = rhs.shape
    it, res = I(), D()
    lib().orc_solve_neumann_poisson_3d(_p(phi), _p(rhs), _p(xlo), _p(xhi), _p(ylo), _p(yhi), _p(zlo), _p(zhi),
                                       I(nx), I(ny), I(nz), D(dx), D(dy), D(dz), D(tolerance), I(max_iterations),
                                       I(check_interval), ctypes.byref(it), ctypes.byref(res))
    return it.value, res.value


def enforce_neumann_compatibility_nonuniform_3d(rhs, xlo, xhi, ylo, yhi, zlo, zhi, dx, dy, dz):
    nx, ny, nz = rhs.shape
    c, m = D(), D()
    lib().orc_enforce_neumann_compatibility_nonuniform_3d(_p(rhs), _p(xlo), _p(xhi), _p(ylo), _p(yhi), _p(zlo),
                                                          _p(zhi), _p(dx), _p(dy), _p(dz), I(nx), I(ny), I(nz),
                                                          ctypes.byref(c), ctypes.byref(m))
    return c.value, m.value


def solve_neumann_poisson_nonuniform_3d(phi, rhs, xlo, xhi, ylo, yhi, zlo, zhi, xc, yc, zc, dx, dy, dz, tolerance,
                                        max_iterations, check_interval):
    nx, ny, nz = rhs.shape
    it, res = I(), D()
    lib().orc_solve_neumann_poisson_nonuniform_3d(_p(phi), _p(rhs), _p(xlo), _p(xhi), _p(ylo), _p(yhi), _p(zlo),
                                                  _p(zhi), _p(xc), _p(yc), _p(zc), _p(dx), _p(dy), _p(dz), I(nx),
                                                  I(ny), I(nz), D(tolerance), I(max_iterations), I(check_interval),
                                                  ctypes.byref(it), ctypes.byref(res))
    return it.value, res.value


def compute_fpm_terms_uniform_3d(phi, u, v, w, ox, oy, oz, ax, ay, az, fluid, dx, dy, dz):
    nx, ny, nz = u.shape
    outs = [np.zeros((nx, ny, nz), order="F") for _ in range(5)]
    totals = np.zeros(2)
    lib().orc_compute_fpm_terms_uniform_3d(_p(phi), _p(u), _p(v), _p(w), _p(ox), _p(oy), _p(oz), _p(ax), _p(ay),
                                           _p(az), _p(fluid), *[_p(o) for o in outs], _p(totals), I(nx), I(ny),
                                           I(nz), D(dx), D(dy), D(dz))
    return (*outs, totals)


def compute_fpm_terms_nonuniform_3d(phi, u, v, w, ox, oy, oz, ax, ay, az, fluid, xc, yc, zc, dx, dy, dz, xlo, xhi,
                                    ylo, yhi, zlo, zhi, bounds):
    nx, ny, nz = u.shape
    outs = [np.zeros((nx, ny, nz), order="F") for _ in range(5)]
    totals = np.zeros(2)
    bd = _f64(bounds)
    _check(lib().orc_compute_fpm_terms_nonuniform_3d(
        _p(phi), _p(u), _p(v), _p(w), _p(ox), _p(oy), _p(oz), _p(ax), _p(ay), _p(az), _p(fluid), _p(xc), _p(yc),
        _p(zc), _p(dx), _p(dy), _p(dz), _p(xlo), _p(xhi), _p(ylo), _p(yhi), _p(zlo), _p(zhi), _p(bd),
        *[_p(o) for o in outs], _p(totals), I(nx), I(ny), I(nz)))
    return (*outs, totals)


# ---------------------------------------------------------------- fpm_partition_2d
def fpm_partition_terms_2d(phi, g, u, v, solid, xf, yf, kin, ring, dt, nu, slip_body=False):
    """Returns (terms[4], vif_density, omega)."""
    nx, ny = u.shape
    terms = np.zeros(4)
    vif = np.zeros((nx, ny), order="F")
    omega = np.zeros((nx, ny), order="F")
    s8 = np.asfortranarray(solid, dtype=np.uint8)
    gg, kk = _f64(g), _f64(kin)
    _check(lib().orc_fpm_partition_terms_2d(_p(phi), _p(gg), _p(u), _p(v), _p(s8), _p(xf), _p(yf), _p(kk),
                                            _p(ring), D(dt), D(nu), I(nx), I(ny), _p(terms), _p(vif), _p(omega),
                                            I(int(bool(slip_body)))))
    return terms, vif, omega


# ---------------------------------------------------------------- test-grid helpers
def stretched_axis(n, lo, hi, amplitude):
    face, center, width = np.zeros(n + 1), np.zeros(n), np.zeros(n)
    lib().orc_stretched_axis(I(n), D(lo), D(hi), D(amplitude), _p(face), _p(center), _p(width))
    return face, center, width


def local_axis(gn, gcenter, gwidth, offset, n):
    center, width = np.zeros(n + 2), np.zeros(n)
    lib().orc_local_axis(I(gn), _p(_f64(gcenter)), _p(_f64(gwidth)), I(offset), I(n), _p(center), _p(width))
    return center, width


def fpm_partition_terms_3d(phi, g, u, v, w, solid, xf, yf, zf, kin, shell, dt, nu, slip_body=False):
    """3-D four-term partition; returns (terms[4], vif_density, omega (3,nx,ny,nz))."""
    nx, ny, nz = u.shape
    terms = np.zeros(4)
    vif = np.zeros((nx, ny, nz), order="F")
    omega = np.zeros((3, nx, ny, nz))
    om = np.zeros(3 * nx * ny * nz)
    s8 = np.asfortranarray(solid, dtype=np.uint8)
    gg, kk = _f64(g), _f64(kin)
    sh = None if shell is None else _f64(shell)
    _check(lib().orc_fpm_partition_terms_3d(_p(phi), _p(gg), _p(u), _p(v), _p(w), _p(s8), _p(_f64(xf)), _p(_f64(yf)),
                                            _p(_f64(zf)), _p(kk), _p(sh) if sh is not None else None, D(dt), D(nu),
                                            I(nx), I(ny), I(nz), _p(terms), _p(vif),
                                            om.ctypes.data_as(ctypes.c_void_p), I(int(bool(slip_body)))))
    for a in range(3):
        omega[a] = om[a * nx * ny * nz:(a + 1) * nx * ny * nz].reshape((nx, ny, nz), order="F")
    return terms, vif, omega
