"""Inputs of the reference's own test programs, restated in numpy.

Each builder follows the reference test it names (tests/*.f90 in the
reference repository) and returns plain numpy arrays in the Fortran layout
(order='F').  The same inputs feed the oracle pins (CPU) and the GPU parity
tests, so both sides always see identical bytes.
"""
from __future__ import annotations

import math

import numpy as np

import oracle as orc


def F(shape, dtype=np.float64):
    return np.zeros(shape, dtype=dtype, order="F")


def axes_from_global(gx, gy, gz):
    """Single-rank local axes (tests/fpm_test_grid.f90:31-43): centres with
    mirrored halo centres.  Each g is (face, center, width) of stretched_axis."""
    xc, dx = orc.local_axis(gx[1].size, gx[1], gx[2], 0, gx[1].size)
    yc, dy = orc.local_axis(gy[1].size, gy[1], gy[2], 0, gy[1].size)
    zc, dz = gz[1].copy(), gz[2].copy()
    return xc, yc, zc, dx, dy, dz


# ----------------------------------------------------------------------------
# tests/test_stairstep_exact_3d.f90
EXACT_G = np.array([0.3, -0.7, 0.5])


def exact_is_solid(i, j, k):
    """tests/test_stairstep_exact_3d.f90:99-105 (1-based global indices)."""
    return ((6 <= i <= 10 and 5 <= j <= 12 and 3 <= k <= 7)
            or (15 <= i <= 19 and 12 <= j <= 16 and 2 <= k <= 9)
            or (15 <= i <= 17 and 8 <= j <= 11 and 2 <= k <= 9)
            or (i >= 22 and j <= 3))


def stairstep_case_exact(exact: bool):
    """Inputs of run_case (tests/test_stairstep_exact_3d.f90:114-165) on one rank.

    exact=True: body and outer face gradients all equal g, so phi = g.x minus
    its fluid mean solves the discrete problem exactly.  exact=False: the FPM
    x influence field (body_grad = e_x, zero outer data)."""
    gnx, gny, nz = 24, 20, 10
    gx = orc.stretched_axis(gnx, 0.0, 1.2, 0.21)
    gy = orc.stretched_axis(gny, 0.0, 1.0, -0.17)
    gz = orc.stretched_axis(nz, 0.0, 0.5, 0.13)
    xc, yc, zc, dx, dy, dz = axes_from_global(gx, gy, gz)
    nx, ny = gnx, gny
    solid = F((nx + 2, ny + 2, nz), np.int32)
    for k in range(1, nz + 1):
        for j in range(1, ny + 1):
            for i in range(1, nx + 1):
                if exact_is_solid(i, j, k):
                    solid[i, j, k - 1] = 1
    orc.exchange_solid_halo_3d(solid)
    rhs = F((nx, ny, nz))
    phi = F((nx + 2, ny + 2, nz))
    if exact:
        g = EXACT_G
        body = g.copy()
        faces = [np.full((ny, nz), g[0], order="F"), np.full((ny, nz), g[0], order="F"),
                 np.full((nx, nz), g[1], order="F"), np.full((nx, nz), g[1], order="F"),
                 np.full((nx, ny), g[2], order="F"), np.full((nx, ny), g[2], order="F")]
    else:
        body = np.array([1.0, 0.0, 0.0])
        faces = [F((ny, nz)), F((ny, nz)), F((nx, nz)), F((nx, nz)), F((nx, ny)), F((nx, ny))]
    X = xc[1:nx + 1][:, None, None]
    Y = yc[1:ny + 1][None, :, None]
    Z = zc[None, None, :]
    one = np.ones((nx, ny, nz))
    flow = {
        "u": np.asfortranarray(1 + np.sin(3 * X) * np.cos(2 * Y) * one),
        "v": np.asfortranarray(0.5 * np.cos(X + Z) * one),
        "w": np.asfortranarray(0.2 * Y * one),
        "ox": np.asfortranarray(np.cos(4 * Z) * one),
        "oy": np.asfortranarray((-0.3 + X * Y) * one),
        "oz": np.asfortranarray(np.sin(5 * Y) * one),
        "ax": np.asfortranarray(0.1 * X * one),
        "ay": np.asfortranarray(-0.2 * one),
        "az": np.asfortranarray(Z * Y * one),
    }
    bounds = np.array([-1.0, 2.0, -1.0, 2.0, -1.0, 1.0])
    return dict(nx=nx, ny=ny, nz=nz, xc=xc, yc=yc, zc=zc, dx=dx, dy=dy, dz=dz, solid=solid, rhs=rhs, phi=phi,
                body=body, faces=faces, flow=flow, bounds=bounds)


def exact_expectations(c, phi, gx, gy, gz, vortex, totals):
    """Errors of tests/test_stairstep_exact_3d.f90:167-194: phi, gradient,
    vortex density and solid cells (Linf) and the closed-form integrals."""
    g = EXACT_G
    nx, ny, nz = c["nx"], c["ny"], c["nz"]
    xc, yc, zc, dx, dy, dz = c["xc"], c["yc"], c["zc"], c["dx"], c["dy"], c["dz"]
    solid = c["solid"][1:nx + 1, 1:ny + 1, :] != 0
    fluid = ~solid
    X = xc[1:nx + 1][:, None, None] * np.ones((nx, ny, nz))
    Y = yc[1:ny + 1][None, :, None] * np.ones((nx, ny, nz))
    Z = zc[None, None, :] * np.ones((nx, ny, nz))
    V = dx[:, None, None] * dy[None, :, None] * dz[None, None, :]
    lin = g[0] * X + g[1] * Y + g[2] * Z
    mean = (V * lin)[fluid].sum() / V[fluid].sum()
    p = phi[1:nx + 1, 1:ny + 1, :]
    fl = c["flow"]
    cx = fl["w"] * fl["oy"] - fl["v"] * fl["oz"]
    cy = fl["u"] * fl["oz"] - fl["w"] * fl["ox"]
    cz = fl["v"] * fl["ox"] - fl["u"] * fl["oy"]
    ev = -(cx * g[0] + cy * g[1] + cz * g[2])
    ea = -(fl["ax"] * g[0] + fl["ay"] * g[1] + fl["az"] * g[2])
    e_phi = np.abs(p - (lin - mean))[fluid].max()
    e_grad = max(np.abs(gx - g[0])[fluid].max(), np.abs(gy - g[1])[fluid].max(), np.abs(gz - g[2])[fluid].max())
    e_vort = np.abs(vortex - ev)[fluid].max()
    e_solid = max(np.abs(p)[solid].max(), np.abs(vortex)[solid].max(), np.abs(gx)[solid].max())
    expected = np.array([(V * ev)[fluid].sum(), (V * ea)[fluid].sum()])
    return np.array([e_phi, e_grad, e_vort, e_solid]), float(np.abs(totals - expected).max())


# ----------------------------------------------------------------------------
# tests/test_stairstep_sphere_3d.f90
SPHERE_A, SPHERE_HALF = 0.5, 1.5


def _dipole(x, y, z):
    a = SPHERE_A
    return -a ** 3 * x / (2 * np.sqrt(x * x + y * y + z * z) ** 3)


def _dipole_grad(axis, x, y, z):
    a = SPHERE_A
    r2 = x * x + y * y + z * z
    c = (x, y, z)[axis - 1]
    return -0.5 * a ** 3 * ((1.0 if axis == 1 else 0.0) / np.sqrt(r2) ** 3 - 3 * x * c / np.sqrt(r2) ** 5)


def sphere_case(n):
    """run_level inputs (tests/test_stairstep_sphere_3d.f90:59-94) on one rank."""
    g = orc.stretched_axis(n, -SPHERE_HALF, SPHERE_HALF, 0.0)
    xc, yc, zc, dx, dy, dz = axes_from_global(g, g, g)
    nx = ny = nz = n
    X = xc[1:nx + 1][:, None, None]
    Y = yc[1:ny + 1][None, :, None]
    Z = zc[None, None, :]
    solid = F((nx + 2, ny + 2, nz), np.int32)
    solid[1:nx + 1, 1:ny + 1, :] = (X ** 2 + Y ** 2 + Z ** 2 < SPHERE_A ** 2).astype(np.int32)
    orc.exchange_solid_halo_3d(solid)
    h = SPHERE_HALF
    yy, zz = np.meshgrid(yc[1:ny + 1], zc, indexing="ij")
    xx2, zz2 = np.meshgrid(xc[1:nx + 1], zc, indexing="ij")
    xx3, yy3 = np.meshgrid(xc[1:nx + 1], yc[1:ny + 1], indexing="ij")
    faces = [np.asfortranarray(_dipole_grad(1, -h, yy, zz)), np.asfortranarray(_dipole_grad(1, h, yy, zz)),
             np.asfortranarray(_dipole_grad(2, xx2, -h, zz2)), np.asfortranarray(_dipole_grad(2, xx2, h, zz2)),
             np.asfortranarray(_dipole_grad(3, xx3, yy3, -h)), np.asfortranarray(_dipole_grad(3, xx3, yy3, h))]
    return dict(nx=nx, ny=ny, nz=nz, xc=xc, yc=yc, zc=zc, dx=dx, dy=dy, dz=dz, solid=solid, rhs=F((nx, ny, nz)),
                phi=F((nx + 2, ny + 2, nz)), body=np.array([1.0, 0.0, 0.0]), faces=faces)


def sphere_errors(c, phi):
    """RMS error, far-field (r > 2a) max error and added-mass coefficient
    (tests/test_stairstep_sphere_3d.f90:95-125)."""
    nx, ny, nz = c["nx"], c["ny"], c["nz"]
    xc, yc, zc, dx, dy, dz = c["xc"], c["yc"], c["zc"], c["dx"], c["dy"], c["dz"]
    s = c["solid"]
    solid = s[1:nx + 1, 1:ny + 1, :] != 0
    fluid = ~solid
    X = xc[1:nx + 1][:, None, None] * np.ones((nx, ny, nz))
    Y = yc[1:ny + 1][None, :, None] * np.ones((nx, ny, nz))
    Z = zc[None, None, :] * np.ones((nx, ny, nz))
    V = dx[:, None, None] * dy[None, :, None] * dz[None, None, :]
    p = phi[1:nx + 1, 1:ny + 1, :]
    dip = _dipole(X, Y, Z)
    mean = (V * (p - dip))[fluid].sum() / V[fluid].sum()
    e = p - dip - mean
    r = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    rms = math.sqrt((V * e * e)[fluid].sum() / V[fluid].sum())
    far = np.abs(e)[fluid & (r > 2 * SPHERE_A)].max()
    A = dy[None, :, None] * dz[None, None, :] * np.ones((nx, ny, nz))
    east_solid = s[2:nx + 2, 1:ny + 1, :] != 0
    west_solid = s[0:nx, 1:ny + 1, :] != 0
    hdx = 0.5 * dx[:, None, None]
    c3 = (-(p + hdx) * A)[fluid & east_solid].sum() + ((p - hdx) * A)[fluid & west_solid].sum()
    cm = -c3 / (4 * math.pi * SPHERE_A ** 3 / 3)
    return rms, float(far), cm


# ----------------------------------------------------------------------------
# tests/test_fpm_3d.f90 (uniform grid, no body)
def manufactured_uniform():
    nx, ny, nz = 12, 10, 8
    dx, dy, dz = 1.0 / nx, 1.0 / ny, 1.0 / nz
    x = (np.arange(1, nx + 1) - 0.5) * dx
    y = (np.arange(1, ny + 1) - 0.5) * dy
    z = (np.arange(1, nz + 1) - 0.5) * dz
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    exact = ((X - .5) ** 2 + (Y - .5) ** 2 + (Z - .5) ** 2) / 6.0
    exact = exact - exact.sum() / (nx * ny * nz)
    return dict(nx=nx, ny=ny, nz=nz, dx=dx, dy=dy, dz=dz, X=X, Y=Y, Z=Z, exact=exact,
                rhs=np.ones((nx, ny, nz), order="F"), phi=F((nx + 2, ny + 2, nz + 2)),
                faces=[F((ny, nz)), F((ny, nz)), F((nx, nz)), F((nx, nz)), F((nx, ny)), F((nx, ny))])


# ----------------------------------------------------------------------------
# tests/test_fpm_3d_nonuniform.f90
def _make_axis(n, amplitude):
    m = np.arange(1, n + 1)
    weight = 1.0 + amplitude * np.sin(2.0 * math.acos(-1.0) * (m - 0.5) / n)
    scale = 1.0 / weight.sum()
    face = np.zeros(n + 1)
    center = np.zeros(n)
    width = np.zeros(n)
    for i in range(1, n + 1):
        width[i - 1] = scale * weight[i - 1]
        face[i] = face[i - 1] + width[i - 1]
        center[i - 1] = 0.5 * (face[i - 1] + face[i])
    return face, center, width


def _nu_field(x, y, z):
    return 0.2 * x * x + 0.3 * y * y - 0.1 * z * z + 0.4 * x - 0.2 * y + 0.3 * z


def _gradx(x):
    return 0.4 * x + 0.4


def _grady(y):
    return 0.6 * y - 0.2


def _gradz(z):
    return -0.2 * z + 0.3


def manufactured_nonuniform():
    nx, ny, nz = 13, 11, 9
    xf, xc, dx = _make_axis(nx, 0.23)
    yf, yc, dy = _make_axis(ny, -0.17)
    zf, zc, dz = _make_axis(nz, 0.19)
    X, Y, Z = np.meshgrid(xc, yc, zc, indexing="ij")
    exact = _nu_field(X, Y, Z)
    V = dx[:, None, None] * dy[None, :, None] * dz[None, None, :]
    exact = exact - (V * exact).sum() / V.sum()
    xlo = np.full((ny, nz), _gradx(xf[0]), order="F")
    xhi = np.full((ny, nz), _gradx(xf[nx]), order="F")
    ylo = np.full((nx, nz), _grady(yf[0]), order="F")
    yhi = np.full((nx, nz), _grady(yf[ny]), order="F")
    zlo = np.full((nx, ny), _gradz(zf[0]), order="F")
    zhi = np.full((nx, ny), _gradz(zf[nz]), order="F")
    rhs = F((nx, ny, nz))
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                e = exact
                gw = xlo[j, k] if i == 0 else (e[i, j, k] - e[i - 1, j, k]) / (xc[i] - xc[i - 1])
                ge = xhi[j, k] if i == nx - 1 else (e[i + 1, j, k] - e[i, j, k]) / (xc[i + 1] - xc[i])
                gs = ylo[i, k] if j == 0 else (e[i, j, k] - e[i, j - 1, k]) / (yc[j] - yc[j - 1])
                gn = yhi[i, k] if j == ny - 1 else (e[i, j + 1, k] - e[i, j, k]) / (yc[j + 1] - yc[j])
                gb = zlo[i, j] if k == 0 else (e[i, j, k] - e[i, j, k - 1]) / (zc[k] - zc[k - 1])
                gt = zhi[i, j] if k == nz - 1 else (e[i, j, k + 1] - e[i, j, k]) / (zc[k + 1] - zc[k])
                rhs[i, j, k] = (ge - gw) / dx[i] + (gn - gs) / dy[j] + (gt - gb) / dz[k]
    return dict(nx=nx, ny=ny, nz=nz, xf=xf, yf=yf, zf=zf, xc=xc, yc=yc, zc=zc, dx=dx, dy=dy, dz=dz, exact=exact,
                rhs=rhs, faces=[xlo, xhi, ylo, yhi, zlo, zhi])


def nonuniform_expected(c, fluid, bounds, gx, gy, gz, vf, af, totals):
    """Gradient, field and integral errors of tests/test_fpm_3d_nonuniform.f90:120-142."""
    nx, ny, nz = c["nx"], c["ny"], c["nz"]
    xf, yf, zf, xc, yc, zc = c["xf"], c["yf"], c["zf"], c["xc"], c["yc"], c["zc"]
    dx, dy, dz = c["dx"], c["dy"], c["dz"]
    ge_ = ef = 0.0
    et = np.zeros(2)
    cx = 3.0 * (-0.25) - 2.0 * 0.75
    cy = 1.0 * 0.75 - 3.0 * 0.5
    cz = 2.0 * 0.5 - 1.0 * (-0.25)
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                gw = _gradx(xf[0]) if i == 0 else _gradx(0.5 * (xc[i - 1] + xc[i]))
                gE = _gradx(xf[nx]) if i == nx - 1 else _gradx(0.5 * (xc[i] + xc[i + 1]))
                gs = _grady(yf[0]) if j == 0 else _grady(0.5 * (yc[j - 1] + yc[j]))
                gn = _grady(yf[ny]) if j == ny - 1 else _grady(0.5 * (yc[j] + yc[j + 1]))
                gb = _gradz(zf[0]) if k == 0 else _gradz(0.5 * (zc[k - 1] + zc[k]))
                gt = _gradz(zf[nz]) if k == nz - 1 else _gradz(0.5 * (zc[k] + zc[k + 1]))
                egx, egy, egz = 0.5 * (gw + gE), 0.5 * (gs + gn), 0.5 * (gb + gt)
                ev = -fluid[i, j, k] * (cx * egx + cy * egy + cz * egz)
                ea = -fluid[i, j, k] * (0.2 * egx - 0.1 * egy + 0.3 * egz)
                ge_ = max(ge_, abs(gx[i, j, k] - egx), abs(gy[i, j, k] - egy), abs(gz[i, j, k] - egz))
                ef = max(ef, abs(vf[i, j, k] - ev), abs(af[i, j, k] - ea))
                inside = (bounds[0] < xc[i] < bounds[1] and bounds[2] < yc[j] < bounds[3]
                          and bounds[4] < zc[k] < bounds[5])
                vol = (1.0 if inside else 0.0) * dx[i] * dy[j] * dz[k]
                et += vol * np.array([ev, ea])
    return ge_, ef, float(np.abs(totals - et).max())


# ----------------------------------------------------------------------------
# tests/test_fpm_partition_2d.f90
def partition_grid(n=160, half=2.0):
    xf, xcg, dxg = orc.stretched_axis(n, -half, half, 0.0)
    xc, dx = orc.local_axis(n, xcg, dxg, 0, n)
    return xf, xc, dx


def fill_ring(u, v):
    """ring(:,c,t) = [west column, east column, south row, north row] of u, v."""
    n1, n2 = u.shape
    ring = np.zeros((2 * n1 + 2 * n2, 2, 2), order="F")
    for t in range(2):
        ring[:, 0, t] = np.concatenate([u[0, :], u[n1 - 1, :], u[:, 0], u[:, n2 - 1]])
        ring[:, 1, t] = np.concatenate([v[0, :], v[n1 - 1, :], v[:, 0], v[:, n2 - 1]])
    return ring
