"""Seeded synthetic workloads with the shapes of the benchmark configurations.

Every generator returns plain numpy arrays in the reference's Fortran layout
(order='F'), ready for the stair-step API: axes with mirrored halo centres
(xc(0:nx+1)), a padded int32 solid flag with a zero physical halo, zero
outer-face data, rhs = 0 and body_grad = e_axis (the FPM influence problem).

Configurations (sizes in cells):
  c1  64x64x32 on [-4,4]^2 x [-2,2], geometric ratio 1.03 away from the
      centre planes, sphere r=0.5 at the origin; flow = U=1 + 8 Gaussian
      z-tubes (core 0.2, circulation N(0,1)), acceleration = 6 Fourier modes.
  c2  256^3, ratio 1.01, four seeded axis-aligned boxes of 8-40 cells per
      side, one touching the outer boundary; phi_x right-hand side.
  c3  384x384x192, ratio 1.02 from a smallest cell of 0.01 at the centre
      planes (so [-21.8,21.8]^2 x [-2.85,2.85]), union of 3 random ellipsoids
      (semi-axes 0.3-1.0, random orientation).
  c4  uneven 2-D foil frames, ratio 1.02 from a smallest cell of 0.01, the
      domain widened to at least [-4,4]^2 for small frames.

The smallest cell fixes the FP64 rounding floor of the solver's convergence
measure, max |src + sum c phi_nb - diag phi|: its terms are of size
diag |phi| ~ 6 |phi| / w^2, so w = 0.01 puts the floor near 1e-12, below the
1e-10 tolerance, while w = 0.0018 (384 cells of ratio 1.02 squeezed into
[-4,4]) puts it at about 1e-10 and no FP64 solver can meet the tolerance.
"""
from __future__ import annotations

import math

import numpy as np


def geometric_axis(n: int, lo: float, hi: float, ratio: float):
    """n cells on [lo, hi], widths growing by `ratio` per cell away from the
    centre plane (symmetric).  Returns (faces(0:n), centres(0:n+1) with
    mirrored halo centres, widths(1:n))."""
    half = n // 2
    if n % 2 == 0:
        side = ratio ** np.arange(half)
        w = np.concatenate([side[::-1], side])
    else:
        side = ratio ** np.arange(1, half + 1)
        w = np.concatenate([side[::-1], [1.0], side])
    w = w * (hi - lo) / w.sum()
    faces = lo + np.concatenate([[0.0], np.cumsum(w)])
    faces[-1] = hi
    c = 0.5 * (faces[:-1] + faces[1:])
    centres = np.concatenate([[c[0] - w[0]], c, [c[-1] + w[-1]]])
    return faces, centres, w


def geometric_axis_w0(n: int, w0: float, ratio: float, min_half: float = 0.0):
    """n cells symmetric about 0, the two centre cells of width w0 and widths
    growing by `ratio` per cell outward; if that spans less than
    [-min_half, min_half] the axis is rescaled to exactly that interval."""
    half = n // 2
    side = ratio ** np.arange(half) if n % 2 == 0 else ratio ** np.arange(1, half + 1)
    extent = w0 * (2 * side.sum() + (0 if n % 2 == 0 else 1.0))
    h = max(0.5 * extent, min_half)
    return geometric_axis(n, -h, h, ratio)


def _empty_faces(nx, ny, nz):
    z = lambda a, b: np.zeros((a, b), order="F")
    return [z(ny, nz), z(ny, nz), z(nx, nz), z(nx, nz), z(nx, ny), z(nx, ny)]


def _frame(nx, ny, nz, ax, ay, az, solid_interior, axis):
    solid = np.zeros((nx + 2, ny + 2, nz), dtype=np.int32, order="F")
    solid[1:nx + 1, 1:ny + 1, :] = solid_interior
    body = np.zeros(3)
    body[axis] = 1.0
    return dict(nx=nx, ny=ny, nz=nz, xf=ax[0], yf=ay[0], zf=az[0], xc=ax[1], yc=ay[1], zc=az[1][1:nz + 1].copy(),
                dx=ax[2], dy=ay[2], dz=az[2], solid=solid, rhs=np.zeros((nx, ny, nz), order="F"),
                phi=np.zeros((nx + 2, ny + 2, nz), order="F"), body=body, faces=_empty_faces(nx, ny, nz))


def boxes_grid(n=256, seed=2025, ratio=1.01, half=4.0, nboxes=4):
    """Weighted-Jacobi bandwidth case: n^3 grid, four axis-aligned boxes of 8-40 cells per side at
    seeded positions, the first one touching the outer boundary (x = -half).  On grids below 160
    cells per side the sides are capped at n/4 so that every box fits."""
    rng = np.random.default_rng(seed)
    ax = geometric_axis(n, -half, half, ratio)
    solid = np.zeros((n, n, n), dtype=np.int32)
    for b in range(nboxes):
        size = np.minimum(rng.integers(8, 41, size=3), max(1, n // 4))
        lo = np.array([rng.integers(0, n - s + 1) for s in size])
        if b == 0:
            lo[0] = 0  # touches the west boundary
        else:
            lo = np.clip(lo, 1, n - 1 - size)
        solid[lo[0]:lo[0] + size[0], lo[1]:lo[1] + size[1], lo[2]:lo[2] + size[2]] = 1
    return _frame(n, n, n, ax, ax, ax, solid, 0)


def sphere_grid(nx=64, ny=64, nz=32, ratio=1.03, radius=0.5, axis=0):
    """Plain-PCG case: stretched grid on [-4,4]^2 x [-2,2], sphere at the origin."""
    ax = geometric_axis(nx, -4.0, 4.0, ratio)
    ay = geometric_axis(ny, -4.0, 4.0, ratio)
    az = geometric_axis(nz, -2.0, 2.0, ratio)
    X = ax[1][1:nx + 1][:, None, None]
    Y = ay[1][1:ny + 1][None, :, None]
    Z = az[1][1:nz + 1][None, None, :]
    solid = ((X ** 2 + Y ** 2 + Z ** 2) < radius ** 2).astype(np.int32)
    return _frame(nx, ny, nz, ax, ay, az, solid, axis)


def _rotation(rng):
    q = rng.standard_normal(4)
    q /= np.linalg.norm(q)
    a, b, c, d = q
    return np.array([[a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
                     [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
                     [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])


def ellipsoids_grid(nx=384, ny=384, nz=192, ratio=1.02, seed=3, count=3, axis=0, w0=0.01):
    """Three-potential PCG case: union of `count` random ellipsoids (semi-axes 0.3-1.0, random
    orientation, centres within 1.0 of the origin, 0.5 in z) on axes of
    smallest cell w0 (at least [-2,2] in z)."""
    rng = np.random.default_rng(seed)
    ax = geometric_axis_w0(nx, w0, ratio, 2.0)
    ay = geometric_axis_w0(ny, w0, ratio, 2.0)
    az = geometric_axis_w0(nz, w0, ratio, 2.0)
    X = ax[1][1:nx + 1][:, None, None]
    Y = ay[1][1:ny + 1][None, :, None]
    Z = az[1][1:nz + 1][None, None, :]
    solid = np.zeros((nx, ny, nz), dtype=bool)
    for _ in range(count):
        semi = rng.uniform(0.3, 1.0, 3)
        cen = rng.uniform(-1.0, 1.0, 3) * np.array([1.0, 1.0, 0.5])
        R = _rotation(rng)
        dX, dY, dZ = X - cen[0], Y - cen[1], Z - cen[2]
        q = 0.0
        for r in range(3):
            comp = R[0, r] * dX + R[1, r] * dY + R[2, r] * dZ
            q = q + (comp / semi[r]) ** 2
        solid |= q < 1.0
    return _frame(nx, ny, nz, ax, ay, az, solid.astype(np.int32), axis)


def flow_c1(frame, seed=11, ntubes=8, core=0.2, nmodes=6):
    """Velocity U=1 plus `ntubes` z-aligned Gaussian (Lamb-Oseen) vortex tubes
    with centres uniform in the fluid and circulation N(0,1), analytic
    vorticity; acceleration = sum of `nmodes` Fourier modes with wavenumbers
    1-3 and amplitudes N(0, 0.1)."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = frame["nx"], frame["ny"], frame["nz"]
    X = frame["xc"][1:nx + 1][:, None, None] * np.ones((nx, ny, nz))
    Y = frame["yc"][1:ny + 1][None, :, None] * np.ones((nx, ny, nz))
    Z = frame["zc"][None, None, :] * np.ones((nx, ny, nz))
    fluid = frame["solid"][1:nx + 1, 1:ny + 1, :] == 0
    u = np.ones((nx, ny, nz))
    v = np.zeros((nx, ny, nz))
    w = np.zeros((nx, ny, nz))
    oz = np.zeros((nx, ny, nz))
    fx, fy = X[fluid], Y[fluid]
    for _ in range(ntubes):
        m = rng.integers(0, fx.size)
        x0, y0 = fx[m], fy[m]
        gam = rng.standard_normal()
        r2 = (X - x0) ** 2 + (Y - y0) ** 2
        r2s = np.where(r2 > 0, r2, 1.0)
        vt = gam / (2 * math.pi) * (1 - np.exp(-r2 / core ** 2)) / r2s
        vt = np.where(r2 > 0, vt, 0.0)
        u += -vt * (Y - y0)
        v += vt * (X - x0)
        oz += gam / (math.pi * core ** 2) * np.exp(-r2 / core ** 2)
    ox = np.zeros((nx, ny, nz))
    oy = np.zeros((nx, ny, nz))
    acc = [np.zeros((nx, ny, nz)) for _ in range(3)]
    for _ in range(nmodes):
        k = rng.integers(1, 4, size=3) * rng.choice([-1, 1], size=3)
        ph = rng.uniform(0, 2 * math.pi)
        amp = rng.normal(0, 0.1, size=3)
        arg = np.sin(k[0] * X + k[1] * Y + k[2] * Z + ph)
        for c in range(3):
            acc[c] += amp[c] * arg
    F = lambda a: np.asfortranarray(a)
    return dict(u=F(u), v=F(v), w=F(w), ox=F(ox), oy=F(oy), oz=F(oz), ax=F(acc[0]), ay=F(acc[1]), az=F(acc[2]))


def foil_frames(nframes=256, seed=4, nmin=96, nmax=512, ratio=1.02, half_x=4.0, half_y=4.0, nvort=12,
                   dt=0.4, nu=1e-4, w0=0.01):
    """Batched-frames case: uneven 2-D frames in the fpm_partition_2d form.  Each frame:
    nx, ny ~ U[nmin, nmax], geometric stretching `ratio` away from the centre
    lines from a smallest cell w0, the domain at least [-half_x, half_x] x
    [-half_y, half_y]; vortex centres lie in that box; an elliptic foil (chord 1, thickness 0.12) at pitch U[-30, 30]
    degrees and heave U[-0.5, 0.5], blocked by cell centre; rigid-body
    kinematics kin ~ N(0,1); velocity U=1 plus `nvort` Lamb-Oseen vortices
    (circulation N(0,1), core U[0.05, 0.2]); the outer ring at t -/+ dt is
    the frame's ring perturbed by N(0, 0.01 dt)."""
    rng = np.random.default_rng(seed)
    frames = []
    for _ in range(nframes):
        nx, ny = (int(v) for v in rng.integers(nmin, nmax + 1, size=2))
        xf, xc, dx = geometric_axis_w0(nx, w0, ratio, half_x)
        yf, yc, dy = geometric_axis_w0(ny, w0, ratio, half_y)
        X = xc[1:nx + 1][:, None] * np.ones((nx, ny))
        Y = yc[1:ny + 1][None, :] * np.ones((nx, ny))
        pitch = math.radians(rng.uniform(-30, 30))
        heave = rng.uniform(-0.5, 0.5)
        cp, sp = math.cos(pitch), math.sin(pitch)
        xr = cp * X + sp * (Y - heave)
        yr = -sp * X + cp * (Y - heave)
        solid = ((xr / 0.5) ** 2 + (yr / 0.06) ** 2 < 1.0).astype(np.uint8)
        if solid.sum() == 0:  # keep at least one blocked cell at the foil centre
            solid[np.argmin(np.abs(xc[1:nx + 1])), np.argmin(np.abs(yc[1:ny + 1] - heave))] = 1
        u = np.ones((nx, ny))
        v = np.zeros((nx, ny))
        for _ in range(nvort):
            x0, y0 = rng.uniform(-half_x, half_x), rng.uniform(-half_y, half_y)
            gam, rc = rng.standard_normal(), rng.uniform(0.05, 0.2)
            r2 = (X - x0) ** 2 + (Y - y0) ** 2
            fac = np.where(r2 > 0, gam / (2 * math.pi) * (1 - np.exp(-r2 / rc ** 2)) / np.where(r2 > 0, r2, 1.0), 0.0)
            u -= fac * (Y - y0)
            v += fac * (X - x0)
        fluid = solid == 0
        u *= fluid
        v *= fluid
        ring = np.zeros((2 * nx + 2 * ny, 2, 2), order="F")
        base_u = np.concatenate([u[0, :], u[nx - 1, :], u[:, 0], u[:, ny - 1]])
        base_v = np.concatenate([v[0, :], v[nx - 1, :], v[:, 0], v[:, ny - 1]])
        for t, sgn in ((0, -1.0), (1, 1.0)):
            ring[:, 0, t] = base_u + sgn * rng.normal(0, 0.01 * dt, base_u.size)
            ring[:, 1, t] = base_v + sgn * rng.normal(0, 0.01 * dt, base_v.size)
        frames.append(dict(nx=nx, ny=ny, xf=xf, yf=yf, xc=xc, yc=yc, dx=dx, dy=dy,
                           solid=np.asfortranarray(solid), u=np.asfortranarray(u), v=np.asfortranarray(v),
                           ring=ring, kin=rng.standard_normal(6), dt=dt, nu=nu))
    return frames


def foil_series(nframes=6, nx=192, ny=160, seed=7, ratio=1.02, half_x=4.0, half_y=4.0, nvort=8, dt=0.05,
                period=2.0, w0=0.01):
    """A time series of 2-D dumps on one grid (FFPM2D02 frame dicts with
    `time`): an elliptic foil (chord 1, thickness 0.12) pitching 20 deg sin(w t)
    and heaving 0.3 sin(w t + 1) (w = 2 pi / period), velocity U = 1 plus
    `nvort` Lamb-Oseen vortices carried downstream at U = 1; dumps every dt,
    each frame's outer ring holding the boundary cells' u, v of the same field
    at t -/+ dt (so interior frames' rings equal their neighbours' boundary
    cells); kin from the analytic rigid-body motion."""
    rng = np.random.default_rng(seed)
    xf, xc, dx = geometric_axis_w0(nx, w0, ratio, half_x)
    yf, yc, dy = geometric_axis_w0(ny, w0, ratio, half_y)
    X = xc[1:nx + 1][:, None] * np.ones((nx, ny))
    Y = yc[1:ny + 1][None, :] * np.ones((nx, ny))
    vort = [(rng.uniform(-half_x, half_x), rng.uniform(-half_y, half_y), rng.standard_normal(), rng.uniform(0.05, 0.2))
            for _ in range(nvort)]
    w = 2 * math.pi / period
    amp_p, amp_h = math.radians(20.0), 0.3

    def motion(t):  # pitch, heave and their first two time derivatives
        return (amp_p * math.sin(w * t), amp_p * w * math.cos(w * t), -amp_p * w * w * math.sin(w * t),
                amp_h * math.sin(w * t + 1), amp_h * w * math.cos(w * t + 1), -amp_h * w * w * math.sin(w * t + 1))

    def solid_at(t):
        pitch, _, _, heave, _, _ = motion(t)
        cp, sp = math.cos(pitch), math.sin(pitch)
        xr = cp * X + sp * (Y - heave)
        yr = -sp * X + cp * (Y - heave)
        return ((xr / 0.5) ** 2 + (yr / 0.06) ** 2 < 1.0).astype(np.uint8)

    def field(t, solid):
        u = np.ones((nx, ny))
        v = np.zeros((nx, ny))
        for x0, y0, gam, rc in vort:
            r2 = (X - x0 - t) ** 2 + (Y - y0) ** 2
            fac = np.where(r2 > 0, gam / (2 * math.pi) * (1 - np.exp(-r2 / rc ** 2)) / np.where(r2 > 0, r2, 1.0), 0.0)
            u -= fac * (Y - y0)
            v += fac * (X - x0 - t)
        fluid = solid == 0
        return u * fluid, v * fluid

    def boundary(a):
        return np.concatenate([a[0, :], a[nx - 1, :], a[:, 0], a[:, ny - 1]])

    frames = []
    for k in range(nframes):
        t = k * dt
        solid = solid_at(t)
        u, v = field(t, solid)
        ring = np.zeros((2 * nx + 2 * ny, 2, 2), order="F")
        for tt, ts in ((0, t - dt), (1, t + dt)):
            ub, vb = field(ts, solid_at(ts))
            ring[:, 0, tt] = boundary(ub)
            ring[:, 1, tt] = boundary(vb)
        pitch, dp, ddp, heave, dh, ddh = motion(t)
        # rotation by the pitch about (0, heave): with U_B = (k1 - k3 y, k2 + k3 x)
        # and a_B = (k4 - k6 y - k3^2 x, k5 + k6 x - k3^2 y), k3 = d(pitch)/dt,
        # k6 = its derivative, k1 = k3 heave, k2 = d(heave)/dt, k4 = k6 heave,
        # k5 = d2(heave)/dt2 + k3^2 heave
        kin = np.array([dp * heave, dh, dp, ddp * heave, ddh + dp * dp * heave, ddp])
        frames.append(dict(nx=nx, ny=ny, xf=xf, yf=yf, xc=xc, yc=yc, dx=dx, dy=dy,
                           solid=np.asfortranarray(solid), u=np.asfortranarray(u), v=np.asfortranarray(v),
                           ring=ring, kin=kin, dt=dt, time=t))
    return frames


def frame_as_stairstep(fr):
    """The reference's 2-D use of the 3-D solver (examples/flapping_foil_fpm.f90:
    nz = 2, dz = 0.5, zero z-face data): padded solid, axes and zero faces."""
    nx, ny, nz = fr["nx"], fr["ny"], 2
    solid = np.zeros((nx + 2, ny + 2, nz), dtype=np.int32, order="F")
    for k in range(nz):
        solid[1:nx + 1, 1:ny + 1, k] = fr["solid"]
    return dict(nx=nx, ny=ny, nz=nz, xc=fr["xc"], yc=fr["yc"], zc=np.array([0.25, 0.75]), dx=fr["dx"], dy=fr["dy"],
                dz=np.array([0.5, 0.5]), solid=solid, rhs=np.zeros((nx, ny, nz), order="F"),
                phi=np.zeros((nx + 2, ny + 2, nz), order="F"), faces=_empty_faces(nx, ny, nz))
