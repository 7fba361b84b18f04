"""GPU parity of the no-body Neumann solvers, their FPM densities and the 2-D
force partition against the CPU oracle on the reference tests' inputs.

Per-cell arithmetic is bit-identical (same expression order, no contraction),
so sweeps, iteration counts, densities and per-cell partition fields match
exactly; only global sums (means, compatibility fluxes, integrals, the four
force terms) differ in summation order, held to 1e-12 relative."""
import math

import numpy as np
import pytest

import oracle as orc
from cases import F, fill_ring, manufactured_nonuniform, manufactured_uniform, partition_grid

pytestmark = pytest.mark.gpu


def close(a, b, rel=1e-12, abs_=1e-15):
    return abs(a - b) <= rel * abs(b) + abs_


def test_uniform_neumann_and_terms(gpu_lib):
    from flowfpmpp_gb300 import laplace as lp
    c = manufactured_uniform()
    nx, ny, nz, dx, dy, dz = c["nx"], c["ny"], c["nz"], c["dx"], c["dy"], c["dz"]
    fo = [f.copy(order="F") for f in c["faces"]]
    fg = [f.copy(order="F") for f in c["faces"]]
    co, io = orc.enforce_neumann_compatibility_3d(c["rhs"], *fo, dx, dy, dz)
    cg, ig = lp.enforce_neumann_compatibility_3d(c["rhs"], *fg, nx, ny, nz, dx, dy, dz)
    assert close(cg, co) and abs(cg - 1.0 / 6) < 1e-12 and abs(ig) < 1e-12
    # The correction is a global sum (960 cells) in another order: 1e-13 relative.
    for a, b in zip(fg, fo):
        assert np.abs(a - b).max() <= 1e-13 * np.abs(b).max()
    po, pg = c["phi"].copy(order="F"), c["phi"].copy(order="F")
    ito, reso = orc.solve_neumann_poisson_3d(po, c["rhs"], *fo, dx, dy, dz, 1e-10, 50000, 25)
    itg, resg = lp.solve_neumann_poisson_3d(pg, c["rhs"], *fo, nx, ny, nz, dx, dy, dz, 1e-10, 50000, 25)
    assert itg == ito and resg <= 1e-10
    assert np.abs(pg - po).max() <= 1e-14
    assert np.abs(pg[1:nx + 1, 1:ny + 1, 1:nz + 1] - c["exact"]).max() < 1e-9
    one = np.ones((nx, ny, nz), order="F")
    flow = [1 * one, 2 * one, 3 * one, 0.5 * one, -0.25 * one, 0.75 * one, 0.2 * one, -0.1 * one, 0.3 * one]
    fluid = np.ones((nx, ny, nz), dtype=np.int32, order="F")
    fluid[3, 4, 2] = 0
    go = orc.compute_fpm_terms_uniform_3d(po, *flow, fluid, dx, dy, dz)
    gg = lp.compute_fpm_terms_uniform_3d(po, *flow, fluid, nx, ny, nz, dx, dy, dz)
    for a, b in zip(gg[:5], go[:5]):
        assert np.array_equal(a, b)
    assert np.abs(gg[5] - go[5]).max() <= 1e-13


def test_nonuniform_neumann_and_terms(gpu_lib):
    from flowfpmpp_gb300 import laplace as lp
    c = manufactured_nonuniform()
    nx, ny, nz = c["nx"], c["ny"], c["nz"]
    rhs37 = np.asfortranarray(c["rhs"] + 0.37)
    fo = [f.copy(order="F") for f in c["faces"]]
    fg = [f.copy(order="F") for f in c["faces"]]
    co, _ = orc.enforce_neumann_compatibility_nonuniform_3d(rhs37, *fo, c["dx"], c["dy"], c["dz"])
    cg, ig = lp.enforce_neumann_compatibility_nonuniform_3d(rhs37, *fg, c["dx"], c["dy"], c["dz"], nx, ny, nz)
    assert close(cg, co) and abs(cg - 0.37 / 6) < 1e-12 and abs(ig) < 1e-12
    po, pg = F((nx, ny, nz)), F((nx, ny, nz))
    args = (c["rhs"], *c["faces"], c["xc"], c["yc"], c["zc"], c["dx"], c["dy"], c["dz"])
    ito, _ = orc.solve_neumann_poisson_nonuniform_3d(po, *args, 1e-10, 100000, 25)
    itg, resg = lp.solve_neumann_poisson_nonuniform_3d(pg, *args, nx, ny, nz, 1e-10, 100000, 25)
    assert itg == ito and resg <= 1e-10
    assert np.abs(pg - po).max() <= 1e-14 and np.abs(pg - c["exact"]).max() < 1e-8
    one = np.ones((nx, ny, nz), order="F")
    flow = [1 * one, 2 * one, 3 * one, 0.5 * one, -0.25 * one, 0.75 * one, 0.2 * one, -0.1 * one, 0.3 * one]
    fluid = np.ones((nx, ny, nz), dtype=np.int32, order="F")
    fluid[nx // 2 - 1, ny // 2 - 1, nz // 2 - 1] = 0
    eps = np.finfo(np.float64).eps
    xc, yc, zc = c["xc"], c["yc"], c["zc"]
    bounds = np.array([xc[1] - eps, xc[nx - 2] + eps, yc[1] - eps, yc[ny - 2] + eps, zc[1] - eps, zc[nz - 2] + eps])
    targs = (po, *flow, fluid, xc, yc, zc, c["dx"], c["dy"], c["dz"], *c["faces"], bounds)
    go = orc.compute_fpm_terms_nonuniform_3d(*targs)
    gg = lp.compute_fpm_terms_nonuniform_3d(*targs, nx, ny, nz)
    for a, b in zip(gg[:5], go[:5]):
        assert np.array_equal(a, b)
    assert np.abs(gg[5] - go[5]).max() <= 1e-13


def _partition_pair(phi, g, u, v, solid, xf, kin, ring, dt, nu, slip=False):
    from flowfpmpp_gb300 import partition as pt
    ro = orc.fpm_partition_terms_2d(phi, g, u, v, solid, xf, xf, kin, ring, dt, nu, slip)
    rg = pt.fpm_partition_terms_2d(phi, g, u, v, solid, xf, xf, kin, ring, dt, nu, slip_body=slip)
    return ro, rg


def test_partition_rotation_uniform_cylinder(gpu_lib):
    n, w0, radius = 160, 0.7, 0.25
    xf, xc, dx = partition_grid(n)
    X = xc[1:n + 1][:, None] * np.ones((n, n))
    Y = xc[1:n + 1][None, :] * np.ones((n, n))
    solid = np.zeros((n, n), dtype=np.uint8, order="F")
    kin = np.zeros(6)
    # rotation
    u, v = np.asfortranarray(-w0 * Y), np.asfortranarray(w0 * X)
    phi = np.ones((n, n), order="F")
    ro, rg = _partition_pair(phi, [1.0, 0.0], u, v, solid, xf, kin, fill_ring(u, v), 1.0, 1e-3)
    assert np.array_equal(rg[1], ro[1]) and np.array_equal(rg[2], ro[2])
    assert np.abs(rg[1][2:n - 2, 2:n - 2] + 2 * w0 ** 2).max() < 1e-10
    assert np.all(np.abs(rg[0] - ro[0]) <= 1e-12 * np.abs(ro[0]).max() + 1e-15)
    # uniform flow: exactly zero
    u, v = np.ones((n, n), order="F"), np.zeros((n, n), order="F")
    phi = np.asfortranarray(X - Y)
    ro, rg = _partition_pair(phi, [1.0, 0.0], u, v, solid, xf, kin, fill_ring(u, v), 1.0, 1e-3)
    assert np.all(rg[0] == 0) and np.all(ro[0] == 0)
    # accelerating cylinder with a GPU-solved potential
    from flowfpmpp_gb300 import stairstep as ss
    nz = 2
    s2 = X ** 2 + Y ** 2 < radius ** 2
    solid3 = F((n + 2, n + 2, nz), np.int32)
    for k in range(nz):
        solid3[1:n + 1, 1:n + 1, k] = s2
    dz, zc = np.array([0.5, 0.5]), np.array([0.25, 0.75])
    faces = [F((n, nz)), F((n, nz)), F((n, nz)), F((n, nz)), F((n, n)), F((n, n))]
    rhs, phi3, body = F((n, n, nz)), F((n + 2, n + 2, nz)), np.array([1.0, 0.0, 0.0])
    ss.enforce_stairstep_compatibility_3d(rhs, solid3, body, *faces, dx, dx, dz)
    ss.solve_stairstep_poisson_3d(phi3, rhs, solid3, body, *faces, xc, xc, zc, dx, dx, dz, 1e-10, 200000, 50)
    z0 = np.zeros((n, n), order="F")
    kin = np.array([0.0, 0.0, 0.0, 1.0, 0.0, 0.0])
    p2 = np.asfortranarray(phi3[1:n + 1, 1:n + 1, 0])
    ro, rg = _partition_pair(p2, [1.0, 0.0], z0, z0, np.asfortranarray(s2.astype(np.uint8)), xf, kin,
                             fill_ring(z0, z0), 1.0, 1e-3)
    cm = -rg[0][0] / (math.pi * radius ** 2)
    assert f"{cm:.2f}" == "1.14" and np.all(rg[0][1:] == 0)
    assert abs(rg[0][0] - ro[0][0]) <= 1e-12 * abs(ro[0][0])


def test_partition_random_frame_with_body_and_ring(gpu_lib):
    """A random frame exercising every face branch (outer, body no-slip and
    slip, interior) with a nonzero ring and kinematics."""
    rng = np.random.default_rng(5)
    nx, ny = 70, 53
    xf = np.concatenate([[0.0], np.cumsum(rng.uniform(0.5, 1.5, nx))])
    yf = np.concatenate([[0.0], np.cumsum(rng.uniform(0.5, 1.5, ny))])
    xc = 0.5 * (xf[:-1] + xf[1:])
    yc = 0.5 * (yf[:-1] + yf[1:])
    X, Y = np.meshgrid(xc, yc, indexing="ij")
    solid = np.asfortranarray(((X - xc.mean()) ** 2 / 100 + (Y - yc.mean()) ** 2 / 30 < 1).astype(np.uint8))
    u = np.asfortranarray(rng.standard_normal((nx, ny)))
    v = np.asfortranarray(rng.standard_normal((nx, ny)))
    phi = np.asfortranarray(rng.standard_normal((nx, ny)))
    ring = np.asfortranarray(rng.standard_normal((2 * nx + 2 * ny, 2, 2)))
    kin = rng.standard_normal(6)
    for slip in (False, True):
        from flowfpmpp_gb300 import partition as pt
        ro = orc.fpm_partition_terms_2d(phi, [0.3, -0.8], u, v, solid, xf, yf, kin, ring, 0.4, 1e-4, slip)
        rg = pt.fpm_partition_terms_2d(phi, [0.3, -0.8], u, v, solid, xf, yf, kin, ring, 0.4, 1e-4,
                                       slip_body=slip)
        assert np.array_equal(rg[1], ro[1]) and np.array_equal(rg[2], ro[2])
        assert np.all(np.abs(rg[0] - ro[0]) <= 1e-12 * np.abs(ro[0]).max())


def test_partition_3d_matches_oracle(gpu_lib):
    """3-D four-term partition: per-cell fields bit-identical to the oracle,
    terms within 1e-12 relative, on a random stretched grid with a blocked
    body, rigid-body kinematics and an outer shell (no-slip and slip)."""
    from flowfpmpp_gb300 import partition as pt
    rng = np.random.default_rng(9)
    nx, ny, nz = 37, 22, 15
    xf, yf, zf = (np.concatenate([[0.0], np.cumsum(rng.uniform(0.5, 1.5, n))]) for n in (nx, ny, nz))
    xc, yc, zc = (0.5 * (f[:-1] + f[1:]) for f in (xf, yf, zf))
    X, Y, Z = np.meshgrid(xc, yc, zc, indexing="ij")
    solid = np.asfortranarray((((X - xc.mean()) / 8) ** 2 + ((Y - yc.mean()) / 5) ** 2
                               + ((Z - zc.mean()) / 4) ** 2 < 1).astype(np.uint8))
    u, v, w, phi = (np.asfortranarray(rng.standard_normal((nx, ny, nz))) for _ in range(4))
    L = 2 * ny * nz + 2 * nx * nz + 2 * nx * ny
    shell = np.asfortranarray(rng.standard_normal((L, 3, 2)))
    kin = rng.standard_normal(12)
    for slip in (False, True):
        ro = orc.fpm_partition_terms_3d(phi, [0.2, -0.5, 0.7], u, v, w, solid, xf, yf, zf, kin, shell, 0.4, 1e-3,
                                        slip)
        rg = pt.fpm_partition_terms_3d(phi, [0.2, -0.5, 0.7], u, v, w, solid, xf, yf, zf, kin, shell, 0.4, 1e-3,
                                       slip_body=slip)
        assert np.array_equal(rg[1], ro[1]) and np.array_equal(rg[2], ro[2])
        assert np.all(np.abs(rg[0] - ro[0]) <= 1e-12 * np.abs(ro[0]).max())
