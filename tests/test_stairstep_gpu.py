"""GPU parity of the stair-step path (libfpm_gb300.so through the C ABI)
against the CPU oracle on the same inputs.

Tolerances: the FP64 Jacobi sweep and the operator build are bit-identical
per cell; max-norm residuals are bit-identical (max is order independent);
the double-float Jacobi must stay within 1e-12 relative of FP64 after 2000
sweeps; converged PCG potentials within 1e-9 relative max-norm of the
oracle's; force densities bit-identical for the same phi and integrals within
1e-12 relative (sum order differs)."""
import ctypes

import numpy as np
import pytest

import oracle as orc
from cases import F, exact_expectations, sphere_case, sphere_errors, stairstep_case_exact
from gpu_util import from_dev, ptr, stream_ptr, to_dev

pytestmark = pytest.mark.gpu

D, I = ctypes.c_double, ctypes.c_int


def gpu_run(c, method, tol, max_it, ci=50):
    from flowfpmpp_gb300 import stairstep as ss
    phi = c["phi"].copy(order="F")
    faces = [f.copy(order="F") for f in c["faces"]]
    corr, imb = ss.enforce_stairstep_compatibility_3d(c["rhs"], c["solid"], c["body"], *faces, c["dx"], c["dy"],
                                                      c["dz"])
    sw, res = ss.solve_stairstep_poisson_3d(phi, c["rhs"], c["solid"], c["body"], *faces, c["xc"], c["yc"], c["zc"],
                                            c["dx"], c["dy"], c["dz"], tol, max_it, ci, method)
    chk = ss.stairstep_residual_3d(phi, c["rhs"], c["solid"], c["body"], *faces, c["xc"], c["yc"], c["zc"], c["dx"],
                                   c["dy"], c["dz"])
    terms = None
    fl = c.get("flow")
    if fl is not None:
        terms = ss.compute_stairstep_fpm_terms_3d(phi, fl["u"], fl["v"], fl["w"], fl["ox"], fl["oy"], fl["oz"],
                                                  fl["ax"], fl["ay"], fl["az"], c["solid"], c["body"], c["xc"],
                                                  c["yc"], c["zc"], c["dx"], c["dy"], c["dz"], *faces, c["bounds"])
    return dict(phi=phi, faces=faces, corr=corr, imb=imb, sweeps=sw, res=res, chk=chk, terms=terms)


def cpu_run(c, method, tol, max_it, ci=50):
    from test_oracle_pins import run_stairstep
    return run_stairstep(c, method, tol, max_it, ci)


def rel_linf(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def test_compatibility_matches_oracle(gpu_lib):
    for exact in (True, False):
        c = stairstep_case_exact(exact)
        g = gpu_run(c, "jacobi", -1.0, 2)
        o = cpu_run(c, "jacobi", -1.0, 2)
        assert abs(g["corr"] - o["corr"]) <= 1e-15 and abs(g["imb"]) < 1e-13
        for fg, fo in zip(g["faces"], o["faces"]):
            assert np.abs(fg - fo).max() <= 1e-15


def test_operator_build_and_fp64_sweeps_bit_identical(gpu_lib):
    """build_operator and 600 FP64 Jacobi sweeps reproduce the oracle bit for bit."""
    c = stairstep_case_exact(False)
    nx, ny, nz = c["nx"], c["ny"], c["nz"]
    faces = [f.copy(order="F") for f in c["faces"]]
    orc.enforce_stairstep_compatibility_3d(c["rhs"], c["solid"], c["body"], *faces, c["dx"], c["dy"], c["dz"])
    coefs = orc.stairstep_coefficients(c["xc"], c["yc"], c["zc"], c["dx"], c["dy"], c["dz"])
    src, diag, rdiag, iso = orc.build_operator(c["rhs"], c["solid"], c["body"], *faces, coefs, c["dx"], c["dy"],
                                               c["dz"], False)
    assert iso == 0
    dfaces = [to_dev(f) for f in faces]
    dax = [to_dev(c[k]) for k in ("xc", "yc", "zc", "dx", "dy", "dz")]
    drhs, dsolid = to_dev(c["rhs"]), to_dev(c["solid"])
    import torch
    n = nx * ny * nz
    gsrc, gdiag, grd = (torch.empty(n, dtype=torch.float64, device="cuda") for _ in range(3))
    iso_g = I()
    bg = np.ascontiguousarray(c["body"])
    rc = gpu_lib.fpm_stairstep_build_operator_dev(ptr(drhs), ptr(dsolid), bg.ctypes.data_as(ctypes.c_void_p),
                                                  *[ptr(f) for f in dfaces], *[ptr(a) for a in dax], I(nx), I(ny),
                                                  I(nz), I(0), ptr(gsrc), ptr(gdiag), ptr(grd), ctypes.byref(iso_g),
                                                  stream_ptr())
    assert rc == 0 and iso_g.value == 0
    for g, o in ((gsrc, src), (gdiag, diag), (grd, rdiag)):
        assert np.array_equal(from_dev(g, (nx, ny, nz)), o)
    # 600 sweeps from a nonzero start, both sides in FP64
    rng = np.random.default_rng(7)
    a = np.zeros((nx + 2, ny + 2, nz), order="F")
    a[1:nx + 1, 1:ny + 1, :] = rng.standard_normal((nx, ny, nz)) * (c["solid"][1:nx + 1, 1:ny + 1, :] == 0)
    b = a.copy(order="F")
    ga, gb = to_dev(a), to_dev(b)
    rc = gpu_lib.fpm_stairstep_jacobi_sweeps_dev(ptr(ga), ptr(gb), ptr(gsrc), ptr(grd), *[ptr(x) for x in dax],
                                                 I(nx), I(ny), I(nz), I(600), I(1), stream_ptr())
    assert rc == 0
    for s in range(600):
        if s % 2 == 0:
            orc.jacobi_sweep(a, b, src, rdiag, coefs)
        else:
            orc.jacobi_sweep(b, a, src, rdiag, coefs)
    assert np.array_equal(from_dev(ga, a.shape), a)
    val = D()
    rc = gpu_lib.fpm_stairstep_operator_residual_dev(ptr(ga), ptr(gsrc), ptr(gdiag), *[ptr(x) for x in dax], I(nx),
                                                     I(ny), I(nz), ctypes.byref(val), stream_ptr())
    assert rc == 0 and val.value == orc.operator_residual(a, src, diag, coefs)


def test_df_sweeps_within_1e12_after_2000(gpu_lib):
    """Double-float sweeps stay within 1e-12 relative of FP64 after 2000 sweeps."""
    c = stairstep_case_exact(False)
    out_g = gpu_run(c, "jacobi_df", -1.0, 2000, ci=2000)
    out_o = cpu_run(c, "jacobi", -1.0, 2000, ci=2000)
    assert out_g["sweeps"] == 2000
    assert rel_linf(out_g["phi"], out_o["phi"]) <= 1e-12
    # The max-norm residual amplifies field differences by the operator norm
    # (about 2e3 here), so it is held to 1e-9 relative.
    assert abs(out_g["res"] - out_o["res"]) <= 1e-9 * out_o["res"]


def test_fma_sweeps_within_1e12_after_2000(gpu_lib):
    """FP64 sweeps with fused multiply-adds stay within 1e-12 relative of the
    separately rounded FP64 oracle after 2000 sweeps."""
    c = stairstep_case_exact(False)
    out_g = gpu_run(c, "jacobi_fma", -1.0, 2000, ci=2000)
    out_o = cpu_run(c, "jacobi", -1.0, 2000, ci=2000)
    assert out_g["sweeps"] == 2000
    assert rel_linf(out_g["phi"], out_o["phi"]) <= 1e-12
    assert abs(out_g["res"] - out_o["res"]) <= 1e-9 * out_o["res"]


def test_tf_sweeps_within_1e12_after_2000(gpu_lib):
    """FP64-storage triple-float sweeps stay within 1e-12 relative of the
    separately rounded FP64 oracle after 2000 sweeps (a bound the FP64 oracle
    itself only meets to its own rounding)."""
    c = stairstep_case_exact(False)
    out_g = gpu_run(c, "jacobi_tf", -1.0, 2000, ci=2000)
    out_o = cpu_run(c, "jacobi", -1.0, 2000, ci=2000)
    assert out_g["sweeps"] == 2000
    assert rel_linf(out_g["phi"], out_o["phi"]) <= 1e-12
    assert abs(out_g["res"] - out_o["res"]) <= 1e-9 * out_o["res"]


def _sweep_longdouble(a, src, rdiag, coefs, nx, ny, nz):
    """One weighted-Jacobi sweep (src/fpm_stairstep_mpi_3d.f90:384-399)
    evaluated in numpy's long double (64- or 113-bit significand), rounded to
    FP64 at the end: the reference the triple-float sweep is held to."""
    L = np.longdouble
    A = a.astype(L)
    cw, ce, cs, cn, cb, ct = (np.asarray(x, dtype=L) for x in coefs)
    s = src.astype(L)
    s = s + cw[:, None, None] * A[0:nx, 1:ny + 1, :]
    s = s + ce[:, None, None] * A[2:nx + 2, 1:ny + 1, :]
    s = s + cs[None, :, None] * A[1:nx + 1, 0:ny, :]
    s = s + cn[None, :, None] * A[1:nx + 1, 2:ny + 2, :]
    kb = [max(k - 1, 0) for k in range(nz)]
    kt = [min(k + 1, nz - 1) for k in range(nz)]
    s = s + cb[None, None, :] * A[1:nx + 1, 1:ny + 1, kb]
    s = s + ct[None, None, :] * A[1:nx + 1, 1:ny + 1, kt]
    b = L(0.2) * A[1:nx + 1, 1:ny + 1, :] + rdiag.astype(L) * s
    # magnitude of the terms, for cells where the sum cancels
    m = np.abs(src) + np.abs(cw[:, None, None] * A[0:nx, 1:ny + 1, :]).astype(np.float64)
    for part in (ce[:, None, None] * A[2:nx + 2, 1:ny + 1, :], cs[None, :, None] * A[1:nx + 1, 0:ny, :],
                 cn[None, :, None] * A[1:nx + 1, 2:ny + 2, :], cb[None, None, :] * A[1:nx + 1, 1:ny + 1, kb],
                 ct[None, None, :] * A[1:nx + 1, 1:ny + 1, kt]):
        m = m + np.abs(part).astype(np.float64)
    mag = 0.2 * np.abs(a[1:nx + 1, 1:ny + 1, :]) + np.abs(rdiag) * m
    return b.astype(np.float64), mag


def test_tf_sweep_rounds_like_wider_arithmetic(gpu_lib):
    """One sweep from a random field: the triple-float result is within one
    FP64 ulp of the long-double evaluation rounded to FP64 in every cell, and
    on average closer to it than the separately rounded FP64 sweep."""
    if np.finfo(np.longdouble).nmant <= 52:
        pytest.skip("numpy long double is FP64 on this host")
    c = stairstep_case_exact(False)
    nx, ny, nz = c["nx"], c["ny"], c["nz"]
    faces = [f.copy(order="F") for f in c["faces"]]
    orc.enforce_stairstep_compatibility_3d(c["rhs"], c["solid"], c["body"], *faces, c["dx"], c["dy"], c["dz"])
    coefs = orc.stairstep_coefficients(c["xc"], c["yc"], c["zc"], c["dx"], c["dy"], c["dz"])
    src, diag, rdiag, _ = orc.build_operator(c["rhs"], c["solid"], c["body"], *faces, coefs, c["dx"], c["dy"],
                                             c["dz"], False)
    rng = np.random.default_rng(11)
    a = np.zeros((nx + 2, ny + 2, nz), order="F")
    a[1:nx + 1, 1:ny + 1, :] = rng.standard_normal((nx, ny, nz)) * (c["solid"][1:nx + 1, 1:ny + 1, :] == 0)
    b = a.copy(order="F")
    ga, gb = to_dev(a), to_dev(b)
    dsrc, drd = to_dev(src), to_dev(rdiag)
    dax = [to_dev(c[k]) for k in ("xc", "yc", "zc", "dx", "dy", "dz")]
    rc = gpu_lib.fpm_stairstep_jacobi_sweeps_dev(ptr(ga), ptr(gb), ptr(dsrc), ptr(drd), *[ptr(x) for x in dax],
                                                 I(nx), I(ny), I(nz), I(1), I(7), stream_ptr())
    assert rc == 0, gpu_lib.fpm_last_error()
    tf = from_dev(gb, a.shape)[1:nx + 1, 1:ny + 1, :]
    ref, mag = _sweep_longdouble(a, src, rdiag, coefs, nx, ny, nz)
    b64 = a.copy(order="F")
    orc.jacobi_sweep(a, b64, src, rdiag, coefs)
    f64 = b64[1:nx + 1, 1:ny + 1, :]
    ulp = np.spacing(np.abs(ref))
    err_tf = np.abs(tf - ref) / ulp
    err_64 = np.abs(f64 - ref) / ulp
    # within one ulp where the sum does not cancel by more than 2^6; elsewhere
    # within one ulp plus 2^-55 of the terms' magnitude (the separately
    # rounded FP64 sweep is off by up to 11 x 2^-55 of it on this field)
    plain = np.abs(ref) >= mag / 64
    assert err_tf[plain].max() <= 1.0, err_tf[plain].max()
    assert (np.abs(tf - ref) <= ulp + 2.0 ** -55 * mag).all()
    assert err_tf.mean() < err_64.mean(), (err_tf.mean(), err_64.mean())
    print(f"ulps from the long-double sweep: triple-float max {err_tf.max():.1f} mean {err_tf.mean():.3f}, "
          f"separately rounded FP64 max {err_64.max():.1f} mean {err_64.mean():.3f}")


@pytest.mark.parametrize("method", ["jacobi", "jacobi_fma", "jacobi_tf", "jacobi_df", "pcg"])
def test_exact_linear_solution_gpu(gpu_lib, method):
    """The reference's exactness test (test_stairstep_exact_3d.f90:40-50) on the GPU."""
    c = stairstep_case_exact(True)
    # The double-float iterate carries a 48-bit significand, so its max-norm
    # residual floors near 1e-11 on this grid; it is held to the PCG tolerance.
    tol = 1e-12 if method in ("jacobi", "jacobi_fma", "jacobi_tf") else 1e-10
    g = gpu_run(c, method, tol, 400000)
    gx, gy, gz, vortex, adv, totals = g["terms"]
    errors, ierr = exact_expectations(c, g["phi"], gx, gy, gz, vortex, totals)
    assert abs(g["corr"]) < 1e-13 and abs(g["imb"]) < 1e-13
    assert g["res"] <= 2 * tol and g["chk"] < 1e-9
    assert errors[0] < 1e-9 and errors[1] < 1e-9 and errors[2] < 1e-9 and errors[3] == 0
    assert ierr < 1e-10 and np.all(np.isfinite([g["res"], g["chk"], *errors, *totals]))
    o = cpu_run(c, "jacobi" if method.startswith("jacobi") else method, tol, 400000)
    assert abs(g["sweeps"] - o["sweeps"]) <= 50


def test_fixed_jacobi_matches_oracle(gpu_lib):
    """600 fixed sweeps (test_stairstep_exact_3d.f90:64): the fields agree to
    the gauge-mean rounding, the max-norm residuals to 1e-13 relative."""
    c = stairstep_case_exact(False)
    g = gpu_run(c, "jacobi", -1.0, 600)
    o = cpu_run(c, "jacobi", -1.0, 600)
    assert g["sweeps"] == 600
    assert np.abs(g["phi"] - o["phi"]).max() < 1e-15
    assert abs(g["res"] - o["res"]) <= 1e-13 * o["res"]
    assert abs(g["chk"] - o["chk"]) <= 1e-13 * o["chk"]


def test_pcg_matches_oracle(gpu_lib):
    """PCG to 1e-11 (test_stairstep_exact_3d.f90:65): potentials within 1e-9
    relative max-norm, integrals within 1e-8 (the reference's threshold)."""
    c = stairstep_case_exact(False)
    g = gpu_run(c, "pcg", 1e-11, 100000)
    o = cpu_run(c, "pcg", 1e-11, 100000)
    assert g["res"] <= 2e-11
    assert rel_linf(g["phi"], o["phi"]) <= 1e-9
    assert np.abs(g["terms"][5] - o["terms"][5]).max() < 1e-8


def test_terms_bit_identical_for_same_phi(gpu_lib):
    from flowfpmpp_gb300 import stairstep as ss
    c = stairstep_case_exact(False)
    o = cpu_run(c, "pcg", 1e-11, 100000)
    fl = c["flow"]
    args = (o["phi"], fl["u"], fl["v"], fl["w"], fl["ox"], fl["oy"], fl["oz"], fl["ax"], fl["ay"], fl["az"],
            c["solid"], c["body"], c["xc"], c["yc"], c["zc"], c["dx"], c["dy"], c["dz"], *o["faces"], c["bounds"])
    g = ss.compute_stairstep_fpm_terms_3d(*args)
    r = orc.compute_stairstep_fpm_terms_3d(*args)
    for a, b in zip(g[:5], r[:5]):
        assert np.array_equal(a, b)
    assert np.abs(g[5] - r[5]).max() <= 1e-12 * np.abs(r[5]).max()
    chk_g = ss.stairstep_residual_3d(o["phi"], c["rhs"], c["solid"], c["body"], *o["faces"], c["xc"], c["yc"],
                                     c["zc"], c["dx"], c["dy"], c["dz"])
    assert chk_g == o["chk"]


@pytest.mark.parametrize("seed", [3, 4])
def test_terms_bit_identical_on_random_stretched_grid(gpu_lib, seed):
    """The densities' face-gradient quotients (spacing reciprocal plus one
    correction step on the GPU, IEEE division in the oracle) agree bit for bit
    on random cell spacings, potentials, bodies, faces and flows."""
    from flowfpmpp_gb300 import stairstep as ss
    rng = np.random.default_rng(seed)
    nx, ny, nz = 23, 17, 11
    axes = []
    for n in (nx, ny):
        c = np.cumsum(rng.uniform(0.01, 2.0, n + 2))
        axes.append(c - c.mean())
    zc = np.cumsum(rng.uniform(0.01, 2.0, nz))
    dxs = [rng.uniform(0.01, 2.0, n) for n in (nx, ny, nz)]
    phi = np.asfortranarray(rng.standard_normal((nx + 2, ny + 2, nz)) * 10.0 ** rng.integers(-6, 3))
    solid = F((nx + 2, ny + 2, nz), np.int32)
    solid[1:nx + 1, 1:ny + 1, :] = rng.random((nx, ny, nz)) < 0.15
    flow = [np.asfortranarray(rng.standard_normal((nx, ny, nz))) for _ in range(9)]
    faces = [np.asfortranarray(rng.standard_normal(sh)) for sh in ((ny, nz), (ny, nz), (nx, nz), (nx, nz),
                                                                   (nx, ny), (nx, ny))]
    bounds = np.array([-1e300, 1e300] * 3)
    args = (phi, *flow, solid, rng.standard_normal(3), axes[0], axes[1], zc, *dxs, *faces, bounds)
    g = ss.compute_stairstep_fpm_terms_3d(*args)
    r = orc.compute_stairstep_fpm_terms_3d(*args)
    for a, b in zip(g[:5], r[:5]):
        assert np.array_equal(a, b)
    assert np.abs(g[5] - r[5]).max() <= 1e-12 * np.abs(r[5]).max()


@pytest.mark.parametrize("n,iters,cm_ref", [(12, 100, 0.897), (24, 200, 0.770)])
def test_sphere_gpu_matches_table(gpu_lib, n, iters, cm_ref):
    c = sphere_case(n)
    g = gpu_run(c, "pcg", 1e-10, 2000000, ci=100)
    rms, far, cm = sphere_errors(c, g["phi"])
    assert g["sweeps"] == iters and round(cm, 3) == pytest.approx(cm_ref, abs=1e-12)


def test_errors_mirror_reference_error_stops(gpu_lib):
    from flowfpmpp_gb300 import FpmError
    from flowfpmpp_gb300 import stairstep as ss
    c = stairstep_case_exact(False)
    args = lambda phi, solid: (phi, c["rhs"], solid, c["body"], *c["faces"], c["xc"], c["yc"], c["zc"], c["dx"],
                               c["dy"], c["dz"], 1e-8, 10, 5)
    with pytest.raises(FpmError) as e:
        ss.solve_stairstep_poisson_3d(*args(c["phi"].copy(order="F"), c["solid"]), method="multigrid")
    assert e.value.code == 1
    # an isolated fluid cell: fluid (1,1,1) walled in by solid on its three inner faces
    solid = c["solid"].copy(order="F")
    solid[2, 1, 0] = 1
    solid[1, 2, 0] = 1
    solid[1, 1, 1] = 1
    solid[1, 1, 0] = 0
    with pytest.raises(FpmError) as e:
        ss.solve_stairstep_poisson_3d(*args(c["phi"].copy(order="F"), solid))
    assert e.value.code == 3


@pytest.mark.parametrize("shape", range(11))
@pytest.mark.parametrize("dims,kchunk", [((37, 29, 11), 3), ((130, 70, 20), 8)])
def test_df_tma_tile_shapes_match_fp64(gpu_lib, monkeypatch, shape, dims, kchunk):
    """Every TMA tile shape and a ragged z-chunk, on grids that are not
    multiples of the tile: 300 double-float sweeps vs 300 FP64 sweeps."""
    import torch
    from flowfpmpp_gb300 import workloads
    nx, ny, nz = dims
    rng = np.random.default_rng(shape)
    ax, ay, az = (workloads.geometric_axis(n, -1.0, 1.0, 1.05) for n in dims)
    solid = np.zeros((nx + 2, ny + 2, nz), dtype=np.int32, order="F")
    solid[3:9, 4:12, 2:6] = 1
    src = np.asfortranarray(rng.standard_normal((nx, ny, nz)) * (solid[1:nx + 1, 1:ny + 1, :] == 0))
    coefs = orc.stairstep_coefficients(ax[1], ay[1], az[1][1:nz + 1].copy(), ax[2], ay[2], az[2])
    rhs = np.asfortranarray(-src)
    faces = [F((ny, nz)), F((ny, nz)), F((nx, nz)), F((nx, nz)), F((nx, ny)), F((nx, ny))]
    osrc, diag, rdiag, _ = orc.build_operator(rhs, solid, [1.0, 0.0, 0.0], *faces, coefs, ax[2], ay[2], az[2], False)
    a = np.zeros((nx + 2, ny + 2, nz), order="F")
    a[1:nx + 1, 1:ny + 1, :] = rng.standard_normal((nx, ny, nz)) * (solid[1:nx + 1, 1:ny + 1, :] == 0)
    dax = [to_dev(x) for x in (ax[1], ay[1], az[1][1:nz + 1].copy(), ax[2], ay[2], az[2])]
    g64 = [to_dev(a), to_dev(a)]
    gdf = [to_dev(a), to_dev(a)]
    ds, dr = to_dev(osrc), to_dev(rdiag)
    monkeypatch.setenv("FPM_DF_SHAPE", str(shape))
    monkeypatch.setenv("FPM_DF_KCHUNK", str(kchunk))
    for meth, bufs in ((1, g64), (2, gdf)):
        rc = gpu_lib.fpm_stairstep_jacobi_sweeps_dev(ptr(bufs[0]), ptr(bufs[1]), ptr(ds), ptr(dr),
                                                     *[ptr(x) for x in dax], I(nx), I(ny), I(nz), I(300), I(meth),
                                                     stream_ptr())
        assert rc == 0, gpu_lib.fpm_last_error()
    r64 = from_dev(g64[0], a.shape)
    rdf = from_dev(gdf[0], a.shape)
    assert np.abs(r64).max() > 0
    assert np.abs(rdf - r64).max() <= 1e-12 * np.abs(r64).max()
    assert np.array_equal(rdf[0], a[0]) and np.array_equal(rdf[:, 0], a[:, 0])  # halos untouched


@pytest.mark.parametrize("method", ["pcg_mixed", "pcg_mg"])
def test_pcg_mixed_matches_fp64_oracle(gpu_lib, method):
    """FP32 PCG (diagonal or multigrid preconditioner) inside FP64 refinement
    reaches the same residual tolerance and potentials within 1e-9 relative
    max-norm of the FP64 oracle."""
    c = stairstep_case_exact(False)
    g = gpu_run(c, method, 1e-11, 100000)
    o = cpu_run(c, "pcg", 1e-11, 100000)
    assert g["res"] <= 2e-11
    assert rel_linf(g["phi"], o["phi"]) <= 1e-9
    assert np.abs(g["terms"][5] - o["terms"][5]).max() < 1e-8
    e = stairstep_case_exact(True)
    ge = gpu_run(e, method, 1e-10, 100000)
    gx, gy, gz, vortex, adv, totals = ge["terms"]
    errors, ierr = exact_expectations(e, ge["phi"], gx, gy, gz, vortex, totals)
    assert ge["res"] <= 2e-10 and errors[0] < 1e-9 and errors[1] < 1e-9 and errors[3] == 0 and ierr < 1e-10


def _multi_rhs_vs_oracle(gpu_lib, f, method, axes=(0, 1, 2)):
    """Potentials for the body moving along each of axes, solved in one call,
    against the FP64 oracle one by one."""
    from flowfpmpp_gb300 import stairstep as ss
    nx, ny, nz = f["nx"], f["ny"], f["nz"]
    n = len(axes)
    phis, rhss, faces_dev, bgs, refs = [], [], [], [], []
    for axis in axes:
        body = np.zeros(3)
        body[axis] = 1.0
        faces = [x.copy(order="F") for x in f["faces"]]
        ss.enforce_stairstep_compatibility_3d(f["rhs"], f["solid"], body, *faces, f["dx"], f["dy"], f["dz"])
        ref = f["phi"].copy(order="F")
        orc.solve_stairstep_poisson_3d(ref, f["rhs"], f["solid"], body, *faces, f["xc"], f["yc"], f["zc"], f["dx"],
                                       f["dy"], f["dz"], 1e-10, 100000, 50, "pcg")
        refs.append(ref)
        phis.append(to_dev(f["phi"]))
        rhss.append(to_dev(f["rhs"]))
        faces_dev += [to_dev(x) for x in faces]
        bgs.append(body)
    dax = [to_dev(f[k]) for k in ("xc", "yc", "zc", "dx", "dy", "dz")]
    VP = ctypes.c_void_p
    phi_arr = (VP * n)(*[t.data_ptr() for t in phis])
    rhs_arr = (VP * n)(*[t.data_ptr() for t in rhss])
    face_arr = (VP * (6 * n))(*[t.data_ptr() for t in faces_dev])
    bg = np.ascontiguousarray(np.concatenate(bgs))
    sweeps = (I * n)()
    res = (D * n)()
    rc = gpu_lib.fpm_solve_stairstep_multi_dev(n, phi_arr, rhs_arr, ptr(to_dev(f["solid"])),
                                               bg.ctypes.data_as(VP), face_arr, *[ptr(x) for x in dax], nx, ny, nz,
                                               D(1e-10), 100000, 50, method, sweeps, res, stream_ptr())
    assert rc == 0, gpu_lib.fpm_last_error()
    for m in range(n):
        assert res[m] <= 2e-10
        assert rel_linf(from_dev(phis[m], refs[m].shape), refs[m]) <= 1e-9


@pytest.mark.parametrize("method", [0, 3, 4])
def test_multi_rhs_three_influence_fields(gpu_lib, method):
    """phi_x, phi_y, phi_z of a stretched-grid sphere in one call (FP64 one
    after the other, mixed precision batched, or multigrid-preconditioned FP32)
    against the FP64 oracle."""
    from flowfpmpp_gb300 import workloads
    _multi_rhs_vs_oracle(gpu_lib, workloads.sphere_grid(nx=40, ny=36, nz=24), method)


@pytest.mark.parametrize("dims,kchunk,axes", [((37, 29, 11), 16, (0, 1, 2)), ((133, 21, 37), 16, (0, 2)),
                                              ((150, 17, 6), 2, (1,)), ((64, 12, 33), 4, (2, 0, 1)),
                                              ((259, 9, 5), 6, (0, 1)),
                                              ((20, 18, 6), 2, (0, 1, 2, 0)),
                                              ((70, 45, 29), None, (0, 1, 2))])
def test_multigrid_tile_edges(gpu_lib, monkeypatch, dims, kchunk, axes):
    """The multigrid path on shapes that end level-0 TMA tiles mid-tile in x
    (nx not a multiple of 4 or of 128) and y (ny not a multiple of 8), chunks
    mid-aggregate in z (odd nz, several chunks, chunks of 2 planes), with one
    to four right-hand sides (the fifth case: level 1 is already the
    coarsest; the last: plane chunks chosen by the library to fill the SMs):
    potentials within 1e-9 of the FP64 oracle."""
    from flowfpmpp_gb300 import workloads
    if kchunk is None:
        monkeypatch.delenv("FPM_MG_KCHUNK", raising=False)
    else:
        monkeypatch.setenv("FPM_MG_KCHUNK", str(kchunk))
    _multi_rhs_vs_oracle(gpu_lib, workloads.sphere_grid(*dims), 4, axes)
