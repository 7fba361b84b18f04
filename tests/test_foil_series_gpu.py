"""A time series of 2-D dumps on one grid (the reference foil example's
frame, examples/flapping_foil_fpm.f90, over consecutive dumps): potentials
warm-started from the previous frame reach the same tolerance and the same
potentials (1e-9 relative) and terms (1e-8 relative) as cold starts (FP64 PCG:
in fewer iterations); the F_BOUND ring built from the neighbouring dumps gives
the terms of the ring stored in the frames (equal by construction here); and a
warm-started dump with the neighbour ring matches the oracle run the same way."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_warm_started_series_matches_cold(gpu_lib):
    from flowfpmpp_gb300 import foil, workloads
    # dumps close enough that the foil moves less than a near-body cell (0.01)
    frames = workloads.foil_series(nframes=4, nx=96, ny=80, dt=0.002)
    for method in ("pcg", "pcg_mg"):
        cold = foil.partition_series(frames, method, warm=False)
        warm = foil.partition_series(frames, method, warm=True)
        nb = foil.partition_series(frames, method, warm=True, ring="neighbours")
        for c, w, n in zip(cold, warm, nb):
            assert (c["residual"] <= 1e-10).all() and (w["residual"] <= 1e-10).all()
            scale = np.abs(c["phi"]).max()
            assert np.abs(w["phi"] - c["phi"]).max() <= 1e-9 * scale
            assert np.allclose(w["terms"], c["terms"], rtol=1e-8, atol=1e-8 * np.abs(c["terms"]).max())
            # same ring values; dt from the dump times may differ in the last bit
            assert np.allclose(n["terms"], w["terms"], rtol=1e-12, atol=1e-12 * np.abs(w["terms"]).max())
        sc = sum(int(r["sweeps"].sum()) for r in cold[1:])
        sw = sum(int(r["sweeps"].sum()) for r in warm[1:])
        print(f"{method}: iterations after the first frame, cold {sc}, warm {sw}")
        if method == "pcg":
            assert sw < sc


def _oracle_frame(fr, phi0=None):
    """foil.partition_frame restated on the CPU oracle (FP64 PCG to 1e-10)."""
    import oracle as orc
    from flowfpmpp_gb300 import foil
    nx, ny, nz = fr["nx"], fr["ny"], 2
    dx, dy, xc, yc = foil.frame_axes(fr)
    dz, zc = np.array([0.5, 0.5]), np.array([0.25, 0.75])
    solid = np.zeros((nx + 2, ny + 2, nz), dtype=np.int32, order="F")
    for k in range(nz):
        solid[1:nx + 1, 1:ny + 1, k] = fr["solid"]
    rhs = np.zeros((nx, ny, nz), order="F")
    out = dict(terms=np.zeros((2, 4)), phi=np.zeros((2, nx, ny)), phi3=[None, None], sweeps=[0, 0])
    for d in range(2):
        body = np.zeros(3)
        body[d] = 1.0
        faces = [np.zeros(s, order="F") for s in ((ny, nz), (ny, nz), (nx, nz), (nx, nz), (nx, ny), (nx, ny))]
        orc.enforce_stairstep_compatibility_3d(rhs, solid, body, *faces, dx, dy, dz)
        phi = np.zeros((nx + 2, ny + 2, nz), order="F") if phi0 is None else np.array(phi0[d], order="F")
        sw, res = orc.solve_stairstep_poisson_3d(phi, rhs, solid, body, *faces, xc, yc, zc, dx, dy, dz, 1e-10,
                                                 2000000, 50, "pcg")
        assert res <= 1e-10
        p2 = np.asfortranarray(phi[1:nx + 1, 1:ny + 1, 0])
        terms, _, _ = orc.fpm_partition_terms_2d(p2, body[:2], fr["u"], fr["v"], fr["solid"], fr["xf"], fr["yf"],
                                                 fr["kin"], fr["ring"], fr["dt"], 1.0 / foil.RE)
        out["terms"][d], out["phi"][d], out["phi3"][d], out["sweeps"][d] = terms, p2, phi, sw
    return out


def test_warm_started_dump_matches_oracle(gpu_lib):
    """The second dump of a series, warm-started from the first dump's
    potentials (src/fpm_stairstep_mpi_3d.f90:110: phi is the initial guess),
    against the oracle warm-started the same way from its own first dump,
    with the F_BOUND ring built from the neighbouring dumps
    (src/fpm_partition_2d.f90:84-87): potentials within 1e-9 relative,
    terms within 1e-8."""
    from flowfpmpp_gb300 import foil, workloads
    frames = workloads.foil_series(nframes=3, nx=96, ny=80, dt=0.002)
    r, dt = foil.ring_from_neighbours(frames[0], frames[2])
    mid = dict(frames[1], ring=r, dt=dt)
    for method in ("pcg", "pcg_mg"):
        gpu = foil.partition_series(frames, method, warm=True, ring="neighbours")[1]
        o0 = _oracle_frame(frames[0])
        o1 = _oracle_frame(mid, phi0=o0["phi3"])
        scale = np.abs(o1["phi"]).max()
        assert np.abs(gpu["phi"] - o1["phi"]).max() <= 1e-9 * scale, method
        tscale = np.abs(o1["terms"]).max()
        assert np.abs(gpu["terms"] - o1["terms"]).max() <= 1e-8 * tscale, (method, gpu["terms"], o1["terms"])
        if method == "pcg":
            assert np.abs(np.asarray(gpu["sweeps"]) - np.asarray(o1["sweeps"])).max() <= 50
