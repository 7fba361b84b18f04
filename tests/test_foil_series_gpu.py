"""A time series of 2-D dumps on one grid (the reference foil example's
frame, examples/flapping_foil_fpm.f90, over consecutive dumps): potentials
warm-started from the previous frame reach the same tolerance and the same
potentials (1e-9 relative) and terms (1e-8 relative) as cold starts (FP64 PCG: in fewer iterations); the
F_BOUND ring built from the neighbouring dumps gives the
terms of the ring stored in the frames (equal by construction here)."""
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
