"""Batched uneven 2-D frames on the GPU against the oracle run frame by frame
(compatibility, FP64 PCG to the same tolerance, four-term partition), on a
small batch of the 256-frame foil generator (elliptic foils, Lamb-Oseen vortices,
noisy outer ring).  Potentials within 1e-9 relative max-norm; force terms
within 1e-8 relative to the frame's largest term."""
import numpy as np
import pytest

import oracle as orc
from cases import F

pytestmark = pytest.mark.gpu


def oracle_frame(fr, tol):
    from flowfpmpp_gb300.workloads import frame_as_stairstep
    s = frame_as_stairstep(fr)
    terms, phis = [], []
    for axis in range(2):
        body = np.zeros(3)
        body[axis] = 1.0
        faces = [x.copy(order="F") for x in s["faces"]]
        orc.enforce_stairstep_compatibility_3d(s["rhs"], s["solid"], body, *faces, s["dx"], s["dy"], s["dz"])
        phi = s["phi"].copy(order="F")
        orc.solve_stairstep_poisson_3d(phi, s["rhs"], s["solid"], body, *faces, s["xc"], s["yc"], s["zc"], s["dx"],
                                       s["dy"], s["dz"], tol, 2000000, 50, "pcg")
        p2 = np.asfortranarray(phi[1:fr["nx"] + 1, 1:fr["ny"] + 1, 0])
        t, _, _ = orc.fpm_partition_terms_2d(p2, body[:2], fr["u"], fr["v"], fr["solid"], fr["xf"], fr["yf"],
                                             fr["kin"], fr["ring"], fr["dt"], fr["nu"])
        terms.append(t)
        phis.append(p2)
    return np.array(terms), phis


def test_batched_frames_match_oracle(gpu_lib):
    from flowfpmpp_gb300 import partition as pt
    from flowfpmpp_gb300 import workloads
    frames = workloads.foil_frames(nframes=5, seed=21, nmin=40, nmax=90)
    tol = 1e-11
    terms, sweeps, res, phis = pt.partition_frames_2d(frames, tolerance=tol, return_phi=True)
    assert np.all(res <= 2 * tol), res
    assert np.all(sweeps > 0)
    for f, fr in enumerate(frames):
        ot, ophi = oracle_frame(fr, tol)
        for r in range(2):
            scale = np.abs(ophi[r]).max()
            assert np.abs(phis[f][r] - ophi[r]).max() <= 1e-9 * scale, (f, r)
            assert np.abs(terms[f, r] - ot[r]).max() <= 1e-8 * np.abs(ot[r]).max(), (f, r, terms[f, r], ot[r])


@pytest.mark.parametrize("rows", [2, 8])
def test_batched_frames_block_tile_heights(gpu_lib, monkeypatch, rows):
    """The frame multigrid's level-0 block tiles of 32 x 16 and 32 x 64 cells
    (FPM_FRAMES_ROWS) reach the tolerance and the potentials of the default
    32 x 32 tiles (1e-9 relative), on frames from 40^2 to 150^2 cells (several
    block tiles, ragged edges)."""
    from flowfpmpp_gb300 import partition as pt
    from flowfpmpp_gb300 import workloads
    frames = workloads.foil_frames(nframes=4, seed=23, nmin=40, nmax=150)
    tol = 1e-11
    monkeypatch.delenv("FPM_FRAMES_ROWS", raising=False)
    t4, _, r4, p4 = pt.partition_frames_2d(frames, tolerance=tol, return_phi=True)
    monkeypatch.setenv("FPM_FRAMES_ROWS", str(rows))
    t, _, res, p = pt.partition_frames_2d(frames, tolerance=tol, return_phi=True)
    assert np.all(res <= 2 * tol) and np.all(r4 <= 2 * tol), (res, r4)
    for f in range(len(frames)):
        for d in range(2):
            scale = np.abs(p4[f][d]).max()
            assert np.abs(p[f][d] - p4[f][d]).max() <= 1e-9 * scale, (rows, f, d)
            assert np.abs(t[f, d] - t4[f, d]).max() <= 1e-8 * np.abs(t4[f, d]).max(), (rows, f, d)
