"""Force partition of one 2-D frame, the GPU counterpart of the reference
example examples/flapping_foil_fpm.f90 (a frame of a flapping-foil
simulation in the FFPM2D02 format).

For x and y: zero outer normal derivative, body_grad = e_dir, compatibility,
stair-step solve to the tolerance (check interval 50, cap 2e6), then the four
FPM terms (F_KINE, F_VIF, F_VIS, F_BOUND) per unit span and density.  The
frame is solved as the reference does it: two z cells of total span 1 with
zero z-face data.

    python -m flowfpmpp_gb300.foil [pcg|pcg_mixed] [input [output [tolerance]]]
"""
from __future__ import annotations

import sys
import time

import numpy as np

from . import partition as pt
from . import stairstep as ss
from .frame_io import read_ffpm2d02, write_partition_output

RE = 1.0e4  # examples/flapping_foil_fpm.f90:180


def frame_axes(fr):
    """dx, dy, xc(0:nx+1), yc(0:ny+1) as examples/flapping_foil_fpm.f90:211-213."""
    dx = fr["xf"][1:] - fr["xf"][:-1]
    dy = fr["yf"][1:] - fr["yf"][:-1]
    xc = np.concatenate([[0.0], 0.5 * (fr["xf"][:-1] + fr["xf"][1:]), [0.0]])
    yc = np.concatenate([[0.0], 0.5 * (fr["yf"][:-1] + fr["yf"][1:]), [0.0]])
    xc[0], xc[-1] = xc[1] - dx[0], xc[-2] + dx[-1]
    yc[0], yc[-1] = yc[1] - dy[0], yc[-2] + dy[-1]
    return dx, dy, xc, yc


def partition_frame(fr, method="pcg", tolerance=1e-10, nu=1.0 / RE, phi0=None):
    """Returns dict(terms (2,4), sweeps (2,), residual (2,), phi (2,nx,ny),
    vif (2,nx,ny), omega (nx,ny), seconds, phi3 (the two padded 3-D
    potentials)).  phi0: the padded potentials to start from (the solver's
    initial guess, src/fpm_stairstep_mpi_3d.f90:110), e.g. the previous
    frame's phi3; default zero."""
    nx, ny, nz = fr["nx"], fr["ny"], 2
    dx, dy, xc, yc = frame_axes(fr)
    dz = np.array([0.5, 0.5])
    zc = np.array([0.25, 0.75])
    solid = np.zeros((nx + 2, ny + 2, nz), dtype=np.int32, order="F")
    for k in range(nz):
        solid[1:nx + 1, 1:ny + 1, k] = fr["solid"]
    rhs = np.zeros((nx, ny, nz), order="F")
    out = dict(terms=np.zeros((2, 4)), sweeps=np.zeros(2, dtype=int), residual=np.zeros(2),
               phi=np.zeros((2, nx, ny)), vif=np.zeros((2, nx, ny)), phi3=[None, None])
    t0 = time.perf_counter()
    for d in range(2):
        body = np.zeros(3)
        body[d] = 1.0
        faces = [np.zeros(s, order="F") for s in ((ny, nz), (ny, nz), (nx, nz), (nx, nz), (nx, ny), (nx, ny))]
        ss.enforce_stairstep_compatibility_3d(rhs, solid, body, *faces, dx, dy, dz)
        phi = np.zeros((nx + 2, ny + 2, nz), order="F") if phi0 is None else np.array(phi0[d], order="F")
        sw, res = ss.solve_stairstep_poisson_3d(phi, rhs, solid, body, *faces, xc, yc, zc, dx, dy, dz, tolerance,
                                                2000000, 50, method)
        p2 = np.asfortranarray(phi[1:nx + 1, 1:ny + 1, 0])
        terms, vif, omega = pt.fpm_partition_terms_2d(p2, body[:2], fr["u"], fr["v"], fr["solid"], fr["xf"],
                                                      fr["yf"], fr["kin"], fr["ring"], fr["dt"], nu)
        out["terms"][d], out["sweeps"][d], out["residual"][d] = terms, sw, res
        out["phi"][d], out["vif"][d] = p2, vif
        out["phi3"][d] = phi
        out["omega"] = omega
    out["seconds"] = time.perf_counter() - t0
    return out


def ring_from_neighbours(prev, nxt):
    """The F_BOUND ring of a frame from its neighbouring dumps: u and v in the
    outer-boundary cells (west column, east column, south row, north row) of
    the dump before and the dump after, and dt half their time distance
    (the layout of the FFPM2D02 ring, src/fpm_partition_2d.f90:84-87)."""
    nx, ny = prev["nx"], prev["ny"]
    ring = np.zeros((2 * nx + 2 * ny, 2, 2), order="F")
    for t, fr in ((0, prev), (1, nxt)):
        for comp, key in ((0, "u"), (1, "v")):
            a = fr[key]
            ring[:, comp, t] = np.concatenate([a[0, :], a[nx - 1, :], a[:, 0], a[:, ny - 1]])
    return ring, 0.5 * (nxt["time"] - prev["time"])


def partition_series(frames, method="pcg_mg", tolerance=1e-10, nu=1.0 / RE, warm=True, ring="file"):
    """Force partition of a time series of dumps on one grid: each frame as
    partition_frame, its potentials started from the previous frame's when
    `warm` (the solver takes phi as its initial guess; cells that turned solid
    are zeroed by the solver), and with ring="neighbours" the F_BOUND ring of
    the interior frames taken from the dumps before and after
    (ring_from_neighbours; the first and last frames keep their own).
    Returns the list of partition_frame results."""
    out, prev = [], None
    for k, fr in enumerate(frames):
        if prev is not None and (fr["nx"], fr["ny"]) != (frames[k - 1]["nx"], frames[k - 1]["ny"]):
            raise ValueError("a series must stay on one grid")
        f = fr
        if ring == "neighbours" and 0 < k < len(frames) - 1:
            r, dt = ring_from_neighbours(frames[k - 1], frames[k + 1])
            f = dict(fr, ring=r, dt=dt)
        res = partition_frame(f, method, tolerance, nu, phi0=prev["phi3"] if (warm and prev is not None) else None)
        out.append(res)
        prev = res
    return out


def main(argv):
    method = argv[1] if len(argv) > 1 else "pcg"
    path = argv[2] if len(argv) > 2 else "flapping_foil_216000.bin"
    output = argv[3] if len(argv) > 3 else "flapping_foil_fpm.bin"
    tol = float(argv[4]) if len(argv) > 4 else 1e-10
    fr = read_ffpm2d02(path)
    print(f"frame: {fr['nx']} x {fr['ny']} cells, {int(fr['solid'].sum())} solid, t = {fr['time']:8.3f}")
    r = partition_frame(fr, method, tol)
    for d in range(2):
        print(f"direction {d + 1}: PCG iterations {r['sweeps'][d]}, residual {r['residual'][d]:10.3e}")
    print(f"solve and partition seconds: {r['seconds']:10.3f}")
    print("force partition per unit span and density (x = drag direction, y = lift):")
    names = ("F_KINE  (body acceleration)", "F_VIF   (vortex-induced)   ", "F_VIS   (viscous)          ",
             "F_BOUND (outer boundary)   ")
    for t, nm in enumerate(names):
        print(f"  {nm}       {r['terms'][0, t]:14.5e}{r['terms'][1, t]:14.5e}")
    s = r["terms"].sum(axis=1)
    print(f"  sum = pressure force             {s[0]:14.5e}{s[1]:14.5e}")
    write_partition_output(output, fr, r["omega"], r["vif"], r["phi"])
    print("wrote " + output)


if __name__ == "__main__":
    main(sys.argv)
