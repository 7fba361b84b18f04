"""Generates tests/golden/c3_phix_oracle.npz: the CPU oracle's plain FP64 PCG
solve of phi_x on the three-ellipsoid 384x384x192 grid (stretching ratio 1.02,
smallest cell 0.01; workloads.ellipsoids_grid with its default seed), to a
1e-10 max-norm residual with check interval 50 -- the reference's
solve_stairstep_poisson_3d(method='pcg') after
enforce_stairstep_compatibility_3d (src/fpm_stairstep_mpi_3d.f90:41-92,
106-330).

The full field (28.3 M cells, 226 MB) is too large to commit, so the fixture
keeps every STRIDE-th interior cell in Fortran order (x fastest) plus
whole-field checksums; the inputs are regenerated from the seeded generator.
OpenMP over z-planes on every core: about an hour on 8 cores.

Usage: python tests/golden/make_c3_oracle.py [threads]
"""
import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle as orc  # noqa: E402
from flowfpmpp_gb300 import workloads  # noqa: E402

STRIDE = 331
OUT = os.path.join(HERE, "c3_phix_oracle.npz")


def inputs_digest(f):
    h = hashlib.sha256()
    for k in ("xc", "yc", "zc", "dx", "dy", "dz", "solid"):
        h.update(np.ascontiguousarray(f[k]).tobytes())
    return h.hexdigest()


def main(threads):
    orc.build()
    f = workloads.ellipsoids_grid()
    nx, ny, nz = f["nx"], f["ny"], f["nz"]
    body = np.array([1.0, 0.0, 0.0])
    faces = [x.copy(order="F") for x in f["faces"]]
    corr, imb = orc.enforce_stairstep_compatibility_3d(f["rhs"], f["solid"], body, *faces, f["dx"], f["dy"], f["dz"])
    phi = f["phi"].copy(order="F")
    orc.set_threads(threads)
    t0 = time.time()
    sw, res = orc.solve_stairstep_poisson_3d(phi, f["rhs"], f["solid"], body, *faces, f["xc"], f["yc"], f["zc"],
                                             f["dx"], f["dy"], f["dz"], 1e-10, 2000000, 50, "pcg")
    el = time.time() - t0
    interior = np.asarray(phi[1:nx + 1, 1:ny + 1, :]).ravel(order="F")
    fluid = (np.asarray(f["solid"][1:nx + 1, 1:ny + 1, :]) == 0).ravel(order="F")
    idx = np.arange(0, interior.size, STRIDE, dtype=np.int64)
    np.savez_compressed(OUT, stride=STRIDE, grid=np.array([nx, ny, nz]), iterations=sw, residual=res,
                        correction=corr, imbalance=imb, sample=interior[idx],
                        checksum=np.array([interior.sum(), np.abs(interior).sum(), np.abs(interior).max()]),
                        fluid_cells=int(fluid.sum()), inputs_sha256=inputs_digest(f), seconds=el, threads=threads)
    print(f"phi_x: {sw} iterations, residual {res:.3e}, {el:.0f} s on {threads} threads -> {OUT}")


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else os.cpu_count())
