"""Generates tests/golden/foil_frame_oracle.json: the CPU oracle run on the
reference's real flapping-foil frame (examples/data/flapping_foil_216000.bin of
the reference repository), exactly as examples/flapping_foil_fpm.f90:71-81 does
it: for x and y, zero outer data, compatibility, PCG to 1e-10 (check interval
50, cap 2e6), then fpm_partition_terms_2d.  Serial oracle (the reference's CPU
reduction order), about ten minutes on one core.

Usage: python tests/golden/make_foil_golden.py /path/to/flapping_foil_216000.bin
The frame itself is not committed (12.9 MB); the JSON keeps its SHA-256.
"""
import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle as orc  # noqa: E402
from flowfpmpp_gb300.frame_io import read_ffpm2d02  # noqa: E402
from flowfpmpp_gb300.workloads import frame_as_stairstep  # noqa: E402


def main(path):
    fr = read_ffpm2d02(path)
    fr["nu"] = 1.0 / 1.0e4  # examples/flapping_foil_fpm.f90:180 (Re = 1e4)
    # axes as the example builds them (:211-213): mirrored halo centres
    dx = fr["xf"][1:] - fr["xf"][:-1]
    dy = fr["yf"][1:] - fr["yf"][:-1]
    xc = np.concatenate([[0.0], 0.5 * (fr["xf"][:-1] + fr["xf"][1:]), [0.0]])
    yc = np.concatenate([[0.0], 0.5 * (fr["yf"][:-1] + fr["yf"][1:]), [0.0]])
    xc[0], xc[-1] = xc[1] - dx[0], xc[-2] + dx[-1]
    yc[0], yc[-1] = yc[1] - dy[0], yc[-2] + dy[-1]
    fr["xc"], fr["yc"], fr["dx"], fr["dy"] = xc, yc, dx, dy
    s = frame_as_stairstep(fr)
    out = {"frame_sha256": hashlib.sha256(open(path, "rb").read()).hexdigest(), "nx": fr["nx"], "ny": fr["ny"],
           "solid_cells": int(fr["solid"].sum()), "tolerance": 1e-10, "directions": []}
    for axis in range(2):
        t0 = time.time()
        body = np.zeros(3)
        body[axis] = 1.0
        faces = [x.copy(order="F") for x in s["faces"]]
        corr, imb = orc.enforce_stairstep_compatibility_3d(s["rhs"], s["solid"], body, *faces, s["dx"], s["dy"],
                                                           s["dz"])
        phi = s["phi"].copy(order="F")
        sw, res = orc.solve_stairstep_poisson_3d(phi, s["rhs"], s["solid"], body, *faces, s["xc"], s["yc"], s["zc"],
                                                 s["dx"], s["dy"], s["dz"], 1e-10, 2000000, 50, "pcg")
        p2 = np.asfortranarray(phi[1:fr["nx"] + 1, 1:fr["ny"] + 1, 0])
        terms, vif, omega = orc.fpm_partition_terms_2d(p2, body[:2], fr["u"], fr["v"], fr["solid"], fr["xf"],
                                                       fr["yf"], fr["kin"], fr["ring"], fr["dt"], fr["nu"])
        out["directions"].append({"axis": "xy"[axis], "iterations": sw, "residual": res, "correction": corr,
                                  "imbalance": imb, "terms": terms.tolist(),
                                  "phi_checksum": [float(p2.sum()), float(np.abs(p2).sum())],
                                  "vif_checksum": [float(vif.sum()), float(np.abs(vif).sum())],
                                  "seconds": time.time() - t0})
        print(out["directions"][-1], flush=True)
    with open(os.path.join(HERE, "foil_frame_oracle.json"), "w") as fh:
        json.dump(out, fh, indent=1)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_foil_golden.py <flapping_foil_216000.bin>")
    main(sys.argv[1])
