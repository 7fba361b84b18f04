"""The one-pass force densities of several potentials
(fpm_compute_stairstep_fpm_terms_3d_multi_dev, double-float per-cell
arithmetic) against the oracle's FP64 compute_stairstep_fpm_terms_3d
(src/fpm_stairstep_mpi_3d.f90:426-497) run on each potential: density fields
within 1e-12 relative max-norm (the double-float arithmetic carries a 48-bit
significand; the required bound is 1e-8) and integrals within 1e-12 of the
largest integral, on the C1 sphere (three potentials) and on a random
stretched grid with interior bounds and random fields (one to four
potentials)."""
import ctypes

import numpy as np
import pytest

import oracle as orc
from gpu_util import from_dev, ptr, stream_ptr, to_dev

pytestmark = pytest.mark.gpu
VP = ctypes.c_void_p


def multi_terms(lib, f, phis, flow, bgs, faces_list, bounds):
    import torch
    nx, ny, nz = f["nx"], f["ny"], f["nz"]
    n3 = nx * ny * nz
    np_ = len(phis)
    dphi = [to_dev(p) for p in phis]
    dflow = [to_dev(flow[k]) for k in ("u", "v", "w", "ox", "oy", "oz", "ax", "ay", "az")]
    dsolid = to_dev(f["solid"])
    dax = [to_dev(f[k]) for k in ("xc", "yc", "zc", "dx", "dy", "dz")]
    dfaces = [to_dev(x) for faces in faces_list for x in faces]
    outs = [torch.empty(n3, dtype=torch.float64, device="cuda") for _ in range(5 * np_)]
    bg = np.ascontiguousarray(np.concatenate(bgs), dtype=np.float64)
    b = np.ascontiguousarray(bounds, dtype=np.float64)
    tot = (ctypes.c_double * (2 * np_))()
    rc = lib.fpm_compute_stairstep_fpm_terms_3d_multi_dev(
        np_, (VP * np_)(*[t.data_ptr() for t in dphi]), *[ptr(t) for t in dflow], ptr(dsolid), bg.ctypes.data_as(VP),
        *[ptr(t) for t in dax], (VP * (6 * np_))(*[t.data_ptr() for t in dfaces]), b.ctypes.data_as(VP),
        (VP * (5 * np_))(*[t.data_ptr() for t in outs]), tot, nx, ny, nz, stream_ptr())
    assert rc == 0, lib.fpm_last_error()
    fields = [[from_dev(outs[5 * m + c], (nx, ny, nz)) for c in range(5)] for m in range(np_)]
    return fields, [(tot[2 * m], tot[2 * m + 1]) for m in range(np_)]


def check(fields, totals, ref):
    scale_t = max(max(abs(a), abs(b)) for (_, (a, b)) in ref) or 1.0
    for m, (fl, (ta, tb)) in enumerate(zip(fields, totals)):
        rf, (ra, rb) = ref[m]
        for c in range(5):
            err = np.abs(fl[c] - rf[c]).max() / max(np.abs(rf[c]).max(), 1e-300)
            assert err <= 1e-12, (m, c, err)
        assert abs(ta - ra) <= 1e-12 * scale_t and abs(tb - rb) <= 1e-12 * scale_t, (m, ta, ra, tb, rb)


def oracle_terms(f, phi, flow, bg, faces, bounds):
    out = orc.compute_stairstep_fpm_terms_3d(phi, flow["u"], flow["v"], flow["w"], flow["ox"], flow["oy"], flow["oz"],
                                             flow["ax"], flow["ay"], flow["az"], f["solid"], bg, f["xc"], f["yc"],
                                             f["zc"], f["dx"], f["dy"], f["dz"], *faces, bounds)
    return list(out[:5]), tuple(out[5])


def test_c1_sphere_three_potentials(gpu_lib):
    from flowfpmpp_gb300 import workloads
    f = workloads.sphere_grid()
    flow = workloads.flow_c1(f)
    bounds = np.array([-1e300, 1e300] * 3)
    phis, bgs, faces_list, ref = [], [], [], []
    for axis in range(3):
        bg = np.zeros(3)
        bg[axis] = 1.0
        faces = [x.copy(order="F") for x in f["faces"]]
        orc.enforce_stairstep_compatibility_3d(f["rhs"], f["solid"], bg, *faces, f["dx"], f["dy"], f["dz"])
        phi = f["phi"].copy(order="F")
        orc.solve_stairstep_poisson_3d(phi, f["rhs"], f["solid"], bg, *faces, f["xc"], f["yc"], f["zc"], f["dx"],
                                       f["dy"], f["dz"], 1e-10, 100000, 50, "pcg")
        phis.append(phi)
        bgs.append(bg)
        faces_list.append(faces)
        ref.append(oracle_terms(f, phi, flow, bg, faces, bounds))
    fields, totals = multi_terms(gpu_lib, f, phis, flow, bgs, faces_list, bounds)
    check(fields, totals, ref)


@pytest.mark.parametrize("npot", [1, 2, 4])
def test_random_grid_interior_bounds(gpu_lib, npot):
    from flowfpmpp_gb300 import workloads
    rng = np.random.default_rng(100 + npot)
    nx, ny, nz = 37, 29, 11
    ax = workloads.geometric_axis(nx, -2.0, 3.0, 1.07)
    ay = workloads.geometric_axis(ny, -1.5, 1.5, 1.04)
    az = workloads.geometric_axis(nz, -1.0, 1.0, 1.1)
    X = ax[1][1:nx + 1][:, None, None]
    Y = ay[1][1:ny + 1][None, :, None]
    Z = az[1][1:nz + 1][None, None, :]
    solid = (((X - 0.3) / 0.8) ** 2 + (Y / 0.6) ** 2 + (Z / 0.5) ** 2 < 1).astype(np.int32)
    f = workloads._frame(nx, ny, nz, ax, ay, az, solid, 0)
    flow = {k: np.asfortranarray(rng.standard_normal((nx, ny, nz)) * 10.0 ** rng.uniform(-3, 2))
            for k in ("u", "v", "w", "ox", "oy", "oz", "ax", "ay", "az")}
    bounds = np.array([-1.2, 2.1, -1.0, 0.9, -0.7, 0.8])
    phis, bgs, faces_list, ref = [], [], [], []
    for m in range(npot):
        phi = np.zeros((nx + 2, ny + 2, nz), order="F")
        phi[1:nx + 1, 1:ny + 1, :] = rng.standard_normal((nx, ny, nz)) * (solid == 0) + 3.0
        bg = rng.standard_normal(3)
        faces = [np.asfortranarray(rng.standard_normal(x.shape)) for x in f["faces"]]
        phis.append(phi)
        bgs.append(bg)
        faces_list.append(faces)
        ref.append(oracle_terms(f, phi, flow, bg, faces, bounds))
    fields, totals = multi_terms(gpu_lib, f, phis, flow, bgs, faces_list, bounds)
    check(fields, totals, ref)
