"""GPU parity at the benchmark configurations' own sizes, against the CPU
oracle on the same seeded inputs (no comparison of the CUDA path with itself):

  C1  64x64x32 sphere, phi_x/phi_y/phi_z to a 1e-10 max-norm residual with
      plain FP64 PCG and the multigrid-preconditioned refinement, then the
      force densities in the C1 flow: potentials within 1e-9 relative
      max-norm, density fields and their integrals within 1e-8 relative
      (the required tolerances).
  C2  256^3 boxes, exactly 2000 weighted-Jacobi sweeps: the FP64
      (fused multiply-add) and double-float sweeps within 1e-12 relative of
      the oracle's 2000 sweeps (the configuration's own check).
  C3  384x384x192 ellipsoids, phi_x with the multigrid refinement and with
      plain FP64 PCG against the oracle's FP64 PCG (fixture
      tests/golden/c3_phix_oracle.npz made by make_c3_oracle.py): within
      1e-9 relative max-norm at the fixture's sampled cells.
"""
import os

import numpy as np
import pytest

import oracle as orc

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
C3_FIXTURE = os.path.join(HERE, "golden", "c3_phix_oracle.npz")


def rel_linf(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def solve_and_terms(mod, f, axis, method, tol, max_it, ci, flow=None):
    body = np.zeros(3)
    body[axis] = 1.0
    faces = [x.copy(order="F") for x in f["faces"]]
    mod.enforce_stairstep_compatibility_3d(f["rhs"], f["solid"], body, *faces, f["dx"], f["dy"], f["dz"])
    phi = f["phi"].copy(order="F")
    sw, res = mod.solve_stairstep_poisson_3d(phi, f["rhs"], f["solid"], body, *faces, f["xc"], f["yc"], f["zc"],
                                             f["dx"], f["dy"], f["dz"], tol, max_it, ci, method)
    terms = None
    if flow is not None:
        bounds = np.array([-1e300, 1e300] * 3)
        terms = mod.compute_stairstep_fpm_terms_3d(phi, flow["u"], flow["v"], flow["w"], flow["ox"], flow["oy"],
                                                   flow["oz"], flow["ax"], flow["ay"], flow["az"], f["solid"], body,
                                                   f["xc"], f["yc"], f["zc"], f["dx"], f["dy"], f["dz"], *faces,
                                                   bounds)
    return phi, sw, res, terms


def test_c1_sphere_three_potentials_and_densities(gpu_lib):
    from flowfpmpp_gb300 import stairstep as ss
    from flowfpmpp_gb300 import workloads
    f = workloads.sphere_grid()
    assert (f["nx"], f["ny"], f["nz"]) == (64, 64, 32)
    flow = workloads.flow_c1(f)
    orc.set_threads(orc.max_threads())
    try:
        for axis in range(3):
            po, swo, reso, to = solve_and_terms(orc, f, axis, "pcg", 1e-10, 2000000, 50, flow)
            assert reso <= 1e-10
            for method in ("pcg", "pcg_mg"):
                pg, swg, resg, tg = solve_and_terms(ss, f, axis, method, 1e-10, 2000000, 50, flow)
                assert resg <= 1e-10, (axis, method, resg)
                assert rel_linf(pg, po) <= 1e-9, (axis, method, rel_linf(pg, po))
                if method == "pcg":
                    assert abs(swg - swo) <= 50, (swg, swo)
                # gx, gy, gz, vortex, advection, totals
                for k in range(5):
                    assert rel_linf(tg[k], to[k]) <= 1e-8, (axis, method, k, rel_linf(tg[k], to[k]))
                scale = max(abs(to[5][0]), abs(to[5][1]))
                assert np.abs(np.asarray(tg[5]) - np.asarray(to[5])).max() <= 1e-8 * scale
    finally:
        orc.set_threads(1)


@pytest.mark.slow
def test_c2_boxes_256cubed_2000_sweeps(gpu_lib):
    from flowfpmpp_gb300 import stairstep as ss
    from flowfpmpp_gb300 import workloads
    f = workloads.boxes_grid(n=256)
    orc.set_threads(orc.max_threads())
    try:
        po, swo, _, _ = solve_and_terms(orc, f, 0, "jacobi", -1.0, 2000, 2000)
    finally:
        orc.set_threads(1)
    assert swo == 2000
    for method in ("jacobi_fma", "jacobi_df"):
        pg, swg, _, _ = solve_and_terms(ss, f, 0, method, -1.0, 2000, 2000)
        assert swg == 2000
        err = rel_linf(pg, po)
        print(f"C2 {method}: rel_linf vs oracle after 2000 sweeps {err:.2e}")
        assert err <= 1e-12, (method, err)


@pytest.mark.slow
def test_c3_phi_x_against_oracle_fixture(gpu_lib):
    from flowfpmpp_gb300 import stairstep as ss
    from flowfpmpp_gb300 import workloads
    fx = np.load(C3_FIXTURE)
    f = workloads.ellipsoids_grid()
    nx, ny, nz = f["nx"], f["ny"], f["nz"]
    assert tuple(int(x) for x in fx["grid"]) == (nx, ny, nz)
    assert int((f["solid"][1:nx + 1, 1:ny + 1, :] == 0).sum()) == int(fx["fluid_cells"])
    stride, ref, scale = int(fx["stride"]), fx["sample"], float(fx["checksum"][2])
    for method in ("pcg_mg", "pcg"):
        phi, sw, res, _ = solve_and_terms(ss, f, 0, method, 1e-10, 2000000, 50)
        assert res <= 1e-10
        flat = phi[1:nx + 1, 1:ny + 1, :].ravel(order="F")
        err = float(np.abs(flat[::stride] - ref).max() / scale)
        print(f"C3 phi_x {method}: {sw} iterations, rel_linf vs oracle at {ref.size} cells {err:.2e}")
        assert err <= 1e-9, (method, err)
        assert abs(flat.sum() - float(fx["checksum"][0])) <= 1e-9 * float(fx["checksum"][1])
        if method == "pcg":
            assert abs(sw - int(fx["iterations"])) <= 100, (sw, int(fx["iterations"]))
