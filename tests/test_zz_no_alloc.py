"""The allocation-free operator residual (fpm_stairstep_operator_residual_noalloc_dev).

It serves callers that cannot allocate GPU memory while they run (fixed
memory pools, allocator policies that forbid cudaMalloc, hard caps on the GPU
footprint): its scratch lives in a fixed device array inside the library.
Through the C ABI, two calls in a row (different fields and grid sizes, so
the shared scratch is reused) must give the same max-norm residual as the
allocating entry point fpm_stairstep_operator_residual_dev -- bit for bit,
the tolerance the other max-norm residual tests use -- and the size limit must
be reported as an error.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

import oracle as orc
from cases import F, stairstep_case_exact
from gpu_util import ptr, stream_ptr, to_dev

pytestmark = pytest.mark.gpu

D, I = ctypes.c_double, ctypes.c_int


def _operator(c):
    nx, ny, nz = c["nx"], c["ny"], c["nz"]
    faces = [f.copy(order="F") for f in c["faces"]]
    orc.enforce_stairstep_compatibility_3d(c["rhs"], c["solid"], c["body"], *faces, c["dx"], c["dy"], c["dz"])
    coefs = orc.stairstep_coefficients(c["xc"], c["yc"], c["zc"], c["dx"], c["dy"], c["dz"])
    src, diag, rdiag, _ = orc.build_operator(c["rhs"], c["solid"], c["body"], *faces, coefs, c["dx"], c["dy"],
                                             c["dz"], True)
    return src, diag


def _case(nx, ny, nz, seed):
    from flowfpmpp_gb300 import workloads
    ax, ay, az = (workloads.geometric_axis(n, -1.0, 1.0, 1.04) for n in (nx, ny, nz))
    solid = F((nx + 2, ny + 2, nz), np.int32)
    solid[2:5, 3:6, 1:3] = 1
    c = dict(nx=nx, ny=ny, nz=nz, xc=ax[1], yc=ay[1], zc=az[1][1:nz + 1].copy(), dx=ax[2], dy=ay[2], dz=az[2],
             solid=solid, rhs=F((nx, ny, nz)), body=np.array([0.0, 1.0, 0.0]),
             faces=[F((ny, nz)), F((ny, nz)), F((nx, nz)), F((nx, nz)), F((nx, ny)), F((nx, ny))])
    rng = np.random.default_rng(seed)
    phi = F((nx + 2, ny + 2, nz))
    phi[1:nx + 1, 1:ny + 1, :] = rng.standard_normal((nx, ny, nz)) * (solid[1:nx + 1, 1:ny + 1, :] == 0)
    return c, phi


def _both(lib, c, phi, src, diag):
    nx, ny, nz = c["nx"], c["ny"], c["nz"]
    dphi, dsrc, ddiag = to_dev(phi), to_dev(src), to_dev(diag)
    dax = [to_dev(c[k]) for k in ("xc", "yc", "zc", "dx", "dy", "dz")]
    ref, new = D(), D()
    rc = lib.fpm_stairstep_operator_residual_dev(ptr(dphi), ptr(dsrc), ptr(ddiag), *[ptr(x) for x in dax], I(nx),
                                                 I(ny), I(nz), ctypes.byref(ref), stream_ptr())
    assert rc == 0, lib.fpm_last_error()
    rc = lib.fpm_stairstep_operator_residual_noalloc_dev(ptr(dphi), ptr(dsrc), ptr(ddiag), *[ptr(x) for x in dax],
                                                         I(nx), I(ny), I(nz), ctypes.byref(new), stream_ptr())
    assert rc == 0, lib.fpm_last_error()
    return ref.value, new.value


def test_no_alloc_residual_matches_allocating_entry_point(gpu_lib):
    # first call: the reference test grid with a random field
    c = stairstep_case_exact(False)
    src, diag = _operator(c)
    rng = np.random.default_rng(3)
    phi = c["phi"].copy(order="F")
    phi[1:c["nx"] + 1, 1:c["ny"] + 1, :] = rng.standard_normal((c["nx"], c["ny"], c["nz"]))
    ref1, new1 = _both(gpu_lib, c, phi, src, diag)
    assert ref1 > 0 and new1 == ref1
    assert new1 == orc.operator_residual(phi, src, diag,
                                         orc.stairstep_coefficients(c["xc"], c["yc"], c["zc"], c["dx"], c["dy"],
                                                                    c["dz"]))
    # second call in a row: another grid size and field, same shared scratch
    c2, phi2 = _case(53, 17, 9, seed=4)
    src2, diag2 = _operator(c2)
    ref2, new2 = _both(gpu_lib, c2, phi2, src2, diag2)
    assert ref2 > 0 and new2 == ref2 and ref2 != ref1


def test_no_alloc_residual_leaves_free_device_memory_unchanged(gpu_lib):
    """The property the entry point exists for: after a first call (which
    loads the kernels and looks the scratch address up), further calls do not
    change the device's free memory."""
    import torch
    c2, phi2 = _case(53, 17, 9, seed=5)
    src2, diag2 = _operator(c2)
    nx, ny, nz = c2["nx"], c2["ny"], c2["nz"]
    dphi, dsrc, ddiag = to_dev(phi2), to_dev(src2), to_dev(diag2)
    dax = [to_dev(c2[k]) for k in ("xc", "yc", "zc", "dx", "dy", "dz")]
    v = D()

    def call():
        rc = gpu_lib.fpm_stairstep_operator_residual_noalloc_dev(ptr(dphi), ptr(dsrc), ptr(ddiag),
                                                                 *[ptr(x) for x in dax], I(nx), I(ny), I(nz),
                                                                 ctypes.byref(v), stream_ptr())
        assert rc == 0, gpu_lib.fpm_last_error()
        return v.value

    first = call()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    values = [call() for _ in range(3)]
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert all(x == first for x in values)


def test_no_alloc_rejects_sizes_beyond_its_limit(gpu_lib):
    c = stairstep_case_exact(False)
    src, diag = _operator(c)
    dphi, dsrc, ddiag = to_dev(c["phi"]), to_dev(src), to_dev(diag)
    dax = [to_dev(c[k]) for k in ("xc", "yc", "zc", "dx", "dy", "dz")]
    v = D()
    rc = gpu_lib.fpm_stairstep_operator_residual_noalloc_dev(ptr(dphi), ptr(dsrc), ptr(ddiag), *[ptr(x) for x in dax],
                                                             I(12000), I(200), I(100), ctypes.byref(v), stream_ptr())
    assert rc == 8 and b"limit" in gpu_lib.fpm_last_error()
