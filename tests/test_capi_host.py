"""CPU-side checks of the C ABI: the library loads, exports every function
include/*.h declares, validates arguments on the host, and refuses to run
without a GPU instead of falling back to the CPU."""
import ctypes

import numpy as np
import pytest

from cases import stairstep_case_exact


def test_library_exports_every_declared_symbol():
    import flowfpmpp_gb300
    from flowfpmpp_gb300._lib import declared_symbols
    lib = flowfpmpp_gb300.lib()
    names = declared_symbols()
    assert len(names) >= 10
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_exchange_solid_halo_is_host_side():
    from flowfpmpp_gb300 import stairstep as ss
    solid = np.ones((6, 5, 3), dtype=np.int32, order="F")
    ss.exchange_solid_halo_3d(solid)
    assert solid[0].sum() == 0 and solid[-1].sum() == 0 and solid[:, 0].sum() == 0 and solid[:, -1].sum() == 0
    assert solid[1:-1, 1:-1].min() == 1


def test_bad_method_and_sizes_are_rejected_before_the_device():
    from flowfpmpp_gb300 import FpmError
    from flowfpmpp_gb300 import stairstep as ss
    c = stairstep_case_exact(False)
    base = (c["rhs"], c["solid"], c["body"], *c["faces"], c["xc"], c["yc"], c["zc"], c["dx"], c["dy"], c["dz"],
            1e-8, 10, 5)
    with pytest.raises(FpmError) as e:
        ss.solve_stairstep_poisson_3d(c["phi"].copy(order="F"), *base, method="gmres")
    assert e.value.code == 1 and "pcg or jacobi" in e.value.message
    import flowfpmpp_gb300
    lib = flowfpmpp_gb300.lib()
    z = ctypes.c_void_p(1)
    sw, res = ctypes.c_int(), ctypes.c_double()
    rc = lib.fpm_solve_stairstep_poisson_3d(*([z] * 16), 4, 4, 1, ctypes.c_double(1e-8), 10, 5, 0,
                                            ctypes.byref(sw), ctypes.byref(res))
    assert rc == 2 and b"nz>=2" in lib.fpm_last_error()
    rc = lib.fpm_solve_stairstep_poisson_3d(*([None] * 16), 4, 4, 4, ctypes.c_double(1e-8), 10, 5, 0,
                                            ctypes.byref(sw), ctypes.byref(res))
    assert rc == 5


def test_no_cpu_fallback_without_gpu():
    """On a machine without a GPU the solve fails loudly (FPM_E_NO_DEVICE or
    a CUDA error) instead of computing on the CPU."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from flowfpmpp_gb300 import FpmError
    from flowfpmpp_gb300 import stairstep as ss
    c = stairstep_case_exact(False)
    with pytest.raises(FpmError) as e:
        ss.solve_stairstep_poisson_3d(c["phi"].copy(order="F"), c["rhs"], c["solid"], c["body"], *c["faces"],
                                      c["xc"], c["yc"], c["zc"], c["dx"], c["dy"], c["dz"], 1e-8, 10, 5)
    assert e.value.code in (6, 7)
