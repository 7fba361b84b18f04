"""GB300-native FlowFPM++ hot path: stair-step influence-potential solve and
force-partitioning densities as hand-written sm_103a CUDA kernels behind a C
ABI (include/fpm_capi.h, libfpm_gb300.so).

The Python modules mirror the reference's Fortran modules (same procedure
names and argument meaning) on top of that C ABI:
  stairstep  -- fpm_stairstep_mpi_3d
"""
from ._lib import FpmError, lib  # noqa: F401
from . import stairstep  # noqa: F401

__all__ = ["FpmError", "lib", "stairstep"]
