"""GB300-native FlowFPM++ hot path: stair-step influence-potential solve and
force-partitioning densities as hand-written sm_103a CUDA kernels behind a C
ABI (include/fpm_capi.h, libfpm_gb300.so).

The Python modules mirror the reference's Fortran modules (same procedure
names and argument meaning) on top of that C ABI:
  stairstep  -- fpm_stairstep_mpi_3d
  laplace    -- fpm_laplace_3d and fpm_terms_3d (no body)
  partition  -- fpm_partition_2d
"""
from ._lib import FpmError, lib  # noqa: F401
from . import laplace, partition, stairstep  # noqa: F401

__all__ = ["FpmError", "lib", "stairstep", "laplace", "partition"]
