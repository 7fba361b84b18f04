"""Reader and writer of the reference's 2-D frame formats.

FFPM2D02 (input, examples/flapping_foil_fpm.f90:163-171 and
README "Example data format"): little-endian Fortran stream,
  character(8) 'FFPM2D02'; int32 nx, ny; real64 xf(0:nx), yf(0:ny);
  real64 u(nx,ny), v(nx,ny); int8 solid(nx,ny); real64 dt;
  real64 ring(2nx+2ny, 2, 2); real64 kin(6); real64 time.
Output (examples/flapping_foil_fpm.f90:242-245): int32 nx, ny; real64
xc(nx), yc(ny), omega(nx,ny), vif_x(nx,ny), vif_y(nx,ny), phi_x(nx,ny),
phi_y(nx,ny), solid(nx,ny) as 0/1 reals.
"""
from __future__ import annotations

import numpy as np

MAGIC = b"FFPM2D02"


def read_ffpm2d02(path):
    """Returns a frame dict (nx, ny, xf, yf, u, v, solid, dt, ring, kin, time).
    A path ending in .xz is decompressed first."""
    if str(path).endswith(".xz"):
        import lzma
        with lzma.open(path, "rb") as fh:
            raw = fh.read()
    else:
        with open(path, "rb") as fh:
            raw = fh.read()
    if raw[:8] != MAGIC:
        raise ValueError("unexpected input format")
    nx, ny = (int(x) for x in np.frombuffer(raw, dtype="<i4", count=2, offset=8))
    if nx < 2 or ny < 2 or nx > 100000 or ny > 100000:
        raise ValueError("implausible grid size (byte order?)")
    off = 16

    def take(dtype, count, shape=None):
        nonlocal off
        a = np.frombuffer(raw, dtype=dtype, count=count, offset=off)
        off += a.nbytes
        return np.asfortranarray(a.reshape(shape, order="F")) if shape else a.copy()

    xf = take("<f8", nx + 1)
    yf = take("<f8", ny + 1)
    u = take("<f8", nx * ny, (nx, ny))
    v = take("<f8", nx * ny, (nx, ny))
    solid = take("i1", nx * ny, (nx, ny))
    dt = float(take("<f8", 1)[0])
    ring = take("<f8", (2 * nx + 2 * ny) * 4, (2 * nx + 2 * ny, 2, 2))
    kin = take("<f8", 6)
    time = float(take("<f8", 1)[0])
    if off != len(raw):
        raise ValueError(f"frame size mismatch: read {off} of {len(raw)} bytes")
    return dict(nx=nx, ny=ny, xf=xf, yf=yf, u=u, v=v, solid=(solid != 0).astype(np.uint8), dt=dt, ring=ring,
                kin=kin, time=time)


def write_partition_output(path, frame, omega, vif, phi):
    """The reference example's output layout; vif and phi are (2, nx, ny)."""
    nx, ny = frame["nx"], frame["ny"]
    xf, yf = frame["xf"], frame["yf"]
    xc = 0.5 * (xf[:-1] + xf[1:])
    yc = 0.5 * (yf[:-1] + yf[1:])
    with open(path, "wb") as fh:
        fh.write(np.array([nx, ny], dtype="<i4").tobytes())
        for a in (xc, yc, omega, vif[0], vif[1], phi[0], phi[1], (np.asarray(frame["solid"]) != 0) * 1.0):
            fh.write(np.asarray(a, dtype="<f8").tobytes(order="F"))
