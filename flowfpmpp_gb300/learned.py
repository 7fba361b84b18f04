"""Learned initial guess for the stair-step solve (host side).

The network, its training kernels and the solver hook are in the CUDA
library (``fpm_net_*`` and ``fpm_solve_stairstep_learned_dev`` in
include/fpm_capi.h); this module drives them:

* :class:`LearnedGuess` owns a network handle (parameters on the GPU) and
  saves / loads the flat parameter vector (``.npy``);
* :func:`random_bodies` and :func:`make_dataset` generate the training set:
  stair-step bodies made of 1-4 random ellipsoids and boxes, each with the
  FP64 PCG potential of one random axis as target;
* :func:`train` runs Adam over the dataset with the library's own forward
  and backward kernels;
* :func:`solve` is the stair-step solve with the learned initial guess.

Device arrays are torch CUDA tensors used as plain device memory.
"""
from __future__ import annotations

import ctypes
import math
import os
from dataclasses import dataclass

import numpy as np

from ._lib import check, lib
from . import stairstep as ss
from . import workloads

VP = ctypes.c_void_p
WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "learned_guess.npy")
TRAIN_DOMAIN = (3.0, 3.0, 1.5)  # half extents of the training / evaluation boxes
TRAIN_RATIO = 1.02


def _t():
    import torch
    return torch


def _p(t):
    return VP(t.data_ptr())


class LearnedGuess:
    """A network handle with its parameters on the current CUDA device."""

    def __init__(self, seed: int = 1, params: np.ndarray | None = None):
        h = VP()
        check(lib().fpm_net_create(ctypes.c_ulonglong(seed), ctypes.byref(h)))
        self.h = h
        lib().fpm_net_param_count.restype = ctypes.c_longlong
        self.n = int(lib().fpm_net_param_count(h))
        if params is not None:
            self.set_params(params)

    @classmethod
    def load(cls, path: str = WEIGHTS) -> "LearnedGuess":
        return cls(params=np.load(path))

    def save(self, path: str = WEIGHTS) -> None:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        np.save(path, self.params())

    def params(self) -> np.ndarray:
        out = np.empty(self.n, dtype=np.float32)
        check(lib().fpm_net_get_params(self.h, out.ctypes.data_as(VP), ctypes.c_longlong(self.n)))
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.n:
            raise ValueError(f"expected {self.n} parameters, got {p.size}")
        check(lib().fpm_net_set_params(self.h, p.ctypes.data_as(VP), ctypes.c_longlong(self.n)))

    def grads(self) -> np.ndarray:
        out = np.empty(self.n, dtype=np.float32)
        check(lib().fpm_net_get_grads(self.h, out.ctypes.data_as(VP), ctypes.c_longlong(self.n)))
        return out

    def forward(self, nx, ny, nz, fluid, mx, my, mz, b):
        torch = _t()
        out = torch.empty(nx * ny * nz, dtype=torch.float32, device=b.device)
        check(lib().fpm_net_forward_dev(self.h, nx, ny, nz, _p(fluid), _p(mx), _p(my), _p(mz), _p(b), _p(out), VP(0)))
        return out

    def backward(self, nx, ny, nz, fluid, mx, my, mz, b, target) -> float:
        loss = ctypes.c_double()
        check(lib().fpm_net_backward_dev(self.h, nx, ny, nz, _p(fluid), _p(mx), _p(my), _p(mz), _p(b), _p(target),
                                         ctypes.byref(loss), VP(0)))
        return loss.value

    def train_step(self, nx, ny, nz, fluid, mx, my, mz, b, target, lr: float) -> float:
        loss = ctypes.c_double()
        check(lib().fpm_net_train_step_dev(self.h, nx, ny, nz, _p(fluid), _p(mx), _p(my), _p(mz), _p(b),
                                           _p(target), ctypes.c_float(lr), ctypes.byref(loss), VP(0)))
        return loss.value

    def close(self) -> None:
        if self.h:
            lib().fpm_net_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- problems
def training_grid(nx: int, ny: int, nz: int):
    """Axes of the training / evaluation boxes: ratio 1.02 away from the centre
    planes, at least [-3,3]^2 x [-1.5,1.5], smallest cell at least 0.01 (so
    the FP64 rounding floor of the max-norm residual stays well below 1e-10)."""
    hx, hy, hz = TRAIN_DOMAIN
    return (workloads.geometric_axis_w0(nx, 0.01, TRAIN_RATIO, hx),
            workloads.geometric_axis_w0(ny, 0.01, TRAIN_RATIO, hy),
            workloads.geometric_axis_w0(nz, 0.01, TRAIN_RATIO, hz))


def random_bodies(rng: np.random.Generator, ax, ay, az) -> np.ndarray:
    """Union of 1-4 random ellipsoids (semi-axes 0.2-0.7, random orientation)
    and axis-aligned boxes (half sizes 0.15-0.6), centres within 1.0 of the
    origin in x, y and 0.3 in z; blocked by cell centre.  Returns (nx, ny, nz) bool."""
    X = ax[1][1:-1][:, None, None]
    Y = ay[1][1:-1][None, :, None]
    Z = az[1][1:-1][None, None, :]
    nx, ny, nz = X.shape[0], Y.shape[1], Z.shape[2]
    solid = np.zeros((nx, ny, nz), dtype=bool)
    for _ in range(int(rng.integers(1, 5))):
        cen = rng.uniform(-1.0, 1.0, 3) * np.array([1.0, 1.0, 0.3])
        if rng.random() < 0.5:
            semi = rng.uniform(0.2, 0.7, 3)
            R = workloads._rotation(rng)
            dX, dY, dZ = X - cen[0], Y - cen[1], Z - cen[2]
            q = 0.0
            for r in range(3):
                comp = R[0, r] * dX + R[1, r] * dY + R[2, r] * dZ
                q = q + (comp / semi[r]) ** 2
            solid |= q < 1.0
        else:
            h = rng.uniform(0.15, 0.6, 3)
            solid |= (np.abs(X - cen[0]) < h[0]) & (np.abs(Y - cen[1]) < h[1]) & (np.abs(Z - cen[2]) < h[2])
    if not solid.any():
        solid[nx // 2, ny // 2, nz // 2] = True
    # fluid pockets enclosed by the body have no outer face: their Neumann
    # problem is incompatible on its own, so they are blocked
    from scipy import ndimage
    lab, _ = ndimage.label(~solid)
    outer = np.unique(np.concatenate([lab[0].ravel(), lab[-1].ravel(), lab[:, 0].ravel(), lab[:, -1].ravel(),
                                      lab[:, :, 0].ravel(), lab[:, :, -1].ravel()]))
    solid |= ~np.isin(lab, outer[outer > 0])
    # the solver rejects fluid cells without a fluid neighbour (as the
    # reference does): block them
    while True:
        fl = ~solid
        nb = np.zeros(solid.shape, dtype=np.int8)
        for axis in range(3):
            for sh in (1, -1):
                r = np.roll(fl, sh, axis=axis)
                idx = [slice(None)] * 3
                idx[axis] = 0 if sh == 1 else -1
                r[tuple(idx)] = False
                nb += r
        lonely = fl & (nb == 0)
        if not lonely.any():
            return solid
        solid |= lonely


def frame_for(solid_interior: np.ndarray, ax, ay, az, axis: int):
    """A stair-step problem dict (workloads layout) for a body and an axis."""
    nx, ny, nz = solid_interior.shape
    return workloads._frame(nx, ny, nz, ax, ay, az, solid_interior.astype(np.int32), axis)


class DeviceProblem:
    """The stair-step problem on the GPU after compatibility, with its operator."""

    def __init__(self, f):
        torch = _t()
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(np.asarray(a).ravel(order="F"))).cuda()
        nx, ny, nz = f["nx"], f["ny"], f["nz"]
        self.nx, self.ny, self.nz = nx, ny, nz
        faces = [x.copy(order="F") for x in f["faces"]]
        ss.enforce_stairstep_compatibility_3d(f["rhs"], f["solid"], f["body"], *faces, f["dx"], f["dy"], f["dz"])
        self.faces = [dev(x) for x in faces]
        self.rhs = dev(f["rhs"])
        self.solid = dev(f["solid"])
        self.axes = [dev(f[k]) for k in ("xc", "yc", "zc", "dx", "dy", "dz")]
        self.body = np.ascontiguousarray(f["body"], dtype=np.float64)
        self.phi0 = f["phi"]
        n = nx * ny * nz
        self.src = torch.empty(n, dtype=torch.float64, device="cuda")
        self.diag = torch.empty(n, dtype=torch.float64, device="cuda")
        rdiag = torch.empty(n, dtype=torch.float64, device="cuda")
        iso = ctypes.c_int()
        check(lib().fpm_stairstep_build_operator_dev(_p(self.rhs), _p(self.solid), self.body.ctypes.data_as(VP),
                                                     *[_p(t) for t in self.faces], *[_p(t) for t in self.axes],
                                                     nx, ny, nz, 1, _p(self.src), _p(self.diag), _p(rdiag),
                                                     ctypes.byref(iso), VP(0)))

    def inputs(self):
        torch = _t()
        n = self.nx * self.ny * self.nz
        fluid = torch.empty(n, dtype=torch.uint8, device="cuda")
        mx, my, mz = (torch.empty(k, dtype=torch.float32, device="cuda") for k in (self.nx, self.ny, self.nz))
        b = torch.empty(n, dtype=torch.float32, device="cuda")
        check(lib().fpm_net_prepare_inputs_dev(_p(self.src), _p(self.diag), _p(self.axes[3]), _p(self.axes[4]),
                                               _p(self.axes[5]), self.nx, self.ny, self.nz, _p(fluid), _p(mx),
                                               _p(my), _p(mz), _p(b), VP(0)))
        return fluid, mx, my, mz, b

    def solve(self, method="pcg", tol=1e-10, max_sweeps=2000000, ci=50, net: LearnedGuess | None = None):
        """(phi padded device tensor, sweeps, residual, fallback)."""
        torch = _t()
        phi = torch.from_numpy(np.ascontiguousarray(self.phi0.ravel(order="F"))).cuda()
        sw = (ctypes.c_int * 1)()
        res = (ctypes.c_double * 1)()
        fb = (ctypes.c_int * 1)()
        args = ((VP * 1)(_p(phi)), (VP * 1)(_p(self.rhs)), _p(self.solid), self.body.ctypes.data_as(VP),
                (VP * 6)(*[_p(t) for t in self.faces]), *[_p(t) for t in self.axes], self.nx, self.ny, self.nz,
                ctypes.c_double(tol), max_sweeps, ci, ss.METHODS[method], sw, res)
        if net is None:
            check(lib().fpm_solve_stairstep_multi_dev(1, *args, VP(0)))
        else:
            check(lib().fpm_solve_stairstep_learned_dev(net.h, 1, *args, fb, VP(0)))
        return phi, sw[0], res[0], fb[0]

    def interior(self, phi_padded):
        nx, ny, nz = self.nx, self.ny, self.nz
        return phi_padded.view(nz, ny + 2, nx + 2)[:, 1:ny + 1, 1:nx + 1].contiguous().view(-1)


@dataclass
class Dataset:
    nx: int
    ny: int
    nz: int
    mx: object
    my: object
    mz: object
    fluid: object   # (count, n) uint8
    b: object       # (count, n) float32
    target: object  # (count, n) float32
    iterations: list


def make_dataset(count: int, nx=128, ny=128, nz=64, seed=7, tol=1e-8, log=None) -> Dataset:
    """`count` random bodies, each with the FP64 PCG potential of a random axis."""
    torch = _t()
    rng = np.random.default_rng(seed)
    ax, ay, az = training_grid(nx, ny, nz)
    n = nx * ny * nz
    fluid = torch.empty((count, n), dtype=torch.uint8, device="cuda")
    b = torch.empty((count, n), dtype=torch.float32, device="cuda")
    target = torch.empty((count, n), dtype=torch.float32, device="cuda")
    its = []
    mx = my = mz = None
    for s in range(count):
        solid = random_bodies(rng, ax, ay, az)
        axis = int(rng.integers(0, 3))
        p = DeviceProblem(frame_for(solid, ax, ay, az, axis))
        f, mx, my, mz, bb = p.inputs()
        phi, sw, res, _ = p.solve("pcg", tol=tol)
        fluid[s] = f
        b[s] = bb
        target[s] = p.interior(phi).float()
        its.append(sw)
        if log and (s + 1) % max(1, count // 10) == 0:
            log(f"dataset {s + 1}/{count}: last PCG {sw} iterations, residual {res:.2e}")
    return Dataset(nx, ny, nz, mx, my, mz, fluid, b, target, its)


def train(net: LearnedGuess, data: Dataset, epochs: int = 8, lr: float = 2e-3, lr_final: float = 1e-4, seed=0,
          log=None) -> list[float]:
    """Adam over the dataset (one sample per step, cosine learning-rate decay).
    Returns the mean loss of every epoch."""
    rng = np.random.default_rng(seed)
    count = data.fluid.shape[0]
    total = epochs * count
    history = []
    step = 0
    for e in range(epochs):
        order = rng.permutation(count)
        acc = 0.0
        for s in order:
            rate = lr_final + 0.5 * (lr - lr_final) * (1 + math.cos(math.pi * step / max(1, total - 1)))
            acc += net.train_step(data.nx, data.ny, data.nz, data.fluid[s], data.mx, data.my, data.mz, data.b[s],
                                  data.target[s], rate)
            step += 1
        history.append(acc / count)
        if log:
            log(f"epoch {e + 1}/{epochs}: mean loss {history[-1]:.4e}")
    return history
