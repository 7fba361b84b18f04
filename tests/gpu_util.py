"""Device-memory plumbing for the GPU tests (torch tensors as raw buffers).

The kernels under test are called through the C ABI with these tensors'
device pointers; torch only allocates and copies."""
import ctypes

import numpy as np


def torch():
    import torch as t
    return t


def to_dev(a):
    """Fortran-ordered numpy array -> flat CUDA tensor with the same bytes."""
    t = torch()
    flat = np.ascontiguousarray(np.asarray(a).ravel(order="F"))
    return t.from_numpy(flat.copy()).to("cuda")


def from_dev(t, shape):
    return np.asfortranarray(t.cpu().numpy().reshape(shape, order="F"))


def ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def stream_ptr():
    return ctypes.c_void_p(torch().cuda.current_stream().cuda_stream)
