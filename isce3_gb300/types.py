"""GSLC sample types and codecs on the GPU (python/packages/isce3/core/types.py).

``complex32`` is isce3's pairs of float16.  ``to_complex32``,
``truncate_mantissa`` and ``read_c4_dataset_as_c8`` keep the reference's
names, arguments, results and error behaviour (types.py:38-165) and run as
byte-bound kernels of libgslc.so (gslc_complex64_to_complex32,
gslc_complex32_to_complex64, gslc_truncate_mantissa).  NumPy arrays are
copied to the GPU and back; CUDA tensors are processed where they are.  The
geocoder applies the same codecs inside its loads and stores (complex32
radar or geo blocks, ``output_nonzero_mantissa_bits``), so a GSLC workflow
need not call these around it.
"""
from __future__ import annotations

import ctypes as C
import logging

import numpy as np
import torch

from . import _lib as L
from .geocode import COMPLEX32

log = logging.getLogger("isce3_gb300.types")

complex32 = COMPLEX32


def _stream(dev):
    return torch.cuda.current_stream(dev)


def _dev(device=None) -> torch.device:
    if device is not None:
        return torch.device(device)
    if not torch.cuda.is_available():
        raise RuntimeError("isce3_gb300.types needs a CUDA GPU")
    return torch.device("cuda", torch.cuda.current_device())


def _run(fn, dev, *args):
    ctx = L.context(dev.index)
    with torch.cuda.device(dev):
        s = _stream(dev)
        L.check(fn(ctx, *args, C.c_void_p(s.cuda_stream)), ctx, fn.__name__)


def to_complex32(z):
    """complex64 -> complex32 (types.py:38-42): each part rounded to float16
    to nearest even, overflow to infinity, as numpy's astype.  Returns a
    NumPy complex32 array for a NumPy input, a torch.complex32 tensor for a
    CUDA tensor."""
    lib = L.lib()
    if isinstance(z, torch.Tensor) and z.device.type == "cuda":
        src = z.to(torch.complex64).contiguous()
        out = torch.empty(tuple(src.shape), dtype=torch.complex32, device=src.device)
        _run(lib.gslc_complex64_to_complex32, src.device, C.c_void_p(src.data_ptr()), C.c_void_p(out.data_ptr()),
             src.numel())
        return out
    zz = np.ascontiguousarray(np.asarray(z), dtype=np.complex64)
    dev = _dev()
    src = torch.from_numpy(zz).to(dev)
    out = torch.empty(zz.shape, dtype=torch.int32, device=dev)
    _run(lib.gslc_complex64_to_complex32, dev, C.c_void_p(src.data_ptr()), C.c_void_p(out.data_ptr()), zz.size)
    return out.cpu().numpy().view(complex32)


def read_c4_dataset_as_c8(ds, key=np.s_[...]):
    """A complex32 dataset (an h5py dataset, or a NumPy array of complex32)
    sliced by ``key``, as complex64 (types.py:45-72; float16 -> float32 is
    exact).  Returns a NumPy complex64 array."""
    if hasattr(ds, "astype") and not isinstance(ds, np.ndarray):
        z = ds.astype(complex32)[key]          # h5py's dtype-cast read
    else:
        z = np.asarray(ds)[key]
    z = np.ascontiguousarray(z)
    if z.dtype != complex32:
        z = z.astype(complex32)
    dev = _dev()
    src = torch.from_numpy(z.view(np.int32)).to(dev)
    out = torch.empty(z.shape, dtype=torch.complex64, device=dev)
    _run(L.lib().gslc_complex32_to_complex64, dev, C.c_void_p(src.data_ptr()), C.c_void_p(out.data_ptr()), z.size)
    return out.cpu().numpy()


def truncate_mantissa(z, significant_bits=10):
    """Zero out all but the leading ``significant_bits`` mantissa bits of
    every element of ``z`` in place (types.py:116-165).  ``z`` is a real or
    complex float16/32/64 NumPy array or CUDA tensor."""
    is_np = isinstance(z, np.ndarray)
    is_cuda = isinstance(z, torch.Tensor) and z.device.type == "cuda"
    if not (is_np or is_cuda):
        err = "argument z is not of type np.ndarray"
        log.info(err)
        raise ValueError(err)
    if is_np:
        if np.iscomplexobj(z):
            word = np.dtype(z.dtype).itemsize // 2
        elif issubclass(z.dtype.type, np.floating):
            word = z.dtype.itemsize
        else:
            err = "argument z is not complex float or float type"
            log.info(err)
            raise ValueError(err)
    else:
        if not (z.dtype.is_floating_point or z.dtype.is_complex):
            raise ValueError("argument z is not complex float or float type")
        word = z.element_size() // (2 if z.dtype.is_complex else 1)
    mant = {2: 10, 4: 23, 8: 52}.get(word)
    if mant is None:
        raise ValueError("argument z is not complex float or float type")
    if significant_bits == mant:
        return
    if not 0 < significant_bits <= mant:
        err = f"Require 0 < {significant_bits=} <= {mant}"
        log.info(err)
        raise ValueError(err)
    lib = L.lib()
    if is_cuda:
        if not z.is_contiguous():
            raise ValueError("arrays must be C-contiguous")
        n = z.numel() * (2 if z.dtype.is_complex else 1)
        _run(lib.gslc_truncate_mantissa, z.device, C.c_void_p(z.data_ptr()), n, word, int(significant_bits))
        return
    if not z.flags.c_contiguous:
        raise ValueError("arrays must be C-contiguous")
    words = z.view({2: np.uint16, 4: np.uint32, 8: np.uint64}[word]).reshape(-1)
    signed = words.view({2: np.int16, 4: np.int32, 8: np.int64}[word])
    dev = _dev()
    buf = torch.from_numpy(signed).to(dev)
    _run(lib.gslc_truncate_mantissa, dev, C.c_void_p(buf.data_ptr()), words.size, word, int(significant_bits))
    signed[...] = buf.cpu().numpy()
