"""Operator surface of a module written by fmmgen.generate_code(..., cython=True).

fmmgen emits `<name>_wrap` with `cpdef` functions over `double[:]` buffers
(fmmgen/writer.py:349-432): the order dispatchers P2M, M2M, M2L, L2L, L2P, M2P
taking a trailing `order`, per-order functions with the underscore dropped
(`P2M_3` -> `P2M3`), P2P, and the FMMGEN_* constants.  `module(...)` returns
an object with the same names; every call runs on the GPU through
libfmmgen_gb300.so and adds into the caller's numpy array in place.  M2P's
field is the exact gradient of its potential (the generated one is not).

Batched device versions (torch tensors, many applications per launch) are the
`*_batch` functions at module level.
"""
import ctypes as C

import numpy as np
import torch

from ._lib import check, lib

_OPS = ("P2M", "M2M", "M2L", "L2L", "L2P", "M2P")


def nterms(p):
    return int(lib().fmmgen_nterms(p))


def msize(order, source_order=0):
    return int(lib().fmmgen_msize(order, source_order))


def lsize(order, source_order=0):
    return int(lib().fmmgen_lsize(order, source_order))


def _buf(a):
    if not isinstance(a, np.ndarray) or a.dtype != np.float64 or not a.flags.c_contiguous:
        raise TypeError("operator buffers must be C-contiguous float64 numpy arrays (double[:])")
    return a.ctypes.data


class OperatorModule:
    """What `import <name>_wrap` exposes after generate_code(order, name, ...)."""

    def __init__(self, order, source_order=0, potential=True, field=True):
        self.FMMGEN_MINORDER = int(lib().fmmgen_minorder(source_order, int(field)))
        self.FMMGEN_MAXORDER = int(order)  # exclusive, as generate_code's `order`
        self.FMMGEN_SOURCEORDER = int(source_order)
        self.FMMGEN_SOURCESIZE = int(lib().fmmgen_sourcesize(source_order))
        self.FMMGEN_OUTPUTSIZE = int(lib().fmmgen_outputsize(int(potential), int(field)))
        if order - 1 > lib().fmmgen_max_order():
            raise ValueError(f"orders above {lib().fmmgen_max_order()} are not supported")
        self._cfg = (source_order, int(potential), int(field), int(order) - 1)

    def _configure(self):
        check(lib().fmmgen_configure(*self._cfg))

    def P2M(self, x, y, z, q, M, order):
        self._configure()
        lib().P2M(x, y, z, q, _buf(M), order)

    def M2M(self, x, y, z, M, Ms, order):
        self._configure()
        lib().M2M(x, y, z, _buf(M), _buf(Ms), order)

    def M2L(self, x, y, z, M, L, order):
        self._configure()
        lib().M2L(x, y, z, _buf(M), _buf(L), order)

    def L2L(self, x, y, z, L, Ls, order):
        self._configure()
        lib().L2L(x, y, z, _buf(L), _buf(Ls), order)

    def L2P(self, x, y, z, L, F, order):
        self._configure()
        lib().L2P(x, y, z, _buf(L), _buf(F), order)

    def M2P(self, x, y, z, M, F, order):
        self._configure()
        lib().M2P(x, y, z, _buf(M), _buf(F), order)

    def P2P(self, x, y, z, S, F):
        self._configure()
        lib().P2P(x, y, z, _buf(S), _buf(F))

    def __getattr__(self, name):
        # per-order functions: P2M3(x, y, z, q, M) == P2M(x, y, z, q, M, 3)
        for op in _OPS:
            if name.startswith(op) and name[len(op):].isdigit():
                p = int(name[len(op):])
                if not (self.FMMGEN_MINORDER <= p < self.FMMGEN_MAXORDER):
                    break
                f = getattr(self, op)
                return lambda *a, _f=f, _p=p: _f(*a, _p)
        raise AttributeError(name)


def module(order, source_order=0, potential=True, field=True):
    return OperatorModule(order, source_order, potential, field)


# ---- batched device operators ----------------------------------------------
def _dev(t, n, width):
    if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
        raise TypeError("batched operators take contiguous float64 CUDA tensors")
    if t.numel() != n * width:
        raise ValueError(f"expected {n}x{width} elements, got {t.numel()}")
    return C.c_void_p(t.data_ptr())


def _st(stream):
    return C.c_void_p((stream or torch.cuda.current_stream()).cuda_stream)


def P2M_batch(d, q, M, order, source_order=0, stream=None):
    n = d.shape[0]
    check(lib().fmmgen_gpu_P2M(n, _dev(d, n, 3), _dev(q, n, 1), _dev(M, n, msize(order, source_order)), order,
                               source_order, _st(stream)))


def M2M_batch(d, M, Ms, order, source_order=0, stream=None):
    n = d.shape[0]
    ms = msize(order, source_order)
    check(lib().fmmgen_gpu_M2M(n, _dev(d, n, 3), _dev(M, n, ms), _dev(Ms, n, ms), order, source_order, _st(stream)))


def M2L_batch(d, M, L, order, source_order=0, stream=None):
    n = d.shape[0]
    check(lib().fmmgen_gpu_M2L(n, _dev(d, n, 3), _dev(M, n, msize(order, source_order)),
                               _dev(L, n, lsize(order, source_order)), order, source_order, _st(stream)))


def L2L_batch(d, L, Ls, order, source_order=0, stream=None):
    n = d.shape[0]
    ls = lsize(order, source_order)
    check(lib().fmmgen_gpu_L2L(n, _dev(d, n, 3), _dev(L, n, ls), _dev(Ls, n, ls), order, source_order, _st(stream)))


def L2P_batch(d, L, F, order, source_order=0, potential=True, field=True, stream=None):
    n = d.shape[0]
    os_ = int(lib().fmmgen_outputsize(int(potential), int(field)))
    check(lib().fmmgen_gpu_L2P(n, _dev(d, n, 3), _dev(L, n, lsize(order, source_order)), _dev(F, n, os_), order,
                               source_order, int(potential), int(field), _st(stream)))


def M2P_batch(d, M, F, order, source_order=0, potential=True, field=True, stream=None):
    n = d.shape[0]
    os_ = int(lib().fmmgen_outputsize(int(potential), int(field)))
    check(lib().fmmgen_gpu_M2P(n, _dev(d, n, 3), _dev(M, n, msize(order, source_order)), _dev(F, n, os_), order,
                               source_order, int(potential), int(field), _st(stream)))


def P2P_batch(d, S, F, source_order=0, potential=True, field=True, stream=None):
    n = d.shape[0]
    ss = int(lib().fmmgen_sourcesize(source_order))
    os_ = int(lib().fmmgen_outputsize(int(potential), int(field)))
    check(lib().fmmgen_gpu_P2P(n, _dev(d, n, 3), _dev(S, n, ss), _dev(F, n, os_), source_order, int(potential),
                               int(field), _st(stream)))
