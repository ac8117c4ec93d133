"""Operator surface of a module written by fmmgen.generate_code(..., cython=True).

fmmgen emits `<name>_wrap` with `cpdef` functions over `double[:]` buffers
(fmmgen/writer.py:349-432): the order dispatchers P2M, M2M, M2L, L2L, L2P, M2P
taking a trailing `order`, per-order functions with the underscore dropped
(`P2M_3` -> `P2M3`), P2P, and the FMMGEN_* constants.  `module(...)` returns
an object with the same names; every call runs on the GPU through
libfmmgen_gb300.so and adds into the caller's numpy array in place.  M2P's
field is the exact gradient of its potential (the generated one is not).
`precision="float"` is the generator's FP32 variant (fmmgen/writer.py:105):
float32 buffers (`float[:]`) and FP32 arithmetic on the device.

Batched device versions (torch tensors, many applications per launch) are the
`*_batch` functions at module level; float32 tensors select the FP32 kernels.
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


_PRECISIONS = {"double": (np.float64, "double[:]", ""), "float": (np.float32, "float[:]", "f")}


def _buf(a, dtype=np.float64, what="double[:]"):
    if not isinstance(a, np.ndarray) or a.dtype != dtype or not a.flags.c_contiguous:
        raise TypeError(f"operator buffers must be C-contiguous {np.dtype(dtype).name} numpy arrays ({what})")
    return a.ctypes.data


class OperatorModule:
    """What `import <name>_wrap` exposes after generate_code(order, name, ...)."""

    def __init__(self, order, source_order=0, potential=True, field=True, precision="double"):
        if precision not in _PRECISIONS:
            raise ValueError("Precision must be float or double")
        self._dtype, self._what, sfx = _PRECISIONS[precision]
        self.precision = precision
        self._fn = {op: getattr(lib(), op + sfx) for op in _OPS + ("P2P",)}
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

    def _b(self, a):
        return _buf(a, self._dtype, self._what)

    def P2M(self, x, y, z, q, M, order):
        self._configure()
        self._fn["P2M"](x, y, z, q, self._b(M), order)

    def M2M(self, x, y, z, M, Ms, order):
        self._configure()
        self._fn["M2M"](x, y, z, self._b(M), self._b(Ms), order)

    def M2L(self, x, y, z, M, L, order):
        self._configure()
        self._fn["M2L"](x, y, z, self._b(M), self._b(L), order)

    def L2L(self, x, y, z, L, Ls, order):
        self._configure()
        self._fn["L2L"](x, y, z, self._b(L), self._b(Ls), order)

    def L2P(self, x, y, z, L, F, order):
        self._configure()
        self._fn["L2P"](x, y, z, self._b(L), self._b(F), order)

    def M2P(self, x, y, z, M, F, order):
        self._configure()
        self._fn["M2P"](x, y, z, self._b(M), self._b(F), order)

    def P2P(self, x, y, z, S, F):
        self._configure()
        self._fn["P2P"](x, y, z, self._b(S), self._b(F))

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


def module(order, source_order=0, potential=True, field=True, precision="double"):
    return OperatorModule(order, source_order, potential, field, precision)


# ---- batched device operators ----------------------------------------------
def _dev(t, n, width, dtype=torch.float64):
    if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == dtype and t.is_contiguous()):
        raise TypeError(f"batched operators take contiguous CUDA tensors of one dtype (here {dtype})")
    if t.numel() != n * width:
        raise ValueError(f"expected {n}x{width} elements, got {t.numel()}")
    return C.c_void_p(t.data_ptr())


def _entry(name, d):
    """The FP64 entry point, or its FP32 twin when the displacements are float32."""
    if isinstance(d, torch.Tensor) and d.dtype == torch.float32:
        return getattr(lib(), name + "_f32"), torch.float32
    return getattr(lib(), name), torch.float64


def _st(stream):
    return C.c_void_p((stream or torch.cuda.current_stream()).cuda_stream)


def P2M_batch(d, q, M, order, source_order=0, stream=None):
    n = d.shape[0]
    fn, dt = _entry("fmmgen_gpu_P2M", d)
    check(fn(n, _dev(d, n, 3, dt), _dev(q, n, 1, dt), _dev(M, n, msize(order, source_order), dt), order,
             source_order, _st(stream)))


def M2M_batch(d, M, Ms, order, source_order=0, stream=None):
    n = d.shape[0]
    fn, dt = _entry("fmmgen_gpu_M2M", d)
    ms = msize(order, source_order)
    check(fn(n, _dev(d, n, 3, dt), _dev(M, n, ms, dt), _dev(Ms, n, ms, dt), order, source_order, _st(stream)))


def M2L_batch(d, M, L, order, source_order=0, stream=None):
    n = d.shape[0]
    fn, dt = _entry("fmmgen_gpu_M2L", d)
    check(fn(n, _dev(d, n, 3, dt), _dev(M, n, msize(order, source_order), dt),
             _dev(L, n, lsize(order, source_order), dt), order, source_order, _st(stream)))


def L2L_batch(d, L, Ls, order, source_order=0, stream=None):
    n = d.shape[0]
    fn, dt = _entry("fmmgen_gpu_L2L", d)
    ls = lsize(order, source_order)
    check(fn(n, _dev(d, n, 3, dt), _dev(L, n, ls, dt), _dev(Ls, n, ls, dt), order, source_order, _st(stream)))


def L2P_batch(d, L, F, order, source_order=0, potential=True, field=True, stream=None):
    n = d.shape[0]
    fn, dt = _entry("fmmgen_gpu_L2P", d)
    os_ = int(lib().fmmgen_outputsize(int(potential), int(field)))
    check(fn(n, _dev(d, n, 3, dt), _dev(L, n, lsize(order, source_order), dt), _dev(F, n, os_, dt), order,
             source_order, int(potential), int(field), _st(stream)))


def M2P_batch(d, M, F, order, source_order=0, potential=True, field=True, stream=None):
    n = d.shape[0]
    fn, dt = _entry("fmmgen_gpu_M2P", d)
    os_ = int(lib().fmmgen_outputsize(int(potential), int(field)))
    check(fn(n, _dev(d, n, 3, dt), _dev(M, n, msize(order, source_order), dt), _dev(F, n, os_, dt), order,
             source_order, int(potential), int(field), _st(stream)))


def P2P_batch(d, S, F, source_order=0, potential=True, field=True, stream=None):
    n = d.shape[0]
    fn, dt = _entry("fmmgen_gpu_P2P", d)
    ss = int(lib().fmmgen_sourcesize(source_order))
    os_ = int(lib().fmmgen_outputsize(int(potential), int(field)))
    check(fn(n, _dev(d, n, 3, dt), _dev(S, n, ss, dt), _dev(F, n, os_, dt), source_order, int(potential),
             int(field), _st(stream)))
