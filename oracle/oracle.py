"""ctypes access to the checker: the CPU restatement (liboracle.so) and, where it
was built, the reference's own tree code + generated operators (oracle/_ref).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg.  The product package never imports this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(HERE, "liboracle.so")
_REF_DIR = os.path.join(HERE, "_ref")

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_lp = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_up = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")


def build():
    subprocess.check_call(["make", "-s", "-C", HERE])


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB):
            build()
        L = C.CDLL(_LIB)
        d, i, l = C.c_double, C.c_int, C.c_long
        L.or_nterms.restype = l
        L.or_nterms.argtypes = [i]
        L.or_index.restype = l
        L.or_index.argtypes = [i, i, i]
        L.or_derivs.argtypes = [d, d, d, i, _dp]
        L.or_P2M.argtypes = [d, d, d, d, _dp, i, i]
        for f in ("or_M2M", "or_M2L", "or_L2L"):
            getattr(L, f).argtypes = [d, d, d, _dp, _dp, i, i]
        L.or_L2P.argtypes = [d, d, d, _dp, _dp, i, i, i, i]
        L.or_P2P.argtypes = [d, d, d, _dp, _dp, i, i, i]
        L.or_tree_build.restype = C.c_void_p
        L.or_tree_build.argtypes = [_dp, _dp, l, l, i, d, i, C.POINTER(C.c_int)]
        L.or_tree_free.argtypes = [C.c_void_p]
        L.or_tree_info.argtypes = [C.c_void_p, _lp]
        L.or_tree_export_cells.argtypes = [C.c_void_p, _up, _lp, _dp, _lp, _lp, _lp, _lp]
        L.or_tree_export_lists.argtypes = [C.c_void_p, _up, _up]
        L.or_tree_set_m2l_orders.argtypes = [C.c_void_p, C.c_void_p]
        L.or_M2P.argtypes = [d, d, d, _dp, _dp, i, i, i, i]
        L.or_tree_evaluate_bh.argtypes = [C.c_void_p, _dp, i, i]
        L.or_tree_evaluate.restype = i
        L.or_tree_evaluate.argtypes = [C.c_void_p, _dp, i, i, l, C.c_void_p, C.c_void_p, _dp]
        L.or_direct.argtypes = [_dp, _dp, l, _lp, l, i, i, i, _dp]
        L.or_num_threads.restype = i
        _lib = L
    return _lib


def nterms(p):
    return int(lib().or_nterms(p))


def sourcesize(so):
    """Components of a source: the degree-so multipole coefficients (1, 3, 6)."""
    return nterms(so) - nterms(so - 1)


def msize(order, so):
    return nterms(order) - nterms(so - 1)


def lsize(order, so):
    return nterms(order - so)


def outsize(potential=True, field=True):
    return (1 if potential else 0) + (3 if field else 0)


# ---- scalar operators (same argument order as fmmgen's generated ABI) ----
def P2M(x, y, z, q, M, order, so=0):
    lib().or_P2M(x, y, z, q, M, order, so)


def M2M(x, y, z, M, Ms, order, so=0):
    lib().or_M2M(x, y, z, M, Ms, order, so)


def M2L(x, y, z, M, L, order, so=0):
    lib().or_M2L(x, y, z, M, L, order, so)


def L2L(x, y, z, L, Ls, order, so=0):
    lib().or_L2L(x, y, z, L, Ls, order, so)


def L2P(x, y, z, L, F, order, so=0, potential=True, field=True):
    lib().or_L2P(x, y, z, L, F, order, so, int(potential), int(field))


def P2P(x, y, z, S, F, so=0, potential=True, field=True):
    lib().or_P2P(x, y, z, S, F, so, int(potential), int(field))


def M2P(x, y, z, M, F, order, so=0, potential=True, field=True):
    lib().or_M2P(x, y, z, M, F, order, so, int(potential), int(field))


def derivs(x, y, z, p):
    D = np.zeros(nterms(p))
    lib().or_derivs(x, y, z, p, D)
    return D


class OracleTree:
    """build_tree + Tree::compute_field_fmm restated on the CPU (FP64, OpenMP)."""

    def __init__(self, pos, S, ncrit, order, theta, source_order=0):
        self.pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        ss = sourcesize(source_order)
        self.S = np.ascontiguousarray(S, dtype=np.float64).reshape(-1, ss)
        self.N = self.pos.shape[0]
        self.ncrit, self.order, self.theta, self.so = ncrit, order, theta, source_order
        err = C.c_int(0)
        self.h = lib().or_tree_build(self.pos.ravel(), self.S.ravel(), self.N, ncrit, order, theta,
                                     source_order, C.byref(err))
        if err.value != 0:
            if self.h:
                lib().or_tree_free(self.h)
                self.h = None
            raise ValueError(f"oracle tree build failed (code {err.value})")
        info = np.zeros(5, dtype=np.int64)
        lib().or_tree_info(self.h, info)
        self.ncells, self.nleaves, self.nm2l, self.np2p, self.maxlevel = (int(v) for v in info)

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_tree_free(self.h)
            self.h = None

    def cells(self):
        nc, nl = self.ncells, self.nleaves
        cid = np.zeros(nc, np.uint64)
        nleaf = np.zeros(nc, np.int64)
        cen = np.zeros(3 * nc)
        lev = np.zeros(nc, np.int64)
        leaf_cell = np.zeros(nl, np.int64)
        leaf_off = np.zeros(nl + 1, np.int64)
        leaf_idx = np.zeros(self.N, np.int64)
        lib().or_tree_export_cells(self.h, cid, nleaf, cen, lev, leaf_cell, leaf_off, leaf_idx)
        return dict(id=cid, nleaf=nleaf, centre=cen.reshape(-1, 3), level=lev, leaf_cell=leaf_cell,
                    leaf_off=leaf_off, leaf_idx=leaf_idx)

    def lists(self):
        m2l = np.zeros(2 * max(self.nm2l, 1), np.uint64)
        p2p = np.zeros(2 * max(self.np2p, 1), np.uint64)
        lib().or_tree_export_lists(self.h, m2l, p2p)
        return m2l[: 2 * self.nm2l].reshape(-1, 2), p2p[: 2 * self.np2p].reshape(-1, 2)

    def set_m2l_orders(self, orders=None):
        """Per-pair M2L orders in the order of lists() (None: the one order)."""
        if orders is None:
            lib().or_tree_set_m2l_orders(self.h, None)
            return
        o = np.ascontiguousarray(orders, dtype=np.uint8)
        if o.shape != (self.nm2l,):
            raise ValueError("one order per M2L pair")
        lib().or_tree_set_m2l_orders(self.h, o.ctypes.data)

    def evaluate_bh(self, potential=True, field=True):
        """Tree::compute_field_bh with a physical M2P field (or_M2P)."""
        F = np.zeros(self.N * outsize(potential, field))
        lib().or_tree_evaluate_bh(self.h, F, int(potential), int(field))
        return F.reshape(self.N, -1)

    def evaluate(self, potential=True, field=True, sample_stride=1, want_ML=False):
        F = np.zeros(self.N * outsize(potential, field))
        times = np.zeros(6)
        M = L = None
        if want_ML:
            M = np.zeros(self.ncells * msize(self.order, self.so))
            L = np.zeros(self.ncells * lsize(self.order, self.so))
        lib().or_tree_evaluate(self.h, F, int(potential), int(field), sample_stride,
                               M.ctypes.data if M is not None else None,
                               L.ctypes.data if L is not None else None, times)
        F = F.reshape(self.N, -1)
        if want_ML:
            return F, times, M.reshape(self.ncells, -1), L.reshape(self.ncells, -1)
        return F, times


def direct(pos, S, targets=None, source_order=0, potential=True, field=True):
    """evaluate_direct (example/calculate.cpp:252-264) on a target subset."""
    pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
    ss = sourcesize(source_order)
    S = np.ascontiguousarray(S, dtype=np.float64).reshape(-1, ss)
    N = pos.shape[0]
    if targets is None:
        targets = np.arange(N, dtype=np.int64)
    targets = np.ascontiguousarray(targets, dtype=np.int64)
    F = np.zeros(len(targets) * outsize(potential, field))
    lib().or_direct(pos.ravel(), S.ravel(), N, targets, len(targets), source_order, int(potential),
                    int(field), F)
    return F.reshape(len(targets), -1)


def num_threads():
    return int(lib().or_num_threads())


# ---------------------------------------------------------------------------
# The reference itself (only where oracle/ref/build_ref.py has built it).
# ---------------------------------------------------------------------------
_refs = {}


def ref_available(so=0):
    return os.path.exists(os.path.join(_REF_DIR, f"libref_so{so}.so"))


def ref(so=0):
    if so not in _refs:
        path = os.path.join(_REF_DIR, f"libref_so{so}.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = C.CDLL(path)
        d, i, l, sz = C.c_double, C.c_int, C.c_long, C.c_size_t
        for f in ("ref_sourceorder", "ref_minorder", "ref_maxorder"):
            getattr(L, f).restype = i
        L.ref_build.restype = C.c_void_p
        L.ref_build.argtypes = [_dp, _dp, sz, sz, sz, d, C.POINTER(C.c_double)]
        L.ref_free.argtypes = [C.c_void_p]
        L.ref_info.argtypes = [C.c_void_p, _lp]
        L.ref_export_cells.argtypes = [C.c_void_p, _up, _lp, _dp, _lp, _lp, _lp]
        L.ref_export_lists.argtypes = [C.c_void_p, _up, _up]
        L.ref_evaluate.restype = d
        L.ref_evaluate.argtypes = [C.c_void_p, _dp]
        L.ref_evaluate_bh.restype = d
        L.ref_evaluate_bh.argtypes = [C.c_void_p, _dp]
        L.ref_M2P.argtypes = [d, d, d, _dp, _dp, i]
        L.ref_cell_M.argtypes = [C.c_void_p, _dp]
        L.ref_cell_L.argtypes = [C.c_void_p, _dp]
        L.ref_P2M.argtypes = [d, d, d, d, _dp, i]
        for f in ("ref_M2M", "ref_M2L", "ref_L2L", "ref_L2P"):
            getattr(L, f).argtypes = [d, d, d, _dp, _dp, i]
        L.ref_P2P_generated.argtypes = [d, d, d, _dp, _dp]
        L.ref_P2P_restated.argtypes = [d, d, d, _dp, _dp]
        _refs[so] = L
    return _refs[so]


class RefTree:
    """The reference's build_tree / compute_field_fmm, unchanged (P2P restated)."""

    def __init__(self, pos, S, ncrit, order, theta, source_order=0):
        self.L = ref(source_order)
        self.pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        ss = sourcesize(source_order)
        self.S = np.ascontiguousarray(S, dtype=np.float64).reshape(-1, ss)
        self.N = self.pos.shape[0]
        self.ncrit, self.order, self.so = ncrit, order, source_order
        sec = C.c_double(0)
        self.h = self.L.ref_build(self.pos.ravel(), self.S.ravel(), self.N, ncrit, order, theta, C.byref(sec))
        self.build_seconds = sec.value
        info = np.zeros(4, dtype=np.int64)
        self.L.ref_info(self.h, info)
        self.ncells, self.nleaves, self.nm2l, self.np2p = (int(v) for v in info)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.ref_free(self.h)
            self.h = None

    def cells(self):
        nc, nl = self.ncells, self.nleaves
        cid = np.zeros(nc, np.uint64)
        nleaf = np.zeros(nc, np.int64)
        cen = np.zeros(3 * nc)
        lev = np.zeros(nc, np.int64)
        leaf_off = np.zeros(nl + 1, np.int64)
        leaf_idx = np.zeros(self.N, np.int64)
        self.L.ref_export_cells(self.h, cid, nleaf, cen, lev, leaf_off, leaf_idx)
        return dict(id=cid, nleaf=nleaf, centre=cen.reshape(-1, 3), level=lev, leaf_off=leaf_off,
                    leaf_idx=leaf_idx)

    def lists(self):
        m2l = np.zeros(2 * max(self.nm2l, 1), np.uint64)
        p2p = np.zeros(2 * max(self.np2p, 1), np.uint64)
        self.L.ref_export_lists(self.h, m2l, p2p)
        return m2l[: 2 * self.nm2l].reshape(-1, 2), p2p[: 2 * self.np2p].reshape(-1, 2)

    def evaluate(self):
        F = np.zeros(self.N * 4)
        sec = self.L.ref_evaluate(self.h, F)
        return F.reshape(self.N, 4), sec

    def evaluate_bh(self):
        """Tree::compute_field_bh; only the potential column is meaningful (the
        generated M2P's field is not the gradient of its potential)."""
        F = np.zeros(self.N * 4)
        sec = self.L.ref_evaluate_bh(self.h, F)
        return F.reshape(self.N, 4), sec

    def ML(self):
        from_ms = msize(self.order, self.so)
        from_ls = lsize(self.order, self.so)
        M = np.zeros(self.ncells * from_ms)
        L = np.zeros(self.ncells * from_ls)
        self.L.ref_cell_M(self.h, M)
        self.L.ref_cell_L(self.h, L)
        return M.reshape(self.ncells, -1), L.reshape(self.ncells, -1)
