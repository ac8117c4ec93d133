"""Host-side mirror of the reference example's tree API (example/tree.hpp:78-103).

    tree = build_tree(pos, S, N, ncrit, order, theta, source_order=0)
    tree.compute_field_fmm(F)      # Tree::compute_field_fmm (example/tree.cpp:243-271)
    tree.compute_field_exact(F)    # Tree::compute_field_exact (example/tree.cpp:295-297)

pos is [N][3], S is [N][SOURCESIZE] and F is [N][OUTPUTSIZE], FP64, in the
caller's particle order, as in the reference.  Device tensors (torch, cuda,
float64) are used in place; host arrays (numpy or CPU tensors) are copied to the
device and F is copied back.  All work runs in libfmmgen_gb300.so on the GPU:
torch supplies device memory and the stream.
"""
import ctypes as C

import numpy as np
import torch

from . import _lib
from ._lib import check, lib

PRECISIONS = {"fp64": _lib.PREC_FP64, "mixed": _lib.PREC_MIXED, "mixed_simt": _lib.PREC_MIXED_SIMT}


def _stream_ptr(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def _as_device(a, shape_tail):
    if isinstance(a, torch.Tensor) and a.is_cuda:
        t = a
    else:
        t = torch.as_tensor(np.asarray(a) if not isinstance(a, torch.Tensor) else a)
        t = t.to(device="cuda")
    t = t.to(torch.float64).reshape(-1, *shape_tail).contiguous()
    return t


def sourcesize(source_order):
    """Components of a source: 1 charge, 3 dipole, 6 quadrupole (xx xy xz yy yz zz)."""
    return {0: 1, 1: 3, 2: 6}[source_order]


def outputsize(potential=True, field=True):
    return (1 if potential else 0) + (3 if field else 0)


class Tree:
    """Device octree + interaction lists for fixed particle positions."""

    def __init__(self, pos, S, ncrit, order, theta, source_order=0, stream=None, sys_off=None):
        if source_order not in (0, 1, 2):
            raise ValueError("source_order must be 0 (charges), 1 (dipoles) or 2 (quadrupoles)")
        # a forest of independent systems when sys_off (nsys + 1 particle offsets) is given
        self.sys_off = None if sys_off is None else np.ascontiguousarray(sys_off, dtype=np.int64)
        self.pos = _as_device(pos, (3,))
        self.N = self.pos.shape[0]
        self.S = _as_device(S, (sourcesize(source_order),)) if S is not None else None
        if self.S is not None and self.S.shape[0] != self.N:
            raise ValueError("S must hold one source per particle")
        self.ncrit, self.order, self.theta, self.source_order = int(ncrit), int(order), float(theta), source_order
        self._h = C.c_void_p(None)
        self.rebuild(stream=stream)

    def rebuild(self, pos=None, stream=None):
        """Rebuild for new positions, reusing the handle's device buffers."""
        if pos is not None:
            self.pos = _as_device(pos, (3,))
            self.N = self.pos.shape[0]
        if self.sys_off is None:
            check(lib().fmmgen_tree_build(C.c_void_p(self.pos.data_ptr()), self.N, self.ncrit, self.order,
                                          self.theta, self.source_order, _stream_ptr(stream), C.byref(self._h)))
        else:
            if self.sys_off[-1] != self.N:
                raise ValueError("the system offsets must end at N")
            check(lib().fmmgen_forest_build(C.c_void_p(self.pos.data_ptr()), self.sys_off.ctypes.data,
                                            len(self.sys_off) - 1, self.ncrit, self.order, self.theta,
                                            self.source_order, _stream_ptr(stream), C.byref(self._h)))
        self._counts()
        return self

    def _counts(self):
        info = np.zeros(8, dtype=np.int64)
        check(lib().fmmgen_tree_counts(self._h, info.ctypes.data))  # does not wait for the device
        (self.ncells, self.nleaves, self.nm2l, self.np2p, self.nlevels, self.nclasses, _, _) = (int(v) for v in info)

    @property
    def p2p_interactions(self):
        """Particle-particle interactions of the P2P list (self pairs excluded);
        waits for the build's work on the device."""
        info = np.zeros(9, dtype=np.int64)
        check(lib().fmmgen_tree_info(self._h, info.ctypes.data))
        return int(info[8])

    def rebuild_compute(self, pos=None, F=None, S=None, potential=True, field=True, precision="mixed",
                        stream=None):
        """rebuild(pos) followed by compute_field_fmm(F, S, ...) in one call: the
        near field and the multipoles run while the build groups the M2L
        lists by class.  Returns F like compute_field_fmm."""
        if pos is not None:
            self.pos = _as_device(pos, (3,))
            self.N = self.pos.shape[0]
        if S is not None:
            self.S = _as_device(S, (sourcesize(self.source_order),))
        if self.S is None or self.S.shape[0] != self.N:
            raise ValueError("S must hold one source per particle")
        os_ = outputsize(potential, field)
        host_out = F is not None and not (isinstance(F, torch.Tensor) and F.is_cuda)
        Fd = F if (F is not None and not host_out) else torch.empty((self.N, os_), dtype=torch.float64,
                                                                     device=self.pos.device)
        if Fd.dtype != torch.float64 or not Fd.is_contiguous() or Fd.numel() != self.N * os_:
            raise ValueError("F must be a contiguous float64 [N][OUTPUTSIZE] array")
        off = self.sys_off
        if off is not None and off[-1] != self.N:
            raise ValueError("the system offsets must end at N")
        check(lib().fmmgen_tree_build_compute(
            C.c_void_p(self.pos.data_ptr()), off.ctypes.data if off is not None else None,
            len(off) - 1 if off is not None else 1, self.N, self.ncrit, self.order, self.theta, self.source_order,
            C.c_void_p(self.S.data_ptr()), C.c_void_p(Fd.data_ptr()), int(potential), int(field),
            PRECISIONS[precision], _stream_ptr(stream), C.byref(self._h)))
        self._counts()
        if host_out:
            F[...] = Fd.reshape(np.shape(F)).cpu().numpy() if isinstance(F, np.ndarray) else Fd.cpu()
            return F
        return Fd

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().fmmgen_tree_free(h)
            except Exception:
                pass
            self._h = C.c_void_p(None)

    # -- evaluation ---------------------------------------------------------
    def compute_field_fmm(self, F=None, S=None, potential=True, field=True, precision="fp64", stream=None):
        """Fill F with phi/E of the FMM; returns F (device tensor unless F is a host array)."""
        if S is not None:
            self.S = _as_device(S, (sourcesize(self.source_order),))
        if self.S is None:
            raise ValueError("no sources")
        os_ = outputsize(potential, field)
        host_out = F is not None and not (isinstance(F, torch.Tensor) and F.is_cuda)
        Fd = F if (F is not None and not host_out) else torch.empty((self.N, os_), dtype=torch.float64,
                                                                     device=self.pos.device)
        if Fd.dtype != torch.float64 or not Fd.is_contiguous() or Fd.numel() != self.N * os_:
            raise ValueError("F must be a contiguous float64 [N][OUTPUTSIZE] array")
        check(lib().fmmgen_tree_compute_field_fmm(self._h, C.c_void_p(self.S.data_ptr()), C.c_void_p(Fd.data_ptr()),
                                                  int(potential), int(field), PRECISIONS[precision],
                                                  _stream_ptr(stream)))
        if host_out:
            F[...] = Fd.reshape(np.shape(F)).cpu().numpy() if isinstance(F, np.ndarray) else Fd.cpu()
            return F
        return Fd

    def compute_field_bh(self, F=None, S=None, potential=True, field=True, stream=None):
        """Tree::compute_field_bh (example/tree.cpp:273-293): Barnes-Hut with the
        tree's order and theta, in FP64; returns F like compute_field_fmm."""
        if S is not None:
            self.S = _as_device(S, (sourcesize(self.source_order),))
        if self.S is None:
            raise ValueError("no sources")
        os_ = outputsize(potential, field)
        host_out = F is not None and not (isinstance(F, torch.Tensor) and F.is_cuda)
        Fd = F if (F is not None and not host_out) else torch.empty((self.N, os_), dtype=torch.float64,
                                                                     device=self.pos.device)
        if Fd.dtype != torch.float64 or not Fd.is_contiguous() or Fd.numel() != self.N * os_:
            raise ValueError("F must be a contiguous float64 [N][OUTPUTSIZE] array")
        check(lib().fmmgen_tree_compute_field_bh(self._h, C.c_void_p(self.S.data_ptr()), C.c_void_p(Fd.data_ptr()),
                                                 int(potential), int(field), _stream_ptr(stream)))
        if host_out:
            F[...] = Fd.reshape(np.shape(F)).cpu().numpy() if isinstance(F, np.ndarray) else Fd.cpu()
            return F
        return Fd

    def compute_field_exact(self, F=None, targets=None, potential=True, field=True, stream=None):
        return direct(self.pos, self.S, targets=targets, source_order=self.source_order, potential=potential,
                      field=field, F=F, stream=stream)

    # -- introspection (host arrays) ------------------------------------------
    def root(self):
        r = np.zeros(4)
        check(lib().fmmgen_tree_root(self._h, r.ctypes.data))
        return r

    def systems(self):
        """(root cubes [nsys][4], system of every cell in level-major order)."""
        n = int(lib().fmmgen_tree_nsys(self._h))
        roots = np.zeros((n, 4))
        csys = np.zeros(self.ncells, dtype=np.int32)
        check(lib().fmmgen_tree_export_systems(self._h, roots.ctypes.data, csys.ctypes.data))
        return roots, csys

    def cells(self):
        nc, nl = self.ncells, self.nleaves
        cid = np.zeros(nc, np.uint64)
        cnt = np.zeros(nc, np.int64)
        cen = np.zeros((nc, 3))
        loff = np.zeros(nl + 1, np.int64)
        lidx = np.zeros(self.N, np.int64)
        check(lib().fmmgen_tree_export_cells(self._h, cid.ctypes.data, cnt.ctypes.data, cen.ctypes.data,
                                             loff.ctypes.data, lidx.ctypes.data))
        return dict(id=cid, count=cnt, centre=cen, leaf_off=loff, leaf_idx=lidx)

    def lists(self):
        m2l = np.zeros((max(self.nm2l, 1), 2), np.uint64)
        p2p = np.zeros((max(self.np2p, 1), 2), np.uint64)
        check(lib().fmmgen_tree_export_lists(self._h, m2l.ctypes.data, p2p.ctypes.data))
        return m2l[: self.nm2l], p2p[: self.np2p]

    def expansions(self):
        ms = int(lib().fmmgen_msize(self.order, self.source_order))
        ls = int(lib().fmmgen_lsize(self.order, self.source_order))
        M = np.zeros((self.ncells, ms))
        L = np.zeros((self.ncells, ls))
        check(lib().fmmgen_tree_export_expansions(self._h, M.ctypes.data, L.ctypes.data))
        return M, L

    def set_graph(self, enable=True):
        """Replay the evaluation pass as one CUDA graph launch while the build and
        the arguments of compute_field_fmm stay the same."""
        check(lib().fmmgen_tree_set_graph(self._h, int(bool(enable))))
        return self

    # -- M2L choices and the autotuner (no counterpart in the reference) -------
    M2L_IMPLS = {-1: "default", 0: "tensor cores", 1: "generated CUDA-core kernels", 2: "contraction engine"}

    def set_tune(self, impl=-1, nslots=0, grouping=0, overlap=0):
        """M2L implementation (-1 default rules, 0 tensor cores with source rows
        gathered row by row, 1 generated CUDA-core kernels, 2 contraction
        engine, 3 tensor cores with source rows boxed from level grids where
        every level is complete, else as 0, 4 class-major and 5 target-major
        CUDA-core kernels; per-pair orders run on 5 unless 2 or 4 is chosen),
        tensor-core pipeline depth
        (0: as deep as fits), cell grouping (0 by octant, 1 Morton) and
        overlap (1 / 2: tensor-core M2L and P2P side by side on the SMs, the
        P2P in blocks of 4 / 2 warps)."""
        check(lib().fmmgen_tree_set_tune(self._h, int(impl), int(nslots), int(grouping), int(overlap)))
        return self

    def get_tune(self):
        v = np.zeros(4, np.int32)
        check(lib().fmmgen_tree_get_tune(self._h, v.ctypes.data))
        return dict(impl=int(v[0]), nslots=int(v[1]), grouping=int(v[2]), overlap=int(v[3]))

    def autotune(self, S=None, precision="mixed", reps=3, stream=None):
        """Time the M2L + P2P phases for every supported (implementation,
        pipeline depth, overlap, grouping) and keep the fastest on this handle;
        returns the chosen setting and the table of median times (ms)."""
        if S is not None:
            self.S = _as_device(S, (sourcesize(self.source_order),))
        if self.S is None:
            raise ValueError("no sources")
        cand = np.zeros((64, 4), np.int32)
        ms = np.zeros(64, np.float32)
        n = C.c_int(0)
        check(lib().fmmgen_tree_autotune(self._h, C.c_void_p(self.S.data_ptr()), PRECISIONS[precision], int(reps), 64,
                                         cand.ctypes.data, ms.ctypes.data, C.byref(n), _stream_ptr(stream)))
        table = [dict(impl=int(c[0]), nslots=int(c[1]), grouping=int(c[2]), overlap=int(c[3]), ms=float(m))
                 for c, m in zip(cand[: n.value], ms[: n.value])]
        return dict(best=self.get_tune(), table=table)

    # -- per-pair M2L orders (no counterpart in the reference) ----------------
    def set_m2l_orders(self, orders=None, stream=None):
        """Apply M2L pair k (export_lists order) at order orders[k] (clamped to
        [source_order + 1, order]) in the evaluations of this build; None
        returns to the one order."""
        if orders is None:
            check(lib().fmmgen_tree_set_m2l_orders(self._h, None, _stream_ptr(stream)))
            return self
        o = orders if isinstance(orders, torch.Tensor) else torch.as_tensor(np.asarray(orders))
        o = o.to(device="cuda", dtype=torch.uint8).contiguous()
        if o.numel() != self.nm2l:
            raise ValueError("one order per M2L pair")
        check(lib().fmmgen_tree_set_m2l_orders(self._h, C.c_void_p(o.data_ptr()), _stream_ptr(stream)))
        (stream or torch.cuda.current_stream()).synchronize()  # the copy has read o
        return self

    def set_order_model(self, params=None, delta=0.0, eps=1e-6):
        """Attach an order model (FP32 parameters on the device, see learned.py)
        for the relative field error target eps: every evaluation predicts each
        pair's order from its own multipoles and near field.  None detaches it."""
        if params is None:
            check(lib().fmmgen_tree_set_order_model(self._h, None, 0.0, 1.0))
            self._order_params = None
            return self
        if not (isinstance(params, torch.Tensor) and params.is_cuda and params.dtype == torch.float32
                and params.is_contiguous() and params.numel() == lib().fmmgen_order_model_nparam()):
            raise ValueError("params must be a contiguous float32 CUDA tensor of the model's size")
        check(lib().fmmgen_tree_set_order_model(self._h, C.c_void_p(params.data_ptr()), float(delta), float(eps)))
        self._order_params = params  # kept alive while attached
        return self

    def m2l_orders(self):
        """Host copy of the per-pair orders the last evaluation used."""
        o = np.zeros(max(self.nm2l, 1), np.uint8)
        check(lib().fmmgen_tree_export_m2l_orders(self._h, o.ctypes.data))
        return o[: self.nm2l]

    def m2l_work(self):
        """Last tensor-core M2L: (class steps, MMA instructions, executed tensor
        flops, 1.0 if its source rows were boxed from level grids else 0.0)."""
        w = np.zeros(4)
        check(lib().fmmgen_tree_m2l_work(self._h, w.ctypes.data))
        return tuple(float(x) for x in w)

    def kernel_ms(self):
        """Device times (ms) of the last evaluate's M2L kernels and P2P kernel
        alone (events on their streams around the launches, preparation
        excluded): {"M2L": ms, "P2P": ms}, -1 where none ran."""
        v = np.zeros(2, np.float32)
        check(lib().fmmgen_tree_kernel_ms(self._h, v.ctypes.data))
        return {"M2L": float(v[0]), "P2P": float(v[1])}

    def times(self):
        b = np.zeros(6, np.float32)
        e = np.zeros(8, np.float32)
        check(lib().fmmgen_tree_times(self._h, b.ctypes.data, e.ctypes.data))
        return (dict(zip(["root", "keys_sort", "cells", "lists", "classes", "total"], b.tolist())),
                dict(zip(["P2M", "M2M", "M2L", "P2P", "L2L", "L2P", "finalize", "total"], e.tolist())))


def build_forest(pos, S, sizes, ncrit=64, order=4, theta=0.5, source_order=0, stream=None):
    """Independent systems in one handle: system s is the next sizes[s] particles
    of pos/S; each gets exactly the tree build_tree would give it alone, and the
    build and evaluation phases run once over all systems."""
    sizes = np.asarray(sizes, dtype=np.int64)
    if sizes.ndim != 1 or len(sizes) < 1 or (sizes < 1).any():
        raise ValueError("sizes must be a non-empty list of positive particle counts")
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    return Tree(pos, S, ncrit, order, theta, source_order=source_order, stream=stream, sys_off=off)


def build_tree(pos, S, N=None, ncrit=64, order=4, theta=0.5, source_order=0, stream=None):
    """build_tree(pos, S, N, ncrit, order, theta) of example/tree.cpp:130-233."""
    pos_t = _as_device(pos, (3,))
    if N is not None and int(N) != pos_t.shape[0]:
        pos_t = pos_t[: int(N)]
    return Tree(pos_t, S, ncrit, order, theta, source_order=source_order, stream=stream)


def direct(pos, S, targets=None, source_order=0, potential=True, field=True, F=None, stream=None):
    """FP64 O(N^2) sum (example/calculate.cpp:252-264) for a target subset."""
    pos = _as_device(pos, (3,))
    S = _as_device(S, (sourcesize(source_order),))
    N = pos.shape[0]
    tgt = None
    nt = N
    if targets is not None:
        tgt = torch.as_tensor(np.asarray(targets) if not isinstance(targets, torch.Tensor) else targets)
        tgt = tgt.to(device=pos.device, dtype=torch.int64).contiguous()
        nt = tgt.numel()
    os_ = outputsize(potential, field)
    Fd = torch.empty((nt, os_), dtype=torch.float64, device=pos.device)
    check(lib().fmmgen_gpu_direct(C.c_void_p(pos.data_ptr()), C.c_void_p(S.data_ptr()), N,
                                  C.c_void_p(tgt.data_ptr() if tgt is not None else None), nt, source_order,
                                  int(potential), int(field), C.c_void_p(Fd.data_ptr()), _stream_ptr(stream)))
    if F is not None:
        if isinstance(F, torch.Tensor):
            F.copy_(Fd)
        else:
            F[...] = Fd.cpu().numpy().reshape(np.shape(F))
        return F
    return Fd
