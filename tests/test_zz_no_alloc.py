"""fmmgen_root_box_noalloc: the root cube computed without allocating device
memory, for callers that cannot call cudaMalloc where they need it.  It must
equal, bit for bit, the root cube of the allocating path (fmmgen_tree_build),
on consecutive calls that reuse the shared static scratch array."""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def root_via_build(fg, pos):
    t = fg.build_tree(pos, torch.ones(pos.shape[0], 1, dtype=torch.float64, device="cuda"), pos.shape[0], 64, 3,
                      0.5)
    return t.root()


def root_noalloc(fg, pos):
    out = torch.full((4,), float("nan"), dtype=torch.float64, device="cuda")
    rc = fg.lib().fmmgen_root_box_noalloc(C.c_void_p(pos.data_ptr()), pos.shape[0], C.c_void_p(out.data_ptr()),
                                          C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, fg.lib().fmmgen_last_error()
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_noalloc_root_box_matches_build_twice(fg):
    rng = np.random.default_rng(123)
    # two calls in a row on different inputs: the second call reuses the scratch
    # (and its stale maxima) left by the first
    a = torch.tensor(rng.uniform(-2, 5, (300_001, 3)), device="cuda")
    b = torch.tensor(0.1 * rng.standard_normal((70_000, 3)), device="cuda")
    ra, rb = root_via_build(fg, a), root_via_build(fg, b)
    na, nb = root_noalloc(fg, a), root_noalloc(fg, b)
    assert np.array_equal(na, ra), (na, ra)
    assert np.array_equal(nb, rb), (nb, rb)
    # and again in the other order
    assert np.array_equal(root_noalloc(fg, b), rb)
    assert np.array_equal(root_noalloc(fg, a), ra)


def test_noalloc_call_allocates_nothing(fg):
    """After a warm-up call on the device (which places the static array and the
    kernels there), a call leaves the device's free memory unchanged."""
    rng = np.random.default_rng(5)
    a = torch.tensor(rng.uniform(0, 1, (200_003, 3)), device="cuda")
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    lib = fg.lib()
    assert lib.fmmgen_root_box_noalloc(C.c_void_p(a.data_ptr()), 1000, C.c_void_p(out.data_ptr()), stream) == 0
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        assert lib.fmmgen_root_box_noalloc(C.c_void_p(a.data_ptr()), a.shape[0], C.c_void_p(out.data_ptr()),
                                           stream) == 0, lib.fmmgen_last_error()
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 == free0, (free0, free1)
    assert np.array_equal(out.cpu().numpy(), root_via_build(fg, a))


def test_noalloc_rejects_oversize(fg):
    from fmmgen_gb300 import _lib

    dummy = torch.zeros(4, dtype=torch.float64, device="cuda")
    rc = fg.lib().fmmgen_root_box_noalloc(C.c_void_p(dummy.data_ptr()), 16777217, C.c_void_p(dummy.data_ptr()), None)
    assert rc == _lib.ERR_ARG
    assert b"FMMGEN_NOALLOC_MAX_N" in fg.lib().fmmgen_last_error()
