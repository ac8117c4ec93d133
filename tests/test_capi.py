"""The C-ABI library loads and exports every symbol include/fmmgen_gb300.h
declares; the host-only entry points answer without a GPU."""
import ctypes

import numpy as np
import pytest


def test_library_exports_header(fg):
    from fmmgen_gb300 import _lib

    names = _lib.header_functions()
    assert len(names) >= 30, names
    L = ctypes.CDLL(_lib.LIB_PATH)
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # every header function is bound with a signature in the Python binding
    assert set(names) <= set(_lib._SIGS), set(names) - set(_lib._SIGS)


def test_layout_constants(fg, oracle_lib):
    L = fg.lib()
    for p in range(0, 13):
        assert L.fmmgen_nterms(p) == oracle_lib.nterms(p)
    for p in range(1, 13):
        for so in (0, 1):
            assert L.fmmgen_msize(p, so) == oracle_lib.msize(p, so)
            assert L.fmmgen_lsize(p, so) == oracle_lib.lsize(p, so)
    assert L.fmmgen_minorder(0, 1) == 1 and L.fmmgen_minorder(1, 1) == 2 and L.fmmgen_minorder(0, 0) == 0
    assert L.fmmgen_sourcesize(0) == 1 and L.fmmgen_sourcesize(1) == 3
    assert L.fmmgen_outputsize(1, 1) == 4 and L.fmmgen_outputsize(0, 1) == 3 and L.fmmgen_outputsize(1, 0) == 1
    assert L.fmmgen_max_order() == 12
    assert b"sm_103a" in L.fmmgen_version()


def test_operator_module_surface(fg):
    from fmmgen_gb300 import operators

    m = operators.module(9, source_order=0)
    assert (m.FMMGEN_MINORDER, m.FMMGEN_MAXORDER, m.FMMGEN_SOURCESIZE, m.FMMGEN_OUTPUTSIZE) == (1, 9, 1, 4)
    d = operators.module(7, source_order=1, potential=False)
    assert (d.FMMGEN_MINORDER, d.FMMGEN_SOURCEORDER, d.FMMGEN_SOURCESIZE, d.FMMGEN_OUTPUTSIZE) == (2, 1, 3, 3)
    assert callable(m.M2L5)
    with pytest.raises(AttributeError):
        m.M2L9  # outside [MINORDER, MAXORDER)
    with pytest.raises(TypeError):
        m.M2M(0.0, 0.0, 0.0, [1.0], np.zeros(4), 1)  # buffers must be float64 arrays


def test_invalid_arguments_rejected_without_gpu(fg):
    from fmmgen_gb300 import _lib

    L = fg.lib()
    assert L.fmmgen_configure(3, 1, 1, 8) == _lib.ERR_ARG  # source orders 0, 1, 2
    assert L.fmmgen_sourcesize(2) == 6 and L.fmmgen_msize(5, 2) == 56 - 4
    assert L.fmmgen_configure(0, 0, 0, 8) == _lib.ERR_ARG
    assert L.fmmgen_configure(0, 1, 1, 13) == _lib.ERR_ARG
    # order above the supported maximum is rejected before any device work
    assert L.fmmgen_gpu_M2L(1, None, None, None, 13, 0, None) == _lib.ERR_ARG
    h = ctypes.c_void_p(None)
    assert L.fmmgen_tree_build(None, 10, 8, 4, 0.5, 0, None, ctypes.byref(h)) == _lib.ERR_ARG
    assert L.fmmgen_tree_info(None, None) == _lib.ERR_STATE
