"""include/operators.h as a drop-in for the generated operators.h.

CPU: a C++ caller shaped like the reference example and a C caller compile
against the header with the generator's choices as -D macros and link against
libfmmgen_gb300.so (every declared symbol resolves); where the reference
checkout is present, its own example sources (example/calculate.cpp, tree.cpp,
utils.cpp, main.cpp) compile unchanged against the header and link too.
GPU: the C++ caller evaluates the reference's own tree (tests/golden, written
by the reference's build_tree / compute_field_fmm) through the scalar
operators alone and matches the reference's F; the C caller's per-order
functions equal the dispatchers."""
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
INC = os.path.join(ROOT, "include")
SRC = os.path.join(HERE, "operators_h")
GOLDEN = os.path.join(HERE, "golden")
REFERENCE = os.environ.get("FMMGEN_REFERENCE_DIR", "/root/reference")


def _link_flags(fg):
    from fmmgen_gb300 import _lib

    d = os.path.dirname(_lib.LIB_PATH)
    return ["-L", d, "-lfmmgen_gb300", f"-Wl,-rpath,{d}"]


def compile_caller(fg, tmp_path, source, so, maxorder, extra=()):
    out = str(tmp_path / f"{os.path.basename(source)}.so{so}.p{maxorder}")
    cc = "g++" if source.endswith(".cpp") else "gcc"
    std = ["-std=c++17"] if cc == "g++" else ["-std=c11"]
    cmd = [cc, "-O1", *std, f"-DFMMGEN_SOURCEORDER={so}", f"-DFMMGEN_MAXORDER={maxorder}", "-I", INC, *extra,
           source, "-o", out, *_link_flags(fg), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, " ".join(cmd) + "\n" + r.stdout + r.stderr
    return out


def test_callers_compile_and_link(fg, tmp_path):
    for so in (0, 1):
        compile_caller(fg, tmp_path, os.path.join(SRC, "fmm_caller.cpp"), so, 9)
        compile_caller(fg, tmp_path, os.path.join(SRC, "per_order.c"), so, 9)


def test_header_rejects_bad_maxorder(fg, tmp_path):
    src = tmp_path / "bad.c"
    src.write_text('#include "operators.h"\nint main(void) { return 0; }\n')
    r = subprocess.run(["gcc", "-DFMMGEN_MAXORDER=14", "-I", INC, "-c", str(src), "-o", str(tmp_path / "bad.o")],
                       capture_output=True, text=True)
    assert r.returncode != 0 and "FMMGEN_MAXORDER" in r.stderr


@pytest.mark.skipif(not os.path.isdir(os.path.join(REFERENCE, "example")), reason="reference checkout absent")
def test_reference_example_compiles_unchanged(fg, tmp_path):
    """The reference's example driver and tree code, unmodified, build against
    include/operators.h (found first on the include path) and link against the
    library: every operator and FMMGEN_* macro they use is provided."""
    ex = os.path.join(REFERENCE, "example")
    srcs = [os.path.join(ex, f) for f in ("calculate.cpp", "tree.cpp", "utils.cpp", "main.cpp")]
    out = str(tmp_path / "example_fmm")
    cmd = ["g++", "-O1", "-std=c++14", "-fopenmp", "-DFMMGEN_SOURCEORDER=0", "-DFMMGEN_MAXORDER=9", "-I", INC,
           "-I", ex, *srcs, "-o", out, *_link_flags(fg)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def write_input(path, g, idx):
    """The reference tree of a golden fixture in fmm_caller's input format;
    cells in canonical-id order (parents before children)."""
    ids = g["cell_id"].astype(np.uint64)
    N, so = int(g["N"]), int(g["source_order"])
    ncells = len(ids)
    pos_of = {int(c): k for k, c in enumerate(ids)}
    parent = np.array([pos_of.get(int(c) >> 3, -1) if k else -1 for k, c in enumerate(ids)], np.int64)
    leafcell = np.array([pos_of[int(c)] for c in g["leaf_id"]], np.int64)
    m2l = np.array([[pos_of[int(b)], pos_of[int(a)]] for b, a in g["m2l"]], np.int64).reshape(-1, 2)
    p2p = np.array([[pos_of[int(a)], pos_of[int(b)]] for a, b in g["p2p"]], np.int64).reshape(-1, 2)
    hdr = np.array([N, ncells, len(leafcell), len(m2l), len(p2p), int(g["order"]), so, 0], np.int64)
    with open(path, "wb") as f:
        for a in (hdr, g["pos"].astype(np.float64), g["S"].astype(np.float64), g["cell_centre"].astype(np.float64),
                  parent, leafcell, g["leaf_off"].astype(np.int64), g["leaf_idx"].astype(np.int64), m2l, p2p):
            f.write(np.ascontiguousarray(a).tobytes())


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["small_charges", "small_dipoles"])
def test_reference_tree_through_scalar_operators(fg, tmp_path, name):
    g = np.load(os.path.join(GOLDEN, f"tree_{name}.npz"))
    so, p = int(g["source_order"]), int(g["order"])
    exe = compile_caller(fg, tmp_path, os.path.join(SRC, "fmm_caller.cpp"), so, p + 1)
    inp, outp = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    write_input(inp, g, None)
    r = subprocess.run([exe, inp, outp], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    F = np.fromfile(outp, dtype=np.float64).reshape(-1, 4)
    Fr = g["F"]
    rel = np.linalg.norm(F - Fr) / np.linalg.norm(Fr)
    assert rel < 1e-12, rel


@pytest.mark.gpu
@pytest.mark.parametrize("so", [0, 1])
def test_per_order_functions_equal_dispatchers(fg, tmp_path, so):
    exe = compile_caller(fg, tmp_path, os.path.join(SRC, "per_order.c"), so, 9)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    mn, mx, sorder, ssize, osize, diff, amax = r.stdout.split()
    assert (int(mn), int(mx), int(sorder), int(ssize), int(osize)) == (so + 1, 9, so, 1 if so == 0 else 3, 4)
    assert float(amax) > 0 and float(diff) == 0.0
