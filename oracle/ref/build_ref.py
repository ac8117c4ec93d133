"""Build the reference's own FMM path into oracle/_ref/ (checker only).

Recipe, run in the development container where the reference checkout exists:
  1. fmmgen.generate_code (the reference generator, imported read-only from the
     checkout) emits operators.{cpp,h} for Coulomb (source_order=0, orders
     1..PMAX0) and dipole (source_order=1, orders 2..PMAX1) sources, with the
     settings of the reference's example/example.py (CSE, harmonic derivatives,
     minpow=11, atomic, C++), and for quadrupole sources (source_order=2,
     orders 3..PMAX2).
  2. g++ compiles the reference's example/tree.cpp, calculate.cpp, utils.cpp
     where they lie in the checkout, plus the generated operators and
     oracle/ref/ref_harness.cpp, into oracle/_ref/libref_so{0,1,2}.so.
     -ffp-contract=off keeps every FP64 expression as written (no FMA
     contraction), which the bit-exact tree/list comparisons rely on.

  3. (--float) fmmgen.generate_code with precision="float" and language="c"
     emits the FP32 operators (the same settings otherwise); gcc compiles
     them alone into oracle/_ref/libref_f32_so{0,1,2}.so, whose plain C
     symbols (P2M, M2M, ... with float arguments) ctypes calls directly.

Outputs are cached: a step is skipped when its output is newer than its inputs.
Nothing here is shipped; the GPU machine never runs it.

Usage: python oracle/ref/build_ref.py [--reference DIR] [--pmax0 8] [--pmax1 6] [--pmax2 5] [--float]
"""
import argparse
import contextlib
import io
import multiprocessing as mp
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_ref")
# the reference checkout: $FMMGEN_REFERENCE_DIR, else where the development container mounts it
DEFAULT_REF = os.environ.get("FMMGEN_REFERENCE_DIR", "/root/reference")


def _generate(args):
    ref, so, pmax, outdir = args[:4]
    precision, language = args[4:] if len(args) > 4 else ("double", "c++")
    sys.path.insert(0, ref)
    import fmmgen  # the reference generator

    os.makedirs(outdir, exist_ok=True)
    cwd = os.getcwd()
    os.chdir(outdir)
    try:
        with contextlib.redirect_stdout(io.StringIO()):
            fmmgen.generate_code(
                pmax + 1,  # the generator's upper order bound is exclusive
                "operators",
                precision=precision,
                CSE=True,
                cython=False,
                potential=True,
                field=True,
                source_order=so,
                atomic=True,
                minpow=11,
                harmonic_derivs=True,
                language=language,
                include_dir=outdir,
                src_dir=outdir,
            )
    finally:
        os.chdir(cwd)
    return outdir


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(ref=DEFAULT_REF, pmax0=8, pmax1=6, pmax2=5, jobs=4, verbose=True):
    """Generate + compile; returns {source_order: path to .so}.  Raises if the
    reference checkout is absent."""
    ex = os.path.join(ref, "example")
    if not os.path.isdir(ex):
        raise FileNotFoundError(f"reference checkout not found at {ref}")
    specs = [(0, pmax0), (1, pmax1), (2, pmax2)]
    gen_jobs = []
    for so, pmax in specs:
        outdir = os.path.join(OUT, f"so{so}_p{pmax}")
        if _stale(os.path.join(outdir, "operators.cpp"), [os.path.join(ref, "fmmgen", "generator.py")]):
            gen_jobs.append((ref, so, pmax, outdir))
    if gen_jobs:
        if verbose:
            print(f"[build_ref] generating operators with fmmgen: {[(j[1], j[2]) for j in gen_jobs]}", flush=True)
        ctx = mp.get_context("spawn")
        with ctx.Pool(len(gen_jobs)) as pool:
            pool.map(_generate, gen_jobs)
    libs = {}
    procs = []
    for so, pmax in specs:
        gdir = os.path.join(OUT, f"so{so}_p{pmax}")
        lib = os.path.join(OUT, f"libref_so{so}.so")
        srcs = [os.path.join(ex, f) for f in ("tree.cpp", "calculate.cpp", "utils.cpp")]
        deps = srcs + [os.path.join(gdir, "operators.cpp"), os.path.join(HERE, "ref_harness.cpp"), __file__]
        libs[so] = lib
        if not _stale(lib, deps):
            continue
        objs = []
        flags = ["-O2", "-std=c++14", "-fopenmp", "-fPIC", "-ffp-contract=off", "-I", gdir, "-I", ex]
        cmds = []
        for s in srcs:
            o = os.path.join(gdir, os.path.basename(s).replace(".cpp", ".o"))
            cmds.append(["g++", *flags, "-c", s, "-o", o])
            objs.append(o)
        o = os.path.join(gdir, "operators.o")
        cmds.append(["g++", *flags, "-DP2P=fmmgen_generated_P2P", "-c", os.path.join(gdir, "operators.cpp"), "-o", o])
        objs.append(o)
        o = os.path.join(gdir, "ref_harness.o")
        cmds.append(["g++", *flags, "-c", os.path.join(HERE, "ref_harness.cpp"), "-o", o])
        objs.append(o)
        procs.append((cmds, objs, lib, flags))
    for cmds, objs, lib, flags in procs:
        if verbose:
            print(f"[build_ref] compiling {lib}", flush=True)
        running = [subprocess.Popen(c) for c in cmds]
        rcs = [p.wait() for p in running]
        if any(rcs):
            raise RuntimeError(f"reference compile failed: {rcs}")
        subprocess.check_call(["g++", "-shared", "-fopenmp", "-o", lib, *objs])
    return libs


def build_float(ref=DEFAULT_REF, pmax0=8, pmax1=6, pmax2=5, verbose=True):
    """The precision="float" operators alone; returns {source_order: path to .so}."""
    if not os.path.isdir(os.path.join(ref, "fmmgen")):
        raise FileNotFoundError(f"reference checkout not found at {ref}")
    specs = [(0, pmax0), (1, pmax1), (2, pmax2)]
    gen = [os.path.join(ref, "fmmgen", f) for f in ("generator.py", "printers.py", "writer.py")]
    jobs = []
    for so, pmax in specs:
        outdir = os.path.join(OUT, f"f32_so{so}_p{pmax}")
        if _stale(os.path.join(outdir, "operators.c"), gen):
            jobs.append((ref, so, pmax, outdir, "float", "c"))
    if jobs:
        if verbose:
            print(f"[build_ref] generating float operators: {[(j[1], j[2]) for j in jobs]}", flush=True)
        with mp.get_context("spawn").Pool(len(jobs)) as pool:
            pool.map(_generate, jobs)
    libs, procs = {}, []
    for so, pmax in specs:
        gdir = os.path.join(OUT, f"f32_so{so}_p{pmax}")
        lib = os.path.join(OUT, f"libref_f32_so{so}.so")
        libs[so] = lib
        src = os.path.join(gdir, "operators.c")
        if _stale(lib, [src, __file__]):
            cmd = ["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-I", gdir, src, "-o", lib, "-lm"]
            if verbose:
                print(f"[build_ref] compiling {lib}", flush=True)
            procs.append(subprocess.Popen(cmd))
    if any(p.wait() for p in procs):
        raise RuntimeError("float operator compile failed")
    return libs


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=DEFAULT_REF)
    ap.add_argument("--pmax0", type=int, default=8)
    ap.add_argument("--pmax1", type=int, default=6)
    ap.add_argument("--pmax2", type=int, default=5)
    ap.add_argument("--float", action="store_true", help="also build the precision=\"float\" operators")
    a = ap.parse_args()
    print(build(a.reference, a.pmax0, a.pmax1, a.pmax2))
    if a.float:
        print(build_float(a.reference, a.pmax0, a.pmax1, a.pmax2))


if __name__ == "__main__":
    main()
