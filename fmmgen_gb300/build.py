"""Compile the CUDA sources in fmmgen_gb300/csrc into fmmgen_gb300/libfmmgen_gb300.so.

nvcc, one -gencode for sm_103a, translation units compiled in parallel, then
linked into a shared library with a plain C ABI (include/fmmgen_gb300.h).
Rebuilds only what changed.  Usage: python -m fmmgen_gb300.build [-v]
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfmmgen_gb300.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(os.path.dirname(HERE), "include", "fmmgen_gb300.h"))
    return hs


def _generate():
    """(Re)write the generated kernels (csrc/m2l_gen.cuh, csrc/m2l_cm*) when
    their generator is newer."""
    from . import gen_m2l, gen_m2l_cm

    out, src = gen_m2l.OUT, os.path.abspath(gen_m2l.__file__)
    if not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(src):
        gen_m2l.generate()
    src = os.path.abspath(gen_m2l_cm.__file__)
    outs = [os.path.join(CSRC, "m2l_cm.cuh")] + [os.path.join(CSRC, gen_m2l_cm.family_file(so, pm))
                                                  for so, pm in gen_m2l_cm.FAMILIES]
    if any(not os.path.exists(o) or os.path.getmtime(o) < os.path.getmtime(src) for o in outs):
        gen_m2l_cm.generate()


def build(verbose=False, ptxas_verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    _generate()
    hdr_mtime = max(os.path.getmtime(h) for h in _headers())
    jobs = []
    objs = []
    for src in _sources():
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), hdr_mtime):
            cmd = [NVCC, *ARCH, *FLAGS, "-c", s, "-o", o]
            if ptxas_verbose:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    failed = []
    with ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for cmd, r in ex.map(run, jobs):
            if r.returncode != 0:
                failed.append((cmd, r))
            elif verbose or ptxas_verbose:
                sys.stdout.write(r.stdout + r.stderr)
    if failed:
        for cmd, r in failed:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError("nvcc failed")
    if jobs or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [NVCC, *ARCH, "-shared", "-o", LIB, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(HERE))
    from fmmgen_gb300 import build as _b

    _b.build(verbose="-v" in sys.argv, ptxas_verbose="--ptxas" in sys.argv)
    print(LIB)
