"""Generate fmmgen_gb300/csrc/m2l_gen.cuh: register-resident FP32 M2L kernels.

For a pair (B -> A) of translation class c the scaled M2L (see csrc/eval.cu) is
    L^_n += sum_m D_c[n + m] * rho^|m| * M~_m,     |n| + |m| <= p, |m| >= so
(the contraction of fmmgen/expansions.py:144-172).  The emitted kernels give
each thread one target cell and one group of its outputs n: the thread loops
over the target's sources, takes the source multipole terms the group needs
into registers (the warp first stages its 32 lanes' source rows in shared
memory with coalesced loads), streams the class's derivative vector in float4
quads, and issues the group's multiply-adds with every index resolved at
generation time.  Outputs are split into groups so that accumulators plus
resident multipole terms stay within the register file; groups are chosen to
balance their multiply-add counts.

Run:  python -m fmmgen_gb300.gen_m2l   (build.py runs it when this file changes)
"""
import os

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "csrc", "m2l_gen.cuh")

# (order, source_order) -> output degree groups (inclusive ranges of |n|)
CONFIGS = {
    (4, 0): [(0, 4)],
    (5, 0): [(0, 5)],
    (6, 0): [(0, 1), (2, 6)],
    (7, 0): [(0, 1), (2, 3), (4, 7)],
    (8, 0): [(0, 1), (2, 3), (4, 8)],
    (4, 1): [(0, 3)],
    (5, 1): [(0, 4)],
    (6, 1): [(0, 1), (2, 5)],
    (7, 1): [(0, 1), (2, 3), (4, 6)],
}
# Outputs with at least this many terms per pair first sum the pair's terms in
# a temporary and then add it to their running total: otherwise every term is
# added to a large running sum and the FP32 rounding grows with the number of
# terms over all sources (~10^5 for L_0 at p=8).
PARTIAL_MIN_TERMS = 21


def nterms(p):
    return 0 if p < 0 else (p + 1) * (p + 2) * (p + 3) // 6


def monomials(p):
    out = []
    for d in range(p + 1):
        for nx in range(d, -1, -1):
            for ny in range(d - nx, -1, -1):
                out.append((nx, ny, d - nx - ny))
    return out


def idx3(n):
    d = sum(n)
    j = d - n[0]
    return nterms(d - 1) + j * (j + 1) // 2 + (j - n[1])


def stride(n):
    return (n + 3) // 4 * 4


def emit_kernel(p, so, g, lo, hi):
    mono = monomials(p)
    moff = nterms(so - 1)
    ms = nterms(p) - moff
    ls = nterms(p - so)
    outs = [i for i in range(ls) if lo <= sum(mono[i]) <= hi]
    # terms: (k = idx(n+m), out slot, m in M layout)
    terms = []
    need_m = set()
    for oi, i in enumerate(outs):
        n = mono[i]
        for j in range(moff, nterms(p)):
            m = mono[j]
            if sum(m) < so or sum(n) + sum(m) > p:
                continue
            k = idx3((n[0] + m[0], n[1] + m[1], n[2] + m[2]))
            terms.append((k, oi, j - moff))
            need_m.add(j - moff)
    terms.sort()
    need_m = sorted(need_m)
    mdeg = {j: sum(mono[j + moff]) for j in need_m}
    name = f"k_m2l_reg_p{p}_s{so}_g{g}"
    L = []
    L.append(f"// order {p}, source order {so}, outputs of degree {lo}..{hi}: {len(outs)} outputs, "
             f"{len(need_m)} multipole terms, {len(terms)} multiply-adds per pair")
    quads = sorted({j // 4 for j in need_m})
    nq = quads[-1] + 1  # the needed terms are a prefix of the multipole row
    # warps per block: the staging buffer (32 rows x (nq + 1) quads per warp) stays within 48 KB
    warps = max(1, min(4, 49152 // (32 * (nq + 1) * 16)))
    L.append(f"__global__ void __launch_bounds__({32 * warps}) {name}(const int *__restrict__ tgt, int ntgt, "
             "const int *__restrict__ off, const int *__restrict__ src, const int *__restrict__ cls, "
             "const float *__restrict__ clsD, const unsigned char *__restrict__ clevel, "
             "const float *__restrict__ M, float *__restrict__ L) {")
    L.append(f"  __shared__ float4 sM[{warps}][32][{nq + 1}];  // per warp: the 32 lanes' source rows (+1 quad pad)")
    L.append("  const int t = blockIdx.x * blockDim.x + threadIdx.x;")
    L.append("  const int lane = threadIdx.x & 31, wq = threadIdx.x >> 5;")
    L.append("  const bool act = t < ntgt;")
    L.append("  const int A = act ? (tgt ? tgt[t] : t) : 0;  // cells without sources store zeros")
    L.append("  const int la = clevel[A];")
    L.append("  const int k0 = act ? off[A] : 0;")
    L.append("  const int n = act ? off[A + 1] - k0 : 0;")
    L.append("  int nmax = n;")
    L.append("  for (int o = 16; o; o >>= 1) nmax = max(nmax, __shfl_xor_sync(0xffffffffu, nmax, o));")
    for oi in range(len(outs)):
        L.append(f"  float a{oi} = 0.f;")
    L.append("  for (int j = 0; j < nmax; j++) {")
    L.append("    const bool on = j < n;")
    L.append("    const int B = on ? src[k0 + j] : -1;")
    L.append("    const int c = on ? cls[k0 + j] : 0;")
    L.append("    // stage the lanes' source rows with asynchronous 16-byte copies: the warp walks the")
    L.append(f"    // 32 x {nq} quads row after row, so each warp-wide copy covers one contiguous segment")
    L.append("    __syncwarp();")
    L.append("#pragma unroll 6")
    L.append(f"    for (int i = lane; i < {32 * nq}; i += 32) {{")
    L.append(f"      const int r = i / {nq}, q = i - r * {nq};")
    L.append("      const int Br = __shfl_sync(0xffffffffu, B, r);")
    L.append("      if (Br >= 0)")
    L.append(f"        cp_async16(&sM[wq][r][q], M + (size_t)Br * {stride(ms)} + 4 * q);")
    L.append("    }")
    L.append("    cp_async_wait_all();")
    L.append("    __syncwarp();")
    L.append("    if (!on) continue;")
    L.append(f"    const float *__restrict__ Dp = clsD + (size_t)c * {stride(nterms(p))};")
    # multipole terms, scaled by rho^|m| = 2^((lA - lB)|m|)
    for q in quads:
        L.append(f"    const float4 mq{q} = sM[wq][lane][{q}];")
    comp = "xyzw"
    for j in need_m:
        L.append(f"    float m{j} = mq{j // 4}.{comp[j % 4]};")
    L.append("    const int dl = la - (int)clevel[B];")
    L.append("    if (dl != 0) {")
    degs = sorted(set(mdeg.values()))
    for d in degs:
        if d == 0:
            continue
        L.append(f"      const float s{d} = __int_as_float((dl * {d} + 127) << 23);")
    for j in need_m:
        if mdeg[j]:
            L.append(f"      m{j} *= s{mdeg[j]};")
    L.append("    }")
    # stream D in quads, multiply-add (per-pair temporaries for long outputs)
    nterm_out = {}
    for k, oi, j in terms:
        nterm_out[oi] = nterm_out.get(oi, 0) + 1
    partial = {oi for oi, c in nterm_out.items() if c >= PARTIAL_MIN_TERMS}
    started = set()
    cur_q = None
    for k, oi, j in terms:
        q = k // 4
        if q != cur_q:
            L.append(f"    const float4 dq{q} = __ldg((const float4 *)(Dp + {4 * q}));")
            cur_q = q
        if oi in partial:
            if oi not in started:
                L.append(f"    float t{oi} = dq{q}.{comp[k % 4]} * m{j};")
                started.add(oi)
            else:
                L.append(f"    t{oi} = fmaf(dq{q}.{comp[k % 4]}, m{j}, t{oi});")
        else:
            L.append(f"    a{oi} = fmaf(dq{q}.{comp[k % 4]}, m{j}, a{oi});")
    for oi in sorted(partial):
        L.append(f"    a{oi} += t{oi};")
    L.append("  }")
    L.append("  if (!act) return;")
    for oi, i in enumerate(outs):
        L.append(f"  L[(size_t)A * {stride(ls)} + {i}] = a{oi};")
    L.append("}")
    return name, 32 * warps, "\n".join(L)


def generate():
    parts = ["// m2l_gen.cuh -- generated by fmmgen_gb300/gen_m2l.py; do not edit.",
             "// Register-resident FP32 M2L kernels, one thread per (target cell, output group).",
             "#pragma once", "#include <cuda_runtime.h>", "",
             "// 16-byte global -> shared copy that bypasses the registers (cp.async, L2 only)",
             "static __device__ __forceinline__ void cp_async16(void *dst, const void *src) {",
             "  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);",
             "  asm volatile(\"cp.async.cg.shared.global [%0], [%1], 16;\\n\" :: \"r\"(d), \"l\"(src) : \"memory\");",
             "}",
             "static __device__ __forceinline__ void cp_async_wait_all() {",
             "  asm volatile(\"cp.async.wait_all;\\n\" ::: \"memory\");",
             "}", ""]
    table = []
    for (p, so), groups in CONFIGS.items():
        names = []
        for g, (lo, hi) in enumerate(groups):
            name, threads, code = emit_kernel(p, so, g, lo, hi)
            parts.append(code)
            parts.append("")
            names.append((name, threads))
        table.append((p, so, names))
    parts.append("typedef void (*m2l_reg_kernel)(const int *, int, const int *, const int *, const int *, "
                 "const float *, const unsigned char *, const float *, float *);")
    parts.append("// kernels of the output groups for (order, source order) and their block sizes;")
    parts.append("// returns 0 when none was generated")
    parts.append("static inline int m2l_reg_kernels(int p, int so, m2l_reg_kernel *k, int *threads) {")
    for p, so, names in table:
        body = " ".join(f"k[{i}] = {n}; threads[{i}] = {t};" for i, (n, t) in enumerate(names))
        parts.append(f"  if (p == {p} && so == {so}) {{ {body} return {len(names)}; }}")
    parts.append("  return 0;")
    parts.append("}")
    text = "\n".join(parts) + "\n"
    with open(OUT, "w") as f:
        f.write(text)
    return OUT


if __name__ == "__main__":
    print(generate())
