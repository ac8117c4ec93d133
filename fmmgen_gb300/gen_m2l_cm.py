"""Generate fmmgen_gb300/csrc/m2l_cm_s{so}.cu: FP32 M2L kernels for every order
up to a family's largest, per-pair orders included.

For a pair (B -> A) of translation class c the scaled M2L (see csrc/eval.cu) is
    L^_n += sum_m D_c[n + m] * rho^|m| * M~_m,     |n| + |m| <= q, |m| >= so
(the contraction of fmmgen/expansions.py:144-172) with q the order of the pair:
the tree's order, or a per-pair order (learned or given).  Since |n + m| =
|n| + |m|, truncating at q keeps exactly the terms whose derivative index k =
n + m has degree <= q.

A thread holds one group of its target's outputs in registers.  Per pair it
stages its source row in shared memory chunk by chunk (asynchronous 16-byte
copies, the next chunk -- or the next pair's first -- in flight while the
current one is multiplied) and issues the multiply-adds with every index
resolved at generation time, nested by the degree of k so that a lane stops at
its pair's order: a warp's pair costs the largest order among its lanes.
Outputs with many terms per pair sum the pair's terms in a temporary first
(FP32 rounding then grows with the number of pairs, not of terms).  The order
is a runtime argument, and blocks of degree above it are skipped by a
warp-uniform branch, so one family covers every order up to its largest.

The code of one kernel is bounded (KERNEL_FMAS multiply-adds): a kernel whose
unrolled body outgrows the SM's instruction cache stalls on instruction fetch
(measured: a 12,000-term body issued a third of the time, warps waiting for
instructions).  An output group's chunks are split over several kernels; the
first stores the group's outputs, the others add to them.

Two schedules of the pairs:
  class-major (k_m2l_cm_*): the tiles of the tensor-core path's class-step
      schedule (128 target cells in M2L processing order; a step gives every
      row its source of one class, or none), one warp per 32 rows walking the
      steps that have a pair in its rows.  The class's derivative vector is
      the same for the whole warp: it is staged once in shared memory and read
      as broadcasts.
  target-major (k_m2l_tp_*): one thread per target cell walking its own pair
      list (by descending order when orders are per pair, so a warp's lanes
      reach pairs of similar order together); the lanes read their own
      classes' derivative vectors through the L1 cache.  No lane idles on a
      class its target does not have -- the better schedule on adaptive trees.

Run:  python -m fmmgen_gb300.gen_m2l_cm   (build.py runs it when this file changes)
"""
import os

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")

# (source order, largest order) of the generated families; a pass of order p
# runs the family of its source order with the smallest largest order >= p (a
# family's kernels are split for its largest order: at lower orders a smaller
# family packs more of its terms into fewer kernels)
FAMILIES = [(0, 6), (0, 8), (0, 12), (1, 6), (1, 8)]


def family_file(so, pmax):
    return f"m2l_cm_s{so}_p{pmax}.cu"
CH = 48                 # multipole terms per staged chunk (a multiple of 4)
KERNEL_FMAS = 3000      # multiply-adds per pair in one kernel's body at most (unless one chunk exceeds it)
RMAX = 208              # register estimate per thread an output group may reach
OVERHEAD = 32           # registers besides accumulators, temporaries and the chunk
PARTIAL_MIN_TERMS = 21  # outputs with at least this many terms per pair (in a kernel) sum per pair first
ROWS = 128              # threads of a block (class-major: rows of a schedule tile)
TP_PREFETCH_QUADS = 2   # target-major: operator quads of the next degree block loaded a block ahead
MIN_BLOCKS = 2          # resident blocks per SM the register allocation must allow


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


def plan(so, pmax):
    """The kernels of a family.  Each is a dict: outs (output indices of its
    group), lo (degree of the group's first output), first (it stores the
    outputs; later kernels of the group add), temps (outputs summed per pair),
    chunks: dicts with mb, me (multipole index range), emin (degree of its
    first term) and terms [(d, k, i, jj)] (degree, derivative index, output
    index, multipole index) sorted by (d, k, i)."""
    mono = monomials(pmax)
    moff = nterms(so - 1)
    nout = nterms(pmax - so)

    def per_pair(i):
        return nterms(pmax - sum(mono[i])) - moff

    def need_of(lo):
        return nterms(pmax - lo) - moff

    def est(i0, i1):
        lo = sum(mono[i0])
        a = i1 - i0
        t = sum(1 for i in range(i0, i1) if per_pair(i) >= PARTIAL_MIN_TERMS)
        ch = min(CH, (need_of(lo) + 3) // 4 * 4)
        return a + t + ch + OVERHEAD

    kernels = []
    i0 = 0
    while i0 < nout:
        i1 = i0 + 1
        while i1 < nout and est(i0, i1 + 1) <= RMAX:
            i1 += 1
        outs = list(range(i0, i1))
        lo = sum(mono[i0])
        chunks = []
        for mb in range(0, need_of(lo), CH):
            me = min(need_of(lo), mb + CH)
            terms = []
            for i in outs:
                n = mono[i]
                for jj in range(mb, me):
                    m = mono[jj + moff]
                    d = sum(n) + sum(m)
                    if d <= pmax:
                        terms.append((d, idx3((n[0] + m[0], n[1] + m[1], n[2] + m[2])), i, jj))
            terms.sort()
            if terms:
                chunks.append({"mb": mb, "me": me, "emin": sum(mono[mb + moff]), "terms": terms})
        # consecutive chunks into kernels of at most KERNEL_FMAS multiply-adds
        runs, cur, nf = [], [], 0
        for c in chunks:
            if cur and nf + len(c["terms"]) > KERNEL_FMAS:
                runs.append(cur)
                cur, nf = [], 0
            cur.append(c)
            nf += len(c["terms"])
        runs.append(cur)
        for r, run in enumerate(runs):
            cnt = {}
            for c in run:
                for (_, _, i, _) in c["terms"]:
                    cnt[i] = cnt.get(i, 0) + 1
            kernels.append({"outs": outs, "lo": lo, "first": r == 0, "chunks": run,
                            "temps": sorted(i for i, v in cnt.items() if v >= PARTIAL_MIN_TERMS)})
        i0 = i1
    return kernels


COMP = "xyzw"


def chunk_body(so, pmax, c, kern, srcexpr, dload, ind, prefetch_quads=0):
    """Multiply one staged chunk: its multipole terms from shared memory
    (scaled by the level difference), the terms nested by degree; with
    prefetch_quads, each degree block first loads that many of the next
    block's operator quads (global loads, whose latency the block's own
    multiply-adds then cover)."""
    mono = monomials(pmax)
    moff = nterms(so - 1)
    i0 = kern["outs"][0]
    temps = set(kern["temps"])
    L = []
    L.append(ind + f"const float4 *src = {srcexpr};")
    used = sorted({jj for (_, _, _, jj) in c["terms"]})
    for q in sorted({(jj - c["mb"]) // 4 for jj in used}):
        L.append(ind + f"const float4 mq{q} = src[{q}];")
    for jj in used:
        L.append(ind + f"float m{jj} = mq{(jj - c['mb']) // 4}.{COMP[(jj - c['mb']) % 4]};")
    degs = sorted({sum(mono[jj + moff]) for jj in used})
    if any(d > 0 for d in degs):
        L.append(ind + "if (dl != 0) {")
        for d in degs:
            if d:
                L.append(ind + f"  const float sc{d} = __int_as_float((dl * {d} + 127) << 23);")
        for jj in used:
            d = sum(mono[jj + moff])
            if d:
                L.append(ind + f"  m{jj} *= sc{d};")
        L.append(ind + "}")
    by_d = {}
    for t in c["terms"]:
        by_d.setdefault(t[0], []).append(t)
    dlo, dhi = min(by_d), max(by_d)
    # the quads each degree block loads first, in order of use
    first = {}
    seen = set()
    for d in range(dlo, dhi + 1):
        first[d] = []
        for (_, k, i, jj) in by_d.get(d, []):
            if k // 4 not in seen:
                seen.add(k // 4)
                first[d].append(k // 4)
    depth = 0
    loaded = set()

    def prefetch(d, ii, guard):
        # the first quads of block d, loaded a block ahead (warp-uniform: d <= qmax <= the pass's order,
        # so every load stays inside the class's row)
        for kq in first.get(d, [])[:prefetch_quads]:
            if guard:
                L.append(ii + f"float4 dq{kq} = make_float4(0.f, 0.f, 0.f, 0.f);")
                L.append(ii + f"if (qmax >= {d}) dq{kq} = {dload(kq)};")
            else:
                L.append(ii + f"const float4 dq{kq} = {dload(kq)};")
            loaded.add(kq)

    if prefetch_quads:
        prefetch(dlo, ind, False)  # the chunk runs only when qmax reaches its lowest degree
    for d in range(dlo, dhi + 1):
        L.append(ind + "  " * depth + f"if (ql >= {d}) {{")
        depth += 1
        ii = ind + "  " * depth
        if prefetch_quads and d < dhi:
            prefetch(d + 1, ii, True)
        for (_, k, i, jj) in by_d.get(d, []):
            kq = k // 4
            if kq not in loaded:
                L.append(ii + f"const float4 dq{kq} = {dload(kq)};")
                loaded.add(kq)
            acc = f"t{i - i0}" if i in temps else f"a{i - i0}"
            L.append(ii + f"{acc} = fmaf(dq{kq}.{COMP[k % 4]}, m{jj}, {acc});")
    for _ in range(depth):
        depth -= 1
        L.append(ind + "  " * depth + "}")
    return L


def stage_chunk(c, chq, chb, bufexpr, bvar, ind):
    """Stage a chunk of the 32 lanes' source rows (lane r's row from cell bvar
    of lane r, skipped when -1): consecutive lanes copy consecutive quads."""
    nq = (c["me"] - c["mb"] + 3) // 4
    qb = c["mb"] // 4
    return [ind + "{",
            ind + f"  float4 *dst = sbuf + ({bufexpr}) * {chb};",
            "#pragma unroll 4",
            ind + f"  for (int i = lane; i < {32 * nq}; i += 32) {{",
            ind + f"    const int r = i / {nq}, q = i - r * {nq};",
            ind + f"    const int Br = __shfl_sync(0xffffffffu, {bvar}, r);",
            ind + f"    if (Br >= 0 && {qb} + q < mq)",
            ind + f"      cm_cp_async16(dst + r * {chq + 1} + q, P.M + (size_t)Br * P.mstr + 4 * ({qb} + q));",
            ind + "  }",
            ind + "}"]


def pipeline(so, pmax, kern, chq, chb, dload, prefetch_next, ind, prefetch_quads=0):
    """The chunks of one pair (or step): chunk j+1 staged while j is multiplied;
    after the last, prefetch_next(ind) stages the next pair's first chunk."""
    chunks = kern["chunks"]
    L = []
    for ci, c in enumerate(chunks):
        L.append(ind + f"if ({ci} < nch) {{  // multipole terms {c['mb']}..{c['me'] - 1}")
        if ci + 1 < len(chunks):
            L.append(ind + f"  if ({ci + 1} < nch) {{")
            L.extend(stage_chunk(chunks[ci + 1], chq, chb, f"(base + {ci + 1}) & 1", "B", ind + "    "))
            L.append(ind + "    cm_cp_async_commit();")
            L.append(ind + "    cm_cp_async_wait<1>();")
            L.append(ind + "  } else {")
        else:
            L.append(ind + "  {")
        L.extend(prefetch_next(ind + "    "))
        L.append(ind + "  }")
        L.append(ind + "  __syncwarp();")
        L.extend(chunk_body(so, pmax, c, kern, f"sbuf + ((base + {ci}) & 1) * {chb} + lane * {chq + 1}", dload,
                            ind + "  ", prefetch_quads))
        L.append(ind + "  __syncwarp();  // the buffer is refilled two chunks on")
        L.append(ind + "}")
    return L


def header_lines(kern, name, so, pmax, params, extra_smem_comment):
    mono = monomials(pmax)
    outs = kern["outs"]
    nf = sum(len(c["terms"]) for c in kern["chunks"])
    c0, c1 = kern["chunks"][0], kern["chunks"][-1]
    return [f"// outputs {outs[0]}..{outs[-1]} (degree {kern['lo']}..{sum(mono[outs[-1]])}), multipole terms "
            f"{c0['mb']}..{c1['me'] - 1}: {len(outs)} accumulators, {len(kern['temps'])} per-pair sums, "
            f"{nf} multiply-adds per pair at order {pmax}; {'stores' if kern['first'] else 'adds to'} the outputs",
            f"__global__ void __launch_bounds__({ROWS}, {MIN_BLOCKS}) {name}(const {params} P) {{",
            f"  // per warp: 2 source-chunk buffers [32 rows][{CH // 4 + 1}] (float4){extra_smem_comment}",
            "  extern __shared__ float4 cm_smem[];",
            "  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;"]


def store_lines(kern):
    i0 = kern["outs"][0]
    L = ["  float *Lr = P.L + (size_t)A * P.lstr;"]
    for i in kern["outs"]:
        if kern["first"]:
            L.append(f"  if ({i} < P.lsize) Lr[{i}] = a{i - i0};")
        else:
            L.append(f"  if ({i} < P.lsize) Lr[{i}] += a{i - i0};")
    return L


def kernel_dmin(kern):
    return kern["lo"] + kern["chunks"][0]["emin"]


def nch_expr(kern):
    return " + ".join(f"(qmax >= {kern['lo'] + c['emin']})" for c in kern["chunks"])


def emit_cm(so, pmax, ki, kern):
    chq = CH // 4
    chb = 32 * (chq + 1)
    dq = (nterms(pmax) + 3) // 4
    i0 = kern["outs"][0]
    temps = set(kern["temps"])
    dmin = kernel_dmin(kern)
    name = f"k_m2l_cm_s{so}_p{pmax}_k{ki}"
    L = header_lines(kern, name, so, pmax, "CmParams", f" and 2 operator buffers [{dq}]")
    L.append(f"  float4 *const sbuf = cm_smem + w * {2 * chb + 2 * dq};")
    L.append(f"  float4 *const dbuf = sbuf + {2 * chb};")
    L.append(f"  const int row = blockIdx.x * {ROWS} + threadIdx.x;")
    L.append("  const int A = row < P.ncells ? P.order[row] : -1;")
    L.append("  const int la = A >= 0 ? (int)P.clevel[A] : 0;")
    for i in kern["outs"]:
        L.append(f"  float a{i - i0} = 0.f;")
    L.append("  const int mq = P.mstr >> 2;")
    L.append("  const int e1 = P.woff[blockIdx.x * 4 + w + 1];")
    L.append("  int e = P.woff[blockIdx.x * 4 + w];")
    L.append("  // the warp's steps (those with a pair in its 32 rows): the current one (staged), the next (slots")
    L.append("  // loaded a step ahead, its operator and rows staged during this step) and the step after")
    L.append(f"#define CM_SRC(ss) ((ss) >= 0 ? P.stab[(size_t)(ss) * {ROWS} + threadIdx.x] : -1)")
    L.append(f"#define CM_ORD(ss, bb) ((bb) >= 0 ? (P.otab ? min(max((int)P.otab[(size_t)(ss) * {ROWS} + threadIdx.x], "
             f"{so + 1}), P.p) : P.p) : -1)")
    L.append("  const int sc0 = e < e1 ? P.wstep[e] : -1, sn0 = e + 1 < e1 ? P.wstep[e + 1] : -1;")
    L.append("  int Bc = CM_SRC(sc0), qc = CM_ORD(sc0, Bc);")
    L.append("  unsigned cc = sc0 >= 0 ? P.sched_cls[sc0] : 0u;")
    L.append("  int Bn = CM_SRC(sn0), qn = CM_ORD(sn0, Bn);")
    L.append("  unsigned cn = sn0 >= 0 ? P.sched_cls[sn0] : 0u;")
    L.append("  int s2 = e + 2 < e1 ? P.wstep[e + 2] : -1;")
    L.append("  bool pf = false;  // the current step's operator and first chunk are staged")
    L.append("  int base = 0, dsel = 0;  // chunk buffer of the step's first chunk, operator buffer of the step")
    L.append("  for (; e < e1; e++) {")
    L.append("    const int s3 = e + 3 < e1 ? P.wstep[e + 3] : -1;")
    L.append("    const int B2 = CM_SRC(s2), q2 = CM_ORD(s2, B2);")
    L.append("    const unsigned c2 = s2 >= 0 ? P.sched_cls[s2] : 0u;")
    L.append(f"    const bool on = qc >= {dmin};")
    L.append("    const int ql = on ? qc : -1;")
    L.append("    bool pfn = false;")
    L.append("    if (__any_sync(0xffffffffu, on)) {")
    L.append("      const int qmax = (int)__reduce_max_sync(0xffffffffu, (unsigned)(on ? ql : 0));")
    L.append("      const int B = on ? Bc : -1;")
    L.append("      const int dl = on ? la - (int)P.clevel[B] : 0;")
    L.append(f"      const int nch = {nch_expr(kern)};")
    L.append(f"      const float4 *const sD = dbuf + dsel * {dq};")

    def stage_op(clsvar, qvar, bufexpr, ind):
        return [ind + "{",
                ind + f"  const float *Dsrc = P.D + (size_t){clsvar} * P.dstr;",
                ind + f"  float4 *dst = dbuf + ({bufexpr}) * {dq};",
                ind + f"  const int nq = ((({qvar}) + 1) * (({qvar}) + 2) * (({qvar}) + 3) / 6 + 3) >> 2;",
                ind + "  for (int i = lane; i < nq; i += 32) cm_cp_async16(dst + i, Dsrc + 4 * i);",
                ind + "}"]

    L.append("      if (!pf) {  // not prefetched: stage the operator and the first chunk now")
    L.extend(stage_op("cc", "qmax", "dsel", "        "))
    L.extend(stage_chunk(kern["chunks"][0], chq, chb, "base", "B", "        "))
    L.append("        cm_cp_async_commit();")
    L.append("      }")
    for i in kern["outs"]:
        if i in temps:
            L.append(f"      float t{i - i0} = 0.f;")

    def prefetch_next(ind):
        return [ind + f"const bool onn = qn >= {dmin};",
                ind + "pfn = __any_sync(0xffffffffu, onn);",
                ind + "if (pfn) {",
                ind + "  const int Bnn = onn ? Bn : -1;",
                ind + "  const int qmaxn = (int)__reduce_max_sync(0xffffffffu, (unsigned)(onn ? qn : 0));"] + \
            stage_op("cn", "qmaxn", "dsel ^ 1", ind + "  ") + \
            stage_chunk(kern["chunks"][0], chq, chb, "(base + nch) & 1", "Bnn", ind + "  ") + \
            [ind + "  cm_cp_async_commit();",
             ind + "  cm_cp_async_wait<1>();",
             ind + "} else {",
             ind + "  cm_cp_async_wait<0>();",
             ind + "}"]

    L.extend(pipeline(so, pmax, kern, chq, chb, lambda kq: f"sD[{kq}]", prefetch_next, "      "))
    for i in kern["outs"]:
        if i in temps:
            L.append(f"      a{i - i0} += t{i - i0};")
    L.append("      base = (base + nch) & 1;")
    L.append("      dsel ^= 1;")
    L.append("    }")
    L.append("    pf = pfn;")
    L.append("    Bc = Bn;")
    L.append("    qc = qn;")
    L.append("    cc = cn;")
    L.append("    Bn = B2;")
    L.append("    qn = q2;")
    L.append("    cn = c2;")
    L.append("    s2 = s3;")
    L.append("  }")
    L.append("#undef CM_SRC")
    L.append("#undef CM_ORD")
    L.append("  if (A < 0) return;")
    L.extend(store_lines(kern))
    L.append("}")
    return name, dmin, 4 * (2 * chb + 2 * dq) * 16, "\n".join(L)


def emit_tp(so, pmax, ki, kern):
    chq = CH // 4
    chb = 32 * (chq + 1)
    i0 = kern["outs"][0]
    temps = set(kern["temps"])
    dmin = kernel_dmin(kern)
    name = f"k_m2l_tp_s{so}_p{pmax}_k{ki}"
    L = header_lines(kern, name, so, pmax, "TpParams", "")
    L.append(f"  float4 *const sbuf = cm_smem + w * {2 * chb};")
    L.append(f"  const int t = blockIdx.x * {ROWS} + threadIdx.x;")
    L.append("  const bool act = t < P.ntgt;")
    L.append("  const int A = act ? (P.tgt ? P.tgt[t] : t) : -1;")
    L.append("  const int la = act ? (int)P.clevel[A] : 0;")
    L.append("  const int k0 = act ? P.off[A] : 0;")
    L.append("  const int n = act ? P.off[A + 1] - k0 : 0;")
    L.append("  const int nmax = (int)__reduce_max_sync(0xffffffffu, (unsigned)n);")
    for i in kern["outs"]:
        L.append(f"  float a{i - i0} = 0.f;")
    L.append("  const int mq = P.mstr >> 2;")
    L.append("  // a lane's pairs (by descending order when orders are per pair): the current one (staged), the")
    L.append("  // next (slots loaded a pair ahead, its row staged during this pair) and the list index of the one after")
    L.append("#define TP_PAIR(jj) ((jj) < n ? (P.perm ? P.perm[k0 + (jj)] : k0 + (jj)) : -1)")
    L.append(f"#define TP_ORD(kk) ((kk) >= 0 ? (P.ord ? min(max((int)P.ord[kk], {so + 1}), P.p) : P.p) : -1)")
    L.append("  const int kc0 = TP_PAIR(0);")
    L.append("  int Bc = kc0 >= 0 ? P.src[kc0] : -1, qc = TP_ORD(kc0), cc = kc0 >= 0 ? P.cls[kc0] : 0;")
    L.append("  const int kn0 = TP_PAIR(1);")
    L.append("  int Bn = kn0 >= 0 ? P.src[kn0] : -1, qn = TP_ORD(kn0), cn = kn0 >= 0 ? P.cls[kn0] : 0;")
    L.append("  int k2 = TP_PAIR(2);")
    L.append("  bool pf = false;  // the current pair's first chunk is staged")
    L.append("  int base = 0;")
    L.append("  for (int j = 0; j < nmax; j++) {")
    L.append("    const int k3 = TP_PAIR(j + 3);")
    L.append("    const int B2 = k2 >= 0 ? P.src[k2] : -1, q2 = TP_ORD(k2), c2 = k2 >= 0 ? P.cls[k2] : 0;")
    L.append(f"    const bool on = qc >= {dmin};")
    L.append("    // no lane has terms here: with pairs by descending order none has any further on")
    L.append("    if (!__any_sync(0xffffffffu, on)) break;")
    L.append("    const int ql = on ? qc : -1;")
    L.append("    const int qmax = (int)__reduce_max_sync(0xffffffffu, (unsigned)(on ? ql : 0));")
    L.append("    const int B = on ? Bc : -1;")
    L.append("    const int dl = on ? la - (int)P.clevel[B] : 0;")
    L.append("    const float *__restrict__ Dp = P.D + (size_t)(on ? cc : 0) * P.dstr;")
    L.append(f"    const int nch = {nch_expr(kern)};")
    L.append("    bool pfn = false;")
    L.append("    if (!pf) {")
    L.extend(stage_chunk(kern["chunks"][0], chq, chb, "base", "B", "      "))
    L.append("      cm_cp_async_commit();")
    L.append("    }")
    for i in kern["outs"]:
        if i in temps:
            L.append(f"    float t{i - i0} = 0.f;")

    def prefetch_next(ind):
        return [ind + f"const bool onn = qn >= {dmin};",
                ind + "pfn = __any_sync(0xffffffffu, onn);",
                ind + "if (pfn) {",
                ind + "  const int Bnn = onn ? Bn : -1;"] + \
            stage_chunk(kern["chunks"][0], chq, chb, "(base + nch) & 1", "Bnn", ind + "  ") + \
            [ind + "  cm_cp_async_commit();",
             ind + "  cm_cp_async_wait<1>();",
             ind + "} else {",
             ind + "  cm_cp_async_wait<0>();",
             ind + "}"]

    L.extend(pipeline(so, pmax, kern, chq, chb, lambda kq: f"__ldg((const float4 *)(Dp + {4 * kq}))",
                      prefetch_next, "    ", TP_PREFETCH_QUADS))
    for i in kern["outs"]:
        if i in temps:
            L.append(f"    a{i - i0} += t{i - i0};")
    L.append("    base = (base + nch) & 1;")
    L.append("    pf = pfn;")
    L.append("    Bc = Bn;")
    L.append("    qc = qn;")
    L.append("    cc = cn;")
    L.append("    Bn = B2;")
    L.append("    qn = q2;")
    L.append("    cn = c2;")
    L.append("    k2 = k3;")
    L.append("  }")
    L.append("#undef TP_PAIR")
    L.append("#undef TP_ORD")
    L.append("  if (!act) return;")
    L.extend(store_lines(kern))
    L.append("}")
    return name, dmin, 4 * 2 * chb * 16, "\n".join(L)


def launcher(fname, params, so, pmax, table, grid):
    L = [f"int {fname}(const {params} &P, cudaStream_t st) {{",
         f"  if (P.p > {pmax} || P.p < {so + 1} || (P.mstr & 3) || (P.dstr & 3)) return FMM_ERR_ARG;",
         f"  const unsigned grid = (unsigned)(({grid} + {ROWS - 1}) / {ROWS});",
         "  if (grid == 0) return FMM_OK;"]
    for name, dmin, smem in table:
        L.append(f"  if (P.p >= {dmin}) {{")
        L.append(f"    FMM_CUDA_TRY(cudaFuncSetAttribute({name}, cudaFuncAttributeMaxDynamicSharedMemorySize, {smem}));")
        L.append(f"    fmm_note_launch(), {name}<<<grid, {ROWS}, {smem}, st>>>(P);")
        L.append("    FMM_CUDA_TRY(cudaGetLastError());")
        L.append("  }")
    L.append("  return FMM_OK;")
    L.append("}")
    return L


def generate_family(so, pmax):
    kernels = plan(so, pmax)
    out = os.path.join(CSRC, family_file(so, pmax))
    parts = [f"// {family_file(so, pmax)} -- generated by fmmgen_gb300/gen_m2l_cm.py; do not edit.",
             f"// FP32 M2L kernels, source order {so}, orders {so + 1}..{pmax}: class-major (k_m2l_cm_*) and",
             "// target-major (k_m2l_tp_*) schedules of the same kernel bodies.",
             '#include "m2l_cm.cuh"', ""]
    tcm, ttp = [], []
    for ki, kern in enumerate(kernels):
        name, dmin, smem, code = emit_cm(so, pmax, ki, kern)
        parts += [code, ""]
        tcm.append((name, dmin, smem))
        name, dmin, smem, code = emit_tp(so, pmax, ki, kern)
        parts += [code, ""]
        ttp.append((name, dmin, smem))
    parts += launcher(f"fmm_m2l_cm_s{so}_p{pmax}", "CmParams", so, pmax, tcm, "P.ncells") + [""]
    parts += launcher(f"fmm_m2l_tp_s{so}_p{pmax}", "TpParams", so, pmax, ttp, "P.ntgt")
    with open(out, "w") as f:
        f.write("\n".join(parts) + "\n")
    return out


HEADER = """// m2l_cm.cuh -- generated by fmmgen_gb300/gen_m2l_cm.py; do not edit.
// FP32 M2L kernels for every order up to a family's largest (m2l_cm_s*.cu):
// parameters and launchers.  Outputs are written, not accumulated.
#pragma once
#include "internal.h"

// class-major schedule: the tiles of the tensor-core class-step schedule
struct CmParams {
  const int *woff;              // [4 ntiles + 1] first entry of each (tile, warp) in wstep
  const int *wstep;             // steps with a pair in the warp's 32 rows, per (tile, warp), increasing
  const unsigned *sched_cls;    // [steps] class of each step
  const int *stab;              // [steps][128] source cell of each row, -1 without a pair
  const unsigned char *otab;    // [steps][128] per-pair order, or null: every pair at order p
  const int *order;             // [ncells] rows -> cells (M2L processing order)
  int ncells, p;
  const float *D;               // [classes][dstr] FP32 class operators
  int dstr;
  const unsigned char *clevel;  // [ncells] level of each cell
  const float *M;               // [ncells][mstr] scaled multipoles (degrees >= source order)
  int mstr;
  float *L;                     // [ncells][lstr] scaled locals
  int lstr, lsize;
};

// target-major schedule: a thread per target cell over its target list
struct TpParams {
  const int *tgt;               // [ntgt] target cells (null: cells 0 .. ntgt - 1)
  int ntgt;
  const int *off, *src, *cls;   // target lists: pairs of cell A are off[A] .. off[A + 1] - 1
  const int *perm;              // pair indices of each list by descending order, or null (list order)
  const unsigned char *ord;     // per-pair orders (list order, needs perm), or null: every pair at order p
  int p;
  const float *D;
  int dstr;
  const unsigned char *clevel;
  const float *M;
  int mstr;
  float *L;
  int lstr, lsize;
};

static __device__ __forceinline__ void cm_cp_async16(void *dst, const void *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\\n" :: "r"(d), "l"(src) : "memory");
}
static __device__ __forceinline__ void cm_cp_async_commit() { asm volatile("cp.async.commit_group;\\n" ::: "memory"); }
template <int N> static __device__ __forceinline__ void cm_cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\\n" :: "n"(N) : "memory");
}

"""


def generate():
    outs = []
    decl = []
    for so, pmax in FAMILIES:
        outs.append(generate_family(so, pmax))
        decl.append(f"int fmm_m2l_cm_s{so}_p{pmax}(const CmParams &P, cudaStream_t st);  // orders {so + 1}..{pmax}")
        decl.append(f"int fmm_m2l_tp_s{so}_p{pmax}(const TpParams &P, cudaStream_t st);")
    fams = sorted(FAMILIES, key=lambda f: (f[0], f[1]))
    table = ["// largest order of the families of each source order (0: none)",
             "static inline int fmm_m2l_cm_pmax(int so) {"]
    for so in sorted({f[0] for f in fams}):
        table.append(f"  if (so == {so}) return {max(pm for s_, pm in fams if s_ == so)};")
    table += ["  return 0;", "}"]
    for kind, params in (("cm", "CmParams"), ("tp", "TpParams")):
        table += [f"// launch the family of source order so with the smallest largest order >= P.p (FMM_ERR_STATE: none)",
                  f"static inline int fmm_m2l_{kind}_launch(int so, const {params} &P, cudaStream_t st) {{"]
        for so, pmax in fams:
            table.append(f"  if (so == {so} && P.p <= {pmax}) return fmm_m2l_{kind}_s{so}_p{pmax}(P, st);")
        table += ["  return FMM_ERR_STATE;", "}"]
    hdr = os.path.join(CSRC, "m2l_cm.cuh")
    with open(hdr, "w") as f:
        f.write(HEADER + "\n".join(decl) + "\n" + "\n".join(table) + "\n")
    outs.append(hdr)
    # generated files of families no longer listed
    keep = {family_file(so, pm) for so, pm in FAMILIES}
    for fn in os.listdir(CSRC):
        if fn.startswith("m2l_cm_s") and fn.endswith(".cu") and fn not in keep:
            os.remove(os.path.join(CSRC, fn))
    return outs


if __name__ == "__main__":
    for o in generate():
        print(o)
