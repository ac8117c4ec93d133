#!/usr/bin/env python
"""Benchmark of the octree FMM evaluation path on GB300.

Workload (one "step"): the full FMM -- device octree + interaction lists +
P2M/M2M/M2L/P2P/L2L/L2P -- of N = 1,000,000 Coulomb charges, positions i.i.d.
uniform in [0,1]^3 and charges uniform in [-1,1] (seeded synthetic data),
expansion order p = 8, ncrit = 128, theta = 0.5, field output, mixed precision.
`value` is particles/s with inputs resident in HBM; `e2e` is the same step
through the public API from pinned host buffers, copies included.  The plain
FP64 GPU FMM is timed beside it, and the field error of both against an FP64
direct sum on a 10,000-particle subset is reported.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--config NAME]

--config selects another configuration of the same path (10^4 charges at p=4;
2x10^6 Plummer dipoles at p=6; 4096 independent systems of 1,000-65,536
charges, log-uniform sizes, p=6, solved as one forest per step; 8x10^6
clustered charges at p_max=12 with learned per-pair M2L orders, the fixed
p=12 pass timed beside it); the default is the headline above.

Multi-GPU: the path is replicated (independent systems per rank, no collective
on the data path); `value` is the job total.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particles/s full FMM, N=1M p=8 at 1e-6 rel field err: mixed/learned vs FP64"
UNIT = "particles/s"


# name -> (N, order, ncrit, theta, source_order, distribution, potential, field)
CONFIGS = {
    # the headline: 1e6 uniform charges, p=8 (Nterms=165), field output
    "uniform_1m_p8": (1_000_000, 8, 128, 0.5, 0, "uniform", False, True),
    # the reference's CPU-runnable case: 1e4 uniform charges, p=4, potential and field
    "uniform_10k_p4": (10_000, 4, 64, 0.5, 0, "uniform", True, True),
    # 2e6 dipoles in a Plummer sphere (scale 0.1, truncated at radius 1), p=6, potential and field
    "plummer_dipole_2m_p6": (2_000_000, 6, 64, 0.5, 1, "plummer", True, True),
    # 4096 independent systems, sizes log-uniform in [1000, 65536], each uniform in its own unit cube,
    # p=6, field output; N is the sum of the sizes
    "batched_4096_p6": (0, 6, 64, 0.5, 0, "batched", False, True),
    # learned per-pair M2L orders: 8e6 charges, half uniform in the unit cube and half in 64 Gaussian
    # clusters (sigma 0.01), p_max=12, field output; the committed order model picks each pair's order
    "learned_8m_p12": (8_000_000, 12, 128, 0.5, 0, "mixture", False, True),
}
NSYS_BATCHED = 4096


def batched_sizes(nsys, seed):
    """Seeded system sizes, log-uniform in [1000, 65536]."""
    rng = np.random.default_rng(seed + 7919)
    return np.floor(np.exp(rng.uniform(np.log(1000.0), np.log(65536.0), nsys))).astype(np.int64)


def args_parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--config", choices=sorted(CONFIGS), default="uniform_1m_p8")
    ap.add_argument("--n", type=int, default=None, help="override the configuration's particle count")
    ap.add_argument("--order", type=int, default=None)
    ap.add_argument("--ncrit", type=int, default=None)
    ap.add_argument("--theta", type=float, default=None)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--nsys", type=int, default=NSYS_BATCHED, help="systems of the batched configuration")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default M2L rules (no autotuner run)")
    ap.add_argument("--tune", default=None,
                    help="impl,nslots,grouping,overlap: set the M2L choice instead of running the autotuner")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--cpu-stride", type=int, default=1,
                    help="CPU baseline evaluates every k-th target cell and scales (1: the full pass, the default)")
    ap.add_argument("--profile-only", action="store_true",
                    help="run warmup + timed steps only (no e2e, FP64, direct sum, CPU baseline): for ncu captures")
    a = ap.parse_args()
    n, order, ncrit, theta, so, dist, pot, fld = CONFIGS[a.config]
    a.sizes = None
    if dist == "batched":
        a.sizes = batched_sizes(a.nsys, a.seed)
        n = int(a.sizes.sum())
    a.n = a.n or n
    a.order = a.order or order
    a.ncrit = a.ncrit or ncrit
    a.theta = a.theta or theta
    a.so, a.dist, a.potential, a.field = so, dist, pot, fld
    a.outsize = (1 if pot else 0) + (3 if fld else 0)
    return a


def metric_name(a):
    if a.config == "uniform_1m_p8" and a.n == 1_000_000:
        return METRIC
    return f"particles/s full FMM, {a.config} (N={a.n})"


def max_over_ranks(x, pg=None, device=None):
    """The job's time: the largest of the ranks' times (replicas run side by side)."""
    if pg is None:
        return x
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return t.item()


def job_throughput(n_per_rank, steps, world, t_max_ms):
    """Particles per second of the whole job: every rank's particles over the
    slowest rank's time."""
    return n_per_rank * steps * world / (t_max_ms / 1e3)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def plummer(rng, n, a=0.1, rmax=1.0):
    """Plummer sphere of scale a truncated at rmax: r = a / sqrt(u^(-2/3) - 1), isotropic directions."""
    out, have = [], 0
    while have < n:
        u = rng.uniform(0.0, 1.0, 2 * (n - have) + 16)
        r = a / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
        r = r[r <= rmax]
        v = rng.standard_normal((len(r), 3))
        v /= np.linalg.norm(v, axis=1, keepdims=True)
        out.append(v * r[:, None])
        have += len(r)
    return np.concatenate(out)[:n]


def mixture(n, seed, nclusters=64, sigma=0.01):
    """Half uniform in the unit cube, half in nclusters isotropic Gaussian
    clusters with centres uniform in the cube (the order model's training
    distribution, fmmgen_gb300.learned.mixture_positions)."""
    rng = np.random.default_rng(seed)
    nu = n // 2
    centres = rng.uniform(0, 1, (nclusters, 3))
    which = rng.integers(0, nclusters, n - nu)
    return np.concatenate([rng.uniform(0, 1, (nu, 3)), centres[which] + sigma * rng.standard_normal((n - nu, 3))])


def workload(a, seed):
    """Seeded synthetic inputs of the configuration's shape (no dataset is involved)."""
    rng = np.random.default_rng(seed)
    if a.dist == "plummer":
        pos = plummer(rng, a.n)
    elif a.dist == "mixture":
        pos = mixture(a.n, seed + 104729)
    else:  # uniform; for the batched configuration each system in its own unit cube
        pos = rng.uniform(0.0, 1.0, (a.n, 3))
    if a.so == 0:
        S = rng.uniform(-1.0, 1.0, (a.n, 1))
    else:
        S = rng.standard_normal((a.n, 3))
    return pos, S


def config(a, world):
    kind = "Coulomb charges" if a.so == 0 else "dipoles"
    where = {"uniform": "uniform in the unit cube", "plummer": "in a Plummer sphere (a=0.1, r<=1)",
             "mixture": "half uniform in the unit cube, half in 64 Gaussian clusters (sigma=0.01)",
             "batched": f"in {len(a.sizes) if a.sizes is not None else 0} independent systems (sizes log-uniform "
                        f"in [1000, 65536], each uniform in its own unit cube), one forest"}[a.dist]
    out = "+".join(x for x, f in (("potential", a.potential), ("field", a.field)) if f)
    orders = (f"p_max={a.order} with learned per-pair M2L orders (MLP 16-64-64-11, features + inference in "
              f"every pass)" if a.dist == "mixture" else f"p={a.order}")
    return {"workload": f"octree FMM, {a.n} {kind} {where}, {orders}, ncrit={a.ncrit}, theta={a.theta}, "
                        f"{out} output, tree+lists+evaluation per step",
            "name": a.config, "N": a.n, "order": a.order, "ncrit": a.ncrit, "theta": a.theta, "source_order": a.so,
            "precision": "mixed (FP32 sweeps/M2L/P2P, FP64 operator assembly and final accumulation)",
            "l2": "flushed between timed steps (512 MB write)", "parallelism": f"replicas x{world}"}


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.gpu)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU baseline: the checker's restatement of the reference path on host cores
# ---------------------------------------------------------------------------
def sys_offsets(a):
    return np.concatenate([[0], np.cumsum(a.sizes)]).astype(np.int64)


def sampled_systems(a, k):
    return np.unique(np.linspace(0, len(a.sizes) - 1, k).astype(np.int64))


def cpu_sample(pos, q, a, stride):
    from oracle import oracle as orc

    if a.sizes is not None:
        # batched: the full build and evaluation of a spread of the systems, one at a time
        off = sys_offsets(a)
        tot_n, tot_t = 0, 0.0
        idx = sampled_systems(a, 8)
        for k in idx:
            sl = slice(off[k], off[k + 1])
            t0 = time.perf_counter()
            ot = orc.OracleTree(pos[sl], q[sl], a.ncrit, a.order, a.theta, a.so)
            t_build = time.perf_counter() - t0
            _, ph = ot.evaluate(potential=a.potential, field=a.field, sample_stride=1)
            tot_n += int(a.sizes[k])
            tot_t += t_build + float(np.sum(ph))
        sample = (f"oracle port (C, OpenMP) on this host: full tree build and evaluation of {len(idx)} of "
                  f"{len(a.sizes)} systems one after another ({tot_n} particles)")
        return tot_n / tot_t, tot_t * a.n / tot_n, sample, orc.num_threads()
    if a.n <= 100_000:
        stride = 1  # small systems run in full
    t0 = time.perf_counter()
    ot = orc.OracleTree(pos, q, a.ncrit, a.order, a.theta, a.so)
    t_build = time.perf_counter() - t0
    _, ph = ot.evaluate(potential=a.potential, field=a.field, sample_stride=stride)
    p2m, m2m, m2l, p2p, l2l, l2p = ph.tolist()
    t_full = t_build + p2m + m2m + l2l + stride * (m2l + p2p + l2p)
    if stride == 1:
        sample = f"oracle port (C, OpenMP) on this host: the full tree build and evaluation, N={a.n}"
    else:
        sample = (f"oracle port (C, OpenMP) on this host: full tree build, P2M, M2M, L2L; M2L, P2P, L2P on every "
                  f"{stride}-th target cell, scaled by {stride}; N={a.n}")
    return a.n / t_full, t_full, sample, orc.num_threads()


def run_reference(a, rank, world):
    """--impl reference: the reference path's CPU implementation on host cores."""
    if rank != 0:
        return
    import subprocess as sp

    sp.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle")])
    pos, q = workload(a, a.seed)
    # every step is the whole workload: tree build and the full evaluation
    # (stride 1, nothing sampled or scaled), timed on the wall clock
    for _ in range(a.warmup):
        cpu_sample(pos, q, a, 1)
    t0 = time.perf_counter()
    est = 0.0
    for _ in range(a.steps):
        ts = time.perf_counter()
        v, t_full, sample, cores = cpu_sample(pos, q, a, 1)
        est += time.perf_counter() - ts
    wall = time.perf_counter() - t0
    value = a.n * a.steps / est
    line = {"impl": "reference", "metric": metric_name(a), "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": 1e3 * est / a.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "config": config(a, world),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": wall}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def main():
    a = args_parse()
    rank, world, local = dist_env()
    if a.impl == "reference":
        run_reference(a, rank, world)
        return
    import torch

    import fmmgen_gb300 as fg
    from fmmgen_gb300 import build as fbuild

    if not os.path.exists(fbuild.LIB) and rank == 0:
        fbuild.build()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
        pg = dist
        dist.barrier()

    def barrier():
        if pg:
            pg.barrier()

    pos_np, q_np = workload(a, a.seed + rank)
    pos = torch.tensor(pos_np, device=dev)
    q = torch.tensor(q_np, device=dev)
    st = torch.cuda.current_stream()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    F = torch.empty((a.n, a.outsize), dtype=torch.float64, device=dev)
    L = fg.lib()

    tree = fg.Tree(pos, q, a.ncrit, a.order, a.theta, source_order=a.so,
                   sys_off=sys_offsets(a) if a.sizes is not None else None)
    autotune = None
    if a.tune:
        impl, nslots, grouping, overlap = (int(v) for v in a.tune.split(","))
        tree.set_tune(impl, nslots, grouping, overlap)
        autotune = {"chosen": tree.get_tune(), "candidates_ms": None, "legend": "set with --tune"}
    elif not a.no_autotune and a.dist != "mixture":
        # the M2L autotuner, once before the warm-up (outside every timed region)
        r = tree.autotune(precision="mixed", reps=3)
        autotune = {"chosen": r["best"], "candidates_ms": [
            [c["impl"], c["nslots"], c["grouping"], c["overlap"], round(c["ms"], 3)] for c in r["table"]],
            "legend": "impl 0 tensor cores (row gather) / 1 generated CUDA-core / 2 contraction engine / 3 tensor cores "
                      "(level-grid boxes) / 4 generated class-major / 5 generated target-major; nslots = tensor-core "
                      "pipeline depth; grouping 0 by octant / 1 Morton; overlap 1 / 2 = M2L and P2P side by side "
                      "(P2P blocks of 4 / 2 warps); "
                      "M2L + P2P median ms"}
    model = None
    if a.dist == "mixture":  # learned per-pair M2L orders: every pass predicts them from its multipoles
        from fmmgen_gb300 import learned

        model = learned.OrderModel.load()
        model.attach(tree)

    def step(precision="mixed"):
        # the build and the evaluation in one call (fmmgen_tree_build_compute)
        tree.rebuild_compute(pos, F, potential=a.potential, field=a.field, precision=precision)

    phase_sum = {}

    def timed(nsteps, fn, collect_phases=False):
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nsteps)]
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(nsteps):
            flush.fill_(float(i))
            evs[i][0].record(st)
            fn()
            evs[i][1].record(st)
            if collect_phases:
                torch.cuda.synchronize()
                b, e = tree.times()
                for k, v in list(b.items()) + list(e.items()):
                    key = ("build_" if k in b and k not in e else "") + k
                    phase_sum[key] = phase_sum.get(key, 0.0) + v
                for k, v in tree.kernel_ms().items():  # the kernels alone, events around their launches
                    phase_sum["kernel_" + k] = phase_sum.get("kernel_" + k, 0.0) + v
        torch.cuda.synchronize()
        barrier()
        wall = time.perf_counter() - t0
        dev_ms = sum(s.elapsed_time(e) for s, e in evs)
        return dev_ms, wall

    # ---- device-resident value (mixed) ----
    for _ in range(a.warmup):
        step()
    n0 = L.fmmgen_launch_count()
    with ClockSampler(local) as clk:
        dev_ms, wall = timed(a.steps, step, collect_phases=True)
    launches = L.fmmgen_launch_count() - n0
    m2l_steps, m2l_mmas, m2l_exec_flops, m2l_boxes = tree.m2l_work()  # of the last timed (mixed) step
    m2l_orders = tree.m2l_orders() if model is not None else None
    t_max = max_over_ranks(dev_ms, pg, dev)
    value = job_throughput(a.n, a.steps, world, t_max)
    ms_per_step = t_max / a.steps
    # ---- eval-only (the reference's timed region, example/main.cpp:154-162): the tree is
    # built once, then the evaluation pass is replayed from its recorded CUDA graph ----
    tree.rebuild(pos)
    tree.set_graph(True)
    tree.compute_field_fmm(F, potential=a.potential, field=a.field, precision="mixed")  # runs, then records
    eval_ms, _ = timed(a.steps, lambda: tree.compute_field_fmm(F, potential=a.potential, field=a.field,
                                                                  precision="mixed"))
    tree.set_graph(False)
    eval_max = max_over_ranks(eval_ms, pg, dev)
    eval_only = {"value": job_throughput(a.n, a.steps, world, eval_max), "unit": UNIT, "ms_per_step": eval_max / a.steps,
                 "note": "P2M..L2P only, tree built once; the pass is replayed from its recorded CUDA graph"}
    if a.profile_only:
        if rank == 0:
            print(json.dumps({"profile_only": True, "value": value, "unit": UNIT, "ms_per_step": ms_per_step,
                              "gpu_launches": launches}), flush=True)
        return

    # ---- e2e through the public API from pinned host memory: a stream of steps
    # (fmmgen_gb300.stream_compute), every step copying its inputs in and its
    # outputs out, the copies of one step overlapped with its neighbours' work ----
    from fmmgen_gb300.pipeline import StepBuffers

    k_e2e = max(3, a.steps // 2)
    pos_h = [torch.tensor(pos_np).pin_memory() for _ in range(2)]
    q_h = [torch.tensor(q_np).pin_memory() for _ in range(2)]
    F_h = [torch.empty((a.n, a.outsize), dtype=torch.float64).pin_memory() for _ in range(2)]
    bufs = StepBuffers(a.n, q_np.shape[1], a.outsize, dev)
    seq = lambda xs, k: [xs[i % 2] for i in range(k)]  # noqa: E731  (host arrays reused every other step)
    fg.stream_compute(tree, seq(pos_h, 2), seq(q_h, 2), seq(F_h, 2), a.potential, a.field, "mixed", bufs)
    flush.fill_(0.0)
    barrier()
    e2e_ms = fg.stream_compute(tree, seq(pos_h, k_e2e), seq(q_h, k_e2e), seq(F_h, k_e2e), a.potential, a.field,
                               "mixed", bufs, timing=True)
    barrier()
    e2e_max = max_over_ranks(e2e_ms, pg, dev)
    e2e_value = job_throughput(a.n, k_e2e, world, e2e_max)
    h2d = pos_h[0].numel() * 8 + q_h[0].numel() * 8
    d2h = F_h[0].numel() * 8
    del bufs
    tree.rebuild(pos)
    tree.S = q

    # ---- accuracy vs FP64 direct sum, and the plain FP64 GPU FMM ----
    if a.sizes is None:
        tg = torch.arange(0, a.n, max(1, a.n // 10000), device=dev)[:10000]
        Fd = fg.direct(pos, q, targets=tg, source_order=a.so, potential=False, field=True)

        def err(Fx):
            E = Fx[tg][:, -3:]  # the field columns, whether or not the potential is output too
            return (torch.linalg.norm(E - Fd) / torch.linalg.norm(Fd)).item()
    else:
        # batched: each sampled system against its own FP64 direct sum on up to 1,000 of its particles
        off = sys_offsets(a)
        checks = []
        for k in sampled_systems(a, 64):
            b0, b1 = int(off[k]), int(off[k + 1])
            tl = torch.arange(0, b1 - b0, max(1, (b1 - b0) // 1000), device=dev)[:1000]
            Fs = fg.direct(pos[b0:b1], q[b0:b1], targets=tl, source_order=a.so, potential=False, field=True)
            checks.append((b0, tl, Fs))

        def err(Fx):
            e = [(torch.linalg.norm(Fx[b0 + tl][:, -3:] - Fs) / torch.linalg.norm(Fs)).item() for b0, tl, Fs in checks]
            return max(e)

    step("mixed")
    err_mixed = err(F)
    learned_info = None
    if model is not None:
        # the fixed-order fallback (p_max for every pair) timed and checked beside the learned pass
        tree.set_order_model(None)
        step("mixed")
        err_fixed = err(F)
        msf, _ = timed(2, lambda: step("mixed"), collect_phases=False)
        _, ef = tree.times()
        from fmmgen_gb300 import learned

        terms = learned.m2l_terms(m2l_orders, a.so)
        terms_fixed = tree.nm2l * learned.pair_terms(a.order, a.so)
        learned_info = {"delta": model.delta, "m2l_multiply_adds": terms, "m2l_multiply_adds_fixed": terms_fixed,
                        "order_histogram": {int(k): int(v) for k, v in
                                            zip(*np.unique(m2l_orders, return_counts=True))},
                        "fixed_pmax": {"value": a.n * 2 / (msf / 1e3), "ms_per_step": msf / 2,
                                       "rel_field_err": err_fixed, "m2l_ms": ef.get("M2L")},
                        "model": os.path.relpath(learned.MODEL_PATH, ROOT)}
        model.attach(tree)
    fp64 = {}
    if not a.no_fp64:
        step("fp64")
        err_fp64 = err(F)
        k64 = 2
        ms64, _ = timed(k64, lambda: step("fp64"))
        fp64 = {"value": a.n * k64 / (ms64 / 1e3), "ms_per_step": ms64 / k64, "rel_field_err": err_fp64}
        _, e64 = tree.times()
        fp64["phases_ms"] = {k: round(v, 3) for k, v in e64.items()}

    # ---- roofline of the dominant kernel (live CUDA-event phase times) ----
    ph = {k: v / a.steps for k, v in phase_sum.items()}
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    sm_max = peaks.get("sm_max_mhz", 2070.0)
    fp32_peak = 152 * 128 * 2 * sm_max * 1e6 / 1e12  # TFLOP/s, nominal at the max SM clock
    p2p_flops = (20.0 if a.so == 0 else 38.0) * tree.p2p_interactions
    m2l_flops = 2.0 * math.comb(a.order + 6, 6) * tree.nm2l
    if learned_info:
        m2l_flops = 2.0 * learned_info["m2l_multiply_adds"]  # at each pair's own order
    # each kernel's own device time (events on its stream around its launches; the M2L phase also holds
    # its schedule and operand preparation), the phase time where a kernel was not timed
    def ktime(k):
        v = ph.get("kernel_" + k, -1.0)
        return v if v > 0 else ph.get(k, 0.0)

    cand = {"P2P": (ktime("P2P"), p2p_flops), "M2L": (ktime("M2L"), m2l_flops)}
    dom = max(cand, key=lambda k: cand[k][0])
    dom_ms, dom_flops = cand[dom]
    traffic, traffic_current = None, None
    if a.config == "uniform_1m_p8" and a.n == 1_000_000:  # the workload the ncu capture ran
        try:
            import hashlib

            for ln in open(os.path.join(ROOT, "profiles", "dram_traffic_uniform_1m_p8.txt")):
                f = ln.split()
                if len(f) == 4 and not ln.startswith("#") and f[0] == dom:
                    traffic = float(f[1])
                    # the capture describes the kernel only while its source is unchanged
                    with open(os.path.join(ROOT, f[2]), "rb") as src:
                        traffic_current = hashlib.sha256(src.read()).hexdigest()[:16] == f[3]
        except OSError:
            pass
    achieved = dom_flops / (dom_ms / 1e3) / 1e12 if dom_ms > 0 else 0.0
    roofline = {"kernel": dom, "bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                "frac": achieved / fp32_peak, "traffic": traffic, "traffic_capture_current": traffic_current,
                "kernel_ms": dom_ms, "time_source": "CUDA events on the kernel's stream around its launches, "
                                                    "mean over the timed steps (M2L and P2P may run side by side)",
                "peak_source": "nominal: 152 SMs x 128 FP32 lanes x 2 flop x sm_max_mhz of MEASURED_PEAKS.json "
                               "(no measured FP32 figure exists)",
                "work": f"{'20 flop x P2P interactions' if dom == 'P2P' else '2*C(p+6,6) flop x M2L pairs'} "
                        f"per launch = {dom_flops:.3e} flop"}
    m2l_ms, _ = cand["M2L"]
    tpeak = peaks.get("bf16_tflops")  # dense 16-bit tensor peak (FP16 runs at the bf16 rate)
    exec_tf = m2l_exec_flops / (m2l_ms / 1e3) / 1e12 if m2l_ms > 0 else 0.0
    alg_tf = m2l_flops / (m2l_ms / 1e3) / 1e12 if m2l_ms > 0 else 0.0
    tuned = tree.get_tune()["impl"]
    if m2l_steps:
        m2l_kernel = ("M2L (k_m2l_tcg, tcgen05 kind::f16, source rows boxed from level grids)" if m2l_boxes
                      else "M2L (k_m2l_tc, tcgen05 kind::f16)")
    elif learned_info:
        m2l_kernel = ("M2L (k_m2l_tp_*, generated FP32, a thread per target, each pair at its own order; the phase "
                      "includes the pairs' features and the order model's inference)")
    else:
        m2l_kernel = {1: "M2L (k_m2l_reg_*, generated FP32, a thread per target)",
                      4: "M2L (k_m2l_cm_*, generated FP32, class-major)",
                      5: "M2L (k_m2l_tp_*, generated FP32, a thread per target)",
                      2: "M2L (k_m2l_pk, FP32 contraction engine)"}.get(tuned, "M2L (CUDA cores)")
    roofline_m2l = {"kernel": m2l_kernel,
                    "bound": "tensor", "achieved": exec_tf, "algorithmic_tflops": alg_tf, "peak": tpeak,
                    "unit": "TFLOP/s", "frac": exec_tf / tpeak if tpeak else None,
                    "algorithmic_frac": alg_tf / tpeak if tpeak else None,
                    "class_steps": m2l_steps, "mma_instructions": m2l_mmas,
                    "executed_flops_per_launch": m2l_exec_flops, "algorithmic_flops_per_launch": m2l_flops,
                    "source_rows": "boxed from level grids (tensor-map copies)" if m2l_boxes else "gathered row by row",
                    "note": "executed = MMA flops issued (3 FP16 products per 16-term chunk, 1 for the chunks of "
                            "degree >= 6 in the level-grid kernel; 128-row tiles over the union of the tile's classes, "
                            "triangular N per chunk); algorithmic = 2*C(p+6,6) per pair; "
                            "peak = measured bf16 dense (MEASURED_PEAKS.json)"}

    if dom == "M2L":
        roofline["kernel"] = m2l_kernel
    if dom == "M2L" and m2l_steps and tpeak:
        # the dominant M2L ran on the tensor cores: its roofline is the measured
        # dense 16-bit tensor peak (algorithmic flops, as for every bound); the
        # FP32 CUDA-core view stays beside it
        roofline_fp32 = roofline
        roofline = {"kernel": roofline_m2l["kernel"], "bound": "tensor", "achieved": alg_tf, "peak": tpeak,
                    "unit": "TFLOP/s", "frac": alg_tf / tpeak, "traffic": traffic,
                    "traffic_capture_current": traffic_current, "kernel_ms": m2l_ms,
                    "time_source": roofline_fp32["time_source"],
                    "peak_source": "measured bf16 dense burst (MEASURED_PEAKS.json bf16_tflops)",
                    "work": roofline_fp32["work"], "executed_achieved": exec_tf, "executed_frac": exec_tf / tpeak,
                    "fp32_view": {k: roofline_fp32[k] for k in ("achieved", "peak", "frac", "peak_source")}}

    line = {"metric": metric_name(a), "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64", "data": "synthetic (seeded positions and sources)",
            "config": config(a, world), "rel_field_err": err_mixed,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches, "eval_only": eval_only, "roofline": roofline, "roofline_m2l": roofline_m2l,
            "fp64_plain": fp64, "speedup_vs_fp64": (value / world) / fp64["value"] if fp64 else None,
            "learned_orders": learned_info, "m2l_autotune": autotune,
            "phases_ms": {k: round(v, 3) for k, v in ph.items()},
            "tree": {"cells": tree.ncells, "leaves": tree.nleaves, "m2l_pairs": tree.nm2l, "p2p_pairs": tree.np2p,
                     "p2p_interactions": tree.p2p_interactions, "m2l_classes": tree.nclasses},
            "clocks": clk.summary(), "wall_s": wall}
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        v, t_full, sample, cores = cpu_sample(pos_np, q_np, a, a.cpu_stride)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg:
        pg.barrier()
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
