"""Write the golden fixtures in tests/golden/ from the reference itself.

Run in the development container after `python oracle/ref/build_ref.py`:
    python tests/golden/make_golden.py
The values come from the reference's own code: fmmgen's generated operators
(P2M/M2M/M2L/L2L/L2P at every order) and the example's build_tree /
interact_dehnen_lazy / compute_field_fmm, linked by oracle/ref/ref_harness.cpp.
The one restated piece is P2P (the generated field is zero at HEAD); its
potential is checked against the generated P2P here before anything is saved.
Barnes-Hut fixtures (compute_field_bh, M2P) keep potentials only: the
generated M2P's field is not the gradient of its potential.
`--bh` writes only the Barnes-Hut fixtures; `--so2` only the quadrupole-source
fixtures (ops_so2.npz, tree_quadrupole_plummer.npz, m2p_potential_so2.npz).
`--trees a,b` writes only the named tree fixtures.
`--f32` (after `build_ref.py --float`) writes ops_f32_so{0,1,2}.npz: the outputs
of the reference's precision="float" operators on the inputs of ops_so*.npz
rounded to float32 -- the accuracy the FP32 variant is held to.
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import oracle as O  # noqa: E402


def list_digest(pairs):
    """SHA-256 of the sorted pair multiset (rows of uint64)."""
    a = np.ascontiguousarray(pairs, dtype=np.uint64).reshape(-1, 2)
    order = np.lexsort((a[:, 1], a[:, 0]))
    return hashlib.sha256(a[order].tobytes()).hexdigest()


def make_ops(specs=((0, (1, 8)), (1, (2, 6))), seed=2024):
    rng = np.random.default_rng(seed)
    for so, (pmin, pmax) in specs:
        R = O.ref(so)
        out = {}
        K = 6
        for p in range(pmin, pmax + 1):
            ms, ls = O.msize(p, so), O.lsize(p, so)
            d = rng.uniform(-1, 1, (K, 3))
            d *= rng.uniform(1.0, 3.0, (K, 1)) / np.linalg.norm(d, axis=1, keepdims=True)
            q = rng.uniform(-1, 1, K)
            Min = rng.standard_normal((K, ms))
            Lin = rng.standard_normal((K, ls))
            res = {k: [] for k in ("P2M", "M2M", "M2L", "L2L", "L2P")}
            for i in range(K):
                a = np.zeros(ms); R.ref_P2M(*d[i], q[i], a, p); res["P2M"].append(a)
                a = np.zeros(ms); R.ref_M2M(*d[i], Min[i].copy(), a, p); res["M2M"].append(a)
                a = np.zeros(ls); R.ref_M2L(*d[i], Min[i].copy(), a, p); res["M2L"].append(a)
                a = np.zeros(ls); R.ref_L2L(*d[i], Lin[i].copy(), a, p); res["L2L"].append(a)
                a = np.zeros(4); R.ref_L2P(*d[i], Lin[i].copy(), a, p); res["L2P"].append(a)
            out[f"p{p}_d"] = d
            out[f"p{p}_q"] = q
            out[f"p{p}_M"] = Min
            out[f"p{p}_L"] = Lin
            for k, v in res.items():
                out[f"p{p}_{k}"] = np.array(v)
        # P2P: restated physics; its potential must equal the generated P2P's
        ss = O.sourcesize(so)
        d = rng.uniform(-1, 1, (16, 3))
        S = rng.standard_normal((16, ss))
        Fr = np.zeros((16, 4))
        Fg = np.zeros((16, 4))
        for i in range(16):
            R.ref_P2P_restated(*d[i], S[i].copy(), Fr[i])
            R.ref_P2P_generated(*d[i], S[i].copy(), Fg[i])
        assert np.allclose(Fr[:, 0], Fg[:, 0], rtol=1e-13, atol=0), "restated P2P potential != generated"
        out["p2p_d"], out["p2p_S"], out["p2p_F"], out["p2p_F_generated"] = d, S, Fr, Fg
        out["pmin"], out["pmax"] = np.int64(pmin), np.int64(pmax)
        np.savez_compressed(os.path.join(HERE, f"ops_so{so}.npz"), **out)
        print(f"ops_so{so}.npz: orders {pmin}..{pmax}")


def make_ops_f32():
    import ctypes as C

    fp = C.POINTER(C.c_float)
    for so in (0, 1, 2):
        lib = C.CDLL(os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle", "_ref", f"libref_f32_so{so}.so"))
        for nm in ("M2M", "M2L", "L2L", "L2P"):
            getattr(lib, nm).argtypes = [C.c_float] * 3 + [fp, fp, C.c_int]
        lib.P2M.argtypes = [C.c_float] * 4 + [fp, C.c_int]
        lib.P2P.argtypes = [C.c_float] * 3 + [fp, fp]

        def ptr(a):
            return a.ctypes.data_as(fp)

        g = np.load(os.path.join(HERE, f"ops_so{so}.npz"))
        pmin, pmax = int(g["pmin"]), int(g["pmax"])
        out = {"pmin": g["pmin"], "pmax": g["pmax"]}
        for p in range(pmin, pmax + 1):
            d = g[f"p{p}_d"].astype(np.float32)
            q = g[f"p{p}_q"].astype(np.float32)
            Min = g[f"p{p}_M"].astype(np.float32)
            Lin = g[f"p{p}_L"].astype(np.float32)
            K = len(d)
            ms, ls = Min.shape[1], Lin.shape[1]
            res = {k: np.zeros((K, w), np.float32) for k, w in (("P2M", ms), ("M2M", ms), ("M2L", ls), ("L2L", ls),
                                                                 ("L2P", 4))}
            for i in range(K):
                x, y, z = (float(v) for v in d[i])
                lib.P2M(x, y, z, float(q[i]), ptr(res["P2M"][i]), p)
                lib.M2M(x, y, z, ptr(Min[i].copy()), ptr(res["M2M"][i]), p)
                lib.M2L(x, y, z, ptr(Min[i].copy()), ptr(res["M2L"][i]), p)
                lib.L2L(x, y, z, ptr(Lin[i].copy()), ptr(res["L2L"][i]), p)
                lib.L2P(x, y, z, ptr(Lin[i].copy()), ptr(res["L2P"][i]), p)
            for k, v in res.items():
                out[f"p{p}_{k}"] = v
        d = g["p2p_d"].astype(np.float32)
        S = g["p2p_S"].astype(np.float32)
        F = np.zeros((len(d), 4), np.float32)
        for i in range(len(d)):
            lib.P2P(*(float(v) for v in d[i]), ptr(S[i].copy()), ptr(F[i]))
        out["p2p_phi"] = F[:, 0].copy()  # the generated P2P's field is zero; its potential is kept
        np.savez_compressed(os.path.join(HERE, f"ops_f32_so{so}.npz"), **out)
        print(f"ops_f32_so{so}.npz: orders {pmin}..{pmax}")


def plummer(rng, n, a=0.1, rmax=1.0):
    pts = []
    while sum(len(p) for p in pts) < n:
        u = rng.uniform(0, 1, 2 * n)
        r = a / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
        r = r[r <= rmax]
        v = rng.standard_normal((len(r), 3))
        v /= np.linalg.norm(v, axis=1, keepdims=True)
        pts.append(v * r[:, None])
    return np.concatenate(pts)[:n]


def clusters(rng, n, k=4, sigma=0.02):
    m = n // 2
    cen = rng.uniform(0, 1, (k, 3))
    lab = rng.integers(0, k, n - m)
    return np.concatenate([rng.uniform(0, 1, (m, 3)), cen[lab] + sigma * rng.standard_normal((n - m, 3))])


CASES = {
    # name: (N, ncrit, order, theta, source_order, generator)
    "uniform10k": (10000, 64, 4, 0.5, 0, "uniform"),
    "deep": (3000, 8, 3, 0.7, 0, "uniform"),
    "dipole_plummer": (4000, 32, 4, 0.5, 1, "plummer"),
    "clustered": (5000, 16, 5, 0.4, 0, "clusters"),
    "tiny": (50, 64, 3, 0.5, 0, "uniform"),
    "example_scaled": (2000, 64, 4, 0.5, 0, "example"),
    "quadrupole_plummer": (3000, 32, 4, 0.5, 2, "plummer"),
    # small enough for a caller that applies every operator through the scalar
    # operators of include/operators.h (tests/test_gpu_operators_h.py)
    "small_charges": (400, 16, 3, 0.5, 0, "uniform"),
    "small_dipoles": (300, 16, 3, 0.5, 1, "plummer"),
}


def make_trees(only=None):
    for seed, (name, (N, ncrit, p, theta, so, gen)) in enumerate(CASES.items()):
        if only is not None and name not in only:
            continue
        rng = np.random.default_rng(seed)
        if gen == "uniform":
            pos = rng.uniform(0, 1, (N, 3))
        elif gen == "plummer":
            pos = plummer(rng, N)
        elif gen == "clusters":
            pos = clusters(rng, N)
        else:  # the example driver's data: U(-1,1) scaled by 1e-9 (example/main.cpp:86-110)
            pos = rng.uniform(-1, 1, (N, 3)) * 1e-9
        S = rng.uniform(-1, 1, (N, 1)) if so == 0 else rng.standard_normal((N, O.sourcesize(so)))
        rt = O.RefTree(pos, S, ncrit, p, theta, so)
        cells = rt.cells()
        m2l, p2p = rt.lists()
        F, _ = rt.evaluate()
        leaf_cell_ids = cells["id"][cells["nleaf"] < ncrit]
        order = np.argsort(cells["id"])
        out = dict(N=np.int64(N), ncrit=np.int64(ncrit), order=np.int64(p), theta=np.float64(theta),
                   source_order=np.int64(so), pos=pos, S=S, F=F,
                   cell_id=cells["id"][order], cell_nleaf=cells["nleaf"][order], cell_centre=cells["centre"][order],
                   leaf_id=leaf_cell_ids, leaf_off=cells["leaf_off"], leaf_idx=cells["leaf_idx"],
                   nm2l=np.int64(len(m2l)), np2p=np.int64(len(p2p)),
                   m2l_sha256=np.array(list_digest(m2l)), p2p_sha256=np.array(list_digest(p2p)))
        if len(m2l) + len(p2p) < 20000:
            o = np.lexsort((m2l[:, 1], m2l[:, 0]))
            out["m2l"] = m2l[o]
            o = np.lexsort((p2p[:, 1], p2p[:, 0]))
            out["p2p"] = p2p[o]
        np.savez_compressed(os.path.join(HERE, f"tree_{name}.npz"), **out)
        print(f"tree_{name}.npz: cells {rt.ncells} leaves {rt.nleaves} m2l {len(m2l)} p2p {len(p2p)}")


BH_CASES = {  # name: (N, ncrit, order, theta, source_order, generator)
    "uniform10k": (10000, 64, 4, 0.5, 0, "uniform"),
    "clustered": (5000, 16, 6, 0.5, 0, "clusters"),
    "dipole_plummer": (3000, 32, 5, 0.5, 1, "plummer"),
}


def make_bh():
    """Barnes-Hut: the reference's compute_field_bh potentials (its M2P field is
    not the gradient of its potential, so only the potential is kept) and the
    generated M2P's potential at every order."""
    for seed, (name, (N, ncrit, p, theta, so, gen)) in enumerate(BH_CASES.items()):
        rng = np.random.default_rng(100 + seed)
        pos = {"uniform": lambda: rng.uniform(0, 1, (N, 3)), "plummer": lambda: plummer(rng, N),
               "clusters": lambda: clusters(rng, N)}[gen]()
        S = rng.uniform(-1, 1, (N, 1)) if so == 0 else rng.standard_normal((N, 3))
        rt = O.RefTree(pos, S, ncrit, p, theta, so)
        F, _ = rt.evaluate_bh()
        np.savez_compressed(os.path.join(HERE, f"bh_{name}.npz"), N=np.int64(N), ncrit=np.int64(ncrit),
                            order=np.int64(p), theta=np.float64(theta), source_order=np.int64(so), pos=pos, S=S,
                            phi=F[:, 0])
        print(f"bh_{name}.npz: N {N} p {p}")
    rng = np.random.default_rng(77)
    out = {}
    for so, (pmin, pmax) in ((0, (1, 8)), (1, (2, 6))):
        R = O.ref(so)
        for p in range(pmin, pmax + 1):
            K = 5
            d = rng.uniform(-1, 1, (K, 3))
            d *= rng.uniform(1.5, 3.0, (K, 1)) / np.linalg.norm(d, axis=1, keepdims=True)
            M = rng.standard_normal((K, O.msize(p, so)))
            phi = np.zeros(K)
            for k in range(K):
                F = np.zeros(4)
                R.ref_M2P(*d[k], np.ascontiguousarray(M[k]), F, p)
                phi[k] = F[0]
            out[f"so{so}_p{p}_d"], out[f"so{so}_p{p}_M"], out[f"so{so}_p{p}_phi"] = d, M, phi
    np.savez_compressed(os.path.join(HERE, "m2p_potential.npz"), **out)
    print("m2p_potential.npz")


def make_m2p(specs, name, seed):
    """The generated M2P's potential at every order of the given source orders."""
    rng = np.random.default_rng(seed)
    out = {}
    for so, (pmin, pmax) in specs:
        R = O.ref(so)
        for p in range(pmin, pmax + 1):
            K = 5
            d = rng.uniform(-1, 1, (K, 3))
            d *= rng.uniform(1.5, 3.0, (K, 1)) / np.linalg.norm(d, axis=1, keepdims=True)
            M = rng.standard_normal((K, O.msize(p, so)))
            phi = np.zeros(K)
            for k in range(K):
                F = np.zeros(4)
                R.ref_M2P(*d[k], np.ascontiguousarray(M[k]), F, p)
                phi[k] = F[0]
            out[f"so{so}_p{p}_d"], out[f"so{so}_p{p}_M"], out[f"so{so}_p{p}_phi"] = d, M, phi
    np.savez_compressed(os.path.join(HERE, name), **out)
    print(name)


if __name__ == "__main__":
    if "--f32" in sys.argv:
        make_ops_f32()
    elif "--so2" in sys.argv:
        make_ops(specs=((2, (3, 5)),), seed=2025)
        make_trees(only={"quadrupole_plummer"})
        make_m2p(((2, (3, 5)),), "m2p_potential_so2.npz", 78)
    elif "--bh" in sys.argv:
        make_bh()
    elif "--trees" in sys.argv:  # --trees name[,name...]: only these tree fixtures
        make_trees(only=set(sys.argv[sys.argv.index("--trees") + 1].split(",")))
    else:
        make_ops()
        make_trees()
        make_bh()
