"""fmmgen_gb300.stream_compute: a stream of build + evaluate steps from host
memory, copies overlapped with the neighbouring steps' work, gives every step
exactly the outputs of a plain rebuild_compute on the same inputs (single
systems and forests)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def inputs(n, k, so, seed):
    rng = np.random.default_rng(seed)
    pos = [torch.tensor(rng.uniform(0, 1, (n, 3))).pin_memory() for _ in range(k)]
    S = [torch.tensor(rng.uniform(-1, 1, (n, 1)) if so == 0 else rng.standard_normal((n, 3))).pin_memory()
         for _ in range(k)]
    return pos, S


@pytest.mark.parametrize("sizes,so", [(None, 0), ([3000, 12000, 5000], 0), (None, 1)])
def test_stream_equals_steps(fg, sizes, so):
    n = 20000 if sizes is None else sum(sizes)
    pos, S = inputs(n, 4, so, 17)
    if sizes is None:
        t = fg.build_tree(pos[0].cuda(), S[0].cuda(), n, 64, 5, 0.5, source_order=so)
    else:
        t = fg.build_forest(pos[0].cuda(), S[0].cuda(), sizes, 64, 5, 0.5, source_order=so)
    osz = 4
    F = [torch.zeros((n, osz), dtype=torch.float64).pin_memory() for _ in range(4)]
    ms = fg.stream_compute(t, pos, S, F, True, True, "mixed", timing=True)
    assert ms > 0
    for i in range(4):
        ref = t.rebuild_compute(pos[i].cuda(), S=S[i].cuda(), potential=True, field=True, precision="mixed")
        assert np.array_equal(F[i].numpy(), ref.cpu().numpy()), i


def test_stream_single_step(fg):
    pos, S = inputs(5000, 1, 0, 3)
    t = fg.build_tree(pos[0].cuda(), S[0].cuda(), 5000, 32, 4, 0.5)
    F = [torch.zeros((5000, 3), dtype=torch.float64).pin_memory()]
    fg.stream_compute(t, pos, S, F, False, True, "fp64")
    ref = t.rebuild_compute(pos[0].cuda(), S=S[0].cuda(), potential=False, field=True, precision="fp64")
    assert np.array_equal(F[0].numpy(), ref.cpu().numpy())
