"""A stream of FMM steps whose inputs and outputs live in host memory.

No counterpart in the reference, whose example builds and evaluates one tree
per call with its arrays already in host memory (example/main.cpp:154-162).
Here every step is `Tree.rebuild_compute` (build_tree + compute_field_fmm,
example/tree.cpp:130-271) on new positions and sources; `stream_compute` runs
a sequence of such steps with the host<->device copies of each step
overlapped with the device work of its neighbours:

    step i-1: ...compute...|  D2H F(i-1)
    step i:     H2D in(i)  |...compute...|  D2H F(i)
    step i+1:               H2D in(i+1)  |...compute...

Inputs are copied on one stream, outputs on another, the steps computed on a
third, with two device buffers of each array and events between them, so a
step's copies cost nothing while they are shorter than a step's device work.
Host arrays should be pinned (torch `pin_memory()`), or the copies are
synchronous.
"""
import torch


class StepBuffers:
    """Two device buffers of each per-step array (positions, sources, outputs)."""

    def __init__(self, n, sourcesize, outputsize, device):
        self.pos = [torch.empty((n, 3), dtype=torch.float64, device=device) for _ in range(2)]
        self.S = [torch.empty((n, sourcesize), dtype=torch.float64, device=device) for _ in range(2)]
        self.F = [torch.empty((n, outputsize), dtype=torch.float64, device=device) for _ in range(2)]


def stream_compute(tree, pos_host, S_host, F_host, potential=True, field=True, precision="mixed", buffers=None,
                   timing=False):
    """Run len(pos_host) steps: step i rebuilds `tree` for pos_host[i], evaluates
    the sources S_host[i] and leaves the outputs in F_host[i] (host tensors,
    [N][3], [N][SOURCESIZE], [N][OUTPUTSIZE], float64, the same N in every
    step).  Returns the device time in ms from the first input copy to the
    last output copy when `timing`, else None; the outputs are complete when
    the call returns."""
    n = len(pos_host)
    if not (len(S_host) == len(F_host) == n) or n == 0:
        raise ValueError("one position, source and output array per step")
    N = pos_host[0].shape[0]
    dev = tree.pos.device
    if buffers is None:
        buffers = StepBuffers(N, S_host[0].shape[1], F_host[0].shape[1], dev)
    comp = torch.cuda.current_stream(dev)
    s_in, s_out = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    ev_in = [torch.cuda.Event() for _ in range(2)]     # inputs of the buffer landed
    ev_done = [torch.cuda.Event() for _ in range(2)]   # the step on the buffer computed
    ev_out = [torch.cuda.Event() for _ in range(2)]    # the buffer's outputs copied out
    t0, t1 = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) if timing else (None, None)

    def copy_in(i):
        b = i % 2
        with torch.cuda.stream(s_in):
            if i >= 2:
                s_in.wait_event(ev_done[b])  # step i - 2 has finished with the buffer
            buffers.pos[b].copy_(pos_host[i], non_blocking=True)
            buffers.S[b].copy_(S_host[i], non_blocking=True)
            ev_in[b].record(s_in)

    if timing:
        t0.record(s_in)
    copy_in(0)
    for i in range(n):
        b = i % 2
        if i + 1 < n:
            copy_in(i + 1)  # beside this step's work
        comp.wait_event(ev_in[b])
        if i >= 2:
            comp.wait_event(ev_out[b])  # the outputs of step i - 2 have left the buffer
        tree.rebuild_compute(buffers.pos[b], buffers.F[b], S=buffers.S[b], potential=potential, field=field,
                             precision=precision, stream=comp)
        ev_done[b].record(comp)
        with torch.cuda.stream(s_out):
            s_out.wait_event(ev_done[b])
            F_host[i].copy_(buffers.F[b], non_blocking=True)
            ev_out[b].record(s_out)
    comp.wait_event(ev_out[(n - 1) % 2])
    if n >= 2:
        comp.wait_event(ev_out[n % 2])
    if timing:
        t1.record(comp)
    comp.synchronize()
    return t0.elapsed_time(t1) if timing else None
