"""Work-item autotuner of the fused step.

The jet kernels walk (subdomain, run of pairs) work items; how many pairs an
item holds trades per-item set-up (weights into shared memory, tensor-core B
operands, the tile pipeline's fill and drain, one gradient partial) against
load balance over the SMs.  The best sizes depend on the network, the jet and
how the pairs spread over the subdomains, so they are measured: every
candidate (adjoint pairs per item, forward pairs per item) builds the work
queues for the actual points and times forward + POU/loss + adjoint with CUDA
events; the fastest is kept on the engine.  The candidates' results are
identical up to the FP32 summation order of the per-item gradient partials.
"""

import torch


def default_candidates(s, m, sms):
    """Around the pair-count heuristic (``engine.work_item_sizes`` with the
    requested 1024 / 4096): adjoint items of half, once and twice its size,
    forward items of 1, 2 and 4 times the adjoint's (at most 8192)."""
    from .engine import work_item_sizes
    adj, _, _ = work_item_sizes(s, m, sms, 1024, 4096)
    out = []
    for a in (max(64, adj // 2), adj, 2 * adj):
        for k in (1, 2, 4):
            if (a, min(a * k, 8192)) not in out:
                out.append((a, min(a * k, 8192)))
    return out


def _pass(engine, ps):
    engine.forward_pairs(ps)
    engine.pou_loss(ps)
    engine.adjoint(ps)


def tune_work_items(engine, x, caps=None, candidates=None, reps=3):
    """Time the step's device work (no parameter update) for each candidate
    (adjoint chunk, forward chunk) on points x and set the fastest on the
    engine (``engine.chunk``, ``engine.forward_chunk``; item sizes are then
    used as given).  Needs ``engine.set_problem`` first.  Returns a dict with
    the choice and every candidate's time in ms.  ``candidates`` defaults to
    ``default_candidates`` for the pair count of x."""
    x = torch.as_tensor(x, dtype=torch.float32).to(engine.device)
    if candidates is None:
        probe = engine.points(x)
        candidates = default_candidates(probe.s, engine.m, engine.sm_count)
        del probe
    engine.adaptive_items = False
    timings = {}
    ev = lambda: torch.cuda.Event(enable_timing=True)
    for adj, fwd in candidates:
        engine.chunk, engine.forward_chunk = int(adj), int(fwd)
        ps = engine.points(x, caps=caps)
        _pass(engine, ps)  # warm-up: per-device kernel attributes, caches
        torch.cuda.synchronize()
        a, b = ev(), ev()
        a.record()
        for _ in range(reps):
            _pass(engine, ps)
        b.record()
        torch.cuda.synchronize()
        ps.check_status()
        timings[(int(adj), int(fwd))] = a.elapsed_time(b) / reps
        del ps
    best = min(timings, key=timings.get)
    engine.chunk, engine.forward_chunk = best
    engine.tuned = {"chunk": best[0], "forward_chunk": best[1],
                    "timings_ms": {f"{k[0]}/{k[1]}": round(v, 4) for k, v in timings.items()}}
    return engine.tuned
