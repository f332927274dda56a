"""Launch autotuner of the fused step.

The jet kernels walk (subdomain, run of pairs) work items.  Four launch
choices trade against each other and depend on the network, the jet and how
the pairs spread over the subdomains, so they are measured on the actual
points rather than guessed:

* the work-item sizes (adjoint pairs per item, forward pairs per item): per-item
  set-up (weights into shared memory, tensor-core B operands, the tile
  pipeline's fill and drain, one gradient partial) against load balance;
* the schedule of each of the two jet launches: ``dynamic`` (a resident grid
  whose CTAs take the next item from a device counter), ``static`` (CTA b takes
  items b, b + grid, ...) or ``per_item`` (one CTA per item, so that CTAs
  retire as they finish and kernels of a higher-priority stream get SMs);
* the CTA count of the adjoint and of the forward launch (0 = every CTA that
  can be resident, else a multiple of the SM count).

The search is coordinate-wise: the item sizes first (dynamic schedules,
resident grids), then the adjoint's schedule, the forward's, then the two
CTA counts; every candidate
builds the work queues for the points and times forward + POU/loss + adjoint
with CUDA events -- for a pipelined step with the next step's lists rebuilt
on the higher-priority side stream at the same time, as in the step itself
(the schedule decides how those list kernels get SMs during the jet
kernels).  The choice is kept on the engine and cached on disk, keyed by the
GPU, the network, the jet, the kernels, the subdomain and point counts and
the pipelining, so that a later run of the same configuration skips the
search.  The candidates' results are identical up to the FP32 summation
order of the per-item gradient partials.
"""

import json
import os
import tempfile

import torch

CACHE_ENV = "FBPINNS_GB300_AUTOTUNE_CACHE"


def cache_path():
    """JSON file of tuned launches: $FBPINNS_GB300_AUTOTUNE_CACHE, else
    ~/.cache/fbpinns_gb300/autotune.json."""
    p = os.environ.get(CACHE_ENV)
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "fbpinns_gb300", "autotune.json")


def config_key(engine, n, pipelined):
    """The configuration a tuned launch is valid for: the GPU, the network and
    its jet, the kernels used (and whether layer 2 is stored for the adjoint),
    whether batches are put in cell order, the subdomain and point counts and whether the
    next step's lists are built alongside (a redrawn batch of the same size
    keeps the key; its pair count is recorded with the choice)."""
    props = torch.cuda.get_device_properties(engine.device)
    return "|".join(str(v) for v in (props.name, props.multi_processor_count, engine.layer_sizes, engine.activation,
                                     engine.d2mask, int(engine.tensor_cores), int(getattr(engine, "tc_adjoint", 0)),
                                     int(bool(getattr(engine, "z2_rows", 0))), int(bool(getattr(engine, "cell_order", 0))),
                                     engine.m, int(n), int(bool(pipelined))))


def _load_cache(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store_cache(path, key, entry):
    """Adds one entry (atomic replace: readers never see a partial file).
    Returns None, or the reason the file could not be written (the choice
    still holds for this run)."""
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        data = _load_cache(path)
        data[key] = entry
        fd, tmp = tempfile.mkstemp(dir=os.path.dirname(path), prefix=".autotune.")
        with os.fdopen(fd, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
        return None
    except OSError as ex:
        return repr(ex)


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


def _apply(engine, choice):
    engine.chunk, engine.forward_chunk = int(choice["chunk"]), int(choice["forward_chunk"])
    engine.schedule = choice["schedule"]
    engine.forward_schedule = choice.get("forward_schedule", choice["schedule"])
    engine.launch_grid = int(choice["grid"])
    engine.forward_grid = int(choice["forward_grid"])
    engine.adaptive_items = False


def _pass(engine, ps, side=None):
    """The step's device work on point set ps.  With side = (stream, point
    set), that set's lists are rebuilt on the (higher-priority) stream at
    the same time, as the pipelined step builds the next step's lists."""
    main = torch.cuda.current_stream()
    if side is not None:
        stream, ps2 = side
        stream.wait_stream(main)
        with torch.cuda.stream(stream):
            ps2.rebuild(stream=stream)
    engine.forward_pairs(ps)
    engine.pou_loss(ps)
    engine.adjoint(ps)
    if side is not None:
        main.wait_stream(side[0])


def tune_work_items(engine, x, caps=None, candidates=None, reps=3, use_cache=True, pipelined=False):
    """Tune the launches of the step's device work on points x and set the
    choice on the engine (``chunk``, ``forward_chunk``, ``schedule``,
    ``launch_grid``, ``forward_grid``).  Needs ``engine.set_problem`` first.
    ``pipelined``: time each candidate with the lists of a second point set
    rebuilt on a higher-priority stream alongside (the pipelined step's
    load).  Returns (and keeps as ``engine.tuned``) the choice, what was
    searched, every candidate's time in ms and whether the cache held it."""
    x = torch.as_tensor(x, dtype=torch.float32).to(engine.device)
    probe = engine.points(x)
    s, n = probe.s, probe.n
    if candidates is None:
        candidates = default_candidates(s, engine.m, engine.sm_count)
    if pipelined and caps is None:
        caps = (int(probe.s * 1.25) + 1024, int(probe.u * 1.25) + 1024)
    del probe
    key = config_key(engine, n, pipelined)
    path = cache_path()
    if use_cache:
        hit = _load_cache(path).get(key)
        if hit is not None:
            _apply(engine, hit["choice"])
            engine.tuned = dict(hit, cache="hit", key=key)
            return engine.tuned
    sms = engine.sm_count
    searched = {"item_sizes": [f"{a}/{f}" for a, f in candidates], "schedule": ["dynamic", "static", "per_item"],
                "forward_schedule": ["dynamic", "static", "per_item"],
                "grid": [0, sms, 2 * sms, 3 * sms], "forward_grid": [0, sms, 2 * sms]}
    timings = {}
    ev = lambda: torch.cuda.Event(enable_timing=True)
    if pipelined:
        side_stream = torch.cuda.Stream(device=engine.device, priority=-1)

    def run(choice):
        tag = f"{choice['chunk']}/{choice['forward_chunk']} {choice['schedule']}/{choice['forward_schedule']} " \
              f"g{choice['grid']} fg{choice['forward_grid']}"
        if tag in timings:
            return timings[tag]
        _apply(engine, choice)
        ps = engine.points(x, caps=caps)
        side = (side_stream, engine.points(x, caps=caps)) if pipelined else None
        _pass(engine, ps, side)  # warm-up: per-device kernel attributes, caches
        torch.cuda.synchronize()
        a, b = ev(), ev()
        a.record()
        for _ in range(reps):
            _pass(engine, ps, side)
        b.record()
        torch.cuda.synchronize()
        ps.check_status()
        del ps, side
        timings[tag] = a.elapsed_time(b) / reps
        return timings[tag]

    best = {"chunk": candidates[0][0], "forward_chunk": candidates[0][1], "schedule": "dynamic",
            "forward_schedule": "dynamic", "grid": 0, "forward_grid": 0}
    best_t = None
    stages = [("size", [dict(chunk=a, forward_chunk=f) for a, f in candidates]),
              ("schedule", [dict(schedule=v) for v in searched["schedule"]]),
              ("forward_schedule", [dict(forward_schedule=v) for v in searched["forward_schedule"]]),
              ("grid", [dict(grid=v) for v in searched["grid"]]),
              ("forward_grid", [dict(forward_grid=v) for v in searched["forward_grid"]])]
    for name, opts in stages:
        if (name == "grid" and best["schedule"] == "per_item") or \
                (name == "forward_grid" and best["forward_schedule"] == "per_item"):
            continue  # one CTA per item: the grid is the item count
        for o in opts:
            c = dict(best, **o)
            t = run(c)
            if best_t is None or t < best_t:
                best, best_t = c, t
    _apply(engine, best)
    entry = {"choice": best, "searched": searched, "best_ms": round(best_t, 4), "pairs": int(s),
             "pipelined": bool(pipelined), "timings_ms": {k: round(v, 4) for k, v in timings.items()}}
    err = _store_cache(path, key, entry) if use_cache else None
    engine.tuned = dict(entry, cache="miss", key=key)
    if err:
        engine.tuned["cache_write_error"] = err
    return engine.tuned
