#!/usr/bin/env python
"""FBPINN train steps/s on one GB300: fused CUDA step vs the plain GPU step.

Workload (the 2D multilevel Poisson configuration): -lap u = f on [0,1]^2,
u = sum_{k=1..6} sin(2^k pi x) sin(2^k pi y) / 2^k, hard zero BC; multilevel
rectangular decomposition with 1, 2^2, 4^2, 8^2, 16^2, 32^2 subdomains
(m = 1365, width 2.9 x spacing, the single level-1 box [0,1]^2); FCN 2-16-16-1
tanh per subdomain; 2^18 uniform collocation points redrawn on the device every
step; Adam lr 1e-3.  A step = sample + interaction lists + sort + work queues +
forward jets + POU/residual/FP64 loss + adjoint + gradient reduce + Adam, one
CUDA graph.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl fused|reference]
Under torchrun (N > 1) every rank runs an independent replica (the step does
not shard across GPUs); value = steps/s summed over ranks, timed by the
slowest rank.  Prints one JSON line on rank 0.
"""

import argparse
import csv
import io
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np
import torch

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

N_POINTS = 1 << 18
LAYERS = [2, 16, 16, 1]
LEVELS = [1, 2, 4, 8, 16, 32]
WIDTH = 2.9
LR = 1e-3
SEED = 0
# DRAM bytes (read + write) of one adjoint launch and the pairs it covered, from an ncu
# capture of this workload at 2^16 points: layer 2 recomputed, and z-jets read from the
# forward's store (the forward then writes 256 B per pair more)
ADJ_DRAM_RECOMPUTE = (52.580352e6 + 0.155392e6, 2342389)
ADJ_DRAM_STORED = (689.641984e6 + 3.272704e6, 2342389)
METRIC = "FBPINN train steps/s, fused adjoint vs plain GPU step, at matched test L1 error"
WORKLOAD = "poisson2d_multilevel_m1365_fcn2-16-16-1_n262144_resampled"


def decomposition_static():
    from fbpinns_gb300.constants import get_subdomain_ws
    from fbpinns_gb300.decompositions import MultilevelRectangularDecompositionND
    sxs = [[np.array([0.5])] * 2] + [[np.linspace(0, 1, k)] * 2 for k in LEVELS[1:]]
    sws = [[np.array([1.0])] * 2] + [get_subdomain_ws(s, WIDTH) for s in sxs[1:]]
    return MultilevelRectangularDecompositionND.init_params(sxs, sws, (0., 1.))[0]


def init_theta(m, seed=SEED):
    from fbpinns_gb300.networks import FCN, pack_layers
    from fbpinns_gb300.trainers import init_subdomain_networks
    _, tr = init_subdomain_networks(FCN, {"layer_sizes": LAYERS}, m, seed)
    return pack_layers(tr["layers"])


def problem_setup():
    from fbpinns_gb300.problems import Poisson2D
    ps = Poisson2D.init_params(n_freq=6, sd=0.1)[0]
    return Poisson2D, {"static": {"problem": ps}, "trainable": {}}


def test_points():
    g = torch.linspace(0, 1, 100)
    X, Y = torch.meshgrid(g, g, indexing="ij")
    return torch.stack([X.reshape(-1), Y.reshape(-1)], 1)


def test_l1(eng, problem, all_params, x_test, u_exact):
    """mean |u - u_exact| of the engine's current parameters at x_test."""
    from fbpinns_gb300.trainers import FBPINNTrainer
    u = FBPINNTrainer.predict(eng, all_params, problem, x_test)
    return float(torch.mean(torch.abs(u_exact.float() - u)).item())


def test_l1_theta(eng, theta, problem, all_params, x_test, u_exact):
    """test_l1 with parameters theta (the engine's are restored afterwards)."""
    keep = eng.theta.clone()
    eng.set_theta(theta)
    l1 = test_l1(eng, problem, all_params, x_test, u_exact)
    eng.theta.copy_(keep)
    return l1


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class NvmlClockSampler:
    """SM clock and clock-event reasons read through NVML (libnvidia-ml, read
    only) every 5 ms on a background thread during the timed region, so that
    even a region of a fraction of a second gets many samples.  Falls back to
    ``ClockSampler`` (nvidia-smi at 200 ms) when NVML cannot be loaded."""
    # nvmlClocksEventReasons bits (nvml.h)
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown"}

    def __init__(self, index):
        import ctypes
        import threading
        self.C, self.threading = ctypes, threading
        # NVML numbers GPUs in PCI order, CUDA fastest-first: look the GPU up by
        # its PCI bus id (then its UUID), never by the CUDA ordinal
        self.bus_id, self.uuid = pci_ids(index)
        self.nvml = self.handle = None
        self.rows = []
        try:
            nv = ctypes.CDLL("libnvidia-ml.so.1")
            if nv.nvmlInit_v2() != 0:
                raise OSError("nvmlInit failed")
            h = ctypes.c_void_p()
            found = False
            if self.bus_id:
                found = nv.nvmlDeviceGetHandleByPciBusId_v2(self.bus_id.encode(), ctypes.byref(h)) == 0
            if not found and self.uuid:
                found = nv.nvmlDeviceGetHandleByUUID(self.uuid.encode(), ctypes.byref(h)) == 0
            if found:
                self.reasons_fn = getattr(nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                    nv.nvmlDeviceGetCurrentClocksThrottleReasons
                self.nvml, self.handle = nv, h
        except (OSError, AttributeError):
            self.nvml = None
        self.fallback = None if self.nvml is not None else ClockSampler(self.bus_id or self.uuid or index)

    def _sample(self):
        C = self.C
        mhz, mx, rs = C.c_uint(), C.c_uint(), C.c_ulonglong()
        self.nvml.nvmlDeviceGetMaxClockInfo(self.handle, 1, C.byref(mx))  # NVML_CLOCK_SM
        while not self._stop.is_set():
            if self.nvml.nvmlDeviceGetClockInfo(self.handle, 1, C.byref(mhz)) == 0 and \
                    self.reasons_fn(self.handle, C.byref(rs)) == 0:
                self.rows.append((mhz.value, mx.value, rs.value))
            self._stop.wait(0.005)

    def start(self):
        if self.fallback is not None:
            return self.fallback.start()
        self._stop = self.threading.Event()
        self.thread = self.threading.Thread(target=self._sample, daemon=True)
        self.thread.start()

    def stop(self):
        if self.fallback is not None:
            return self.fallback.stop()
        self._stop.set()
        self.thread.join(timeout=5)
        rows = self.rows
        reasons = sorted({name for _, _, r in rows for bit, name in self.REASONS.items() if r & bit})
        return {"sm_mhz": float(np.median([r[0] for r in rows])) if rows else None,
                "sm_max_mhz": float(max(r[1] for r in rows)) if rows else None,
                "reasons": reasons, "samples": len(rows), "source": "nvml, 5 ms", "pci_bus_id": self.bus_id}


def pci_ids(index):
    """(PCI bus id as NVML writes it, 'GPU-<uuid>') of CUDA device ``index``,
    either None when torch does not report it."""
    try:
        pr = torch.cuda.get_device_properties(index)
    except Exception:
        return None, None
    bus = None
    if all(hasattr(pr, a) for a in ("pci_domain_id", "pci_bus_id", "pci_device_id")):
        bus = "%08x:%02x:%02x.0" % (pr.pci_domain_id, pr.pci_bus_id, pr.pci_device_id)
    uid = getattr(pr, "uuid", None)
    uid = None if uid is None else ("GPU-" + str(uid) if not str(uid).startswith("GPU-") else str(uid))
    return bus, uid


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index  # a PCI bus id, a UUID or (last resort) an nvidia-smi index
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.TemporaryFile(mode="w+")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, ValueError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.seek(0)
        rows = [r for r in csv.reader(io.StringIO(self.f.read())) if len(r) >= 9]
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].strip().lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "source": "nvidia-smi, 200 ms", "gpu": str(self.index)}


# ---------------------------------------------------------------------------
# CPU baseline: the C restatement of the reference step (oracle/cstep.c) on
# the host cores, on the full workload (all 2^18 points, all 1365 subdomains)
# ---------------------------------------------------------------------------
def cpu_reference_step(static, theta_cpu, threads):
    from oracle import cstep
    p = static["subdomain"]["params"]
    return cstep.PoissonStep([t.numpy() for t in p], static["subdomain"]["pou"].numpy(), theta_cpu.numpy(),
                             LAYERS[1], sd=0.1, n_freq=6, threads=threads, lr=LR)


def cpu_steps(ref, n_points, steps, warmup, seed=1, budget_s=None):
    """Seconds per step of ``ref`` on fresh uniform points (drawn inside the
    timed loop, as the GPU step draws its own), after ``warmup`` steps; with
    ``budget_s`` it stops after that many seconds (at least 3 steps).
    Returns (seconds per step, steps timed, per-stage seconds of the last step)."""
    rng = np.random.default_rng(seed)
    for _ in range(warmup):
        ref.step(rng.uniform(0, 1, (n_points, 2)).astype(np.float32))
    t0 = time.perf_counter()
    k = 0
    while k < steps:
        ref.step(rng.uniform(0, 1, (n_points, 2)).astype(np.float32))
        k += 1
        if budget_s is not None and k >= 3 and time.perf_counter() - t0 > budget_s:
            break
    return (time.perf_counter() - t0) / k, k, ref.times.copy()


CPU_KIND = ("C restatement of the reference step (oracle/cstep.c): dense point-in-box lists, per-pair FCN jets "
            "(u, grad u, u_xx, u_yy) with activations stored for the reverse pass, POU segment sums, hard "
            "constraint, FP64 loss sum, reverse-mode gradient, optax Adam; FP32, pthreads")


# ---------------------------------------------------------------------------
def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend)
    return world, rank, local


def max_over_ranks(v, world):
    """Largest value over the ranks (the slowest rank's time)."""
    if world == 1:
        return v
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def run_reference(args, world, rank):
    """The reference arm: the reference step restated in C, timed on the full
    workload (2^18 points redrawn every step, all 1365 subdomains) on every
    host core, --warmup then --steps steps; plus a sweep of the point count."""
    if rank != 0:
        return
    static = decomposition_static()
    theta = init_theta(static["m"])
    threads = os.cpu_count() or 1
    ref = cpu_reference_step(static, theta, threads)
    t_step, k, stages = cpu_steps(ref, N_POINTS, args.steps, args.warmup)
    value = 1.0 / t_step
    sweep = {}
    for n in (1024, 16384, N_POINTS):
        r2 = cpu_reference_step(static, theta, threads)
        ts, ks, _ = cpu_steps(r2, n, 3, 1, seed=2)
        sweep[str(n)] = {"ms_per_step": 1000.0 * ts, "steps": ks, "pairs": r2.pairs}
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world,
            "steps": k, "warmup": args.warmup, "ms_per_step": 1000.0 * t_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": "synthetic (uniform points redrawn each step)",
            "config": {"workload": WORKLOAD, "m": static["m"], "n_points": N_POINTS, "pairs_per_step": ref.pairs,
                       "layers": LAYERS},
            "cpu_baseline": {"value": value, "unit": "steps/s", "cores": threads, "kind": "port",
                             "sample": f"{k} full steps of the workload ({N_POINTS} points, {ref.pairs} pairs); "
                                       + CPU_KIND,
                             "stage_s": {"lists": stages[0], "forward": stages[1], "pou_loss": stages[2],
                                         "reverse": stages[3], "adam": stages[4]}},
            "sample_sweep": sweep,
            "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_fused(args, world, rank, local):
    from fbpinns_gb300 import _lib
    from fbpinns_gb300.engine import FBPINNEngine
    from fbpinns_gb300.optim import adam
    from fbpinns_gb300.plain import PlainStep
    from fbpinns_gb300.trainers import FusedStep

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib = _lib.load()
    static = decomposition_static()
    problem, all_params = problem_setup()
    spec = problem.fused_spec(all_params)
    theta0 = init_theta(static["m"])
    opt = adam(LR)
    seed = SEED + 1000 * rank

    tc = False if args.fma_forward else None
    # the Poisson residual needs only the Laplacian: jets (u, u_x, u_y, u_xx + u_yy)
    d2 = 3 if args.per_dim_jets else 3 | _lib.D2_LAPLACIAN
    tca = args.tc_adjoint
    eng = FBPINNEngine(static, LAYERS, d2mask=d2, device=dev, chunk=args.chunk, grid=args.grid, tensor_cores=tc,
                       schedule=args.schedule, forward_chunk=args.forward_chunk, tc_adjoint=tca,
                       store_z2=args.store_z2, cell_order=args.cell_order)
    eng.set_theta(theta0)
    npts = args.points
    step = FusedStep(eng, spec, opt, resample=(npts, [0.0, 0.0], [1.0, 1.0], seed), use_graph=True,
                     autotune=args.autotune)
    for _ in range(max(args.warmup, 3)):
        step.step()
    torch.cuda.synchronize()
    pairs = int(step.ps.takes.pt_off[npts].item())
    slots = int(step.ps.takes.np_off[npts].item())

    clk = NvmlClockSampler(local)
    barrier(world)
    torch.cuda.synchronize()
    clk.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        step.step()
    e1.record()
    torch.cuda.synchronize()
    barrier(world)
    clocks = clk.stop()
    ms = e0.elapsed_time(e1) / args.steps
    ms_max = max_over_ranks(ms, world)
    step.check()
    loss_last = float(eng.loss.item())
    value = world * 1000.0 / ms_max
    if args.only_timed:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": "steps/s", "ms_per_step": ms_max,
                              "n_points": npts, "pairs_per_step": pairs, "only_timed": True}), flush=True)
        return

    # ---- end to end through the public step API with host buffers ----------
    e2e = None
    try:
        # the work-item sizes of the resampled step (autotuned there)
        eng2 = FBPINNEngine(static, LAYERS, d2mask=d2, device=dev, chunk=args.chunk, grid=args.grid,
                            tensor_cores=tc, schedule=args.schedule, forward_chunk=args.forward_chunk,
                            tc_adjoint=tca, store_z2=args.store_z2, cell_order=args.cell_order)
        eng2.set_theta(theta0)
        rng = np.random.default_rng(seed + 7)
        nh = 4
        host = [torch.from_numpy(rng.uniform(0, 1, (N_POINTS, 2)).astype(np.float32)).pin_memory() for _ in range(nh)]
        # pipelined: each call copies the next step's points in and builds their lists on a
        # second stream while the step trains on the current ones
        # the same configuration as the timed step: its tuned launch comes from the cache
        hstep = FusedStep(eng2, spec, opt, host_points=N_POINTS, x_probe=host[0], use_graph=True, pipeline=True,
                          autotune=args.autotune)
        e2e_tuned = getattr(eng2, "tuned", None)
        for k in range(max(args.warmup, 3)):
            hstep.step(host[k % nh], host[(k + 1) % nh])
        torch.cuda.synchronize()
        barrier(world)
        t0 = time.perf_counter()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record()
        for k in range(args.steps):
            hstep.step(host[k % nh], host[(k + 1) % nh])
        f1.record()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        barrier(world)
        ms_e = max(f0.elapsed_time(f1), 1000 * wall) / args.steps
        ms_e = max_over_ranks(ms_e, world)
        hstep.check()
        e2e = {"value": world * 1000.0 / ms_e, "unit": "steps/s", "h2d_bytes_per_step": N_POINTS * 2 * 4,
               "d2h_bytes_per_step": 8, "autotune_cache": e2e_tuned and e2e_tuned.get("cache")}
        del hstep, eng2
    except Exception as ex:  # reported, not hidden
        e2e = {"value": None, "unit": "steps/s", "error": repr(ex)[:200]}

    # ---- per-kernel timing (eager, CUDA events on the launching stream) ----
    ps = step.ps
    ev = lambda: torch.cuda.Event(enable_timing=True)
    reps = 5
    timings = {}

    def timed(name, fn):
        fn()
        torch.cuda.synchronize()
        a, b = ev(), ev()
        a.record()
        for _ in range(reps):
            fn()
        b.record()
        torch.cuda.synchronize()
        timings[name] = a.elapsed_time(b) / reps

    timed("takes_sort_work", lambda: ps.rebuild())
    timed("forward_pairs", lambda: eng.forward_pairs(ps))
    if eng.tensor_cores:  # the CUDA-core FMA forward on the same pairs, for comparison
        eng.tensor_cores = False
        timed("forward_pairs_fma", lambda: eng.forward_pairs(ps))
        eng.tensor_cores = True
    timed("pou_loss", lambda: eng.pou_loss(ps))
    timed("adjoint_pairs", lambda: eng.adjoint(ps, reduce=False))
    if ps.zs is not None:  # the same two kernels without the stored layer-2 z-jets, for comparison
        timed("forward_pairs_nostore", lambda: eng.forward_pairs(ps, z2=False))
        timed("adjoint_pairs_recompute", lambda: eng.adjoint(ps, reduce=False, z2=False))
    if lib.fbp_has_tc_adjoint_shape(2, LAYERS[1], LAYERS[2], d2, _lib.ACT_TANH):
        # the other adjoint variant on the same pairs, for comparison
        eng.tc_adjoint = not eng.tc_adjoint
        timed("adjoint_pairs_tc" if eng.tc_adjoint else "adjoint_pairs_fma", lambda: eng.adjoint(ps, reduce=False))
        eng.tc_adjoint = not eng.tc_adjoint
    timed("grad_reduce", lambda: eng.reduce_grad(ps))
    timed("adam", lambda: eng.adam(0.0))
    sig = float(sum(a * b for a, b in zip(LAYERS[:-1], LAYERS[1:])))
    J = eng.J
    fl_fwd = pairs * 2 * J * sig
    fl_adj = pairs * 4 * J * sig
    # FP32 FMA throughput probe (roofline denominator)
    sink = torch.zeros(256, device=dev)
    import ctypes as C
    flops = C.c_double()
    best = 0.0
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    for _ in range(3):
        a, b = ev(), ev()
        a.record()
        _lib.check(lib.fbp_fma_probe(_lib.ptr(sink), sms * 8, 8192, C.byref(flops), _lib.stream_ptr()))
        b.record()
        torch.cuda.synchronize()
        best = max(best, flops.value / (a.elapsed_time(b) * 1e-3) / 1e12)
    dom = max(("forward_pairs", "adjoint_pairs"), key=lambda k: timings[k])
    ach = (fl_adj if dom == "adjoint_pairs" else fl_fwd) / (timings[dom] * 1e-3) / 1e12
    # DRAM traffic of the adjoint per launch: ncu dram__bytes_read.sum + dram__bytes_write.sum of
    # adjoint_pairs_kernel<Cfg<2,16,16,11>> in one capture of this workload at 2^16 points, scaled
    # by this run's pairs (traffic grows with the pairs); per variant (bytes, pairs of the capture)
    adj_dram = ADJ_DRAM_STORED if ps.zs is not None else ADJ_DRAM_RECOMPUTE
    traffic = adj_dram[0] / adj_dram[1] * pairs if (dom == "adjoint_pairs" and J == 4 and adj_dram) else None
    roofline = {"bound": "fp32", "kernel": dom, "achieved": ach, "peak": best, "unit": "TFLOP/s", "frac": ach / best,
                "peak_source": "FP32 FMA probe (fbp_fma_probe) measured in this run; MEASURED_PEAKS.json has no FP32 figure",
                "traffic": traffic,
                "traffic_source": "ncu DRAM bytes of the adjoint at 2^16 points scaled by pairs" if traffic else None,
                "kernel_ms": {k: round(v, 4) for k, v in timings.items()},
                "algorithmic_flops_per_launch": {"forward_pairs": fl_fwd, "adjoint_pairs": fl_adj}}

    # ---- plain GPU step (torch autograd), then the matched test error ----
    # Both arms start from theta0 with step count 0 and draw the same points
    # each step (the Philox stream is keyed by the seed and the step count);
    # after the plain arm's 2 warm-up + kp timed steps, both give their test L1
    # on a 100 x 100 grid against the exact solution (mean |u - u_exact|, as
    # the reference's _test, fbpinns/trainers.py:727-774).
    plain = None
    l1_fused = None
    x_test = test_points().to(dev)
    u_exact = problem.exact_solution(all_params, x_test).to(dev)
    if not args.no_plain:
        try:
            eng3 = FBPINNEngine(static, LAYERS, d2mask=3, device=dev, chunk=args.chunk, cell_order=args.cell_order)
            eng3.set_theta(theta0)
            pstep = PlainStep(eng3, problem, all_params, ((0, (0, 0)), (0, (1, 1))), opt,
                              resample=(N_POINTS, [0.0, 0.0], [1.0, 1.0], seed))
            for _ in range(2):
                pstep.step()
            torch.cuda.synchronize()
            kp = max(3, min(args.steps, 10))
            a, b = ev(), ev()
            a.record()
            for _ in range(kp):
                pstep.step()
            b.record()
            torch.cuda.synchronize()
            pstep.check()
            ms_p = max_over_ranks(a.elapsed_time(b) / kp, world)
            k_match = 2 + kp
            l1_plain = test_l1(eng3, problem, all_params, x_test, u_exact)
            del pstep, eng3
            # the fused step (the benchmarked configuration) over the same k_match steps
            eng4 = FBPINNEngine(static, LAYERS, d2mask=d2, device=dev, chunk=args.chunk, grid=args.grid,
                                tensor_cores=tc, schedule=args.schedule, forward_chunk=args.forward_chunk,
                                tc_adjoint=tca, store_z2=args.store_z2, cell_order=args.cell_order)
            eng4.set_theta(theta0)
            fstep = FusedStep(eng4, spec, opt, resample=(N_POINTS, [0.0, 0.0], [1.0, 1.0], seed), use_graph=True,
                              autotune=args.autotune)
            for _ in range(k_match):
                fstep.step()
            torch.cuda.synchronize()
            fstep.check()
            match_tuned = getattr(eng4, "tuned", None)
            l1_fused = test_l1(eng4, problem, all_params, x_test, u_exact)
            l1_0 = test_l1_theta(eng4, theta0, problem, all_params, x_test, u_exact)
            del fstep, eng4
            plain = {"value": world * 1000.0 / ms_p, "unit": "steps/s", "ms_per_step": ms_p, "steps": kp,
                     "fused_over_plain": ms_p / ms_max, "test_l1": l1_plain,
                     "matched": {"steps": k_match, "test_l1_initial": l1_0, "test_l1_fused": l1_fused,
                                 "test_l1_plain": l1_plain, "rel_gap": abs(l1_fused - l1_plain) / l1_plain,
                                 "autotune_cache": match_tuned and match_tuned.get("cache"),
                                 "test_points": "100 x 100 grid on [0,1]^2"}}
        except Exception as ex:
            plain = {"value": None, "error": repr(ex)[:300]}
        torch.cuda.empty_cache()

    # ---- CPU baseline (rank 0 only): full steps of the same workload, ~10 s ----
    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        ref = cpu_reference_step(static, theta0.cpu(), threads)
        t_cpu, nsteps, _ = cpu_steps(ref, N_POINTS, 30, 1, budget_s=10.0)
        cpu = {"value": 1.0 / t_cpu, "unit": "steps/s", "cores": threads, "kind": "port",
               "sample": f"{nsteps} full steps of the workload ({N_POINTS} points, {ref.pairs} pairs); " + CPU_KIND}
        # the GPU step against the restatement at the full size: loss and gradient of the
        # initial parameters on one batch of the workload, computed by both
        try:
            xb = np.random.default_rng(SEED + 7).uniform(0, 1, (N_POINTS, 2)).astype(np.float32)
            loss_c, grad_c = cpu_reference_step(static, theta0.cpu(), threads).loss_grad(xb)
            engp = FBPINNEngine(static, LAYERS, d2mask=d2, device=dev, tensor_cores=tc, cell_order=False)
            engp.set_theta(theta0)
            engp.set_problem(spec)
            psp = engp.points(torch.from_numpy(xb).to(dev))
            engp.forward_pairs(psp)
            loss_g = float(engp.pou_loss(psp).item())
            grad_g = engp.adjoint(psp).cpu().numpy()
            psp.check_status()
            cpu["agreement"] = {"points": N_POINTS, "pairs": int(psp.s), "loss_gpu": loss_g, "loss_cpu": loss_c,
                                "loss_rel_diff": abs(loss_g - loss_c) / abs(loss_c),
                                "grad_max_abs_diff_over_max_abs": float(np.abs(grad_g - grad_c).max()
                                                                        / np.abs(grad_c).max()),
                                "against": "the C restatement above (FP32 arithmetic, FP64 loss sum) on the "
                                           "initial parameters and one batch; the FP64 oracle is the tests' pin"}
            del engp, psp
        except Exception as ex:  # reported, not hidden
            cpu["agreement"] = {"error": repr(ex)[:200]}

    # launches of our kernels in one step (counted from the C-ABI calls of the step body; each
    # scan of up to 4096 tiles of 2048 is two launches, all of them at this size): sample (1),
    # cell order (4), inside count (1), pair and slot offsets (2 + 2), fill (1), subdomain sort
    # (hist 1, scan 2, scatter 1, starts 1), two work queues (count 1, scan 2, fill 1 each),
    # forward, POU/loss, loss finalize, adjoint, gradient reduce, Adam + step count (1+1+1+1+1+2)
    per_step = 1 + (4 if eng.cell_order else 0) + 1 + 4 + 1 + 5 + 2 * 4 + 7
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "fp32", "data": "synthetic (uniform points redrawn each step)",
                "config": {"workload": WORKLOAD, "m": static["m"], "n_points": N_POINTS, "pairs_per_step": pairs,
                           "slots_per_step": slots, "layers": LAYERS, "jet_components": J,
                           "parallelism": f"replicas x{world}", "chunk": step.ps.chunk,
                           "forward_chunk": step.ps.fwd_chunk, "schedule": eng.schedule,
                           "forward_schedule": eng.fwd_schedule(),
                           "grid": eng.launch_grid, "forward_grid": eng.forward_grid,
                           "autotuned": getattr(eng, "tuned", None),
                           "forward_kernel": "tcgen05 3xTF32" if eng.tensor_cores else "fp32 fma",
                           "adjoint_kernel": "tcgen05 3xTF32 layer-2 recompute + fp32 fma" if eng.tc_adjoint
                           else ("fp32 fma, layer-2 z-jets stored by the forward" if ps.zs is not None
                                 else "fp32 fma, layer 2 recomputed"),
                           "jet": "u, grad u, u_xx, u_yy" if args.per_dim_jets else "u, grad u, laplacian u",
                           "point_order": "morton cells of ~64 points" if eng.cell_order else "as drawn",
                           "l2": "per-step working set ~%.0f MB > 129 MB L2; no flush" %
                                 ((pairs * (2 * J * 4 + 16) + slots * 2 * J * 4
                                   + (pairs * J * LAYERS[2] * 4 if ps.zs is not None else 0)) / 1e6)},
                "e2e": e2e, "gpu_launches": per_step * args.steps, "clocks": clocks, "roofline": roofline,
                "cpu_baseline": cpu, "plain": plain, "test_l1": l1_fused, "loss_last": loss_last,
                "evals_per_s": value * pairs}
        print(json.dumps(line), flush=True)


def run_profile_plain(args):
    """One plain GPU step of the workload between cudaProfilerStart and
    cudaProfilerStop (after two warm-up steps), for a launch list of exactly
    that step: ``ncu --profile-from-start off --metrics gpu__time_duration.sum
    ... python bench.py --profile-plain``.  Prints the step's wall time."""
    from fbpinns_gb300.engine import FBPINNEngine
    from fbpinns_gb300.optim import adam
    from fbpinns_gb300.plain import PlainStep
    dev = torch.device("cuda", 0)
    static = decomposition_static()
    problem, all_params = problem_setup()
    eng = FBPINNEngine(static, LAYERS, d2mask=3, device=dev)
    eng.set_theta(init_theta(static["m"]))
    pstep = PlainStep(eng, problem, all_params, ((0, (0, 0)), (0, (1, 1))), adam(LR),
                      resample=(N_POINTS, [0.0, 0.0], [1.0, 1.0], SEED))
    for _ in range(2):
        pstep.step()
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    t0 = time.perf_counter()
    pstep.step()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    torch.cuda.profiler.stop()
    print(json.dumps({"metric": "plain step", "workload": WORKLOAD, "wall_ms": 1000 * wall}), flush=True)


def run_extras(args):
    """Measurements of the paths either side of the step, on the same Poisson
    workload (one JSON line; not part of the default run):
      * the fused step with the other compiled networks (SIREN, AdaptiveFCN,
        AdaptiveSIREN with 16-16 hidden layers, FourierFCN with 8 features and
        one hidden layer of 32), steps/s;
      * test-step inference (forward jets + POU combination at every point of
        a fixed 2^18-point set, all subdomains): points/s;
      * the interaction lists rebuilt on the device after a scheduler change
        (work queues for a new active set, no host synchronisation): ms."""
    from fbpinns_gb300 import _lib
    from fbpinns_gb300.engine import FBPINNEngine
    from fbpinns_gb300.optim import adam
    from fbpinns_gb300.trainers import FusedStep, init_subdomain_networks
    from fbpinns_gb300 import networks as NW
    dev = torch.device("cuda", 0)
    static = decomposition_static()
    m = static["m"]
    problem, all_params = problem_setup()
    spec = problem.fused_spec(all_params)
    d2 = 3 | _lib.D2_LAPLACIAN
    out = {"metric": "extras", "workload": WORKLOAD, "networks": {}}

    def timed_steps(step, k):
        for _ in range(3):
            step.step()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(k):
            step.step()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / k

    nets = [("SIREN", NW.SIREN, {"layer_sizes": LAYERS}), ("AdaptiveFCN", NW.AdaptiveFCN, {"layer_sizes": LAYERS}),
            ("AdaptiveSIREN", NW.AdaptiveSIREN, {"layer_sizes": LAYERS}),
            ("FourierFCN", NW.FourierFCN, {"layer_sizes": [2, 32, 1], "mu": 0.0, "sd": 1.0, "n_features": 8})]
    for name, cls, kw in nets:
        st_, tr = init_subdomain_networks(cls, kw, m, SEED)
        ls, act, layers, _ = NW.engine_network(cls, st_, tr["layers"], kw["layer_sizes"])
        eng = FBPINNEngine(static, ls, d2mask=d2, device=dev, activation=act)
        eng.set_theta(NW.pack_layers(layers))
        step = FusedStep(eng, spec, adam(LR), resample=(N_POINTS, [0.0, 0.0], [1.0, 1.0], SEED), use_graph=True)
        ms = timed_steps(step, max(args.steps, 10))
        step.check()
        out["networks"][name] = {"layers": ls, "activation": act, "ms_per_step": ms, "steps_per_s": 1000.0 / ms}
        del step, eng
    # inference on a fixed point set (the test step)
    eng = FBPINNEngine(static, LAYERS, d2mask=0, device=dev, store_z2=False)
    eng.set_theta(init_theta(m))
    g = torch.Generator(device="cpu").manual_seed(SEED)
    xt = torch.rand((N_POINTS, 2), generator=g).to(dev)
    ps = eng.points(xt)
    for _ in range(3):
        eng.forward_pairs(ps)
        eng.pou_forward(ps)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    k = 20
    a.record()
    for _ in range(k):
        eng.forward_pairs(ps)
        eng.pou_forward(ps)
    b.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / k
    out["inference"] = {"points": N_POINTS, "pairs": ps.s, "jet": "u, grad u", "forward_kernel":
                        "tcgen05 3xTF32" if eng.tensor_cores else "fp32 fma", "ms": ms,
                        "points_per_s": N_POINTS / (ms * 1e-3)}
    # scheduler change: a new active set -> work queues rebuilt on the device
    eng2 = FBPINNEngine(static, LAYERS, d2mask=d2, device=dev)
    eng2.set_theta(init_theta(m))
    ps2 = eng2.points(xt)
    masks = [np.where(np.arange(m) % 2 == i, 1, 2) for i in range(2)]
    times = []
    for i in range(12):
        eng2.set_state(masks[i % 2])
        torch.cuda.synchronize()
        a.record()
        ps2.build_work()
        b.record()
        torch.cuda.synchronize()
        times.append(a.elapsed_time(b))
    out["scheduler_change"] = {"ms_median": float(np.median(times[2:])), "what": "work queues of a new active set "
                               "(forward: all subdomains with pairs; adjoint: the active ones), on the device"}
    a.record()
    ps2.rebuild()
    b.record()
    torch.cuda.synchronize()
    out["list_rebuild_ms"] = a.elapsed_time(b)
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="fused", choices=["fused", "reference"])
    ap.add_argument("--chunk", type=int, default=1024, help="pairs per adjoint work item")
    ap.add_argument("--forward-chunk", type=int, default=0, help="pairs per forward work item (0: 4 x --chunk)")
    ap.add_argument("--grid", type=int, default=0)
    ap.add_argument("--fma-forward", action="store_true", help="forward jets on the CUDA-core FMA kernel")
    ap.add_argument("--tc-adjoint", action="store_true",
                    help="adjoint with the layer-2 recompute on the tensor cores (fbp_adjoint_pairs_tc)")
    ap.add_argument("--store-z2", action="store_const", const=True, default=None,
                    help="the forward stores the layer-2 z-jets and the adjoint reads them instead of recomputing "
                         "(default: only for hidden layers at least 32 wide, so not for this workload)")
    ap.add_argument("--no-cell-order", dest="cell_order", action="store_false",
                    help="keep each drawn batch in the sampler's order (default: Morton cell order)")
    ap.add_argument("--per-dim-jets", action="store_true",
                    help="carry u_xx and u_yy as separate jet components instead of the Laplacian")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="use --chunk/--forward-chunk instead of measuring the work-item sizes on the first batch")
    ap.add_argument("--schedule", default="dynamic", choices=["dynamic", "static", "per_item"],
                    help="how the jet kernels' CTAs take work items")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--only-timed", action="store_true",
                    help="run only the warm-up and timed fused steps (for profiler launch lists)")
    ap.add_argument("--points", type=int, default=N_POINTS, help="collocation points per step")
    ap.add_argument("--extras", action="store_true",
                    help="instead of the bench line: other networks, inference and scheduler-change timings")
    ap.add_argument("--profile-plain", action="store_true",
                    help="instead of the bench line: one plain GPU step bracketed for a profiler launch list")
    args = ap.parse_args()
    if args.extras:
        run_extras(args)
        return
    if args.profile_plain:
        run_profile_plain(args)
        return
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_fused(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
