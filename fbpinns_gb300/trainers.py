"""FBPINN trainer (the reference's ``fbpinns/trainers.py`` API) on the GPU engine.

``FBPINNTrainer(c).train()`` follows the reference's loop
(fbpinns/trainers.py:577-687): initialise parameters, iterate the scheduler,
rebuild the training inputs when the active mask changes, take a step, and
report (summary line, test L1, model pickles).  The step itself is one of:

* ``FusedStep`` — built-in problems: the fused CUDA forward / POU / residual /
  FP64 loss / adjoint / Adam sequence, optionally resampling the collocation
  points on the device each step, captured in a CUDA graph;
* ``GenericStep`` — any problem: ``FBPINNJet`` gives the per-point jets,
  ``constraining_fn`` and ``loss_fn`` run in torch autograd on them, the
  gradient comes back through the CUDA adjoint.
"""

import ctypes
import logging
import os
import pickle
import sys
import time

import numpy as np
import torch

from . import _lib
from .engine import FBPINNEngine, FBPINNJet, constrained_jets, d2mask_of, jet_index
from .networks import (fcn_param_count, pack_layers, unpack_layers, engine_network,  # noqa: F401
                       NETWORK_ACTIVATIONS, FCN, SIREN, AdaptiveFCN, AdaptiveSIREN, FourierFCN)
from .optim import adam_update
from .takes import get_inputs, split_takes, inside_models, grid_of  # noqa: F401  (re-exported API)

logger = logging.getLogger("fbpinns_gb300")
if not logger.handlers:
    _h = logging.StreamHandler(stream=sys.stdout)
    _h.setFormatter(logging.Formatter(fmt="[%(levelname)s] %(asctime)s - %(message)s", datefmt="%Y-%m-%d %H:%M:%S"))
    logger.addHandler(_h)
    logger.setLevel(logging.INFO)


def _to_dev(v, dev):
    return v.to(dev) if torch.is_tensor(v) else v


class GenericStep:
    """Loss and gradients of any problem through the CUDA jets.

    ``constraints`` are the per-constraint lists without ``required_ujs``
    ([x_batch, *values]); their points are concatenated into one point set and
    each constraint owns a contiguous row range (fbpinns/trainers.py:249-267).
    """

    def __init__(self, engine, problem, all_params, constraints, required_ujss, ps=None):
        self.eng, self.problem, self.all_params = engine, problem, all_params
        dev = engine.device
        self.constraints = [[_to_dev(torch.as_tensor(c_), dev) if not torch.is_tensor(c_) else c_.to(dev)
                             for c_ in con] for con in constraints]
        self.required = required_ujss
        self.sizes = [con[0].shape[0] for con in self.constraints]
        self.offsets = np.cumsum([0] + self.sizes[:-1]).tolist()
        x = torch.cat([con[0].float() for con in self.constraints]) if self.constraints else None
        self.ps = ps if ps is not None else engine.points(x)
        self.xd = engine.xd

    def _trainable_problem(self):
        tp = self.all_params.get("trainable", {}).get("problem", {})
        return {k: v for k, v in tp.items() if torch.is_tensor(v)}

    def loss(self, theta):
        eng = self.eng
        U = FBPINNJet.apply(theta, eng, self.ps)
        cons_ = []
        for ic, con in enumerate(self.constraints):
            a, b = self.offsets[ic], self.offsets[ic] + self.sizes[ic]
            x = self.ps.x[a:b]
            ks = [jet_index(self.xd, eng.d2mask, ixs) for _, ixs in self.required[ic]]
            Uc = constrained_jets(self.problem.constraining_fn, self.all_params, x, U[a:b], self.xd, eng.d2mask,
                                  need=ks)
            ujs = [Uc[:, k:k + 1] for k in ks]
            cons_.append(list(con) + ujs)
        return self.problem.loss_fn(self.all_params, cons_)

    def loss_and_grads(self, theta):
        tp = self._trainable_problem()
        leaves = [theta] + list(tp.values())
        for v in tp.values():
            v.requires_grad_(True)
        loss = self.loss(theta)
        gs = torch.autograd.grad(loss, leaves, allow_unused=True)
        gs = [torch.zeros_like(l) if g is None else g for g, l in zip(gs, leaves)]
        return loss.detach(), gs[0], dict(zip(tp.keys(), gs[1:]))

    def step(self, opt):
        eng = self.eng
        theta = eng.theta.detach().clone().requires_grad_(True)
        loss, gtheta, gprob = self.loss_and_grads(theta)
        tp = self._trainable_problem()
        if tp:
            count = int(eng.count.item())  # the shared Adam step count (a host read only when needed)
            if not hasattr(self, "_pm"):
                self._pm = {k: (torch.zeros_like(v), torch.zeros_like(v)) for k, v in tp.items()}
            with torch.no_grad():
                for k, v in tp.items():
                    m1, m2 = self._pm[k]
                    adam_update(v, gprob[k], m1, m2, count, opt["learning_rate"], opt["b1"], opt["b2"], opt["eps"],
                                opt["eps_root"])
        eng.adam(opt["learning_rate"], opt["b1"], opt["b2"], opt["eps"], opt["eps_root"], grad=gtheta)
        return loss

    def check(self):
        """Raise if the point set's status word records an overflow."""
        self.ps.check_status()


class StepGraph:
    """A captured CUDA graph instantiated by the library with per-node
    priorities: kernel nodes keep the priority of the stream they were captured
    on (torch's own replay would run every node at the launching stream's
    priority).  Owns torch's graph (and its memory pool) and the executable."""

    def __init__(self):
        self.graph = torch.cuda.CUDAGraph(keep_graph=True)
        self.exec = None

    def instantiate(self):
        lib = _lib.load()
        out = ctypes.c_void_p()
        _lib.check(lib.fbp_graph_instantiate(ctypes.c_void_p(self.graph.raw_cuda_graph()), 1, ctypes.byref(out)),
                   "fbp_graph_instantiate")
        self.exec = out

    def replay(self):
        _lib.check(_lib.load().fbp_graph_launch(self.exec, _lib.stream_ptr()), "fbp_graph_launch")

    def __del__(self):
        if self.exec is not None:
            try:
                _lib.load().fbp_graph_exec_destroy(self.exec)
            except Exception:  # interpreter shutdown: the CUDA driver releases it with the context
                pass


class FusedStep:
    """The fused CUDA step for a built-in problem.

    Point modes:
      ``x=...``          fixed collocation points (exact buffer sizes);
      ``resample=(n, xmin, xmax, seed)``  n new uniform points drawn on the
                         device every step (stream offset = device step count);
      ``host_points=n``  the caller passes each step's points from (pinned)
                         host memory to ``step(x_host)``.
    In the last two modes the interaction lists are rebuilt every step into
    fixed-capacity buffers (``headroom`` x the first batch's sizes), so the step
    has no host synchronisation and is captured in one CUDA graph when
    ``use_graph``.

    With ``pipeline`` two point sets alternate: while step t trains on one, a
    second stream builds step t+1's lists into the other.  With ``resample``
    (pipelined by default) it also draws step t+1's points (stream offset =
    the count at step t's start + 1, the offset step t+1 would use); with
    ``host_points`` (``pipeline=True`` opt-in) the caller passes the next
    step's points as well, ``step(x_host, x_next)``, and they are copied in
    before the step.  The results are bit-identical to the serial step.

    ``autotune`` first times candidate work-item sizes on the first batch of
    points and keeps the fastest on the engine (``autotune.tune_work_items``).
    """

    def __init__(self, engine, spec, opt, x=None, resample=None, host_points=None, x_probe=None, use_graph=True,
                 headroom=1.25, pipeline=None, autotune=False, scheduled=False):
        self.eng, self.opt = engine, opt
        self.scheduled = bool(scheduled)
        engine.set_problem(spec)
        if autotune:
            # launches measured on this step's first batch of points (with the next
            # step's lists built alongside when the step is pipelined)
            from .autotune import tune_work_items
            if resample is not None:
                xt = torch.empty((resample[0], engine.xd), dtype=torch.float32, device=engine.device)
                engine.sample(xt, int(resample[3]), 1 << 32, list(resample[1]), list(resample[2]))
            else:
                xt = x_probe if host_points is not None else x
            piped = (resample is not None or host_points is not None) and \
                (bool(pipeline) if pipeline is not None else resample is not None)
            if xt is not None:
                tune_work_items(engine, xt, pipelined=piped)
        self.resample = resample
        self.host = host_points is not None
        self.use_graph = use_graph
        self.graph = None
        dev = engine.device
        if resample is not None or self.host:
            if resample is not None:
                n, xmin, xmax, seed = resample
                self.xmin, self.xmax, self.seed = list(xmin), list(xmax), int(seed)
                x0 = torch.empty((n, engine.xd), dtype=torch.float32, device=dev)
                engine.sample(x0, self.seed, 1 << 32, self.xmin, self.xmax)
            else:
                x0 = torch.as_tensor(x_probe, dtype=torch.float32).to(dev)
                assert x0.shape[0] == host_points
            probe = engine.points(x0)
            caps = (int(probe.s * headroom) + 1024, int(probe.u * headroom) + 1024)
            del probe
            self.ps = engine.points(x0, caps=caps, scheduled=self.scheduled)
        else:
            self.ps = engine.points(torch.as_tensor(x, dtype=torch.float32).to(dev), scheduled=self.scheduled)
        self.loss_host = torch.zeros(1, dtype=torch.float64, pin_memory=True)
        if pipeline is None:
            pipeline = resample is not None
        self.pipeline = bool(pipeline) and (resample is not None or self.host)
        # host batches land in a staging buffer and enter the point set in Morton
        # cell order (engine.cell_order: the same batch, in an order with locality)
        self.order_host = self.host and engine.cell_order
        if self.order_host:
            # the cell grid spans the probe batch (later batches: the same
            # distribution; points outside it gather in its edge cells, which
            # stays correct but slows the ordering); no order for a probe
            # with non-finite coordinates or no extent along a dim
            lo, hi = x0.min(0).values.double(), x0.max(0).values.double()
            ok = bool(torch.isfinite(lo).all() and torch.isfinite(hi).all() and (hi > lo).all())
            self.order_host = ok
        if self.order_host:
            self.ps.x_stage = torch.empty_like(self.ps.x)
            pad = 1e-6 * torch.clamp(hi - lo, min=1.0)
            self.order_box = ((lo - pad).cpu().tolist(), (hi + pad).cpu().tolist())
        if self.pipeline:
            self.sets = [self.ps, engine.points(self.ps.x.clone(), caps=caps, scheduled=self.scheduled)]
            if self.order_host:
                self.sets[1].x_stage = torch.empty_like(self.ps.x)
            self.cur = 0
            self.started = False
            self.snap = torch.zeros(1, dtype=torch.int32, device=dev)  # count at the step's start
            # higher priority (kept inside the graphs, see StepGraph): as CTAs of the step's
            # kernels retire, the block scheduler starts the list kernels' CTAs first
            self.side = torch.cuda.Stream(device=dev, priority=-1)
            self.graphs = [None, None]
            if resample is not None:
                self._prologue()

    def _prologue(self):
        """The current point set's points and lists for the current step count."""
        ps = self.sets[self.cur]
        if self.resample is not None:
            self.eng.sample(ps.x, self.seed, 0, self.xmin, self.xmax, counter=self.eng.count)
        ps.rebuild()
        self.ps = ps

    def set_state(self, active):
        """A new scheduler mask.  Scheduled steps take the mask as the scheduler
        yields it (0, 1, 2): one host-to-device copy, then the training points,
        subdomain states, pair sort and work queues are derived on the device,
        and the captured graphs replay unchanged (their buffers are the same).
        Other steps take the masked state (get_inputs' ``active``) and rebuild
        their work queues."""
        sets = self.sets if self.pipeline else [self.ps]
        if self.scheduled:
            self.eng.set_raw_state(active)
            for ps in sets:
                ps.rebuild_scheduled()
            return
        self.eng.set_state(active)
        for ps in sets:
            ps.build_work()
        self.graph = None
        if self.pipeline:
            self.graphs = [None, None]

    def _body_pipelined(self, cur):
        """Step on point set cur while the other set is rebuilt for the next step."""
        eng, o = self.eng, self.opt
        main = torch.cuda.current_stream()
        a, b = self.sets[cur], self.sets[1 - cur]
        self.snap.copy_(eng.count)
        with torch.cuda.stream(self.side):
            self.side.wait_stream(main)
            if self.resample is not None:
                eng.sample(b.x, self.seed, 1, self.xmin, self.xmax, counter=self.snap, stream=self.side)
            elif self.order_host:
                eng.order_points(b.x_stage, b.x, stream=self.side, box=self.order_box)
            b.rebuild(stream=self.side)
        loss = eng.fused_step(a, o["learning_rate"], stream=main, b1=o["b1"], b2=o["b2"], eps=o["eps"],
                              eps_root=o["eps_root"])
        main.wait_stream(self.side)
        return loss

    def _body(self, stream=None):
        eng, o = self.eng, self.opt
        if self.resample is not None:
            eng.sample(self.ps.x, self.seed, 0, self.xmin, self.xmax, counter=eng.count, stream=stream)
            self.ps.rebuild(stream=stream)
        elif self.host:
            if self.order_host:
                eng.order_points(self.ps.x_stage, self.ps.x, stream=stream, box=self.order_box)
            self.ps.rebuild(stream=stream)
        return eng.fused_step(self.ps, o["learning_rate"], stream=stream, b1=o["b1"], b2=o["b2"], eps=o["eps"],
                              eps_root=o["eps_root"])

    def capture(self, warmup=2):
        """Capture the step in a CUDA graph (one per point set when pipelined)
        after ``warmup`` eager steps on a side stream; the warm-up steps'
        updates (parameters, Adam moments, step count, hence also the sampler's
        stream offset) are rolled back, so capturing does not advance training."""
        eng = self.eng
        self.captures = getattr(self, "captures", 0) + 1
        saved = [t.clone() for t in (eng.theta, eng.m1, eng.m2, eng.count)]
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            for w in range(warmup):
                if self.pipeline:
                    self._body_pipelined(w % 2)
                else:
                    self._body()
        torch.cuda.current_stream().wait_stream(s)
        for dst, src in zip((eng.theta, eng.m1, eng.m2, eng.count), saved):
            dst.copy_(src)
        if self.pipeline:
            for cur in (0, 1):
                g = StepGraph()
                with torch.cuda.graph(g.graph):
                    self._body_pipelined(cur)
                g.instantiate()
                self.graphs[cur] = g
            if self.resample is not None:
                self.cur = 0
                self._prologue()  # the current set again, for the rolled-back count
            else:
                self.sets[self.cur].rebuild()  # the warm-up rebuilt both sets from their points
            self.graph = self.graphs
            return
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self._body()
        self.graph = g

    def step(self, x_host=None, x_next=None):
        """One training step; returns the device loss.  In host mode x_host
        (n, xd) float32, ideally pinned, is copied in first and the loss is
        copied back to ``loss_host`` (read it after a synchronisation); when
        pipelined, x_next holds the next step's points (x_host is then read
        only on the first call: later steps use the previous call's x_next)."""
        if self.host and self.pipeline:
            if x_next is None:
                raise ValueError("a pipelined host-point step needs the next step's points (x_next)")
            if not self.started:
                cur = self.sets[self.cur]
                if self.order_host:
                    cur.x_stage.copy_(x_host, non_blocking=True)
                    self.eng.order_points(cur.x_stage, cur.x, box=self.order_box)
                else:
                    cur.x.copy_(x_host, non_blocking=True)
                cur.rebuild()
                self.started = True
            nxt = self.sets[1 - self.cur]
            (nxt.x_stage if self.order_host else nxt.x).copy_(x_next, non_blocking=True)
        elif self.host:
            (self.ps.x_stage if self.order_host else self.ps.x).copy_(x_host, non_blocking=True)
        if self.pipeline:
            if self.use_graph:
                if self.graph is None:
                    self.capture()
                self.graphs[self.cur].replay()
            else:
                self._body_pipelined(self.cur)
            self.cur = 1 - self.cur
            self.ps = self.sets[self.cur]  # holds the next step's lists
        elif self.use_graph:
            if self.graph is None:
                self.capture()
            self.graph.replay()
        else:
            self._body()
        if self.host:
            self.loss_host.copy_(self.eng.loss, non_blocking=True)
        return self.eng.loss

    def check(self):
        for ps in (self.sets if self.pipeline else [self.ps]):
            ps.check_status()


def init_subdomain_networks(network, kwargs, m, seed):
    """Per-subdomain network init from split seeds (fbpinns/trainers.py:601-607)."""
    g = torch.Generator().manual_seed(int(seed))
    seeds = torch.randint(0, 2 ** 62, (m,), generator=g).tolist()
    per = [network.init_params(s, **kwargs) for s in seeds]
    # static network parameters are per subdomain too (FourierFCN's omega: (m, F, xd))
    static = {k: torch.stack([torch.as_tensor(p[0][k]) for p in per]) for k in per[0][0]}
    layers = [tuple(torch.stack([p[1]["layers"][li][k] for p in per]) for k in range(len(per[0][1]["layers"][li])))
              for li in range(len(per[0][1]["layers"]))]
    return static, {"layers": layers}


class FBPINNTrainer:
    """``FBPINNTrainer(c).train() -> all_params`` (fbpinns/trainers.py:479-774)."""

    def __init__(self, c):
        self.c = c
        if getattr(c, "save_models", False):
            c.get_outdirs()
            c.save_constants_file()
        self.u_test_losses = []
        self.history = []

    def _print_summary(self, i, loss, rate, start):
        logger.info("[i: %i/%i] loss: %.4f rate: %.1f elapsed: %.2f hr %s" % (
            i, self.c.n_steps, loss, rate, (time.time() - start) / 3600, self.c.run))
        self.history.append({"i": i, "loss": loss, "rate": rate})

    def _save_model(self, i, model):
        with open(self.c.model_out_dir + f"model_{i:08d}.jax", "wb") as f:
            pickle.dump(model, f)

    def train(self):
        c = self.c
        dev = torch.device(c.device)
        torch.manual_seed(c.seed)
        np.random.seed(c.seed)
        all_params = {"static": {}, "trainable": {}}
        domain, problem, decomposition = c.domain, c.problem, c.decomposition
        for tag, cl, kw in zip(["domain", "problem", "decomposition"], [domain, problem, decomposition],
                               [c.domain_init_kwargs, c.problem_init_kwargs, c.decomposition_init_kwargs]):
            ps_ = cl.init_params(**kw)
            if ps_[0]:
                all_params["static"][tag] = ps_[0]
            if ps_[1]:
                all_params["trainable"][tag] = ps_[1]
        st_dec = all_params["static"]["decomposition"]
        m, xd = st_dec["m"], st_dec["xd"]
        assert all_params["static"]["domain"]["xd"] == all_params["static"]["problem"]["dims"][1] == xd
        logger.info(f"Total number of subdomains: {m}")
        net_static, net_tr = init_subdomain_networks(c.network, c.network_init_kwargs, m, c.seed)
        # the kernels' layers (FourierFCN: its frozen feature layer first)
        layer_sizes, activation, eng_layers, self.frozen_layers = engine_network(
            c.network, net_static, net_tr["layers"], c.network_init_kwargs["layer_sizes"])
        if net_static:  # (model pickles carry them from the start)
            all_params["static"]["network"] = {"subdomain": net_static}
        scheduler = c.scheduler(all_params=all_params, n_steps=c.n_steps, **c.scheduler_kwargs)

        # constraints (sampled once, as the reference does; or resampled per step)
        constraints_global = problem.sample_constraints(all_params=all_params, domain=domain, key=c.seed,
                                                        sampler=c.sampler, batch_shapes=c.ns)
        required = [con[-1] for con in constraints_global]
        constraints_global = [con[:-1] for con in constraints_global]
        d2 = d2mask_of(required, xd)
        if c.engine not in ("fused", "generic", "plain"):
            raise ValueError(f"engine must be 'fused', 'generic' or 'plain', not {c.engine!r}")
        spec = problem.fused_spec(all_params) if c.engine == "fused" else None
        single = len(constraints_global) == 1 and not all_params["trainable"].get("problem")
        use_fused = spec is not None and single
        group = spec.get("d2_group", 0) if use_fused else 0
        if group and (d2 & group) == group:
            # the residual uses these second derivatives only through their sum: one jet slot for it
            d2g = d2 | (_lib.D2_LAPLACIAN if group == (d2 & 7) else _lib.D2_GROUP(group))
            if _lib.load().fbp_has_shape(xd, layer_sizes[1], layer_sizes[2] if len(layer_sizes) == 4 else 0, d2g,
                                         _lib.ACTIVATIONS[activation]):
                d2 = d2g
        eng = FBPINNEngine(st_dec, layer_sizes, d2, device=dev, chunk=c.chunk, grid=c.launch_grid,
                           tensor_cores=getattr(c, "tensor_cores", None), activation=activation,
                           forward_chunk=getattr(c, "forward_chunk", None), store_z2=getattr(c, "store_z2", None))
        eng.set_theta(pack_layers(eng_layers))
        for k, v in list(all_params["trainable"].get("problem", {}).items()):
            all_params["trainable"]["problem"][k] = torch.as_tensor(v, dtype=torch.float32).to(dev).clone()
        all_params["static"]["problem"] = {k: _to_dev(v, dev) for k, v in all_params["static"]["problem"].items()}
        opt = c.optimiser(**c.optimiser_kwargs)
        use_plain = c.engine == "plain"
        if use_plain and not single:
            raise NotImplementedError("the plain step handles one constraint without trainable problem params")
        if c.resample and not (use_fused or use_plain):
            raise NotImplementedError("per-step resampling is implemented for the fused and plain steps")
        # test data (fbpinns/trainers.py:463-470, 620-624)
        x_test = domain.sample_interior(all_params, None, "grid", c.n_test)
        u_exact = problem.exact_solution(all_params, x_test, c.n_test)
        self.x_test, self.u_exact = x_test, u_exact
        self.engine, self.all_params = eng, all_params
        ps_test = None

        x_global = torch.cat([con[0] for con in constraints_global]).float()
        sizes = [con[0].shape[0] for con in constraints_global]
        offs = np.cumsum([0] + sizes)
        step = None
        start0 = start1 = time.time()
        report_time = 0.0
        lossval = None
        # Fused steps follow scheduler changes on the device: one point set over all
        # global points, the mask copied in, the training points / states / work
        # queues derived by kernels, the captured step replayed unchanged
        # (resampled all-active runs keep the unmasked step: every point trains)
        from .schedulers import AllActiveSchedulerND
        device_sched = use_fused and getattr(c, "device_schedule", True)
        masked = not (c.resample and c.scheduler is AllActiveSchedulerND)
        for i, active_ in enumerate(scheduler):
            if active_ is not None and device_sched:
                if step is not None:
                    step.check()  # the steps since the last check ran on complete lists
                t0 = time.time()
                active = np.array(active_).copy()
                if step is None:
                    res = None
                    if c.resample:
                        d = all_params["static"]["domain"]
                        res = (int(np.prod(c.ns[0])), d["xmin"].tolist(), d["xmax"].tolist(), c.seed)
                    step = FusedStep(eng, spec, opt, x=None if c.resample else x_global, resample=res,
                                     use_graph=c.use_graph, headroom=c.pair_headroom,
                                     autotune=c.autotune and getattr(eng, "tuned", None) is None, scheduled=masked)
                if masked:
                    step.set_state(active)
                else:
                    eng.set_state(np.where(active == 0, 1, active))
                logger.info(f"[i: {i}/{c.n_steps}] Updating active inputs done ({time.time() - t0:.2f} s)")
            elif active_ is not None:
                if step is not None:
                    step.check()  # the steps since the last check ran on complete lists
                t0 = time.time()
                active = np.array(active_).copy()
                # points inside models with raw state 1 (fbpinns/trainers.py:482-507)
                ims = np.arange(m)[active == 1]
                if use_fused and c.resample:
                    training_x, cons = None, None
                else:
                    ips = inside_models(st_dec, x_global, ims)[0].long().cpu()
                    training_x = x_global[ips]
                    cons = []
                    for ic, con in enumerate(constraints_global):
                        sel = ips[(ips >= offs[ic]) & (ips < offs[ic + 1])] - offs[ic]
                        cons.append([v[sel] if torch.is_tensor(v) and v.shape[:1] == con[0].shape[:1] else v
                                     for v in con])
                # active/fixed masks after the training-point cut (fbpinns/trainers.py:347-357)
                xs_for_mask = training_x if training_x is not None else None
                state = active.copy()
                state[state == 0] = 1
                if xs_for_mask is not None and xs_for_mask.shape[0]:
                    tk = eng.points(xs_for_mask.to(dev))
                    has = (tk.subdomain_counts() > 0).cpu().numpy()
                    del tk
                else:
                    has = np.ones(m, dtype=bool)
                state = state * has
                eng.set_state(state)
                res = None
                if c.resample:
                    d = all_params["static"]["domain"]
                    res = (int(np.prod(c.ns[0])), d["xmin"].tolist(), d["xmax"].tolist(), c.seed)
                if use_fused:
                    if step is not None and training_x is None:
                        step.set_state(state)
                    else:
                        step = FusedStep(eng, spec, opt, x=training_x, resample=res, use_graph=c.use_graph,
                                         headroom=c.pair_headroom,
                                         autotune=c.autotune and getattr(eng, "tuned", None) is None)
                elif use_plain:
                    from .plain import PlainStep
                    step = PlainStep(eng, problem, all_params, required[0], opt, x=training_x, resample=res,
                                     headroom=c.pair_headroom)
                else:
                    step = GenericStep(eng, problem, all_params, cons, required)
                logger.info(f"[i: {i}/{c.n_steps}] Updating active inputs done ({time.time() - t0:.2f} s)")
            if i == 0:
                self._test(i, eng, all_params, problem)
            lossval = step.step(opt) if isinstance(step, GenericStep) else step.step()
            i1 = i + 1
            if i1 % c.summary_freq == 0:
                lv = float(lossval.item())
                # the status word is sticky: an overflow of a fixed-capacity list in any
                # step since the last check raises here (this read follows the loss's sync)
                step.check()
                rate = c.summary_freq / max(time.time() - start1 - report_time, 1e-9)
                self._print_summary(i1, lv, rate, start0)
                start1, report_time = time.time(), 0.0
            if i1 % c.test_freq == 0 or (c.save_models and i1 % c.model_save_freq == 0):
                t2 = time.time()
                if i1 % c.test_freq == 0:
                    self._test(i1, eng, all_params, problem)
                if c.save_models and i1 % c.model_save_freq == 0:
                    self._save_model(i1, self.model_tuple(i1, eng, all_params))
                report_time += time.time() - t2
        if step is not None:
            torch.cuda.synchronize()
            step.check()
        all_params["trainable"]["network"] = {"subdomain": {"layers": [
            tuple(t.detach().cpu().clone() for t in layer)
            for layer in unpack_layers(eng.theta, layer_sizes, eng.extra)[self.frozen_layers:]]}}
        if net_static:
            all_params["static"]["network"] = {"subdomain": net_static}
        logger.info(f"[i: {c.n_steps}/{c.n_steps}] Training complete")
        return all_params

    @staticmethod
    def _numpy_tree(d):
        """Copy of a params tree with tensors as numpy arrays and private keys dropped."""
        if isinstance(d, dict):
            return {k: FBPINNTrainer._numpy_tree(v) for k, v in d.items() if not str(k).startswith("_")}
        if isinstance(d, (list, tuple)):
            return type(d)(FBPINNTrainer._numpy_tree(v) for v in d)
        if torch.is_tensor(d):
            return d.detach().cpu().numpy().copy()
        return d

    def model_tuple(self, i, eng, all_params):
        """(i, all_params, all_opt_states, active, u_test_losses) as numpy, the
        layout of the reference's model pickles (fbpinns/trainers.py:721)."""
        ls, skip = eng.layer_sizes, getattr(self, "frozen_layers", 0)
        def tree(t):
            return [tuple(x.cpu().numpy().copy() for x in layer) for layer in unpack_layers(t, ls, eng.extra)[skip:]]
        layers, mu, nu = tree(eng.theta), tree(eng.m1), tree(eng.m2)
        ap = {"static": self._numpy_tree(all_params["static"]),
              "trainable": {"network": {"subdomain": {"layers": layers}},
                            **{k: self._numpy_tree(v) for k, v in all_params["trainable"].items() if k != "network"}}}
        opt = {"count": int(eng.count.item()), "mu": {"network": {"subdomain": {"layers": mu}}},
               "nu": {"network": {"subdomain": {"layers": nu}}}}
        return (i, ap, opt, eng.state.cpu().numpy().astype(int), np.array(self.u_test_losses))

    def _test(self, i, eng, all_params, problem):
        """Test L1 on the grid test points (fbpinns/trainers.py:727-765)."""
        u_test = self.predict(eng, all_params, problem, self.x_test)
        ue = torch.as_tensor(self.u_exact).reshape(-1, 1).to(u_test.device).float()
        l1 = torch.mean(torch.abs(ue - u_test)).item()
        l1n = l1 / ue.std().item()
        self.u_test_losses.append([i, l1, l1n])
        logger.info(f"[i: {i}/{self.c.n_steps}] test L1: {l1:.4e} (normalised {l1n:.4e})")
        return l1

    @staticmethod
    def predict(eng, all_params, problem, x):
        """FBPINN solution at points x with all subdomains (the test-step inference)."""
        x = torch.as_tensor(x, dtype=torch.float32).to(eng.device)
        key = "_test_points"
        cache = getattr(eng, key, None)
        if cache is None or cache[0] is not x and not torch.equal(cache[0], x):
            ps = eng.points(x)
            setattr(eng, key, (x, ps))
        ps = getattr(eng, key)[1]
        with torch.no_grad():
            eng.forward_pairs(ps, z2=False)
            U = eng.pou_forward(ps)
            return problem.constraining_fn(all_params, x, U[:, 0:1])


class PINNTrainer(FBPINNTrainer):
    """A single network over the whole domain (fbpinns/trainers.py:780-943).

    Run as the m = 1 case of the FBPINN engine: one box equal to the domain,
    so the subdomain normalisation is the domain's ``norm_fn``, the window flag
    is 0 (w = 1), the POU sum is the network output, and the unnormalisation
    uses ``decomposition_init_kwargs["unnorm"]`` as the reference's PINN does.
    """

    def train(self):
        from .decompositions import RectangularDecompositionND
        from .schedulers import AllActiveSchedulerND
        c = self.c
        lo = np.asarray(c.domain_init_kwargs["xmin"], dtype=np.float64)
        hi = np.asarray(c.domain_init_kwargs["xmax"], dtype=np.float64)
        unnorm = c.decomposition_init_kwargs.get("unnorm", (0., 1.))
        saved = (c.decomposition, c.decomposition_init_kwargs, c.scheduler, c.scheduler_kwargs)
        c.decomposition = RectangularDecompositionND
        c.decomposition_init_kwargs = dict(subdomain_xs=[np.array([(a + b) / 2]) for a, b in zip(lo, hi)],
                                           subdomain_ws=[np.array([b - a]) for a, b in zip(lo, hi)],
                                           unnorm=unnorm)
        c.scheduler, c.scheduler_kwargs = AllActiveSchedulerND, {}
        try:
            return super().train()
        finally:
            c.decomposition, c.decomposition_init_kwargs, c.scheduler, c.scheduler_kwargs = saved
