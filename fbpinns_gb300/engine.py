"""Device engine for the FBPINN training step.

``FBPINNEngine`` owns the packed subdomain parameters (theta (m, P), the Adam
moments, the shared step count) and launches the CUDA kernels of
``libfbpgpu`` on point sets.  ``PointSet`` owns everything derived from one set
of collocation points: the interaction lists, the subdomain-major pair order,
the work queues and the per-pair / per-slot jet buffers.

Step (fused path, built-in problems), all stream-ordered, no host sync:

    forward_pairs   per-pair jets of u*w and w            (K-fwd)
    pou_loss        POU combination, hard constraint, PDE residual,
                    FP64 loss partials, per-slot seeds    (K-seg + K-loss)
    loss_finalize   deterministic FP64 sum
    adjoint_pairs   per-pair recompute + adjoint, one gradient partial per
                    work item                             (K-adj)
    grad_reduce     partials -> grad (m, P) in item order
    adam            masked Adam with the shared count     (K-adam)

With ``resample=True`` a step also draws new uniform points (Philox) and
rebuilds the interaction lists on the device into fixed-capacity buffers, so
the whole step can be captured in one CUDA graph.

The generic path (any problem) uses ``FBPINNJet``: a torch.autograd.Function
whose forward returns the per-point jets of the POU-combined network output
and whose backward runs the adjoint kernels; ``constraining_fn`` and
``loss_fn`` then run in torch autograd on the per-point jets only.
"""

import ctypes as C
import math

import numpy as np
import torch

from . import _lib
from .networks import fcn_param_count
from .takes import PointTakes, grid_of


def d2mask_of(required_ujss, xd):
    """Bit mask of dims needing a pure second derivative; checks the orders.

    Supports what the compiled jets carry: u, all first derivatives, and pure
    second derivatives (the derivative tree of fbpinns/trainers.py:63-107
    restricted to order <= 2 without mixed terms).
    """
    mask = 0
    for req in required_ujss:
        for iu, ixs in req:
            if iu != 0:
                raise NotImplementedError("only scalar solutions (ud=1) are compiled")
            if len(ixs) > 2:
                raise NotImplementedError(f"derivative order {len(ixs)} > 2 is not compiled")
            if len(ixs) == 2:
                if ixs[0] != ixs[1]:
                    raise NotImplementedError(f"mixed derivative {ixs} is not compiled")
                mask |= 1 << ixs[0]
            for ix in ixs:
                if not 0 <= ix < xd:
                    raise ValueError(f"derivative index {ix} out of range for xd={xd}")
    return mask


def jet_index(xd, d2mask, ixs):
    """Component of the jet layout holding d^len(ixs) u / dx_ixs."""
    if len(ixs) == 0:
        return 0
    if len(ixs) == 1:
        return 1 + ixs[0]
    d = ixs[0]
    group = _lib.d2_group(d2mask)
    if (group >> d) & 1:
        raise ValueError(f"d2mask {d2mask} sums d2/dx{d}^2 into its group slot (no single component)")
    singles = d2mask & 7 & ~group
    return 1 + xd + (1 if group else 0) + bin(singles & ((1 << d) - 1)).count("1")


def laplacian_index(xd, d2mask):
    """Component holding the sum of the group's pure second derivatives
    (FBP_D2_LAPLACIAN or FBP_D2_GROUP)."""
    if not _lib.d2_group(d2mask):
        raise ValueError(f"d2mask {d2mask} has no Laplacian slot")
    return 1 + xd


def jet_size(xd, d2mask):
    group = _lib.d2_group(d2mask)
    return 1 + xd + (1 if group else 0) + bin(d2mask & 7 & ~group).count("1")


def record_stride(J):
    """Row stride (floats) of the pair / slot jet records: 2J rounded up to 4."""
    return (2 * J + 3) // 4 * 4


def _pow2_floor(v):
    v = max(int(v), 1)
    return 1 << (v.bit_length() - 1)


def work_item_sizes(s_cap, m, sms, chunk, forward_chunk, adaptive=True):
    """(adjoint pairs per item, forward pairs per item, counter schedule?) for
    up to s_cap pairs over m subdomains on sms SMs.  The requested sizes are
    cut to powers of two (at least 128) so that a small step still gives
    every SM about 8 adjoint and 4 forward items; the counter-based schedule
    pays only with more items than resident CTAs (4 per SM)."""
    adj, fwd = int(chunk), max(int(chunk), int(forward_chunk))
    if adaptive:
        adj = min(adj, max(128, _pow2_floor(s_cap // (8 * sms))))
        fwd = min(fwd, max(adj, _pow2_floor(s_cap // (4 * sms))))
    return adj, fwd, s_cap // adj + m > 4 * sms


class PointSet:
    """Interaction lists, subdomain-major pair order, work queues and jet buffers
    of one set of points ``x`` (n, xd) on the device.

    Sizes are either read back once (``caps=None``; like the reference's
    ``s.item()``) or fixed capacities (``caps=(s_cap, u_cap)``), in which case
    ``rebuild`` runs without any host synchronisation and overflow is
    reported in ``status``.
    """

    def __init__(self, engine, x, select=None, caps=None, chunk=None, scheduled=False):
        self.eng = engine
        g = engine.grid
        self.n = int(x.shape[0])
        self.x = x.to(g.device, torch.float32).contiguous()
        self.J = engine.J
        # scheduled training: the training points of the engine's scheduler mask
        # (eng.raw) are selected on the device; only their pairs are sorted into
        # the work queues and only they enter the loss
        self.scheduled = bool(scheduled)
        if self.scheduled:
            self.pt_keep = torch.zeros(max(self.n, 1), dtype=torch.uint8, device=g.device)
            self.n_keep = torch.zeros(1, dtype=torch.int32, device=g.device)
        # requested pairs per adjoint / forward work item (the sizes used are set
        # with the buffers: smaller for small pair counts, see _allocate)
        self.chunk_req = int(chunk or engine.chunk)
        self.fwd_req = max(self.chunk_req, engine.forward_chunk)
        self.select = select
        s_cap, u_cap = (None, None) if caps is None else caps
        self.takes = PointTakes(g, self.n, s_cap=s_cap, u_cap=u_cap)
        self.fixed_caps = caps is not None
        self._sized = False
        if caps is not None:
            self._allocate(int(s_cap), int(u_cap))
        self.rebuild()

    # -- buffers -----------------------------------------------------------
    def _allocate(self, s_cap, u_cap):
        eng, dev, m = self.eng, self.eng.device, self.eng.m
        self.s_cap, self.u_cap = s_cap, u_cap
        i32 = dict(dtype=torch.int32, device=dev)
        self.sd_start = torch.zeros(m + 1, **i32)
        # sorted pair records (pair, point, slot, 0); the three views below
        self.sd_rec = torch.zeros((max(s_cap, 1), 4), **i32)
        self.sd_pair, self.sd_point, self.sd_slot = self.sd_rec[:, 0], self.sd_rec[:, 1], self.sd_rec[:, 2]
        lib = _lib.load()
        self.sort_scratch = torch.empty(int(lib.fbp_sort_scratch_bytes(s_cap, m)) // 4 + 1, **i32)
        self.work_scratch = torch.empty(int(lib.fbp_work_scratch_bytes(m)) // 4 + 1, **i32)
        # Work-item sizes: the requested ones, cut (to powers of two) so that a
        # small step still gives every SM several adjoint items and a few
        # forward items; a dynamic schedule only when there are more items than
        # resident CTAs (otherwise its counter reset costs more than it saves)
        self.chunk, self.fwd_chunk, self.dynamic = work_item_sizes(s_cap, m, eng.sm_count, self.chunk_req,
                                                                   self.fwd_req, eng.adaptive_items)
        self.items_cap = s_cap // self.chunk + m + 1
        self.forward_items_cap = s_cap // self.fwd_chunk + m + 1  # the forward queue's items fit in this
        self.items_all = torch.zeros(3 * self.items_cap, **i32)
        self.items_act = torch.zeros(3 * self.items_cap, **i32)
        self.item_start_all = torch.zeros(m + 1, **i32)
        self.item_start_act = torch.zeros(m + 1, **i32)
        self.n_items_all = torch.zeros(1, **i32)
        self.n_items_act = torch.zeros(1, **i32)
        # work-item counters of the forward [0] and adjoint [1] launches (dynamic schedule)
        self.item_ctr = torch.zeros(2, **i32)
        R = record_stride(self.J)
        self.pair_out = torch.empty((max(s_cap, 1), R), dtype=torch.float32, device=dev)
        self.slot_out = torch.empty((max(u_cap, 1), R), dtype=torch.float32, device=dev)
        self.grad_part = torch.empty((self.items_cap, eng.P), dtype=torch.float32, device=dev)
        self.U = torch.empty((self.n, self.J), dtype=torch.float32, device=dev)
        # layer-2 z-jets of every sorted pair, written by the forward and read by
        # the adjoint of a training step (fbp_pairs.zs): J * h2 rows of s_cap
        self.zs = None
        if eng.z2_rows and eng.z2_rows * max(s_cap, 1) * 4 <= eng.z2_limit:
            self.zs = torch.empty((eng.z2_rows, max(s_cap, 1)), dtype=torch.float32, device=dev)
        self._sized = True

    def rebuild(self, stream=None, state=None):
        """(Re)build lists, sort and work queues for the current points and state."""
        eng = self.eng
        lib = _lib.load()
        st = _lib.stream_ptr(stream)
        sizes = self.takes.build(self.x, self.select, stream, count_models=False)
        if sizes is not None:
            s, u = sizes
            if not self._sized or s > self.s_cap or u > self.u_cap:
                self._allocate(s, u)
            self.s, self.u = s, u
        if self.scheduled:
            self.rebuild_scheduled(stream)
            return
        t = self.takes
        _lib.check(lib.fbp_sort_pairs(_lib.ptr(t.m_take), _lib.ptr(t.n_take), _lib.ptr(t.p_take),
                                      _lib.ptr(t.pt_off[self.n:]), self.s_cap, eng.m, _lib.ptr(self.sd_start),
                                      _lib.ptr(self.sd_rec), _lib.ptr(self.sort_scratch), self.sort_scratch.numel() * 4, st),
                   "fbp_sort_pairs")
        self.build_work(stream, state)

    def rebuild_scheduled(self, stream=None):
        """For the lists of this point set (unchanged): the training points and
        subdomain states of the engine's scheduler mask (eng.raw), the sort of
        the training points' pairs and the work queues -- all on the device,
        no host synchronisation (fbpinns/trainers.py:482-575 per mask change)."""
        eng, t = self.eng, self.takes
        lib = _lib.load()
        st = _lib.stream_ptr(stream)
        _lib.check(lib.fbp_train_mask(_lib.ptr(t.pt_off), _lib.ptr(t.m_take), self.n, self.s_cap, _lib.ptr(eng.raw),
                                      eng.m, _lib.ptr(self.pt_keep), _lib.ptr(self.n_keep), _lib.ptr(eng.state),
                                      _lib.ptr(eng.active), st), "fbp_train_mask")
        _lib.check(lib.fbp_sort_pairs_kept(_lib.ptr(t.m_take), _lib.ptr(t.n_take), _lib.ptr(t.p_take),
                                           _lib.ptr(self.pt_keep), _lib.ptr(t.pt_off[self.n:]), self.s_cap, eng.m,
                                           _lib.ptr(self.sd_start), _lib.ptr(self.sd_rec), _lib.ptr(self.sort_scratch),
                                           self.sort_scratch.numel() * 4, st), "fbp_sort_pairs_kept")
        self.build_work(stream)

    def build_work(self, stream=None, state=None):
        """Work queues: all subdomains with pairs (forward) and the active ones (adjoint)."""
        eng = self.eng
        lib = _lib.load()
        st = _lib.stream_ptr(stream)
        ws = self.work_scratch.numel() * 4
        _lib.check(lib.fbp_build_work(_lib.ptr(self.sd_start), eng.m, None, self.fwd_chunk, _lib.ptr(self.items_all),
                                      _lib.ptr(self.item_start_all), _lib.ptr(self.n_items_all), self.items_cap,
                                      _lib.ptr(t_status(self)), _lib.ptr(self.work_scratch), ws, st),
                   "fbp_build_work")
        active = eng.active if state is None else state
        self.adj_select = active.contiguous()
        _lib.check(lib.fbp_build_work(_lib.ptr(self.sd_start), eng.m, _lib.ptr(self.adj_select), self.chunk,
                                      _lib.ptr(self.items_act), _lib.ptr(self.item_start_act),
                                      _lib.ptr(self.n_items_act), self.items_cap, _lib.ptr(t_status(self)),
                                      _lib.ptr(self.work_scratch), ws, st), "fbp_build_work")

    def pairs_struct(self, adjoint=False, z2=True):
        """The launch's fbp_pairs; z2: pass the stored layer-2 z-jets buffer
        (when this point set has one) -- only for a forward and the adjoint
        that follows it with the same parameters."""
        p = _lib.Pairs()
        p.sd_start, p.sd_rec = _lib.ptr(self.sd_start), _lib.ptr(self.sd_rec)
        if adjoint:
            p.items, p.n_items = _lib.ptr(self.items_act), _lib.ptr(self.n_items_act)
        else:
            p.items, p.n_items = _lib.ptr(self.items_all), _lib.ptr(self.n_items_all)
        p.items_cap = self.items_cap
        p.slots_cap = self.slot_out.shape[0]
        sched = self.eng.schedule if adjoint else self.eng.fwd_schedule()
        if sched == "dynamic" and self.dynamic:
            p.item_ctr = _lib.ptr(self.item_ctr[1 if adjoint else 0])
        if z2 and self.zs is not None:
            p.zs, p.zs_cap = _lib.ptr(self.zs), self.zs.shape[1]
        return p

    def subdomain_counts(self):
        """Pairs per subdomain (from the subdomain-major order), int64 on the device."""
        st = self.sd_start.long()
        return st[1:] - st[:-1]

    def check_status(self):
        self.takes.check_status()


def t_status(ps):
    return ps.takes.status


def tc_supported(xd, h1, h2, d2mask=3 | _lib.D2_LAPLACIAN, act=_lib.ACT_TANH):
    """True where the tensor-core forward kernel is compiled (xd = 2, two
    16-wide hidden layers; the jet masks and activations of fbp_has_tc_shape)."""
    return bool(_lib.load().fbp_has_tc_shape(xd, h1, h2, d2mask, act))


class FBPINNEngine:
    """Packed parameters + kernel launches for one decomposition and network shape."""

    def __init__(self, static_decomp, layer_sizes, d2mask, device="cuda", chunk=1024, grid=None, tensor_cores=None,
                 activation="tanh", schedule="dynamic", forward_chunk=None, adaptive_items=True, tc_adjoint=None,
                 store_z2=None, cell_order=True):
        if not torch.cuda.is_available():
            raise _lib.FBPLibraryError("the FBPINN engine needs a CUDA device (no CPU fallback)")
        _lib.load()
        self.device = torch.device(device)
        self.grid = grid_of(static_decomp, self.device)
        self.m, self.xd = self.grid.m, self.grid.xd
        ls = list(layer_sizes)
        if ls[0] != self.xd:
            raise ValueError(f"network input {ls[0]} != decomposition xd {self.xd}")
        if ls[-1] != 1:
            raise NotImplementedError("only scalar-output networks are compiled (ud=1)")
        if len(ls) not in (3, 4):
            raise NotImplementedError("the compiled FCN jets have one or two hidden layers")
        self.layer_sizes = ls
        self.h1 = ls[1]
        self.h2 = ls[2] if len(ls) == 4 else 0
        self.P = None  # set below from the activation's parameter count
        self.d2mask = int(d2mask)
        if activation not in _lib.ACTIVATIONS:
            raise ValueError(f"activation must be one of {sorted(_lib.ACTIVATIONS)}, not {activation!r}")
        self.activation = activation
        self.act = _lib.ACTIVATIONS[activation]
        self.extra = _lib.ACT_EXTRA[activation]  # activation parameters per neuron and layer
        self.P = fcn_param_count(ls, self.extra)
        if not _lib.load().fbp_has_shape(self.xd, self.h1, self.h2, self.d2mask, self.act):
            raise _lib.FBPLibraryError(
                f"no compiled jet kernels for layer sizes {ls} ({activation}) with second derivatives along dims "
                f"{[d for d in range(self.xd) if (self.d2mask >> d) & 1]}"
                f"{' (Laplacian slot)' if self.d2mask & _lib.D2_LAPLACIAN else ''}; "
                f"add the shape to csrc/jet_inst_*.cu")
        self.J = jet_size(self.xd, self.d2mask)
        self.chunk = int(chunk)
        # forward work items may be longer: its per-item set-up (weights, B
        # operands, the tile pipeline's fill and drain) is larger
        self.forward_chunk = int(forward_chunk) if forward_chunk else 4 * self.chunk
        self.launch_grid = int(grid) if grid else 0
        # CTAs of the forward launch when set (0 = every CTA that can be
        # resident); None: the same as launch_grid.  Set by the autotuner.
        self.forward_grid = None
        # how the jet kernels' CTAs take work items (the results do not depend on it):
        #   "dynamic"   a resident grid; each CTA takes the next item from a device counter
        #   "static"    a resident grid; CTA b takes items b, b + grid, ...
        #   "per_item"  one CTA per item (grid = the queue's capacity); CTAs retire
        #               as they finish, so kernels of a higher-priority stream get
        #               SM slots during the launch
        if schedule not in ("dynamic", "static", "per_item"):
            raise ValueError(f"schedule must be 'dynamic', 'static' or 'per_item', not {schedule!r}")
        self.schedule = schedule
        # the forward launch's own schedule when set (None: the same as schedule);
        # set by the autotuner, which searches the two separately
        self.forward_schedule = None
        # cut the work-item sizes for small pair counts (PointSet._allocate)
        self.adaptive_items = bool(adaptive_items)
        self.sm_count = torch.cuda.get_device_properties(self.device).multi_processor_count
        # forward jets on the tensor cores (3xTF32) where that kernel is compiled:
        # None = for the plain tanh FCN wherever available (for the other
        # activations, whose sin/cos/tanh calls dominate, the FMA kernel is as
        # fast), True = required, False = CUDA-core FMA kernel
        tc_ok = tc_supported(self.xd, self.h1, self.h2, self.d2mask, self.act)
        if tensor_cores and not tc_ok:
            raise _lib.FBPLibraryError(f"no tensor-core forward kernel for layer sizes {ls} ({activation}, "
                                       f"d2mask {self.d2mask}); compiled: 2-16-16-1 networks")
        self.tensor_cores = (tc_ok and self.act == _lib.ACT_TANH) if tensor_cores is None else bool(tensor_cores)
        # adjoint with the layer-2 recompute on the tensor cores (fbp_adjoint_pairs_tc):
        # None = off unless requested; True = required; False = off
        tca_ok = bool(_lib.load().fbp_has_tc_adjoint_shape(self.xd, self.h1, self.h2, self.d2mask, self.act))
        if tc_adjoint and not tca_ok:
            raise _lib.FBPLibraryError(f"no tensor-core adjoint kernel for layer sizes {ls} ({activation}, "
                                       f"d2mask {self.d2mask}); compiled: xd-16-16-1 tanh networks")
        self.tc_adjoint = bool(tc_adjoint) and tca_ok
        # store_z2: the forward of a training step stores the layer-2 z-jets of
        # every pair (J * h2 floats) and the FMA adjoint reads them instead of
        # recomputing layer 2 (h1 multiply-adds per stored value); a point set
        # keeps the buffer while it takes at most z2_limit bytes (an eighth of
        # the device memory), else the adjoint recomputes.  None: where the first
        # hidden layer is at least 32 wide (measured: 3-32-32-1 gains, 2-16-16-1
        # loses -- its stores cost the forward more than the reads save in the
        # latency-bound adjoint)
        if store_z2 is None:
            store_z2 = self.h1 >= 32
        self.z2_rows = self.J * self.h2 if (store_z2 and self.h2 > 0 and not self.tc_adjoint) else 0
        self.z2_limit = torch.cuda.get_device_properties(self.device).total_memory // 8
        # sample(): uniform batches in the order of a Morton cell grid (locality of
        # the lists and jets; the same points, so the same batch)
        self.cell_order = bool(cell_order)
        self._order_bufs = {}
        # the decomposition's bounding box: the cell grid of batches given by the caller
        self.extent = (self.grid.xmins.min(0).values.double().cpu().tolist(),
                       self.grid.xmaxs.max(0).values.double().cpu().tolist())
        dev = self.device
        self.theta = torch.zeros((self.m, self.P), dtype=torch.float32, device=dev)
        self.m1 = torch.zeros_like(self.theta)
        self.m2 = torch.zeros_like(self.theta)
        self.count = torch.zeros(1, dtype=torch.int32, device=dev)
        self.state = torch.ones(self.m, dtype=torch.uint8, device=dev)
        self.active = torch.ones(self.m, dtype=torch.uint8, device=dev)  # state == 1, the adjoint's selection
        # the scheduler's raw mask (0 inactive, 1 active, 2 fixed) for point sets that
        # derive state and active from it on the device (PointSet(scheduled=True))
        self.raw = torch.ones(self.m, dtype=torch.uint8, device=dev)
        self.grad = torch.zeros_like(self.theta)
        nparts = 8 * torch.cuda.get_device_properties(dev).multi_processor_count + 1
        self.loss_part = torch.zeros(nparts, dtype=torch.float64, device=dev)
        self.loss = torch.zeros(1, dtype=torch.float64, device=dev)
        self.npou = self.grid.npou
        self._problem = None

    def fwd_schedule(self):
        return self.schedule if self.forward_schedule is None else self.forward_schedule

    # -- parameters ----------------------------------------------------------
    def set_theta(self, theta):
        self.theta.copy_(theta.to(self.device, torch.float32).reshape(self.m, self.P))

    def set_state(self, active):
        """active: (m,) ints, 0 = not trained, 1 = active, 2 = fixed (after get_inputs masking)."""
        self.state.copy_(torch.as_tensor(np.asarray(active), dtype=torch.uint8).to(self.device))
        self.active.copy_((self.state == 1).to(torch.uint8))

    def set_raw_state(self, active):
        """The scheduler's mask as it yields it (0, 1, 2 per subdomain), for
        scheduled point sets; one host-to-device copy of m bytes."""
        a = np.asarray(active)
        if a.shape != (self.m,) or not np.isin(a, (0, 1, 2)).all():
            raise ValueError(f"scheduler mask must be ({self.m},) with values 0, 1, 2")
        self.raw.copy_(torch.as_tensor(a.astype(np.uint8)), non_blocking=False)

    def net_struct(self, theta=None, d2mask=None):
        g = self.grid
        n = _lib.Net()
        n.xd, n.h1, n.h2, n.ud = self.xd, self.h1, self.h2, 1
        n.d2mask = self.d2mask if d2mask is None else d2mask
        n.nparam = self.P
        n.act = self.act
        n.theta = _lib.ptr(self.theta if theta is None else theta)
        n.xmins, n.xmaxs, n.flags, n.unnorms = _lib.ptr(g.xmins), _lib.ptr(g.xmaxs), _lib.ptr(g.flags), _lib.ptr(g.unnorms)
        n.m = self.m
        n.window, n.wmins, n.wmaxs = g.window, _lib.ptr(g.wmins), _lib.ptr(g.wmaxs)
        return n

    def set_problem(self, spec):
        """Fused residual of a built-in problem (problems.Problem.fused_spec)."""
        if spec is None:
            self._problem = None
            return
        pr = _lib.Problem()
        pr.kind = int(spec["kind"])
        pr.n_int = int(spec.get("n_int", 0))
        for i, v in enumerate(spec.get("p", [])):
            pr.p[i] = float(v)
        gauss = spec.get("gauss")
        if gauss is not None:
            self._gauss = torch.as_tensor(gauss, dtype=torch.float32).to(self.device).contiguous()
            pr.gauss, pr.ng = _lib.ptr(self._gauss), int(self._gauss.shape[0])
        else:
            self._gauss = None
            pr.gauss, pr.ng = None, 0
        self._problem = pr

    # -- kernels -------------------------------------------------------------
    def points(self, x, select=None, caps=None, chunk=None, scheduled=False):
        return PointSet(self, x, select=select, caps=caps, chunk=chunk, scheduled=scheduled)

    def forward_pairs(self, ps, theta=None, stream=None, z2=True):
        """Per-pair jets into ps.pair_out; z2: also store the layer-2 z-jets
        for an adjoint that follows (False for jets that are not differentiated)."""
        lib = _lib.load()
        net = self.net_struct(theta)
        pr = ps.pairs_struct(False, z2)
        grid = ps.forward_items_cap if self.fwd_schedule() == "per_item" else \
            (self.launch_grid if self.forward_grid is None else self.forward_grid)
        if self.tensor_cores:
            _lib.check(lib.fbp_forward_pairs_tc(C.byref(net), _lib.ptr(ps.x), C.byref(pr), _lib.ptr(ps.pair_out),
                                                _lib.ptr(ps.takes.status), grid, _lib.stream_ptr(stream)),
                       "fbp_forward_pairs_tc")
            return
        _lib.check(lib.fbp_forward_pairs(C.byref(net), _lib.ptr(ps.x), C.byref(pr), _lib.ptr(ps.pair_out),
                                         grid, _lib.stream_ptr(stream)), "fbp_forward_pairs")

    def pou_forward(self, ps, stream=None):
        lib = _lib.load()
        t = ps.takes
        _lib.check(lib.fbp_pou_forward(self.xd, self.d2mask, ps.n, self.npou, _lib.ptr(t.pt_off), _lib.ptr(t.p_take),
                                       _lib.ptr(ps.pair_out), _lib.ptr(ps.slot_out), _lib.ptr(ps.U),
                                       ps.pair_out.shape[0], ps.slot_out.shape[0], _lib.ptr(t.status),
                                       _lib.stream_ptr(stream)), "fbp_pou_forward")
        return ps.U

    def pou_backward(self, ps, Ubar, stream=None):
        lib = _lib.load()
        Ubar = Ubar.to(torch.float32).contiguous()
        _lib.check(lib.fbp_pou_backward(self.xd, self.d2mask, ps.n, self.npou, _lib.ptr(ps.takes.np_off),
                                        _lib.ptr(Ubar), _lib.ptr(ps.slot_out), ps.slot_out.shape[0],
                                        _lib.stream_ptr(stream)),
                   "fbp_pou_backward")

    def pou_loss(self, ps, U_out=None, stream=None):
        if self._problem is None:
            raise RuntimeError("set_problem() first: the fused loss needs a built-in problem")
        lib = _lib.load()
        t = ps.takes
        st = _lib.stream_ptr(stream)
        pr = self._problem
        pr.pt_keep, pr.n_keep = (_lib.ptr(ps.pt_keep), _lib.ptr(ps.n_keep)) if ps.scheduled else (None, None)
        _lib.check(lib.fbp_pou_loss(self.xd, self.d2mask, C.byref(self._problem), ps.n, self.npou, _lib.ptr(ps.x),
                                    _lib.ptr(t.pt_off), _lib.ptr(t.np_off), _lib.ptr(t.p_take), _lib.ptr(ps.pair_out),
                                    _lib.ptr(ps.slot_out), _lib.ptr(U_out), ps.pair_out.shape[0], ps.slot_out.shape[0],
                                    _lib.ptr(self.loss_part),
                                    self.loss_part.numel(), _lib.ptr(t.status), st), "fbp_pou_loss")
        # a scheduled point set's partials are already divided by its training-point count
        _lib.check(lib.fbp_loss_finalize(_lib.ptr(self.loss_part), self.loss_part.numel(),
                                         1.0 if ps.scheduled else 1.0 / ps.n, _lib.ptr(self.loss), st),
                   "fbp_loss_finalize")
        return self.loss

    def adjoint(self, ps, theta=None, out=None, stream=None, reduce=True, z2=True):
        """Gradient partials of the loss seeds in ps.slot_out; z2: read the
        layer-2 z-jets stored by the forward_pairs(..., z2=True) that preceded
        it with the same parameters (False: recompute them)."""
        lib = _lib.load()
        st = _lib.stream_ptr(stream)
        net = self.net_struct(theta)
        pr = ps.pairs_struct(True, z2)
        grid = ps.items_cap if self.schedule == "per_item" else self.launch_grid
        if self.tc_adjoint:
            _lib.check(lib.fbp_adjoint_pairs_tc(C.byref(net), _lib.ptr(ps.x), C.byref(pr), _lib.ptr(ps.slot_out),
                                                _lib.ptr(ps.grad_part), _lib.ptr(ps.takes.status), grid, st),
                       "fbp_adjoint_pairs_tc")
        else:
            _lib.check(lib.fbp_adjoint_pairs(C.byref(net), _lib.ptr(ps.x), C.byref(pr), _lib.ptr(ps.slot_out),
                                             _lib.ptr(ps.grad_part), grid, st), "fbp_adjoint_pairs")
        if not reduce:
            return None
        return self.reduce_grad(ps, out, stream)

    def reduce_grad(self, ps, out=None, stream=None):
        """grad[j] = sum of subdomain j's work-item partials, in item order."""
        lib = _lib.load()
        out = self.grad if out is None else out
        _lib.check(lib.fbp_grad_reduce(_lib.ptr(ps.grad_part), _lib.ptr(ps.item_start_act), self.m, self.P,
                                       _lib.ptr(out), _lib.stream_ptr(stream)), "fbp_grad_reduce")
        return out

    def adam(self, lr, b1=0.9, b2=0.999, eps=1e-8, eps_root=0.0, grad=None, stream=None):
        lib = _lib.load()
        g = self.grad if grad is None else grad
        _lib.check(lib.fbp_adam(_lib.ptr(self.theta), _lib.ptr(self.m1), _lib.ptr(self.m2), _lib.ptr(g),
                                _lib.ptr(self.state), self.m, self.P, lr, b1, b2, eps, eps_root,
                                _lib.ptr(self.count), _lib.stream_ptr(stream)), "fbp_adam")

    def fused_step(self, ps, lr, stream=None, **adam_kw):
        """One training step on point set ps; returns the device loss (float64, 1 elem)."""
        self.forward_pairs(ps, stream=stream)
        loss = self.pou_loss(ps, stream=stream)
        self.adjoint(ps, stream=stream)
        self.adam(lr, stream=stream, **adam_kw)
        return loss

    def sample(self, x_out, seed, offset, xmin, xmax, counter=None, stream=None, order=None):
        """Uniform points into x_out; the stream offset is offset + *counter.
        order (None: the engine's cell_order): the drawn batch in the order of
        the Morton cells of [xmin, xmax] (fbp_sort_points_cells), the same
        points for the same seed and offset."""
        lib = _lib.load()
        lo = (C.c_double * 3)(*[float(v) for v in xmin])
        hi = (C.c_double * 3)(*[float(v) for v in xmax])
        n = int(x_out.shape[0])
        order = (self.cell_order if order is None else bool(order)) and n > 0
        dst = self._order_buffers(n)[0] if order else x_out
        _lib.check(lib.fbp_sample_uniform(_lib.ptr(dst), n, self.xd, lo, hi, int(seed), int(offset),
                                          _lib.ptr(counter), _lib.stream_ptr(stream)), "fbp_sample_uniform")
        if order:
            self.order_points(dst, x_out, stream, (xmin, xmax))

    def _order_buffers(self, n):
        """(drawn batch, sort scratch) for batches of n points, kept per size:
        the resampled and host-point steps order one batch at a time, on one stream."""
        buf = self._order_bufs.get(n)
        if buf is None:
            nb = int(_lib.load().fbp_sort_points_scratch_bytes(n, self.xd))
            buf = (torch.empty((n, self.xd), dtype=torch.float32, device=self.device),
                   torch.empty(nb // 4 + 1, dtype=torch.int32, device=self.device))
            self._order_bufs[n] = buf
        return buf

    def order_points(self, x_in, x_out, stream=None, box=None):
        """x_out = the points x_in in Morton cell order over box (default: the
        decomposition's bounding box), fbp_sort_points_cells."""
        lib = _lib.load()
        n = int(x_in.shape[0])
        if n == 0:
            return
        xmin, xmax = self.extent if box is None else box
        lo = (C.c_double * 3)(*[float(v) for v in xmin])
        hi = (C.c_double * 3)(*[float(v) for v in xmax])
        scratch = self._order_buffers(n)[1]
        _lib.check(lib.fbp_sort_points_cells(_lib.ptr(x_in), n, self.xd, lo, hi, _lib.ptr(x_out), _lib.ptr(scratch),
                                             scratch.numel() * 4, _lib.stream_ptr(stream)), "fbp_sort_points_cells")


class FBPINNJet(torch.autograd.Function):
    """theta (m, P) -> per-point jets U (n, J) of the POU-combined network output.

    forward: per-pair jet kernel + POU combination; backward: POU seeds +
    per-pair adjoint kernel + gradient reduction.  Replaces the nested jvp of
    ``FBPINN_model`` under ``value_and_grad`` (fbpinns/trainers.py:126-177,
    197-247, 292) up to the constraining operator.
    """

    @staticmethod
    def forward(ctx, theta, engine, ps):
        theta = theta.contiguous()
        # autograd may run other forwards on ps before this backward: no stored z-jets
        engine.forward_pairs(ps, theta, z2=False)
        U = engine.pou_forward(ps).clone()
        ctx.engine, ctx.ps = engine, ps
        ctx.save_for_backward(theta)
        return U

    @staticmethod
    def backward(ctx, Ubar):
        (theta,) = ctx.saved_tensors
        eng, ps = ctx.engine, ctx.ps
        eng.pou_backward(ps, Ubar)
        grad = torch.empty_like(theta)
        eng.adjoint(ps, theta, out=grad, z2=False)
        return grad, None, None


def constrained_jets(cfn, all_params, x, U, xd, d2mask, need=None):
    """Jets of constraining_fn(all_params, x, u(x)) from the jets U of u.

    For each dim d the Taylor model u(x + t e_d) = U0 + t U_d + t^2/2 U_dd is
    pushed through cfn with nested forward-mode jvp in t (torch.func), which
    gives d/dx_d and d^2/dx_d^2 of the constrained solution exactly, for any
    constraining_fn; reverse mode through it is plain autograd.

    A constraining_fn that returns its u argument itself (the identity of the
    reference's soft-constraint problems) leaves the jets as they are: U is
    returned.  ``need`` (optional jet indices) limits the work to the dims
    whose components are needed; the other components are zero.
    """
    n = x.shape[0]
    J = U.shape[1]
    out = [None] * J
    u0 = U[:, 0:1]
    out[0] = cfn(all_params, x, u0)
    if out[0] is u0:
        return U
    ones = torch.ones((n, 1), dtype=x.dtype, device=x.device)
    zero = torch.zeros((n, 1), dtype=x.dtype, device=x.device)
    for d in range(xd):
        comps = {1 + d} | ({jet_index(xd, d2mask, (d, d))} if (d2mask >> d) & 1 else set())
        if need is not None and not (comps & set(need)):
            for k in comps:
                out[k] = torch.zeros_like(out[0])
            continue
        e = torch.zeros((1, xd), dtype=x.dtype, device=x.device)
        e[0, d] = 1.0
        ud = U[:, 1 + d:2 + d]
        has2 = (d2mask >> d) & 1
        if has2:
            k = jet_index(xd, d2mask, (d, d))
            udd = U[:, k:k + 1]

            def h(t, ud=ud, udd=udd, e=e):
                return cfn(all_params, x + t * e, u0 + t * ud + 0.5 * t * t * udd)

            def g(t, h=h):
                return torch.func.jvp(h, (t,), (ones,))[1]

            d1, d2 = torch.func.jvp(g, (zero,), (ones,))
            out[1 + d], out[k] = d1, d2
        else:
            def h(t, ud=ud, e=e):
                return cfn(all_params, x + t * e, u0 + t * ud)

            out[1 + d] = torch.func.jvp(h, (zero,), (ones,))[1]
    return torch.cat(out, dim=1)


def inference_d2mask(layer_sizes, activation="tanh"):
    """A compiled jet mask for value-only evaluation of this network shape."""
    lib = _lib.load()
    xd = layer_sizes[0]
    h1 = layer_sizes[1]
    h2 = layer_sizes[2] if len(layer_sizes) == 4 else 0
    act = _lib.ACTIVATIONS[activation]
    for mask in list(range(1 << xd)) + [m | _lib.D2_LAPLACIAN for m in range(1, 1 << xd)]:
        if lib.fbp_has_shape(xd, h1, h2, mask, act):
            return mask
    raise _lib.FBPLibraryError(f"no compiled jet kernels for layer sizes {list(layer_sizes)} ({activation})")
