"""Interaction lists on the GPU (the reference's ``inside_points`` /
``inside_models`` / ``get_inputs`` integer work).

``PointTakes`` owns the device buffers of one point set: per-point counts and
level masks, their scans, the point-major pair lists (n_take, m_take, p_take)
and the unique (point, level) slots (np_take).  Results equal the reference's
bit for bit (fbpinns/decompositions_base.py:24-84, fbpinns/trainers.py:332-419).
"""

import ctypes as C

import numpy as np
import torch

from . import _lib
from .decompositions import build_cell_grid, subdomain_arrays, npou_of


class CellGrid:
    """Device copy of a decomposition's boxes and their uniform cell grid."""

    def __init__(self, static, device="cuda"):
        xmins, xmaxs, flags, unnorms, pou = subdomain_arrays(static)
        if int(pou.min()) < 0 or int(pou.max()) >= 64:
            raise ValueError("POU levels must lie in [0, 64) for the GPU interaction lists")
        self.m, self.xd = xmins.shape
        if self.xd > 3:
            raise ValueError(f"xd={self.xd}: only 1-3 input dimensions are compiled")
        g = build_cell_grid(xmins.numpy(), xmaxs.numpy())
        self.device = torch.device(device)
        self.xmins = xmins.to(self.device).contiguous()
        self.xmaxs = xmaxs.to(self.device).contiguous()
        self.flags = flags.to(self.device).contiguous()
        self.unnorms = unnorms.to(self.device).contiguous()
        self.pou = pou.to(self.device).contiguous()
        # window of the subdomain networks and the overlap widths the sigmoid window reads
        from .decompositions import WINDOWS
        self.window = WINDOWS.index(static.get("window", "cosine"))
        p = static["subdomain"]["params"]
        self.wmins = p[2].float().to(self.device).contiguous()
        self.wmaxs = p[3].float().to(self.device).contiguous()
        self.cell_start = torch.as_tensor(g["cell_start"], device=self.device)
        self.cell_boxes = torch.as_tensor(g["cell_boxes"], device=self.device)
        self.ncell, self.lo, self.inv_h = g["ncell"], g["lo"], g["inv_h"]
        self.npou = npou_of(static)

    def boxes(self, select=None):
        b = _lib.Boxes()
        b.xmins, b.xmaxs, b.pou = _lib.ptr(self.xmins), _lib.ptr(self.xmaxs), _lib.ptr(self.pou)
        b.select = _lib.ptr(select) if select is not None else None
        b.m, b.xd = self.m, self.xd
        for d in range(self.xd):
            b.ncell[d] = int(self.ncell[d])
            b.lo[d] = float(self.lo[d])
            b.inv_h[d] = float(self.inv_h[d])
        b.cell_start, b.cell_boxes = _lib.ptr(self.cell_start), _lib.ptr(self.cell_boxes)
        return b


def grid_of(static, device="cuda"):
    """The cached CellGrid of a decomposition's static params."""
    key = "_gpu_cell_grid"
    g = static.get(key)
    if g is None or g.device != torch.device(device):
        g = CellGrid(static, device)
        static[key] = g
    return g


def _scan(lib, src, dst, n, stream):
    scratch = torch.empty(int(lib.fbp_scan_scratch_bytes(n)) // 4 + 1, dtype=torch.int32, device=src.device)
    _lib.check(lib.fbp_scan_i32(_lib.ptr(src), _lib.ptr(dst), n, _lib.ptr(scratch), scratch.numel() * 4, stream),
               "fbp_scan_i32")


class PointTakes:
    """Interaction lists of one point set, built by count -> scan -> fill.

    With ``s_cap``/``u_cap`` given, no host synchronisation happens (the
    capacity must cover the pairs; overflow is reported in ``status``); without
    them the exact sizes are read back first, like the reference's
    ``s.item()`` (fbpinns/decompositions_base.py:74).
    """

    def __init__(self, grid, n, s_cap=None, u_cap=None):
        self.grid, self.n = grid, int(n)
        dev = grid.device
        self.pt_count = torch.zeros(self.n, dtype=torch.int32, device=dev)
        self.pt_nlvl = torch.zeros(self.n, dtype=torch.int32, device=dev)
        self.pt_lvl = torch.zeros(self.n, dtype=torch.int64, device=dev)
        # hits of the count pass as candidate-list masks, read by the fill pass
        self.pt_hit = torch.zeros(self.n, dtype=torch.int64, device=dev)
        self.pt_cand = torch.zeros(self.n, dtype=torch.int32, device=dev)
        self.use_hit_masks = True
        self.pt_off = torch.zeros(self.n + 1, dtype=torch.int32, device=dev)
        self.np_off = torch.zeros(self.n + 1, dtype=torch.int32, device=dev)
        self.model_count = torch.zeros(grid.m, dtype=torch.int32, device=dev)
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        lib = _lib.load()
        self._scan_scratch = torch.empty(int(lib.fbp_scan_scratch_bytes(self.n)) // 4 + 1, dtype=torch.int32,
                                         device=dev)
        self.s_cap = s_cap
        self.u_cap = u_cap
        self._alloc(s_cap or 0, u_cap or 0)

    def _alloc(self, s_cap, u_cap):
        dev = self.grid.device
        if getattr(self, "n_take", None) is None or self.n_take.numel() < s_cap:
            self.n_take = torch.empty(max(s_cap, 1), dtype=torch.int32, device=dev)
            self.m_take = torch.empty(max(s_cap, 1), dtype=torch.int32, device=dev)
            self.p_take = torch.empty(max(s_cap, 1), dtype=torch.int32, device=dev)
        if getattr(self, "np_take", None) is None or self.np_take.numel() < u_cap:
            self.np_take = torch.empty(max(u_cap, 1), dtype=torch.int32, device=dev)

    def build(self, x, select=None, stream=None, count_models=True):
        """Count, scan and fill for points x (n, xd) float32 on the device.

        ``count_models`` also fills ``model_count`` (points per box, with
        atomics); the training step leaves it off and reads the per-subdomain
        counts from the pair sort instead.  Returns (s, u) as python ints when
        sizes were read back, else None.
        """
        lib = _lib.load()
        st = _lib.stream_ptr(stream)
        b = self.grid.boxes(select)
        assert x.is_cuda and x.dtype == torch.float32 and x.shape == (self.n, self.grid.xd)
        x = x.contiguous()
        # the status word is sticky: cleared only by reset_status()
        if count_models:
            self.model_count.zero_()
        _lib.check(lib.fbp_inside_count(_lib.ptr(x), self.n, C.byref(b), _lib.ptr(self.pt_count),
                                        _lib.ptr(self.pt_nlvl), _lib.ptr(self.pt_lvl),
                                        _lib.ptr(self.model_count) if count_models else None,
                                        _lib.ptr(self.pt_hit), _lib.ptr(self.pt_cand), st),
                   "fbp_inside_count")
        sb = self._scan_scratch.numel() * 4
        _lib.check(lib.fbp_scan_i32(_lib.ptr(self.pt_count), _lib.ptr(self.pt_off), self.n,
                                    _lib.ptr(self._scan_scratch), sb, st), "fbp_scan_i32")
        _lib.check(lib.fbp_scan_i32(_lib.ptr(self.pt_nlvl), _lib.ptr(self.np_off), self.n,
                                    _lib.ptr(self._scan_scratch), sb, st), "fbp_scan_i32")
        sizes = None
        if self.s_cap is None:
            s = int(self.pt_off[self.n].item())
            u = int(self.np_off[self.n].item())
            self._alloc(s, u)
            s_cap, u_cap = s, u
            sizes = (s, u)
        else:
            s_cap, u_cap = self.n_take.numel(), self.np_take.numel()
        _lib.check(lib.fbp_inside_fill(_lib.ptr(x), self.n, C.byref(b), _lib.ptr(self.pt_off), _lib.ptr(self.np_off),
                                       _lib.ptr(self.pt_lvl),
                                       _lib.ptr(self.pt_hit) if self.use_hit_masks else None,
                                       _lib.ptr(self.pt_cand) if self.use_hit_masks else None,
                                       _lib.ptr(self.n_take), _lib.ptr(self.m_take),
                                       _lib.ptr(self.p_take), _lib.ptr(self.np_take), s_cap, u_cap,
                                       _lib.ptr(self.status), st), "fbp_inside_fill")
        self._sizes = sizes
        return sizes

    def sizes(self):
        """(s, u) read back from the device."""
        return int(self.pt_off[self.n].item()), int(self.np_off[self.n].item())

    def reset_status(self):
        self.status.zero_()

    def check_status(self):
        w = int(self.status.item())
        if w:
            raise _lib.FBPLibraryError(f"interaction lists: {_lib.decode_status(w)}")


def _x_dev(x_batch, device):
    return torch.as_tensor(x_batch, dtype=torch.float32).to(device).contiguous()


def inside_points(static, x_batch):
    """(n_take, m_take, inside_ims), int32 device tensors (fbpinns/decompositions.py:202-208)."""
    g = grid_of(static)
    x = _x_dev(x_batch, g.device)
    t = PointTakes(g, x.shape[0])
    s, _ = t.build(x)
    inside_ims = torch.nonzero(t.model_count > 0).reshape(-1).to(torch.int32)
    return t.n_take[:s].clone(), t.m_take[:s].clone(), inside_ims


def inside_models(static, x_batch, ims):
    """(inside_ips, d): points inside any box of ``ims`` and the average
    points per box per dim (fbpinns/decompositions.py:211-215)."""
    g = grid_of(static)
    x = _x_dev(x_batch, g.device)
    ims = torch.as_tensor(np.asarray(ims), dtype=torch.long, device=g.device)
    sel = torch.zeros(g.m, dtype=torch.uint8, device=g.device)
    sel[ims] = 1
    t = PointTakes(g, x.shape[0], s_cap=0, u_cap=0)
    lib = _lib.load()
    b = g.boxes(sel)
    st = _lib.stream_ptr()
    t.model_count.zero_()
    _lib.check(lib.fbp_inside_count(_lib.ptr(x), t.n, C.byref(b), _lib.ptr(t.pt_count), None, None,
                                    _lib.ptr(t.model_count), None, None, st), "fbp_inside_count")
    ips = compact_flags(t.pt_count)
    counts = t.model_count[ims].double()
    d = float(counts.mean() ** (1.0 / g.xd)) if ims.numel() else float("nan")
    return ips, d


def compact_flags(flag):
    """Indices i with flag[i] != 0, ascending (GPU compaction)."""
    lib = _lib.load()
    n = flag.numel()
    out = torch.empty(max(n, 1), dtype=torch.int32, device=flag.device)
    cnt = torch.zeros(1, dtype=torch.int32, device=flag.device)
    scratch = torch.empty(int(lib.fbp_compact_scratch_bytes(n)) // 4 + 1, dtype=torch.int32, device=flag.device)
    _lib.check(lib.fbp_compact_flags(_lib.ptr(flag.to(torch.int32).contiguous()), n, _lib.ptr(out), _lib.ptr(cnt),
                                     _lib.ptr(scratch), scratch.numel() * 4, _lib.stream_ptr()), "fbp_compact_flags")
    return out[:int(cnt.item())]


def gather_i32(src, inv):
    lib = _lib.load()
    out = torch.empty_like(src)
    _lib.check(lib.fbp_gather_i32(_lib.ptr(src), src.numel(), None, _lib.ptr(inv), _lib.ptr(out), _lib.stream_ptr()),
               "fbp_gather_i32")
    return out


def get_inputs(x_batch, active, all_params, decomposition=None):
    """``fbpinns/trainers.py:332-419`` (``get_inputs``) on the GPU.

    Returns ``takes = (m_take, n_take, p_take, np_take, npou)`` (m_take
    re-indexed to positions in ``all_ims``), ``all_ims`` and
    ``(active, active_ims, fixed_ims)``; tensors are int32 on the device.
    """
    static = all_params["static"]["decomposition"]
    g = grid_of(static)
    m = g.m
    active = np.array(active).copy()
    assert np.isin(active, np.array([0, 1, 2])).all()
    assert active.shape == (m,)
    x = _x_dev(x_batch, g.device)
    t = PointTakes(g, x.shape[0])
    s, u = t.build(x)
    t.check_status()
    training = (t.model_count > 0).cpu().numpy()
    active[active == 0] = 1
    active = active * training.astype(active.dtype)
    ims_ = np.arange(m)
    active_ims, fixed_ims = ims_[active == 1], ims_[active == 2]
    all_ims = np.concatenate([active_ims, fixed_ims])
    inv = np.zeros(m, dtype=np.int32)
    inv[all_ims] = np.arange(len(all_ims), dtype=np.int32)
    m_take = gather_i32(t.m_take[:s].contiguous(), torch.as_tensor(inv, device=g.device))
    takes = (m_take, t.n_take[:s].clone(), t.p_take[:s].clone(), t.np_take[:u].clone(), g.npou)
    return takes, torch.as_tensor(all_ims, dtype=torch.int32, device=g.device), (active, active_ims, fixed_ims)


def split_takes(takes, offsets, n_points):
    """Per-constraint re-indexed takes (fbpinns/trainers.py:544-571).

    The training points of constraint ic are the contiguous index range
    [offsets[ic], offsets[ic+1]) of x_batch (constraints are concatenated in
    order and the cut of the global points preserves order), and n_take is
    sorted, so each constraint owns a contiguous run of pairs and of slots;
    re-indexing is a subtraction of the run starts.
    """
    m_take, n_take, p_take, np_take, npou = takes
    bounds = list(offsets) + [n_points]
    dev = n_take.device
    out = []
    for ic in range(len(offsets)):
        a, b = bounds[ic], bounds[ic + 1]
        e0 = int(torch.searchsorted(n_take, torch.tensor([a], dtype=torch.int32, device=dev)).item())
        e1 = int(torch.searchsorted(n_take, torch.tensor([b], dtype=torch.int32, device=dev)).item())
        u0 = int(torch.searchsorted(np_take, torch.tensor([a], dtype=torch.int32, device=dev)).item())
        u1 = int(torch.searchsorted(np_take, torch.tensor([b], dtype=torch.int32, device=dev)).item())
        out.append((m_take[e0:e1], n_take[e0:e1] - a, p_take[e0:e1] - u0, np_take[u0:u1] - a, npou))
    return out
