"""Domain decompositions (the reference's ``fbpinns/decompositions.py`` API).

Parameters are built on the host (numpy float64, then float32 tensors like the
reference's ``jnp.array``); the point-in-box tests run on the GPU through
``libfbpgpu`` over a uniform cell grid built here.

Static parameter layout (same keys as the reference)::

    {"m", "xd", "subdomain": {"params": [xmins, xmaxs, wmins, wmaxs, flags, unnorms],
                               "pou": pous}, "xmins0", "xmaxs0"}
"""

import math

import numpy as np
import torch

from . import windows
from . import networks


class Decomposition:
    """Base class: static methods only, as in ``fbpinns/decompositions.py:31-94``."""

    @staticmethod
    def init_params(*args):
        raise NotImplementedError

    @staticmethod
    def norm_fn(params, x):
        raise NotImplementedError

    @staticmethod
    def unnorm_fn(params, u):
        raise NotImplementedError

    @staticmethod
    def window_fn(params, x):
        raise NotImplementedError

    @staticmethod
    def inside_points(all_params, x_batch):
        raise NotImplementedError

    @staticmethod
    def inside_models(all_params, x_batch, ims):
        raise NotImplementedError


def _overlap_widths(xmins, xmaxs):
    """Per-dim overlap widths with the grid neighbours (fbpinns/decompositions.py:145-160).

    ``xmins``/``xmaxs`` have shape (xd, *nm).  Along each grid axis the overlap
    of cell k with cell k+1 is ``xmax_k - xmin_{k+1}``; it is cell k's upper
    width and cell k+1's lower width.  The first cell's lower width copies its
    upper one and the last cell's upper width copies its lower one; an axis
    with a single cell keeps half the cell width on both sides.
    """
    xd = xmins.shape[0]
    half = 0.5 * (xmaxs - xmins)
    lower, upper = half.copy(), half.copy()
    for i in range(xd):
        lo_i = np.moveaxis(lower[i], i, 0)  # views
        up_i = np.moveaxis(upper[i], i, 0)
        xmax_i = np.moveaxis(xmaxs[i], i, 0)
        xmin_i = np.moveaxis(xmins[i], i, 0)
        if lo_i.shape[0] > 1:
            ov = xmax_i[:-1] - xmin_i[1:]
            up_i[:-1] = ov
            lo_i[1:] = ov
        lo_i[0] = up_i[0]
        up_i[-1] = lo_i[-1]
    if (lower <= 0).any() or (upper <= 0).any():
        raise ValueError("some subdomains are not overlapping!")
    return lower, upper


def level_params(il, xd, subdomain_xs, subdomain_ws, unnorm):
    """One level of rectangular subdomains on a regular grid of centres.

    Follows ``RectangularDecompositionND._get_level_params``
    (fbpinns/decompositions.py:136-181).  Returns numpy float64 arrays
    [xmins, xmaxs, wmins, wmaxs, flags, unnorms, pous], each with m rows in
    C order of the centre grid (last dim fastest).
    """
    xs = np.stack(np.meshgrid(*[np.asarray(v, dtype=np.float64) for v in subdomain_xs], indexing="ij"), 0)
    ws = np.stack(np.meshgrid(*[np.asarray(v, dtype=np.float64) for v in subdomain_ws], indexing="ij"), 0)
    if xs.shape != ws.shape:
        raise ValueError("shape of subdomain_ws not same as subdomain_xs")
    xmins, xmaxs = xs - ws / 2, xs + ws / 2
    wmins, wmaxs = _overlap_widths(xmins, xmaxs)
    flat = lambda a: a.reshape(xd, -1).T
    xmins, xmaxs, wmins, wmaxs = flat(xmins), flat(xmaxs), flat(wmins), flat(wmaxs)
    m = xmins.shape[0]
    flags = np.full((m, 1), 0.0 if m == 1 else 1.0)
    unnorms = np.tile(np.array([[float(unnorm[0]), float(unnorm[1])]]), (m, 1))
    pous = np.full((m, 1), float(il))
    return [xmins, xmaxs, wmins, wmaxs, flags, unnorms, pous]


WINDOWS = ("cosine", "sigmoid", "bump", "wendland", "rbf")  # fbpinns/windows.py, FBP_WINDOW_* order


def _static_from_levels(levels, xd, window="cosine"):
    if window not in WINDOWS:
        raise ValueError(f"window must be one of {WINDOWS}, not {window!r}")
    ps = [np.concatenate([lv[k] for lv in levels]) for k in range(7)]
    xmins0 = ps[0] + ps[2] / 2  # centre lines of the overlap regions (scheduler)
    xmaxs0 = ps[1] - ps[3] / 2
    t = [torch.as_tensor(p, dtype=torch.float32) for p in ps]
    return {
        "m": int(ps[0].shape[0]),
        "xd": int(xd),
        "subdomain": {"params": t[:-1], "pou": t[-1]},
        "xmins0": xmins0,
        "xmaxs0": xmaxs0,
        "window": window,
    }


class RectangularDecompositionND(Decomposition):
    """ND hyperrectangular subdomains on a regular grid (fbpinns/decompositions.py:101-335)."""

    @staticmethod
    def init_params(subdomain_xs, subdomain_ws, unnorm, window="cosine"):
        """``window`` (this engine's extension; the reference's decompositions
        always use the cosine window, decompositions.py:197-199): one of the
        window functions of fbpinns/windows.py, computed with its derivative
        jets in the kernels -- "cosine", "sigmoid", "bump", "wendland", "rbf"."""
        xd = len(subdomain_xs)
        return _static_from_levels([level_params(0, xd, subdomain_xs, subdomain_ws, unnorm)], xd, window), {}

    # per-point functions, batched over pairs: params are the gathered per-pair
    # subdomain params (xmins (s,xd), xmaxs, flags (s,1), unnorms (s,2))
    @staticmethod
    def norm_fn(params, x):
        xmin, xmax = params["static"]["decomposition"]["subdomain"]["params"][:2]
        return networks.norm((xmax + xmin) / 2, (xmax - xmin) / 2, x)

    @staticmethod
    def unnorm_fn(params, u):
        un = params["static"]["decomposition"]["subdomain"]["params"][5]
        return networks.unnorm(un[..., 0:1], un[..., 1:2], u)

    @staticmethod
    def window_fn(params, x):
        dec = params["static"]["decomposition"]
        p = dec["subdomain"]["params"]
        return p[4] * window_values(dec.get("window", "cosine"), p, x) + (1 - p[4])

    @staticmethod
    def inside_points(all_params, x_batch):
        """(n_take, m_take, inside_ims) on the GPU, point-major / box-minor order.

        Replaces fbpinns/decompositions.py:202-208 (``inside_points_batch``).
        """
        from .takes import inside_points
        return inside_points(all_params["static"]["decomposition"], x_batch)

    @staticmethod
    def inside_models(all_params, x_batch, ims):
        """(inside_ips, d): points inside at least one box of ``ims`` (GPU).

        Replaces fbpinns/decompositions.py:211-215 (``inside_models_batch``).
        """
        from .takes import inside_models
        return inside_models(all_params["static"]["decomposition"], x_batch, ims)


class MultilevelRectangularDecompositionND(RectangularDecompositionND):
    """Several rectangular levels concatenated; pou = level index
    (fbpinns/decompositions.py:338-375)."""

    @staticmethod
    def init_params(subdomain_xss, subdomain_wss, unnorm, window="cosine"):
        nms = [tuple(len(x) for x in sx) for sx in subdomain_xss]
        if any(len(nm) != len(nms[0]) for nm in nms):
            raise ValueError("subdomain_xss are not all the same dimensionality")
        xd = len(subdomain_xss[0])
        levels = [level_params(il, xd, sx, sw, unnorm)
                  for il, (sx, sw) in enumerate(zip(subdomain_xss, subdomain_wss))]
        return _static_from_levels(levels, xd, window), {}


# ---------------------------------------------------------------------------
# uniform cell grid over the boxes (host side of the point-in-box kernels)
# ---------------------------------------------------------------------------

def cell_coord(v, lo, inv_h, nc):
    """Cell index along one dim: clamp(floor((double(v) - lo) * inv_h), 0, nc-1).

    IEEE double subtraction then multiplication, the same operations as the
    device (``__dsub_rn``, ``__dmul_rn``), so the host registration and the
    device lookup agree exactly and are monotone in v.
    """
    t = np.floor((np.asarray(v, dtype=np.float32).astype(np.float64) - lo) * inv_h)
    t = np.where(np.isnan(t), 0.0, t)
    return np.clip(t, 0, nc - 1).astype(np.int64)


def build_cell_grid(xmins, xmaxs, cells_per_width=4, max_cells=1 << 21):
    """CSR cell lists of the boxes.  Every box is registered in all cells
    between the cells of its two corners, so by monotonicity of ``cell_coord``
    every box containing a point is a candidate of that point's cell; the exact
    closed-box test is then done on the device in float32.

    Returns dict(ncell (xd,), lo (xd,), inv_h (xd,), cell_start, cell_boxes).
    """
    xmins = np.asarray(xmins, dtype=np.float32)
    xmaxs = np.asarray(xmaxs, dtype=np.float32)
    m, xd = xmins.shape
    lo = xmins.astype(np.float64).min(0)
    hi = xmaxs.astype(np.float64).max(0)
    ext = np.maximum(hi - lo, 1e-30)
    wmin = np.maximum((xmaxs.astype(np.float64) - xmins.astype(np.float64)).min(0), 1e-30)
    nc = np.maximum(1, np.ceil(ext / wmin * cells_per_width)).astype(np.int64)
    while np.prod(nc) > max_cells:
        nc = np.maximum(1, nc // 2)
    inv_h = nc / ext
    c_lo = np.stack([cell_coord(xmins[:, d], lo[d], inv_h[d], nc[d]) for d in range(xd)], 1)
    c_hi = np.stack([cell_coord(xmaxs[:, d], lo[d], inv_h[d], nc[d]) for d in range(xd)], 1)
    cells, boxes = [], []
    strides = np.cumprod(np.concatenate([[1], nc[:-1]]))
    for j in range(m):
        rng = [np.arange(c_lo[j, d], c_hi[j, d] + 1) for d in range(xd)]
        g = np.stack(np.meshgrid(*rng, indexing="ij"), -1).reshape(-1, xd)
        cells.append(g @ strides)
        boxes.append(np.full(g.shape[0], j))
    cells = np.concatenate(cells)
    boxes = np.concatenate(boxes)
    order = np.argsort(cells, kind="stable")  # boxes stay ascending within a cell
    ncells = int(np.prod(nc))
    counts = np.bincount(cells, minlength=ncells)
    start = np.zeros(ncells + 1, dtype=np.int64)
    np.cumsum(counts, out=start[1:])
    return {"ncell": nc, "lo": lo, "inv_h": inv_h, "cell_start": start.astype(np.int32),
            "cell_boxes": boxes[order].astype(np.int32)}


def window_values(name, p, x):
    """The named window of fbpinns/windows.py for boxes p (the subdomain
    params [xmins, xmaxs, wmins, wmaxs, ...], broadcastable against x)."""
    if name == "sigmoid":
        return windows.sigmoid(p[0], p[1], p[2], p[3], x)
    return getattr(windows, name)(p[0], p[1], x)


def subdomain_arrays(static):
    """(xmins, xmaxs, flags (m,), unnorms (m,2), pou int32 (m,)) float32 tensors."""
    p = static["subdomain"]["params"]
    return (p[0].float(), p[1].float(), p[4].float().reshape(-1), p[5].float(),
            static["subdomain"]["pou"].reshape(-1).to(torch.int32))


def npou_of(static):
    """Number of distinct POU levels over all subdomains (fbpinns/trainers.py:388)."""
    return int(torch.unique(static["subdomain"]["pou"].reshape(-1).to(torch.int64)).numel())
