"""Shared builders for the parity tests: the same decomposition, weights and
points for the CUDA engine (float32) and the CPU oracle (float64)."""

import math

import numpy as np
import torch

from conftest import golden
from fbpinns_gb300.constants import get_subdomain_ws
from fbpinns_gb300 import decompositions as D
from fbpinns_gb300.networks import pack_layers
from oracle import model as OM


def decomposition(recipe, window="cosine"):
    """Product static decomposition params for a named recipe (float32 tensors)."""
    if window != "cosine":
        st = decomposition(recipe)
        st = {k: v for k, v in st.items() if not k.startswith("_")}
        st["window"] = window
        return st
    if recipe in ("ho", "ho2c", "ho_hardbc"):
        sx = [np.linspace(0, 1, 15)]
        return D.RectangularDecompositionND.init_params(sx, get_subdomain_ws(sx, 2.0), (0., 1.))[0]
    if recipe.startswith("burgers"):
        sx = [np.linspace(-1, 1, 16), np.linspace(0, 1, 8)]
        return D.RectangularDecompositionND.init_params(sx, get_subdomain_ws(sx, 2.9), (0., 1.))[0]
    if recipe in ("multilevel", "multilevel4"):
        sxs = [[np.array([0.5])] * 2] + [[np.linspace(0, 1, k)] * 2 for k in (2, 4, 8)]
        sws = [[np.array([1.0])] * 2] + [get_subdomain_ws(s, 2.9) for s in sxs[1:]]
        return D.MultilevelRectangularDecompositionND.init_params(sxs, sws, (0., 1.))[0]
    if recipe in ("poisson", "poisson16"):
        sxs = [[np.array([0.5])] * 2] + [[np.linspace(0, 1, k)] * 2 for k in (2, 4, 8, 16, 32)]
        sws = [[np.array([1.0])] * 2] + [get_subdomain_ws(s, 2.9) for s in sxs[1:]]
        return D.MultilevelRectangularDecompositionND.init_params(sxs, sws, (0., 1.))[0]
    if recipe == "wave_full":  # the wave configuration: 15x15x4 boxes, width 2.9 x spacing
        sx = [np.linspace(-1, 1, 15), np.linspace(-1, 1, 15), np.linspace(0, 1, 4)]
        return D.RectangularDecompositionND.init_params(sx, get_subdomain_ws(sx, 2.9), (0., 1.))[0]
    if recipe in ("wave", "wave3d"):
        sx = [np.linspace(-1, 1, 5), np.linspace(-1, 1, 4), np.linspace(0, 1, 3)]
        return D.RectangularDecompositionND.init_params(sx, get_subdomain_ws(sx, 2.0), (0.5, 2.0))[0]
    raise KeyError(recipe)


def boxes_static(xmin, xmax, pou=None):
    """A static decomposition dict from raw boxes (flag 1, unnorm (0,1))."""
    m, xd = xmin.shape
    z = torch.zeros((m, xd))
    pou = torch.zeros((m, 1)) if pou is None else torch.as_tensor(pou, dtype=torch.float32).reshape(m, 1)
    params = [torch.as_tensor(xmin), torch.as_tensor(xmax), z, z, torch.ones((m, 1)),
              torch.tensor([[0.0, 1.0]]).repeat(m, 1)]
    return {"m": m, "xd": xd, "subdomain": {"params": params, "pou": pou}}


def wave_sources(seed=0, n=12, wlo=0.02):
    """The wave configuration's initial field: n Gaussians (centres U[-0.5,
    0.5]^2, widths U[wlo, 0.2], amplitude 1) in the (k, 4) source layout."""
    rng = np.random.default_rng(seed)
    return np.concatenate([rng.uniform(-0.5, 0.5, (n, 2)), rng.uniform(wlo, 0.2, (n, 1)), np.ones((n, 1))], 1)


def golden_layers(g):
    """Layer tuples (W, b[, a] or [, c, o]) of a golden model fixture; for a
    FourierFCN fixture (``omega`` saved) the frozen feature layer
    (W = [omega; omega], b = [0; pi/2]) comes first, as the engine packs it."""
    out, i = [], 0
    if "omega" in g:
        om = torch.tensor(g["omega"])
        m, F = om.shape[0], om.shape[1]
        out.append((torch.cat([om, om], 1),
                    torch.cat([torch.zeros((m, F), dtype=om.dtype), torch.full((m, F), math.pi / 2, dtype=om.dtype)], 1)))
    while f"W{i}" in g:
        layer = [torch.tensor(g[f"W{i}"]), torch.tensor(g[f"b{i}"])]
        layer += [torch.tensor(g[f"{k}{i}"]) for k in "AO" if f"{k}{i}" in g]
        out.append(tuple(layer))
        i += 1
    return out


GOLDEN_ACTIVATION = {"siren": "sin", "adafcn": "adaptive_tanh", "adasiren": "adaptive_sin", "fourier": "fourier"}


def golden_activation(tag):
    """Activation of a golden model tag (suffix _siren, _adafcn, _adasiren, _fourier; else tanh)."""
    return GOLDEN_ACTIVATION.get(tag.rsplit("_", 1)[-1], "tanh")


def golden_base(tag):
    """The decomposition recipe of a golden model tag."""
    return tag.rsplit("_", 1)[0] if tag.rsplit("_", 1)[-1] in GOLDEN_ACTIVATION else tag


def layer_sizes(layers):
    return [layers[0][0].shape[2]] + [layer[0].shape[1] for layer in layers]


def oracle_params(static, layers64, problem=None):
    """Oracle parameter dict (float64) from the product static params."""
    p = static["subdomain"]["params"]
    P = {"xmins": p[0].double(), "xmaxs": p[1].double(), "flags": p[4].double(), "unnorms": p[5].double(),
         "pou": static["subdomain"]["pou"].double(), "layers": [tuple(t.double() for t in l) for l in layers64],
         "problem": problem or {}, "problem_trainable": {}, "wmins": p[2].double(), "wmaxs": p[3].double(),
         "window": static.get("window", "cosine")}
    return P


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def random_layers(sizes, m, seed):
    g = torch.Generator().manual_seed(seed)
    out = []
    for fi, fo in zip(sizes[:-1], sizes[1:]):
        v = 1.0 / np.sqrt(fi)
        out.append(((torch.rand((m, fo, fi), generator=g, dtype=torch.float64) * 2 - 1) * v,
                    (torch.rand((m, fo), generator=g, dtype=torch.float64) * 2 - 1) * v))
    return out
