"""Window functions (the reference's ``fbpinns/windows.py``), batched in torch.

Each takes box bounds broadcastable against ``x`` (..., xd) and returns the
product over dims, shape (..., 1).  ``heaviside1(v)`` is 1 for v >= 0 and 0
otherwise, with zero derivative like ``jnp.heaviside(v, 1)``.
"""

import math

import torch


def heaviside1(v):
    return (v >= 0).to(v.dtype)


def prod_dims(ws):
    """Product over the last dim (the spatial dims, at most 3), keepdim --
    as torch.prod, but as plain multiplications: torch.prod's backward goes
    through generic scan kernels, which made them most of a plain GPU step's
    time under double backward."""
    out = ws[..., 0:1]
    for d in range(1, ws.shape[-1]):
        out = out * ws[..., d:d + 1]
    return out


def sigmoid(xmin, xmax, wmin, wmax, x, tol=1e-8):
    """fbpinns/windows.py:11-22: product of two logistic ramps per dim."""
    t = math.log((1 - tol) / tol)
    mu_min, sd_min = xmin + wmin / 2, wmin / (2 * t)
    mu_max, sd_max = xmax - wmax / 2, wmax / (2 * t)
    ws = torch.sigmoid((x - mu_min) / sd_min) * torch.sigmoid((mu_max - x) / sd_max)
    return prod_dims(ws)


def cosine(xmin, xmax, x):
    """fbpinns/windows.py:25-35: ((1 + cos(pi (x-mu)/sd)) / 2)^2 inside the box."""
    mu, sd = (xmin + xmax) / 2, (xmax - xmin) / 2
    ws = ((1 + torch.cos(math.pi * (x - mu) / sd)) / 2) ** 2
    ws = heaviside1(x - xmin) * heaviside1(xmax - x) * ws
    return prod_dims(ws)


def bump(xmin, xmax, x):
    """fbpinns/windows.py:38-46."""
    mu, sd = (xmin + xmax) / 2, (xmax - xmin) / 2
    ws = torch.exp(3 / (((x - mu) / sd) ** 2 - 1.001)) / math.exp(-3)
    return prod_dims(ws)


def wendland(xmin, xmax, x):
    """fbpinns/windows.py:49-59."""
    mu, sd = (xmin + xmax) / 2, (xmax - xmin) / 2
    r = torch.abs((x - mu) / sd)
    ws = ((1 - r) ** 4) * (4 * r + 1)
    ws = heaviside1(x - xmin) * heaviside1(xmax - x) * ws
    return prod_dims(ws)


def rbf(xmin, xmax, x):
    """fbpinns/windows.py:62-68."""
    mu, sd = (xmin + xmax) / 2, (xmax - xmin) / 2
    return torch.exp(-0.5 * torch.sum(((x - mu) / (0.25 * sd)) ** 2, dim=-1, keepdim=True))
