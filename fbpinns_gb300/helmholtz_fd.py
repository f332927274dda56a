"""Reference field for the 2D Helmholtz problem: a sparse finite-difference solve.

-(u_xx + u_yy) - k^2 u = f on [0,1]^2, u = 0 on the boundary, with the
5-point Laplacian on an N x N interior grid (N chosen for >= 16 points per
wavelength 2 pi / k), solved directly by scipy.sparse; values at arbitrary
points by bilinear interpolation.  Test-time only (it feeds the test L1).
"""

import math

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla
import torch

from .wave_fd import bilinear


def helmholtz_grid(k, source, n=None):
    if n is None:
        n = int(min(1000, max(400, math.ceil(60 * k / (2 * math.pi)))))
    h = 1.0 / (n + 1)
    xs = np.linspace(0, 1, n + 2)
    X, Y = np.meshgrid(xs[1:-1], xs[1:-1], indexing="ij")
    f = np.zeros_like(X)
    for mx, my, sd, amp in np.asarray(source, dtype=np.float64):
        f += amp * np.exp(-0.5 * ((X - mx) ** 2 + (Y - my) ** 2) / sd ** 2)
    e = np.ones(n)
    T = sp.diags([-e[:-1], 2 * e, -e[:-1]], [-1, 0, 1]) / h ** 2
    I = sp.identity(n)
    A = (sp.kron(T, I) + sp.kron(I, T) - k * k * sp.identity(n * n)).tocsc()
    u = spla.spsolve(A, f.ravel()).reshape(n, n)
    U = np.zeros((n + 2, n + 2))
    U[1:-1, 1:-1] = u
    return xs, U


def helmholtz_exact(all_params, x_batch):
    p = all_params["static"]["problem"]
    xb = torch.as_tensor(x_batch).double().cpu().numpy()
    xs, U = helmholtz_grid(p["k"], torch.as_tensor(p["source"]).double().cpu().numpy())
    return torch.as_tensor(bilinear(xs, xs, U, xb[:, 0], xb[:, 1]).reshape(-1, 1), dtype=torch.float32)
