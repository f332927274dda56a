"""Reference field for the (2+1)D wave problems: a finite-difference solve.

The reference computes its "exact" wave field with a 2D acoustic CPML
finite-difference code (fbpinns/problems.py:408-474).  Here the same role is
played by a second-order leapfrog solve of u_tt = c(x)^2 (u_xx + u_yy) with
u(x, y, 0) = the Gaussian source sum and u_t(x, y, 0) = 0, on a grid padded by
c_max * t_max on every side with u = 0 on the padded boundary, so reflections
cannot return into the domain before t_max.  Test-time only (it feeds the
test L1), on the host in float64.
"""

import math

import numpy as np
import torch


def _gauss_sum_np(src, x, y):
    f = np.zeros_like(x)
    for mx, my, sd, amp in np.asarray(src, dtype=np.float64):
        f += amp * np.exp(-0.5 * ((x - mx) ** 2 + (y - my) ** 2) / sd ** 2)
    return f


def wave_field(c_of_xy, source, xmin, xmax, ymin, ymax, tmax, nt_out, points_per_width=12, max_cells=6_000_000):
    """Leapfrog solve; returns (xs, ys, ts, U (nx, ny, nt_out)) on the padded grid."""
    src = np.asarray(source, dtype=np.float64)
    wmin = src[:, 2].min()
    cmax = float(np.max(c_of_xy(np.array([[0.5 * (xmin + xmax), 0.5 * (ymin + ymax)]]))))
    pad = cmax * tmax * 1.05
    lx, ly = (xmax - xmin) + 2 * pad, (ymax - ymin) + 2 * pad
    dx = wmin / points_per_width
    while (lx / dx) * (ly / dx) > max_cells:
        dx *= 1.25
    nx, ny = int(math.ceil(lx / dx)) + 1, int(math.ceil(ly / dx)) + 1
    xs = xmin - pad + dx * np.arange(nx)
    ys = ymin - pad + dx * np.arange(ny)
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    c2 = c_of_xy(np.stack([X.ravel(), Y.ravel()], 1)).reshape(nx, ny) ** 2 if callable(c_of_xy) else None
    dt_out = tmax / (nt_out - 1)
    dt = 0.4 * dx / cmax
    sub = int(math.ceil(dt_out / dt))
    dt = dt_out / sub
    u0 = _gauss_sum_np(src, X, Y)
    u0[0, :] = u0[-1, :] = u0[:, 0] = u0[:, -1] = 0.0
    r = c2 * (dt / dx) ** 2

    def lap(u):
        out = np.zeros_like(u)
        out[1:-1, 1:-1] = u[2:, 1:-1] + u[:-2, 1:-1] + u[1:-1, 2:] + u[1:-1, :-2] - 4 * u[1:-1, 1:-1]
        return out

    out = np.empty((nx, ny, nt_out))
    out[:, :, 0] = u0
    prev, cur = u0, u0 + 0.5 * r * lap(u0)  # zero initial velocity
    k = 1
    for step in range(1, sub * (nt_out - 1) + 1):
        if step % sub == 0:
            out[:, :, step // sub] = cur
        if step == sub * (nt_out - 1):
            break
        prev, cur = cur, 2 * cur - prev + r * lap(cur)
    return xs, ys, np.linspace(0, tmax, nt_out), out


def bilinear(xs, ys, F, x, y):
    """Bilinear interpolation of F (nx, ny[, ...]) on a uniform grid at points (x, y)."""
    dx, dy = xs[1] - xs[0], ys[1] - ys[0]
    fx = np.clip((x - xs[0]) / dx, 0, len(xs) - 1 - 1e-9)
    fy = np.clip((y - ys[0]) / dy, 0, len(ys) - 1 - 1e-9)
    i, j = np.floor(fx).astype(int), np.floor(fy).astype(int)
    a, b = fx - i, fy - j
    return ((1 - a) * (1 - b) * F[i, j] + a * (1 - b) * F[i + 1, j] + (1 - a) * b * F[i, j + 1] + a * b * F[i + 1, j + 1])


def wave_exact(all_params, x_batch, batch_shape):
    """Field at x_batch, a (nx, ny, nt) 'ij' grid flattened like the grid sampler."""
    p = all_params["static"]["problem"]
    xb = torch.as_tensor(x_batch).double().cpu().numpy()
    c_fn = p["c_fn"]

    def c_of_xy(xy):
        v = c_fn(all_params, torch.as_tensor(np.concatenate([xy, np.zeros((xy.shape[0], 1))], 1)))
        v = np.asarray(torch.as_tensor(v).double().cpu())
        return np.broadcast_to(v.reshape(-1), (xy.shape[0],)).copy()

    (xmin, ymin, tmin), (xmax, ymax, tmax) = xb.min(0), xb.max(0)
    nt = batch_shape[2]
    src = torch.as_tensor(p["source"]).double().cpu().numpy()
    xs, ys, ts, U = wave_field(c_of_xy, src, xmin, xmax, ymin, ymax, tmax, nt)
    T = np.rint((xb[:, 2] - 0) / (ts[1] - ts[0])).astype(int).clip(0, nt - 1)
    vals = np.empty(xb.shape[0])
    for k in range(nt):
        sel = T == k
        if sel.any():
            vals[sel] = bilinear(xs, ys, U[:, :, k], xb[sel, 0], xb[sel, 1])
    return torch.as_tensor(vals.reshape(-1, 1), dtype=torch.float32)
