"""torch restatement of the reference PDE problems (constraints and losses).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

``P["problem"]`` holds the static problem parameters and
``P["problem_trainable"]`` the trainable ones, as in the reference's
``all_params["static"]["problem"]`` / ``all_params["trainable"]["problem"]``.

The 2D Poisson and 2D Helmholtz problems do not exist in the reference
library; their definitions here restate the ones of
``fbpinns_gb300/problems.py`` (the engine's own specification of those two
workloads) so that the CUDA kernels have an independent float64 check.
"""

import math

import torch


class HarmonicOscillator1D:
    """``fbpinns/problems.py:68-146``."""

    @staticmethod
    def constraining_fn(P, x_batch, u):
        return u

    @staticmethod
    def loss_fn(P, constraints):
        # problems.py:117-132
        mu, k = P["problem"]["mu"], P["problem"]["k"]
        _, u, ut, utt = constraints[0]
        phys = torch.mean((utt + mu * ut + k * u) ** 2)
        _, uc, utc, u, ut = constraints[1]
        if len(uc):
            boundary = 1e6 * torch.mean((u - uc) ** 2) + 1e2 * torch.mean((ut - utc) ** 2)
        else:
            boundary = 0
        return phys + boundary

    @staticmethod
    def exact_solution(P, x_batch):
        # problems.py:135-146
        d, w0 = P["problem"]["d"], P["problem"]["w0"]
        w = math.sqrt(w0 ** 2 - d ** 2)
        phi = math.atan(-d / w)
        A = 1 / (2 * math.cos(phi))
        return torch.exp(-d * x_batch) * 2 * A * torch.cos(phi + w * x_batch)


class HarmonicOscillator1DHardBC(HarmonicOscillator1D):
    """``fbpinns/problems.py:149-206``."""

    @staticmethod
    def constraining_fn(P, x_batch, u):
        sd = P["problem"]["sd"]
        x = x_batch[:, 0:1]
        return 1 + (torch.tanh(x / sd) ** 2) * u

    @staticmethod
    def loss_fn(P, constraints):
        mu, k = P["problem"]["mu"], P["problem"]["k"]
        _, u, ut, utt = constraints[0]
        return torch.mean((utt + mu * ut + k * u) ** 2)


class HarmonicOscillator1DInverse(HarmonicOscillator1D):
    """``fbpinns/problems.py:209-271``."""

    @staticmethod
    def loss_fn(P, constraints):
        mu, k = P["problem_trainable"]["mu"], P["problem"]["k"]
        _, u, ut, utt = constraints[0]
        phys = torch.mean((utt + mu * ut + k * u) ** 2)
        _, uc, u = constraints[1]
        return phys + 1e6 * torch.mean((u - uc) ** 2)


class BurgersEquation2D:
    """``fbpinns/problems.py:276-341``."""

    @staticmethod
    def constraining_fn(P, x_batch, u):
        sd = P["problem"]["sd"]
        x, t = x_batch[:, 0:1], x_batch[:, 1:2]
        tanh = torch.tanh
        return tanh((x + 1) / sd) * tanh((1 - x) / sd) * tanh((t - 0) / sd) * u - torch.sin(math.pi * x)

    @staticmethod
    def loss_fn(P, constraints):
        nu = P["problem"]["nu"]
        _, u, ux, ut, uxx = constraints[0]
        phys = ut + (u * ux) - (nu * uxx)
        return torch.mean(phys ** 2)


def _gauss_sum(params, x):
    """Sum of isotropic 2D Gaussians ``params (k,4) = [mx, my, sd, amp]``."""
    p = params[:, None, :]
    xx = x[None, :, :]
    return (p[:, :, 3:4] * torch.exp(-0.5 * ((xx - p[:, :, 0:2]) ** 2).sum(2, keepdim=True)
                                     / (p[:, :, 2:3] ** 2))).sum(0)


class WaveEquationConstantVelocity3D:
    """``fbpinns/problems.py:346-481``."""

    @staticmethod
    def c_fn(P, x_batch):
        return torch.tensor([[float(P["problem"]["c0"])]], dtype=x_batch.dtype)

    @classmethod
    def constraining_fn(cls, P, x_batch, u):
        # problems.py:383-398
        c0, source = P["problem"]["c0"], P["problem"]["source"].to(x_batch.dtype)
        x, t = x_batch[:, 0:2], x_batch[:, 2:3]
        f = _gauss_sum(source, x)
        t1 = source[:, 2].min() / c0
        f = torch.exp(-0.5 * (1.5 * t / t1) ** 2) * f
        tt = torch.tanh(2.5 * t / t1) ** 2
        return f + tt * u

    @classmethod
    def loss_fn(cls, P, constraints):
        # problems.py:401-405
        x_batch, uxx, uyy, utt = constraints[0]
        phys = (uxx + uyy) - (1 / cls.c_fn(P, x_batch) ** 2) * utt
        return torch.mean(phys ** 2)


class WaveEquationGaussianVelocity3D(WaveEquationConstantVelocity3D):
    """``fbpinns/problems.py:484-522``."""

    @staticmethod
    def c_fn(P, x_batch):
        c0, mixture = P["problem"]["c0"], P["problem"]["mixture"].to(x_batch.dtype)
        return c0 + _gauss_sum(mixture, x_batch[:, 0:2])


def _box_ansatz(x_batch, sd):
    """tanh(x/sd) tanh((1-x)/sd) tanh(y/sd) tanh((1-y)/sd) on [0,1]^2."""
    x, y = x_batch[:, 0:1], x_batch[:, 1:2]
    t = torch.tanh
    return t(x / sd) * t((1 - x) / sd) * t(y / sd) * t((1 - y) / sd)


class Poisson2D:
    """-lap u = f on [0,1]^2, u = sum_k sin(2^k pi x) sin(2^k pi y) / 2^k, hard zero BC."""

    @staticmethod
    def constraining_fn(P, x_batch, u):
        return _box_ansatz(x_batch, P["problem"]["sd"]) * u

    @staticmethod
    def source(P, x_batch):
        x, y = x_batch[:, 0:1], x_batch[:, 1:2]
        f = torch.zeros_like(x)
        for k in range(1, int(P["problem"]["n_freq"]) + 1):
            a = (2 ** k) * math.pi
            f = f + (2.0 ** (k + 1)) * math.pi ** 2 * torch.sin(a * x) * torch.sin(a * y)
        return f

    @classmethod
    def loss_fn(cls, P, constraints):
        x_batch, uxx, uyy = constraints[0]
        return torch.mean((uxx + uyy + cls.source(P, x_batch)) ** 2)

    @staticmethod
    def exact_solution(P, x_batch):
        x, y = x_batch[:, 0:1], x_batch[:, 1:2]
        u = torch.zeros_like(x)
        for k in range(1, int(P["problem"]["n_freq"]) + 1):
            a = (2 ** k) * math.pi
            u = u + torch.sin(a * x) * torch.sin(a * y) / (2 ** k)
        return u


class Helmholtz2D:
    """-lap u - k^2 u = f on [0,1]^2, f = sum of Gaussians, hard zero BC."""

    @staticmethod
    def constraining_fn(P, x_batch, u):
        return _box_ansatz(x_batch, P["problem"]["sd"]) * u

    @staticmethod
    def source(P, x_batch):
        return _gauss_sum(P["problem"]["source"].to(x_batch.dtype), x_batch[:, 0:2])

    @classmethod
    def loss_fn(cls, P, constraints):
        x_batch, u, uxx, uyy = constraints[0]
        k = P["problem"]["k"]
        return torch.mean((uxx + uyy + k * k * u + cls.source(P, x_batch)) ** 2)
