"""PDE problems (the reference's ``fbpinns/problems.py`` API), in torch.

Each problem keeps the reference interface: ``init_params``,
``sample_constraints`` -> ``[[x_batch, *values, required_ujs], ...]``,
``constraining_fn(all_params, x_batch, u)``, ``loss_fn(all_params,
constraints)`` and ``exact_solution``.  Problems whose hard constraint and
residual are compiled into the fused CUDA loss kernel also describe themselves
through ``fused_spec`` (kind, scalar parameters, Gaussian table); any other
problem runs through the generic path, where the CUDA kernels produce the
per-point derivative jets and torch autograd evaluates ``constraining_fn`` and
``loss_fn``.

``Poisson2D`` and ``Helmholtz2D`` are not in the reference library; they are
defined here for the 2D Poisson and 2D Helmholtz workloads.
"""

import math

import numpy as np
import torch

from . import _lib


class Problem:
    """Base class (fbpinns/problems.py:19-62)."""

    @staticmethod
    def init_params(*args):
        raise NotImplementedError

    @staticmethod
    def sample_constraints(all_params, domain, key, sampler, batch_shapes):
        raise NotImplementedError

    @staticmethod
    def constraining_fn(all_params, x_batch, u):
        return u

    @staticmethod
    def loss_fn(all_params, constraints):
        raise NotImplementedError

    @staticmethod
    def exact_solution(all_params, x_batch, batch_shape=None):
        raise NotImplementedError

    @classmethod
    def fused_spec(cls, all_params):
        """None, or dict(kind=_lib.PROBLEM_*, p=[floats], n_int=int, gauss=(k,4) tensor or None)."""
        return None


def _dev(x, ref):
    return torch.as_tensor(x, dtype=ref.dtype, device=ref.device)


class HarmonicOscillator1D(Problem):
    """m u'' + mu u' + k u = 0, u(0)=1, u'(0)=0 with soft boundary terms
    (fbpinns/problems.py:68-146)."""

    @staticmethod
    def init_params(d=2, w0=20):
        return {"dims": (1, 1), "d": d, "w0": w0, "mu": 2 * d, "k": w0 ** 2}, {}

    @staticmethod
    def sample_constraints(all_params, domain, key, sampler, batch_shapes):
        x_phys = domain.sample_interior(all_params, key, sampler, batch_shapes[0])
        req_phys = ((0, ()), (0, (0,)), (0, (0, 0)))
        x_b = torch.zeros((1, 1))
        u_b = torch.ones((1, 1))
        ut_b = torch.zeros((1, 1))
        return [[x_phys, req_phys], [x_b, u_b, ut_b, ((0, ()), (0, (0,)))]]

    @staticmethod
    def loss_fn(all_params, constraints):
        p = all_params["static"]["problem"]
        _, u, ut, utt = constraints[0]
        phys = torch.mean((utt + p["mu"] * ut + p["k"] * u) ** 2)
        _, uc, utc, u, ut = constraints[1]
        if len(uc):
            boundary = 1e6 * torch.mean((u - uc) ** 2) + 1e2 * torch.mean((ut - utc) ** 2)
        else:
            boundary = 0
        return phys + boundary

    @staticmethod
    def exact_solution(all_params, x_batch, batch_shape=None):
        p = all_params["static"]["problem"]
        d, w0 = p["d"], p["w0"]
        w = math.sqrt(w0 ** 2 - d ** 2)
        phi = math.atan(-d / w)
        A = 1 / (2 * math.cos(phi))
        return torch.exp(-d * x_batch) * 2 * A * torch.cos(phi + w * x_batch)


class HarmonicOscillator1DHardBC(HarmonicOscillator1D):
    """Hard-constrained oscillator u = 1 + tanh(t/sd)^2 NN (fbpinns/problems.py:149-206)."""

    @staticmethod
    def init_params(d=2, w0=20, sd=0.1):
        return {"dims": (1, 1), "d": d, "w0": w0, "mu": 2 * d, "k": w0 ** 2, "sd": sd}, {}

    @staticmethod
    def sample_constraints(all_params, domain, key, sampler, batch_shapes):
        x_phys = domain.sample_interior(all_params, key, sampler, batch_shapes[0])
        return [[x_phys, ((0, ()), (0, (0,)), (0, (0, 0)))]]

    @staticmethod
    def constraining_fn(all_params, x_batch, u):
        sd = all_params["static"]["problem"]["sd"]
        return 1 + torch.tanh(x_batch[:, 0:1] / sd) ** 2 * u

    @staticmethod
    def loss_fn(all_params, constraints):
        p = all_params["static"]["problem"]
        _, u, ut, utt = constraints[0]
        return torch.mean((utt + p["mu"] * ut + p["k"] * u) ** 2)

    @classmethod
    def fused_spec(cls, all_params):
        p = all_params["static"]["problem"]
        return {"kind": _lib.PROBLEM_HO_HARDBC, "p": [p["sd"], p["mu"], p["k"]], "n_int": 0, "gauss": None}


class HarmonicOscillator1DInverse(HarmonicOscillator1D):
    """Learns mu from 13 observations of the exact solution (fbpinns/problems.py:209-271)."""

    @staticmethod
    def init_params(d=2, w0=20):
        return ({"dims": (1, 1), "d": d, "w0": w0, "mu_true": 2 * d, "k": w0 ** 2},
                {"mu": torch.tensor(0.0)})

    @staticmethod
    def sample_constraints(all_params, domain, key, sampler, batch_shapes):
        x_phys = domain.sample_interior(all_params, key, sampler, batch_shapes[0])
        x_data = torch.linspace(0, 1, 13, dtype=torch.float64).float().reshape(13, 1)
        u_data = HarmonicOscillator1DInverse.exact_solution(all_params, x_data)
        return [[x_phys, ((0, ()), (0, (0,)), (0, (0, 0)))], [x_data, u_data, ((0, ()),)]]

    @staticmethod
    def loss_fn(all_params, constraints):
        mu, k = all_params["trainable"]["problem"]["mu"], all_params["static"]["problem"]["k"]
        _, u, ut, utt = constraints[0]
        phys = torch.mean((utt + mu * ut + k * u) ** 2)
        _, uc, u = constraints[1]
        return phys + 1e6 * torch.mean((u - uc) ** 2)


def burgers_exact(nu, x, t, n_quad=60):
    """Cole-Hopf solution of u_t + u u_x = nu u_xx, u(x,0) = -sin(pi x), u(+-1,t) = 0.

    u(x,t) = - int sin(pi(x-c q)) f(x-c q) e^{-q^2} dq / int f(x-c q) e^{-q^2} dq
    with f(y) = exp(-cos(pi y) / (2 pi nu)) and c = 2 sqrt(nu t) (Basdevant et
    al. 1986), evaluated by Gauss-Hermite quadrature with ``n_quad`` nodes.
    ``x``, ``t`` are 1D float64 arrays; returns the (len(x), len(t)) field.
    """
    q, wq = np.polynomial.hermite.hermgauss(n_quad)
    x = np.asarray(x, dtype=np.float64)[:, None, None]
    t = np.asarray(t, dtype=np.float64)[None, :, None]
    c = 2.0 * np.sqrt(nu * t)
    y = x - c * q[None, None, :]
    e = -np.cos(np.pi * y) / (2.0 * np.pi * nu)
    e = e - e.max(axis=2, keepdims=True)  # common factor cancels in the ratio
    f = np.exp(e) * wq[None, None, :]
    u = -(np.sin(np.pi * y) * f).sum(2) / f.sum(2)
    u0 = -np.sin(np.pi * x[:, :, 0])
    return np.where(t[:, :, 0] == 0.0, u0, u)


class BurgersEquation2D(Problem):
    """Viscous Burgers u_t + u u_x = nu u_xx on [-1,1] x [0,1] with the hard
    constraint tanh((x+1)/sd) tanh((1-x)/sd) tanh(t/sd) NN - sin(pi x)
    (fbpinns/problems.py:276-341)."""

    @staticmethod
    def init_params(nu=0.01 / math.pi, sd=0.1):
        return {"dims": (1, 2), "nu": nu, "sd": sd}, {}

    @staticmethod
    def sample_constraints(all_params, domain, key, sampler, batch_shapes):
        x_phys = domain.sample_interior(all_params, key, sampler, batch_shapes[0])
        return [[x_phys, ((0, ()), (0, (0,)), (0, (1,)), (0, (0, 0)))]]

    @staticmethod
    def constraining_fn(all_params, x_batch, u):
        sd = all_params["static"]["problem"]["sd"]
        x, t = x_batch[:, 0:1], x_batch[:, 1:2]
        return torch.tanh((x + 1) / sd) * torch.tanh((1 - x) / sd) * torch.tanh(t / sd) * u - torch.sin(math.pi * x)

    @staticmethod
    def loss_fn(all_params, constraints):
        nu = all_params["static"]["problem"]["nu"]
        _, u, ux, ut, uxx = constraints[0]
        return torch.mean((ut + u * ux - nu * uxx) ** 2)

    @staticmethod
    def exact_solution(all_params, x_batch, batch_shape):
        nu = all_params["static"]["problem"]["nu"]
        xb = torch.as_tensor(x_batch).double().cpu()
        vx = np.linspace(xb[:, 0].min().item(), xb[:, 0].max().item(), batch_shape[0])
        vt = np.linspace(xb[:, 1].min().item(), xb[:, 1].max().item(), batch_shape[1])
        return torch.as_tensor(burgers_exact(nu, vx, vt).reshape(-1, 1), dtype=torch.float32)

    @classmethod
    def fused_spec(cls, all_params):
        p = all_params["static"]["problem"]
        return {"kind": _lib.PROBLEM_BURGERS, "p": [p["sd"], p["nu"]], "n_int": 0, "gauss": None}


def gaussian_sum(params, x):
    """sum_k amp_k exp(-0.5 |x - m_k|^2 / sd_k^2) for params (k,4)=[mx,my,sd,amp], x (n,2)."""
    p = params.to(x.dtype).to(x.device)
    d2 = ((x[None, :, :] - p[:, None, 0:2]) ** 2).sum(2, keepdim=True)
    return (p[:, None, 3:4] * torch.exp(-0.5 * d2 / p[:, None, 2:3] ** 2)).sum(0)


class WaveEquationConstantVelocity3D(Problem):
    """(2+1)D wave u_xx + u_yy - u_tt / c^2 = 0 with Gaussian initial field and
    zero initial velocity as a hard constraint (fbpinns/problems.py:346-481)."""

    @staticmethod
    def init_params(c0=1, source=np.array([[0., 0., 0.2, 1.]])):
        return {"dims": (1, 3), "c0": c0, "c_fn": WaveEquationConstantVelocity3D.c_fn,
                "source": torch.as_tensor(np.asarray(source), dtype=torch.float32)}, {}

    @staticmethod
    def sample_constraints(all_params, domain, key, sampler, batch_shapes):
        x_phys = domain.sample_interior(all_params, key, sampler, batch_shapes[0])
        return [[x_phys, ((0, (0, 0)), (0, (1, 1)), (0, (2, 2)))]]

    @staticmethod
    def constraining_fn(all_params, x_batch, u):
        p = all_params["static"]["problem"]
        c0, source = p["c0"], p["source"].to(x_batch.device)
        x, t = x_batch[:, 0:2], x_batch[:, 2:3]
        f = gaussian_sum(source, x)
        t1 = source[:, 2].min().to(x_batch.dtype) / c0
        f = torch.exp(-0.5 * (1.5 * t / t1) ** 2) * f
        return f + torch.tanh(2.5 * t / t1) ** 2 * u

    @staticmethod
    def loss_fn(all_params, constraints):
        c_fn = all_params["static"]["problem"]["c_fn"]
        x_batch, uxx, uyy, utt = constraints[0]
        return torch.mean(((uxx + uyy) - (1 / c_fn(all_params, x_batch) ** 2) * utt) ** 2)

    @staticmethod
    def c_fn(all_params, x_batch):
        return torch.tensor([[float(all_params["static"]["problem"]["c0"])]], dtype=x_batch.dtype,
                            device=x_batch.device)

    @staticmethod
    def exact_solution(all_params, x_batch, batch_shape):
        from .wave_fd import wave_exact
        return wave_exact(all_params, x_batch, batch_shape)

    @classmethod
    def fused_spec(cls, all_params):
        if cls.c_fn is not WaveEquationConstantVelocity3D.c_fn:
            return None
        p = all_params["static"]["problem"]
        src = p["source"]
        t1 = float(src[:, 2].min()) / float(p["c0"])
        return {"kind": _lib.PROBLEM_WAVE_C, "p": [float(p["c0"]), t1], "n_int": 0, "gauss": src,
                "d2_group": 3}  # the residual needs u_xx + u_yy and u_tt


class WaveEquationGaussianVelocity3D(WaveEquationConstantVelocity3D):
    """Wave equation with velocity c0 + Gaussian mixture (fbpinns/problems.py:484-522)."""

    @staticmethod
    def init_params(c0=1, source=np.array([[0., 0., 0.2, 1.]]), mixture=np.array([[0.5, 0.5, 1., 0.2]])):
        return {"dims": (1, 3), "c0": c0, "c_fn": WaveEquationGaussianVelocity3D.c_fn,
                "source": torch.as_tensor(np.asarray(source), dtype=torch.float32),
                "mixture": torch.as_tensor(np.asarray(mixture), dtype=torch.float32)}, {}

    @staticmethod
    def c_fn(all_params, x_batch):
        p = all_params["static"]["problem"]
        return p["c0"] + gaussian_sum(p["mixture"], x_batch[:, 0:2])


def _box_ansatz(x_batch, sd):
    x, y = x_batch[:, 0:1], x_batch[:, 1:2]
    t = torch.tanh
    return t(x / sd) * t((1 - x) / sd) * t(y / sd) * t((1 - y) / sd)


class Poisson2D(Problem):
    """-lap u = f on [0,1]^2 with the manufactured solution
    u = sum_{k=1..K} sin(2^k pi x) sin(2^k pi y) / 2^k, so
    f = sum_k 2^{k+1} pi^2 sin(2^k pi x) sin(2^k pi y); u = 0 on the boundary
    through the hard constraint tanh(x/sd) tanh((1-x)/sd) tanh(y/sd) tanh((1-y)/sd) NN.
    Not in the reference library (its 2D Poisson lives on an unpublished branch)."""

    @staticmethod
    def init_params(n_freq=6, sd=0.1):
        return {"dims": (1, 2), "n_freq": int(n_freq), "sd": sd}, {}

    @staticmethod
    def sample_constraints(all_params, domain, key, sampler, batch_shapes):
        x_phys = domain.sample_interior(all_params, key, sampler, batch_shapes[0])
        return [[x_phys, ((0, (0, 0)), (0, (1, 1)))]]

    @staticmethod
    def constraining_fn(all_params, x_batch, u):
        return _box_ansatz(x_batch, all_params["static"]["problem"]["sd"]) * u

    @staticmethod
    def source(all_params, x_batch):
        x, y = x_batch[:, 0:1], x_batch[:, 1:2]
        f = torch.zeros_like(x)
        for k in range(1, all_params["static"]["problem"]["n_freq"] + 1):
            a = (2 ** k) * math.pi
            f = f + (2.0 ** (k + 1)) * math.pi ** 2 * torch.sin(a * x) * torch.sin(a * y)
        return f

    @staticmethod
    def loss_fn(all_params, constraints):
        x_batch, uxx, uyy = constraints[0]
        return torch.mean((uxx + uyy + Poisson2D.source(all_params, x_batch)) ** 2)

    @staticmethod
    def exact_solution(all_params, x_batch, batch_shape=None):
        x, y = x_batch[:, 0:1].double(), x_batch[:, 1:2].double()
        u = torch.zeros_like(x)
        for k in range(1, all_params["static"]["problem"]["n_freq"] + 1):
            a = (2 ** k) * math.pi
            u = u + torch.sin(a * x) * torch.sin(a * y) / (2 ** k)
        return u.to(x_batch.dtype)

    @classmethod
    def fused_spec(cls, all_params):
        p = all_params["static"]["problem"]
        return {"kind": _lib.PROBLEM_POISSON2D, "p": [p["sd"]], "n_int": p["n_freq"], "gauss": None,
                "d2_group": 3}  # the residual needs only u_xx + u_yy


def seeded_gaussians(n, seed, centre=(0.1, 0.9), width=(0.02, 0.1), amp=(-1.0, 1.0)):
    """(n,4) table [mx, my, sd, amp] of Gaussians drawn from a seeded numpy generator."""
    rng = np.random.default_rng(seed)
    return np.concatenate([rng.uniform(*centre, (n, 2)), rng.uniform(*width, (n, 1)),
                           rng.uniform(*amp, (n, 1))], axis=1)


class Helmholtz2D(Problem):
    """-lap u - k^2 u = f on [0,1]^2, f a sum of Gaussians, u = 0 on the
    boundary through the same hard constraint as Poisson2D.  Not in the
    reference library."""

    @staticmethod
    def init_params(k=40 * math.pi, n_sources=64, seed=0, sd=0.1, source=None):
        src = seeded_gaussians(n_sources, seed) if source is None else np.asarray(source)
        return {"dims": (1, 2), "k": float(k), "sd": sd,
                "source": torch.as_tensor(src, dtype=torch.float32)}, {}

    @staticmethod
    def sample_constraints(all_params, domain, key, sampler, batch_shapes):
        x_phys = domain.sample_interior(all_params, key, sampler, batch_shapes[0])
        return [[x_phys, ((0, ()), (0, (0, 0)), (0, (1, 1)))]]

    @staticmethod
    def constraining_fn(all_params, x_batch, u):
        return _box_ansatz(x_batch, all_params["static"]["problem"]["sd"]) * u

    @staticmethod
    def loss_fn(all_params, constraints):
        p = all_params["static"]["problem"]
        x_batch, u, uxx, uyy = constraints[0]
        return torch.mean((uxx + uyy + p["k"] ** 2 * u + gaussian_sum(p["source"], x_batch)) ** 2)

    @staticmethod
    def exact_solution(all_params, x_batch, batch_shape=None):
        from .helmholtz_fd import helmholtz_exact
        return helmholtz_exact(all_params, x_batch)

    @classmethod
    def fused_spec(cls, all_params):
        p = all_params["static"]["problem"]
        return {"kind": _lib.PROBLEM_HELMHOLTZ2D, "p": [p["sd"], p["k"]], "n_int": 0, "gauss": p["source"],
                "d2_group": 3}  # the residual needs only u_xx + u_yy
