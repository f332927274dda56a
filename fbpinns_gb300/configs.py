"""The five workload configurations as ``Constants``, and a runner.

    python -m fbpinns_gb300.configs --config ho|burgers|poisson|wave|helmholtz
                                    [--steps N] [--engine fused|plain] [--small]

Each returns a ``Constants`` for ``FBPINNTrainer``.  ``small=True`` shrinks
the point counts and decompositions for quick checks (same code paths).
"""

import argparse
import json
import math
import time

import numpy as np

from . import decompositions, domains, networks, problems, schedulers
from .constants import Constants, get_subdomain_ws


def ho(n_steps=10000, small=False):
    """1D damped harmonic oscillator, d=2, w0=80, hard BC; 15 subdomains (width
    2x spacing); FCN 1-32-32-1; 200 grid points; Adam 1e-3; test on 1000 points."""
    sx = [np.linspace(0, 1, 15)]
    return Constants(run="ho", domain=domains.RectangularDomainND,
                     domain_init_kwargs=dict(xmin=np.array([0.]), xmax=np.array([1.])),
                     problem=problems.HarmonicOscillator1DHardBC,
                     problem_init_kwargs=dict(d=2, w0=80, sd=0.1),
                     decomposition=decompositions.RectangularDecompositionND,
                     decomposition_init_kwargs=dict(subdomain_xs=sx, subdomain_ws=get_subdomain_ws(sx, 2.0),
                                                    unnorm=(0., 1.)),
                     network=networks.FCN, network_init_kwargs=dict(layer_sizes=[1, 32, 32, 1]),
                     ns=((200,),), n_test=(1000,), n_steps=n_steps, optimiser_kwargs=dict(learning_rate=1e-3),
                     summary_freq=max(1, n_steps // 10), test_freq=max(1, n_steps // 5))


def ho_example(n_steps=20000, small=False):
    """The reference's own hard-constraint oscillator example
    (examples/2. Using hard constraints - 1D harmonic oscillator.ipynb):
    d=2, w0=80, 15 subdomains of width 0.15, FCN 1-32-1, 200 grid points,
    Adam 1e-3, 20,000 steps, test on 500 points -- the run behind the
    README's FBPINN test-loss curve."""
    c = ho(n_steps=n_steps, small=small)
    c.run = "ho_example"
    c.decomposition_init_kwargs = dict(subdomain_xs=[np.linspace(0, 1, 15)], subdomain_ws=[0.15 * np.ones((15,))],
                                       unnorm=(0., 1.))
    c.network_init_kwargs = dict(layer_sizes=[1, 32, 1])
    c.n_test = (500,)
    return c


def burgers(n_steps=10000, small=False):
    """(1+1)D viscous Burgers: 16x8 subdomains (width 2.9x spacing), FCN
    2-16-16-1, 200x200 grid, line scheduler from x=0 along t."""
    sx = [np.linspace(-1, 1, 16), np.linspace(0, 1, 8)]
    ns = (50, 50) if small else (200, 200)
    return Constants(run="burgers", domain=domains.RectangularDomainND,
                     domain_init_kwargs=dict(xmin=np.array([-1., 0.]), xmax=np.array([1., 1.])),
                     problem=problems.BurgersEquation2D, problem_init_kwargs=dict(),
                     decomposition=decompositions.RectangularDecompositionND,
                     decomposition_init_kwargs=dict(subdomain_xs=sx, subdomain_ws=get_subdomain_ws(sx, 2.9),
                                                    unnorm=(0., 1.)),
                     network=networks.FCN, network_init_kwargs=dict(layer_sizes=[2, 16, 16, 1]),
                     scheduler=schedulers.LineSchedulerRectangularND,
                     scheduler_kwargs=dict(point=[0.], iaxis=0),
                     ns=(ns,), n_test=(100, 50), n_steps=n_steps, optimiser_kwargs=dict(learning_rate=1e-3),
                     summary_freq=max(1, n_steps // 10), test_freq=max(1, n_steps // 5))


def poisson(n_steps=10000, small=False):
    """2D multilevel Poisson: levels 1,2^2,...,32^2 (m=1365), FCN 2-16-16-1,
    2^18 uniform points redrawn every step."""
    levels = [1, 2, 4, 8] if small else [1, 2, 4, 8, 16, 32]
    sxs = [[np.array([0.5])] * 2] + [[np.linspace(0, 1, k)] * 2 for k in levels[1:]]
    sws = [[np.array([1.0])] * 2] + [get_subdomain_ws(s, 2.9) for s in sxs[1:]]
    n = (128, 128) if small else (512, 512)  # 2^14 / 2^18 points
    return Constants(run="poisson", domain=domains.RectangularDomainND,
                     domain_init_kwargs=dict(xmin=np.array([0., 0.]), xmax=np.array([1., 1.])),
                     problem=problems.Poisson2D, problem_init_kwargs=dict(n_freq=4 if small else 6, sd=0.1),
                     decomposition=decompositions.MultilevelRectangularDecompositionND,
                     decomposition_init_kwargs=dict(subdomain_xss=sxs, subdomain_wss=sws, unnorm=(0., 1.)),
                     network=networks.FCN, network_init_kwargs=dict(layer_sizes=[2, 16, 16, 1]),
                     ns=(n,), sampler="uniform", resample=True, n_test=(100, 100), n_steps=n_steps,
                     optimiser_kwargs=dict(learning_rate=1e-3),
                     summary_freq=max(1, n_steps // 10), test_freq=max(1, n_steps // 5))


def wave(n_steps=10000, small=False, seed=0, min_width=None):
    """(2+1)D wave, c=1: 15x15x4 subdomains (width 2.9x spacing), FCN 3-32-32-1,
    58^3 grid, 12 seeded Gaussian sources (widths U[min_width, 0.2], min_width
    0.02 by default)."""
    rng = np.random.default_rng(seed)
    wlo = min_width if min_width is not None else (0.1 if small else 0.02)
    src = np.concatenate([rng.uniform(-0.5, 0.5, (12, 2)), rng.uniform(wlo, 0.2, (12, 1)), np.ones((12, 1))], 1)
    sx = [np.linspace(-1, 1, 15), np.linspace(-1, 1, 15), np.linspace(0, 1, 4)]
    g = 20 if small else 58
    return Constants(run="wave", domain=domains.RectangularDomainND,
                     domain_init_kwargs=dict(xmin=np.array([-1., -1., 0.]), xmax=np.array([1., 1., 1.])),
                     problem=problems.WaveEquationConstantVelocity3D,
                     problem_init_kwargs=dict(c0=1.0, source=src),
                     decomposition=decompositions.RectangularDecompositionND,
                     decomposition_init_kwargs=dict(subdomain_xs=sx, subdomain_ws=get_subdomain_ws(sx, 2.9),
                                                    unnorm=(0., 1.)),
                     network=networks.FCN, network_init_kwargs=dict(layer_sizes=[3, 32, 32, 1]),
                     ns=((g, g, g),), n_test=(40, 40, 10), n_steps=n_steps,
                     optimiser_kwargs=dict(learning_rate=1e-3),
                     summary_freq=max(1, n_steps // 10), test_freq=max(1, n_steps // 5))


def helmholtz(n_steps=10000, small=False):
    """2D Helmholtz, k=40pi, f = 64 seeded Gaussians; 64x64 subdomains (width
    2.9x spacing), FCN 2-32-32-1, 2^22 uniform points redrawn every step."""
    k = 16 if small else 64
    sx = [np.linspace(0, 1, k)] * 2
    n = (256, 256) if small else (2048, 2048)  # 2^16 / 2^22 points
    return Constants(run="helmholtz", domain=domains.RectangularDomainND,
                     domain_init_kwargs=dict(xmin=np.array([0., 0.]), xmax=np.array([1., 1.])),
                     problem=problems.Helmholtz2D,
                     problem_init_kwargs=dict(k=(10 if small else 40) * math.pi, n_sources=64, seed=0),
                     decomposition=decompositions.RectangularDecompositionND,
                     decomposition_init_kwargs=dict(subdomain_xs=sx, subdomain_ws=get_subdomain_ws(sx, 2.9),
                                                    unnorm=(0., 1.)),
                     network=networks.FCN, network_init_kwargs=dict(layer_sizes=[2, 32, 32, 1]),
                     ns=(n,), sampler="uniform", resample=True, n_test=(200, 200), n_steps=n_steps,
                     optimiser_kwargs=dict(learning_rate=1e-3),
                     summary_freq=max(1, n_steps // 10), test_freq=max(1, n_steps // 5))


CONFIGS = {"ho": ho, "ho_example": ho_example, "burgers": burgers, "poisson": poisson, "wave": wave,
           "helmholtz": helmholtz}


def main():
    from .trainers import FBPINNTrainer
    import torch
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", required=True, choices=sorted(CONFIGS))
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--engine", default="fused", choices=["fused", "plain"])
    ap.add_argument("--small", action="store_true")
    ap.add_argument("--layers", default=None, help="network layer sizes, e.g. 1,32,1 (default: the config's)")
    ap.add_argument("--test-every", type=int, default=0, help="steps between test-L1 evaluations (default n/5)")
    ap.add_argument("--min-width", type=float, default=None, help="wave: lower bound of the source widths")
    ap.add_argument("--z2", default="auto", choices=["auto", "store", "recompute"],
                    help="layer-2 z-jets for the adjoint: stored by the forward or recomputed (auto: by width)")
    a = ap.parse_args()
    kw = {} if a.min_width is None else {"min_width": a.min_width}
    c = CONFIGS[a.config](n_steps=a.steps, small=a.small, **kw)
    c.engine = a.engine
    c.store_z2 = {"auto": None, "store": True, "recompute": False}[a.z2]
    if a.layers:
        c.network_init_kwargs = dict(c.network_init_kwargs, layer_sizes=[int(v) for v in a.layers.split(",")])
    if a.test_every:
        c.test_freq = a.test_every
    tr = FBPINNTrainer(c)
    t0 = time.time()
    tr.train()
    torch.cuda.synchronize()
    wall = time.time() - t0
    rates = [h["rate"] for h in tr.history[1:]] or [h["rate"] for h in tr.history]
    print(json.dumps({"config": a.config, "engine": a.engine, "steps": a.steps, "small": a.small, **kw,
                      "z2": a.z2,
                      "layers": c.network_init_kwargs["layer_sizes"],
                      "test_l1_normalised": [r[2] for r in tr.u_test_losses],
                      "wall_s": round(wall, 2), "steps_per_s": float(np.median(rates)) if rates else None,
                      "test_l1": [r[1] for r in tr.u_test_losses], "test_l1_steps": [r[0] for r in tr.u_test_losses],
                      "loss": [h["loss"] for h in tr.history]}))


if __name__ == "__main__":
    main()
