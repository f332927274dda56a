"""Per-point jets, fused loss, adjoint gradient and Adam on the GPU against the
reference's golden vectors and the float64 oracle.

Tolerances (FP32 kernels vs FP64 oracle), stated per check: jets and loss
1e-5 relative to the component's max magnitude; gradients 1e-5: the largest
difference over all parameters relative to the largest gradient magnitude
(FP32 sums over ~1e3-1e4 pairs); trainable problem parameters 1e-4."""

import math

import numpy as np
import pytest
import torch

from conftest import golden
from helpers import (decomposition, golden_activation, golden_base, golden_layers, layer_sizes, oracle_params,
                     rel_err, random_layers, wave_sources)
from oracle import model as OM
from oracle import problems as OP
from oracle import takes as OT
from fbpinns_gb300.engine import FBPINNEngine, FBPINNJet, constrained_jets, jet_index, d2mask_of
from fbpinns_gb300.networks import pack_layers
from fbpinns_gb300 import problems as PR
from fbpinns_gb300 import _lib

pytestmark = pytest.mark.gpu

JET_TOL = 1e-5
GRAD_TOL = 1e-5


def _engine(static, layers, d2mask, chunk=64, activation="tanh", tensor_cores=None, tc_adjoint=None):
    eng = FBPINNEngine(static, layer_sizes(layers), d2mask, chunk=chunk, activation=activation,
                       tensor_cores=tensor_cores, tc_adjoint=tc_adjoint)
    eng.set_theta(pack_layers([tuple(t.float() for t in layer) for layer in layers]))
    return eng


@pytest.mark.parametrize("tag,dims,d2", [("ho_hardbc", [0], 1), ("burgers", [0, 1], 1), ("wave", [0, 1, 2], 7),
                                         ("multilevel", [0, 1], 3), ("ho_hardbc_siren", [0], 1),
                                         ("multilevel_siren", [0, 1], 3), ("ho_hardbc_adafcn", [0], 1),
                                         ("multilevel_adafcn", [0, 1], 3), ("ho_hardbc_adasiren", [0], 1),
                                         ("multilevel_adasiren", [0, 1], 3), ("ho_hardbc_fourier", [0], 1),
                                         ("multilevel_fourier", [0, 1], 3)])
def test_jets_vs_reference_golden(cuda, tag, dims, d2):
    """POU-combined network jets (before the constraint) vs the reference's
    forward values and their float64 finite differences (FCN, SIREN,
    AdaptiveFCN, AdaptiveSIREN, FourierFCN)."""
    g = golden(f"model_{tag}.npz")
    static = decomposition(golden_base(tag))
    layers = golden_layers(g)
    eng = _engine(static, layers, d2, activation=golden_activation(tag))
    ps = eng.points(torch.tensor(g["x_batch"], dtype=torch.float32))
    U = FBPINNJet.apply(eng.theta, eng, ps).double().cpu().numpy()
    xd = len(static["subdomain"]["params"][0][0])
    assert rel_err(U[:, 0:1], g["u_raw"]) < JET_TOL
    for d in range(xd):
        assert rel_err(U[:, 1 + d:2 + d], g[f"raw_d{d}"]) < JET_TOL, d
        if (d2 >> d) & 1:
            k = jet_index(xd, d2, (d, d))
            assert rel_err(U[:, k:k + 1], g[f"raw_d{d}{d}"]) < JET_TOL, (d, d)



@pytest.mark.parametrize("lap", [False, True])
@pytest.mark.parametrize("tc", [True, False])
def test_benchmarked_jets_vs_reference_golden(cuda, tc, lap):
    """The benchmarked network shape (2-16-16-1) on the full six-level
    decomposition (levels 1, 2, 4, 8, 16, 32 per dim, m = 1365): POU-combined
    jets vs the reference model's values and float64 finite differences, with
    the tensor-core and the FMA forward, per-dim second derivatives and the
    Laplacian slot (u_xx + u_yy)."""
    g = golden("model_poisson16.npz")
    static = decomposition("poisson16")
    assert static["m"] == 1365
    layers = golden_layers(g)
    d2 = 3 | (_lib.D2_LAPLACIAN if lap else 0)
    eng = _engine(static, [tuple(t.double() for t in layer) for layer in layers], d2, chunk=1024, tensor_cores=tc)
    assert eng.tensor_cores == tc
    ps = eng.points(torch.tensor(g["x_batch"], dtype=torch.float32))
    U = FBPINNJet.apply(eng.theta, eng, ps).double().cpu().numpy()
    ps.check_status()
    assert rel_err(U[:, 0:1], g["u_raw"]) < JET_TOL
    for d in range(2):
        assert rel_err(U[:, 1 + d:2 + d], g[f"raw_d{d}"]) < JET_TOL, d
    if lap:
        assert rel_err(U[:, 3:4], g["raw_d00"] + g["raw_d11"]) < JET_TOL
    else:
        for d in range(2):
            assert rel_err(U[:, 3 + d:4 + d], g[f"raw_d{d}{d}"]) < JET_TOL, (d, d)

CASES = {
    # name: (recipe, layer sizes, problem class (product), product init kwargs, oracle class, oracle params, d2)
    "ho_hardbc": ("ho_hardbc", [1, 32, 32, 1], PR.HarmonicOscillator1DHardBC, dict(d=2, w0=80, sd=0.1),
                  OP.HarmonicOscillator1DHardBC, {"sd": 0.1, "mu": 4, "k": 6400}, 1),
    "burgers": ("burgers", [2, 16, 16, 1], PR.BurgersEquation2D, dict(),
                OP.BurgersEquation2D, {"sd": 0.1, "nu": 0.01 / math.pi}, 1),
    "poisson": ("multilevel", [2, 8, 8, 1], PR.Poisson2D, dict(n_freq=6, sd=0.1),
                OP.Poisson2D, {"sd": 0.1, "n_freq": 6}, 3),
    "wave": ("wave", [3, 8, 8, 1], PR.WaveEquationConstantVelocity3D,
             dict(c0=1.0, source=np.array([[0.1, -0.2, 0.3, 1.0], [-0.3, 0.2, 0.25, 0.5]])),
             OP.WaveEquationConstantVelocity3D,
             {"c0": 1.0, "source": torch.tensor([[0.1, -0.2, 0.3, 1.0], [-0.3, 0.2, 0.25, 0.5]], dtype=torch.float64)}, 7),
    "helmholtz": ("multilevel", [2, 32, 32, 1], PR.Helmholtz2D, dict(k=8 * math.pi, n_sources=4, seed=3),
                  OP.Helmholtz2D, None, 3),
    # the benchmarked Poisson step: six-level decomposition (m = 1365), 2-16-16-1
    "poisson_bench": ("poisson", [2, 16, 16, 1], PR.Poisson2D, dict(n_freq=6, sd=0.1),
                      OP.Poisson2D, {"sd": 0.1, "n_freq": 6}, 3),
    # the wave configuration: 15x15x4 boxes, 3-32-32-1, its 12 seeded sources
    "wave_bench": ("wave_full", [3, 32, 32, 1], PR.WaveEquationConstantVelocity3D,
                   dict(c0=1.0, source=wave_sources()), OP.WaveEquationConstantVelocity3D,
                   {"c0": 1.0, "source": torch.tensor(wave_sources(), dtype=torch.float64)}, 7),
}


def _points(recipe, n, seed):
    rng = np.random.default_rng(seed)
    if recipe == "ho_hardbc":
        return rng.uniform(0, 1, (n, 1)).astype(np.float32)
    if recipe == "burgers":
        return np.stack([rng.uniform(-1, 1, n), rng.uniform(0, 1, n)], 1).astype(np.float32)
    if recipe in ("wave", "wave_full"):
        return np.stack([rng.uniform(-1, 1, n), rng.uniform(-1, 1, n), rng.uniform(0, 1, n)], 1).astype(np.float32)
    return rng.uniform(0, 1, (n, 2)).astype(np.float32)


def _required(name):
    return {"ho_hardbc": ((0, ()), (0, (0,)), (0, (0, 0))), "burgers": ((0, ()), (0, (0,)), (0, (1,)), (0, (0, 0))),
            "poisson": ((0, (0, 0)), (0, (1, 1))), "wave": ((0, (0, 0)), (0, (1, 1)), (0, (2, 2))),
            "helmholtz": ((0, ()), (0, (0, 0)), (0, (1, 1))), "poisson_bench": ((0, (0, 0)), (0, (1, 1))),
            "wave_bench": ((0, (0, 0)), (0, (1, 1)), (0, (2, 2)))}[name]


def _oracle_loss_grad(name, static, layers64, x, prob_static):
    recipe, ls, pcls, pkw, ocls, opar, d2 = CASES[name]
    if opar is None:
        opar = {"sd": prob_static["sd"], "k": prob_static["k"], "source": prob_static["source"].double()}
    P = oracle_params(static, layers64, opar)
    p = static["subdomain"]["params"]
    takes, all_ims, (active, a_ims, f_ims) = OT.get_inputs(x, np.ones(static["m"], dtype=int), p[0].numpy(),
                                                          p[1].numpy(), static["subdomain"]["pou"].numpy())
    loss, grads, _ = OM.value_and_grad(P, a_ims, f_ims, [[torch.tensor(x, dtype=torch.float64)]], [takes],
                                       [OM.get_jmaps(_required(name))], ocls)
    gpack = torch.cat([t.reshape(len(a_ims), -1) for dw, db in grads for t in (dw, db)], 1).numpy()
    return loss.item(), gpack, a_ims, active


@pytest.mark.parametrize("name,lap", [("ho_hardbc", False), ("burgers", False), ("poisson", False),
                                      ("poisson", True), ("wave", False), ("wave", True), ("helmholtz", False),
                                      ("helmholtz", True)])
def test_fused_loss_and_gradient_vs_oracle(cuda, name, lap):
    """Fused loss and per-subdomain gradients vs the float64 oracle.  lap=True
    carries one jet slot for u_xx + u_yy instead of u_xx and u_yy (the wave
    keeps u_tt in a slot of its own)."""
    recipe, ls, pcls, pkw, ocls, opar, d2 = CASES[name]
    static = decomposition(recipe)
    layers64 = random_layers(ls, static["m"], seed=5)
    layers32 = [(w.float().double(), b.float().double()) for w, b in layers64]
    x = _points(recipe if recipe != "multilevel" else "poisson", 600, 17)
    prob_static = pcls.init_params(**pkw)[0]
    loss_ref, g_ref, a_ims, active = _oracle_loss_grad(name, static, layers32, x, prob_static)
    assert d2mask_of([_required(name)], x.shape[1]) | d2 == d2
    eng = _engine(static, layers32, d2 | (0 if not lap else _lib.D2_LAPLACIAN if d2 == 3 else _lib.D2_GROUP(3)))
    eng.set_state(active)
    eng.set_problem(pcls.fused_spec({"static": {"problem": prob_static}}))
    ps = eng.points(torch.tensor(x))
    eng.forward_pairs(ps)
    loss = eng.pou_loss(ps).item()
    grad = eng.adjoint(ps).cpu().numpy()
    ps.check_status()
    assert abs(loss - loss_ref) <= JET_TOL * abs(loss_ref), (loss, loss_ref)
    assert (e := rel_err(grad[a_ims], g_ref)) < GRAD_TOL, e
    inactive = np.setdiff1d(np.arange(static["m"]), a_ims)
    assert np.all(grad[inactive] == 0)


_BENCH_ORACLE = {}


def _bench_case(name, n):
    """Inputs and float64 oracle loss/gradient of a benchmarked-shape case
    (computed once per (name, n): the parametrisations share them)."""
    if (name, n) not in _BENCH_ORACLE:
        recipe, ls, pcls, pkw, ocls, opar, d2 = CASES[name]
        static = decomposition(recipe)
        layers64 = random_layers(ls, static["m"], seed=5)
        layers32 = [(w.float().double(), b.float().double()) for w, b in layers64]
        x = _points(recipe, n, 19)
        prob_static = pcls.init_params(**pkw)[0]
        _BENCH_ORACLE[(name, n)] = (static, layers32, x, prob_static,
                                    _oracle_loss_grad(name, static, layers32, x, prob_static))
    return _BENCH_ORACLE[(name, n)]


@pytest.mark.parametrize("name,lap,tc,tca,n", [("poisson_bench", True, True, False, 3000),
                                               ("poisson_bench", True, False, False, 3000),
                                               ("poisson_bench", False, True, False, 3000),
                                               ("poisson_bench", False, False, False, 3000),
                                               ("poisson_bench", True, True, True, 3000),
                                               ("poisson_bench", False, True, True, 3000),
                                               ("wave_bench", True, False, False, 1500),
                                               ("wave_bench", False, False, False, 1500)])
def test_benchmarked_shapes_loss_and_gradient_vs_oracle(cuda, name, lap, tc, tca, n):
    """The kernel instantiations that the benchmark and the full-size
    configurations run, at their real shapes, against the float64 oracle:
    Poisson 2-16-16-1 on the six-level decomposition (m = 1365) with the
    Laplacian slot (the benchmark's Cfg<2,16,16,11>) or per-dim slots
    (Cfg<2,16,16,3>), tensor-core and FMA forward, tensor-core and FMA
    adjoint; the wave 3-32-32-1 on the
    15x15x4 decomposition with its 12 sources, with the grouped u_xx + u_yy
    slot (Cfg<3,32,32,55>) or per-dim slots (Cfg<3,32,32,7>).  The
    benchmark's work-item sizes (1024 adjoint / 4096 forward pairs, cut for
    the small pair count as in any run).  Loss 1e-5 relative, gradient 1e-5
    of the largest gradient."""
    recipe, ls, pcls, pkw, ocls, opar, d2 = CASES[name]
    static, layers32, x, prob_static, (loss_ref, g_ref, a_ims, active) = _bench_case(name, n)
    d2e = d2 | (0 if not lap else _lib.D2_LAPLACIAN if d2 == 3 else _lib.D2_GROUP(3))
    eng = _engine(static, layers32, d2e, chunk=1024, tensor_cores=tc, tc_adjoint=tca)
    assert eng.tensor_cores == tc and eng.tc_adjoint == tca and eng.forward_chunk == 4096
    eng.set_state(active)
    eng.set_problem(pcls.fused_spec({"static": {"problem": prob_static}}))
    ps = eng.points(torch.tensor(x))
    eng.forward_pairs(ps)
    loss = eng.pou_loss(ps).item()
    grad = eng.adjoint(ps).cpu().numpy()
    ps.check_status()
    assert abs(loss - loss_ref) <= JET_TOL * abs(loss_ref), (loss, loss_ref)
    assert (e := rel_err(grad[a_ims], g_ref)) < GRAD_TOL, e
    inactive = np.setdiff1d(np.arange(static["m"]), a_ims)
    assert np.all(grad[inactive] == 0)


@pytest.mark.parametrize("act", ["sin", "adaptive_tanh", "adaptive_sin"])
@pytest.mark.parametrize("name,lap", [("ho_hardbc", False), ("poisson", False), ("poisson", True)])
def test_network_fused_loss_and_gradient_vs_oracle(cuda, name, lap, act):
    """SIREN, AdaptiveFCN and AdaptiveSIREN networks (adaptive parameters drawn
    away from 1): fused loss and per-subdomain gradients -- W, b and the
    activation parameters -- vs the float64 oracle."""
    recipe, ls, pcls, pkw, ocls, opar, d2 = CASES[name]
    ls = [ls[0], 8, 8, 1]
    static = decomposition(recipe)
    scale = 1.0 if act == "adaptive_tanh" else math.sqrt(6.0)
    gen = torch.Generator().manual_seed(71)
    nx = {"sin": 0, "adaptive_tanh": 1, "adaptive_sin": 2}[act]
    layers64 = [(w * scale, b * scale) + tuple(0.5 + torch.rand(b.shape, generator=gen, dtype=torch.float64)
                                               for _ in range(nx))
                for w, b in random_layers(ls, static["m"], seed=7)]
    layers32 = [tuple(t.float().double() for t in layer) for layer in layers64]
    x = _points(recipe if recipe != "multilevel" else "poisson", 500, 23)
    prob_static = pcls.init_params(**pkw)[0]
    P = oracle_params(static, layers32, opar)
    P["activation"] = act
    p = static["subdomain"]["params"]
    takes, all_ims, (active, a_ims, f_ims) = OT.get_inputs(x, np.ones(static["m"], dtype=int), p[0].numpy(),
                                                          p[1].numpy(), static["subdomain"]["pou"].numpy())
    loss_ref, grads, _ = OM.value_and_grad(P, a_ims, f_ims, [[torch.tensor(x, dtype=torch.float64)]], [takes],
                                           [OM.get_jmaps(_required(name))], ocls)
    g_ref = torch.cat([t.reshape(len(a_ims), -1) for layer in grads for t in layer], 1).numpy()
    eng = _engine(static, layers32, d2 | (_lib.D2_LAPLACIAN if lap else 0), activation=act)
    assert not eng.tensor_cores
    eng.set_state(active)
    eng.set_problem(pcls.fused_spec({"static": {"problem": prob_static}}))
    ps = eng.points(torch.tensor(x))
    eng.forward_pairs(ps)
    loss = eng.pou_loss(ps).item()
    grad = eng.adjoint(ps).cpu().numpy()
    ps.check_status()
    assert abs(loss - loss_ref.item()) <= JET_TOL * abs(loss_ref.item()), (loss, loss_ref.item())
    assert (e := rel_err(grad[a_ims], g_ref)) < GRAD_TOL, e


@pytest.mark.parametrize("name,lap", [("ho_hardbc", False), ("poisson", False), ("poisson", True)])
def test_fourier_fused_loss_and_gradient_vs_oracle(cuda, name, lap):
    """FourierFCN (4 features, one hidden layer of 8): fused loss and the
    gradients of the trainable layers vs the float64 oracle, which computes
    [sin(omega x), cos(omega x)] as the reference does; the frozen feature
    layer's gradient is exactly zero."""
    from fbpinns_gb300.networks import fourier_feature_layer
    recipe, ls, pcls, pkw, ocls, opar, d2 = CASES[name]
    static = decomposition(recipe)
    m, xd = static["m"], ls[0]
    gen = torch.Generator().manual_seed(83)
    omega = (2 * math.pi * 0.5 * torch.randn((m, 4, xd), generator=gen, dtype=torch.float64)).float()
    feat = tuple(t.double() for t in fourier_feature_layer(omega))
    layers32 = [feat] + [tuple(t.float().double() for t in layer) for layer in random_layers([8, 8, 1], m, seed=9)]
    x = _points(recipe if recipe != "multilevel" else "poisson", 500, 29)
    prob_static = pcls.init_params(**pkw)[0]
    P = oracle_params(static, layers32, opar)
    P["activation"] = "fourier"
    p = static["subdomain"]["params"]
    takes, all_ims, (active, a_ims, f_ims) = OT.get_inputs(x, np.ones(m, dtype=int), p[0].numpy(),
                                                          p[1].numpy(), static["subdomain"]["pou"].numpy())
    loss_ref, grads, _ = OM.value_and_grad(P, a_ims, f_ims, [[torch.tensor(x, dtype=torch.float64)]], [takes],
                                           [OM.get_jmaps(_required(name))], ocls)
    g_ref = torch.cat([t.reshape(len(a_ims), -1) for layer in grads[1:] for t in layer], 1).numpy()
    eng = _engine(static, layers32, d2 | (_lib.D2_LAPLACIAN if lap else 0), activation="fourier")
    assert eng.layer_sizes == [xd, 8, 8, 1]
    eng.set_state(active)
    eng.set_problem(pcls.fused_spec({"static": {"problem": prob_static}}))
    ps = eng.points(torch.tensor(x))
    eng.forward_pairs(ps)
    loss = eng.pou_loss(ps).item()
    grad = eng.adjoint(ps).cpu().numpy()
    ps.check_status()
    n_feat = 8 * xd + 8  # W1 and b1 of the feature layer
    assert abs(loss - loss_ref.item()) <= JET_TOL * abs(loss_ref.item()), (loss, loss_ref.item())
    assert np.all(grad[:, :n_feat] == 0)
    assert (e := rel_err(grad[a_ims][:, n_feat:], g_ref)) < GRAD_TOL, e


def test_laplacian_jets_match_sum_of_second_derivatives(cuda):
    """A Laplacian jet (FBP_D2_LAPLACIAN) equals u_xx + u_yy of the per-dim
    jet; value and gradient components agree too (FP32 rounding only)."""
    static = decomposition("poisson")
    for ls in ([2, 16, 16, 1], [2, 32, 32, 1], [2, 8, 8, 1]):
        layers = random_layers(ls, static["m"], seed=21)
        x = torch.tensor(_points("poisson", 5000, 3))
        Us = []
        for d2 in (3, 3 | _lib.D2_LAPLACIAN):
            eng = _engine(static, layers, d2)
            ps = eng.points(x)
            Us.append(FBPINNJet.apply(eng.theta, eng, ps).double().cpu().numpy())
        U, L = Us
        assert L.shape[1] == 4 and U.shape[1] == 5
        for c in range(3):
            assert rel_err(L[:, c], U[:, c]) < JET_TOL, (ls, c)
        assert rel_err(L[:, 3], U[:, 3] + U[:, 4]) < JET_TOL, ls


def test_grouped_wave_jets_match_per_dim_jets(cuda):
    """7 | FBP_D2_GROUP(3): the jet carries u_xx + u_yy and u_tt; they equal
    the per-dim jet's components (FP32 rounding only)."""
    static = decomposition("wave")
    layers = random_layers([3, 8, 8, 1], static["m"], seed=33)
    g = np.random.default_rng(8)
    x = torch.tensor(g.uniform([-1, -1, 0], [1, 1, 1], (3000, 3)).astype(np.float32))
    Us = []
    for d2 in (7, 7 | _lib.D2_GROUP(3)):
        eng = _engine(static, layers, d2)
        Us.append(FBPINNJet.apply(eng.theta, eng, eng.points(x)).double().cpu().numpy())
    U, G = Us
    assert U.shape[1] == 7 and G.shape[1] == 6
    for c in range(4):
        assert rel_err(G[:, c], U[:, c]) < JET_TOL, c
    assert rel_err(G[:, 4], U[:, 4] + U[:, 5]) < JET_TOL
    assert rel_err(G[:, 5], U[:, 6]) < JET_TOL


def test_generic_path_matches_fused(cuda):
    """FBPINNJet + constrained_jets + loss_fn in torch == the fused kernel path."""
    name = "burgers"
    recipe, ls, pcls, pkw, ocls, opar, d2 = CASES[name]
    static = decomposition(recipe)
    layers = random_layers(ls, static["m"], seed=9)
    x = torch.tensor(_points(recipe, 500, 4))
    eng = _engine(static, layers, d2)
    prob_static = pcls.init_params(**pkw)[0]
    all_params = {"static": {"problem": prob_static}, "trainable": {}}
    eng.set_problem(pcls.fused_spec(all_params))
    ps = eng.points(x)
    eng.forward_pairs(ps)
    loss_f = eng.pou_loss(ps).item()
    grad_f = eng.adjoint(ps).clone()
    theta = eng.theta.clone().requires_grad_(True)
    U = FBPINNJet.apply(theta, eng, ps)
    xc = ps.x
    Uc = constrained_jets(pcls.constraining_fn, all_params, xc, U, 2, d2)
    ujs = [Uc[:, jet_index(2, d2, ixs):jet_index(2, d2, ixs) + 1] for _, ixs in _required(name)]
    loss_g = pcls.loss_fn(all_params, [[xc] + ujs])
    loss_g.backward()
    assert abs(loss_g.item() - loss_f) <= 1e-5 * abs(loss_f)
    assert (e := rel_err(theta.grad.cpu().numpy(), grad_f.cpu().numpy())) < GRAD_TOL, e


def test_generic_two_constraints_and_inverse_vs_oracle(cuda):
    """Soft-BC oscillator (two constraints, one with a single point) and the
    inverse problem's trainable mu, through the generic path."""
    from fbpinns_gb300.trainers import GenericStep
    static = decomposition("ho")
    layers = random_layers([1, 8, 8, 1], static["m"], seed=2)
    for pcls, ocls, pkw in [(PR.HarmonicOscillator1D, OP.HarmonicOscillator1D, dict(d=2, w0=20)),
                            (PR.HarmonicOscillator1DInverse, OP.HarmonicOscillator1DInverse, dict(d=2, w0=20))]:
        ps_, pt_ = pcls.init_params(**pkw)
        all_params = {"static": {"problem": ps_, "decomposition": static},
                      "trainable": {"problem": {k: v.clone().float().cuda() for k, v in pt_.items()}}}
        from fbpinns_gb300.domains import RectangularDomainND
        dom_ps = RectangularDomainND.init_params(np.array([0.]), np.array([1.]))[0]
        all_params["static"]["domain"] = dom_ps
        cons = pcls.sample_constraints(all_params, RectangularDomainND, 0, "grid", ((50,),))
        eng = FBPINNEngine(static, [1, 8, 8, 1], d2mask_of([c[-1] for c in cons], 1), chunk=64)
        eng.set_theta(pack_layers([(w.float(), b.float()) for w, b in layers]))
        step = GenericStep(eng, pcls, all_params, [c[:-1] for c in cons], [c[-1] for c in cons])
        theta = eng.theta.clone().requires_grad_(True)
        loss, gtheta, gprob = step.loss_and_grads(theta)
        # oracle
        x_all = np.concatenate([c[0].numpy() for c in cons]).astype(np.float32)
        offs = np.cumsum([0] + [c[0].shape[0] for c in cons[:-1]])
        cf = np.zeros((x_all.shape[0], len(cons)), bool)
        for ic, c in enumerate(cons):
            cf[offs[ic]:offs[ic] + c[0].shape[0], ic] = True
        p = static["subdomain"]["params"]
        takes, all_ims, (active, a_ims, f_ims) = OT.get_inputs(x_all, np.ones(static["m"], dtype=int), p[0].numpy(),
                                                              p[1].numpy(), static["subdomain"]["pou"].numpy())
        takess = OT.split_takes(takes, cf, x_all.shape[0])
        ocons = [[torch.tensor(c[0].numpy(), dtype=torch.float64)] + [torch.as_tensor(v).double() for v in c[1:-1]]
                 for c in cons]
        layers32 = [(w.float().double(), b.float().double()) for w, b in layers]
        P = oracle_params(static, layers32, {k: (v if not torch.is_tensor(v) else v.double()) for k, v in ps_.items()
                                             if k != "c_fn"})
        P["problem_trainable"] = {k: v.double() for k, v in pt_.items()}
        lref, gref, gpr = OM.value_and_grad(P, a_ims, f_ims, ocons, takess, [OM.get_jmaps(c[-1]) for c in cons], ocls,
                                            trainable_problem_keys=tuple(pt_.keys()))
        assert abs(loss.item() - lref.item()) <= 1e-5 * abs(lref.item()), (pcls.__name__, loss.item(), lref.item())
        gpack = torch.cat([t.reshape(len(a_ims), -1) for dw, db in gref for t in (dw, db)], 1).numpy()
        assert (e := rel_err(gtheta.cpu().numpy()[a_ims], gpack)) < GRAD_TOL, (e, pcls.__name__)
        for k in pt_:
            assert abs(gprob[k].item() - gpr[k].item()) <= 1e-4 * max(abs(gpr[k].item()), 1e-6)


def test_adam_matches_optax_semantics(cuda):
    static = decomposition("ho")
    eng = FBPINNEngine(static, [1, 8, 8, 1], d2mask=1)
    m, P = eng.m, eng.P
    g = torch.Generator().manual_seed(0)
    theta0 = torch.randn((m, P), generator=g)
    eng.set_theta(theta0)
    state = np.ones(m, dtype=int)
    state[3] = 2
    state[5] = 0
    eng.set_state(state)
    th, mu, nu, cnt = theta0.double(), torch.zeros(m, P, dtype=torch.float64), torch.zeros(m, P, dtype=torch.float64), 0
    for it in range(3):
        grad = torch.randn((m, P), generator=g)
        eng.adam(1e-3, grad=grad.cuda())
        mask = torch.tensor(state == 1)[:, None]
        th2, mu2, nu2, cnt2 = OM.adam_update(th, grad.double(), mu, nu, cnt, 1e-3)
        th = torch.where(mask, th2, th)
        mu = torch.where(mask, mu2, mu)
        nu = torch.where(mask, nu2, nu)
        cnt = cnt2
    assert int(eng.count.item()) == 3
    got = eng.theta.cpu().double()
    assert torch.equal(got[3], theta0[3].double()) and torch.equal(got[5], theta0[5].double())
    assert (got - th).abs().max().item() < 1e-6


def test_plain_step_matches_fused(cuda):
    """The plain torch-autograd drop-in step computes the same loss and gradient."""
    from fbpinns_gb300.plain import PlainStep
    from fbpinns_gb300.optim import adam
    static = decomposition("multilevel")
    layers = random_layers([2, 8, 8, 1], static["m"], seed=4)
    x = torch.tensor(_points("poisson", 1500, 8))
    prob_static = PR.Poisson2D.init_params(n_freq=6, sd=0.1)[0]
    all_params = {"static": {"problem": prob_static}, "trainable": {}}
    eng = _engine(static, layers, 3)
    eng.set_problem(PR.Poisson2D.fused_spec(all_params))
    ps = eng.points(x)
    eng.forward_pairs(ps)
    loss_f = eng.pou_loss(ps).item()
    grad_f = eng.adjoint(ps).cpu().numpy()
    pstep = PlainStep(eng, PR.Poisson2D, all_params, _required("poisson"), adam(1e-3), x=x)
    theta = eng.theta.detach().clone().requires_grad_(True)
    loss_p = pstep.loss(theta)
    (g,) = torch.autograd.grad(loss_p, [theta])
    assert abs(loss_p.item() - loss_f) <= 1e-5 * abs(loss_f)
    assert (e := rel_err(g.cpu().numpy(), grad_f)) < GRAD_TOL, e


def test_resampled_graph_step_is_deterministic_and_matches_eager(cuda):
    """Device resampling + interaction lists + fused step captured in a CUDA graph
    gives bit-identical parameters to the same steps run eagerly."""
    from fbpinns_gb300.trainers import FusedStep
    from fbpinns_gb300.optim import adam
    static = decomposition("poisson")
    layers = random_layers([2, 16, 16, 1], static["m"], seed=1)
    prob_static = PR.Poisson2D.init_params(n_freq=6, sd=0.1)[0]
    spec = PR.Poisson2D.fused_spec({"static": {"problem": prob_static}})
    results = []
    for use_graph, calls in ((True, 4), (False, 4)):  # capture's warm-up steps are rolled back
        eng = _engine(static, layers, 3, chunk=512)
        st = FusedStep(eng, spec, adam(1e-3), resample=(1 << 14, [0., 0.], [1., 1.], 3), use_graph=use_graph)
        for _ in range(calls):
            loss = st.step()
        torch.cuda.synchronize()
        st.check()
        results.append((eng.theta.cpu().clone(), loss.item(), int(eng.count.item())))
    (t_g, l_g, c_g), (t_e, l_e, c_e) = results
    assert c_g == c_e == 4
    assert np.isfinite(l_g) and l_g == l_e
    assert torch.equal(t_g, t_e)


def test_pipelined_resampling_matches_serial_steps(cuda):
    """Building the next step's lists on a second stream while the current step
    trains (two point sets, two graphs) gives bit-identical parameters, loss
    and step count to the serial resampled step."""
    from fbpinns_gb300.trainers import FusedStep
    from fbpinns_gb300.optim import adam
    static = decomposition("poisson")
    layers = random_layers([2, 16, 16, 1], static["m"], seed=2)
    prob_static = PR.Poisson2D.init_params(n_freq=6, sd=0.1)[0]
    spec = PR.Poisson2D.fused_spec({"static": {"problem": prob_static}})
    results = []
    for pipeline, use_graph in ((False, True), (True, True), (True, False)):
        eng = _engine(static, layers, 3 | _lib.D2_LAPLACIAN, chunk=512)
        st = FusedStep(eng, spec, adam(1e-3), resample=(1 << 14, [0., 0.], [1., 1.], 5), use_graph=use_graph,
                       pipeline=pipeline)
        losses = [st.step().item() for _ in range(5)]
        torch.cuda.synchronize()
        st.check()
        results.append((eng.theta.cpu().clone(), losses, int(eng.count.item())))
    ref = results[0]
    for theta, losses, count in results[1:]:
        assert count == ref[2] == 5
        assert losses == ref[1]
        assert torch.equal(theta, ref[0])


@pytest.mark.parametrize("tensor_cores", [True, False])
def test_work_item_schedules_give_identical_steps(cuda, tensor_cores):
    """The dynamic (device counter), static-stride and one-CTA-per-item
    schedules of the jet kernels give bitwise the same loss and parameters,
    and so do different resident grids."""
    from fbpinns_gb300.optim import adam
    static = decomposition("poisson")
    layers = random_layers([2, 16, 16, 1], static["m"], seed=4)
    prob_static = PR.Poisson2D.init_params(n_freq=6, sd=0.1)[0]
    spec = PR.Poisson2D.fused_spec({"static": {"problem": prob_static}})
    x = torch.rand((1 << 14, 2), generator=torch.Generator().manual_seed(3))
    results = []
    for schedule, grid in (("dynamic", None), ("static", None), ("per_item", None), ("dynamic", 37), ("static", 37)):
        eng = FBPINNEngine(static, layer_sizes(layers), 3 | _lib.D2_LAPLACIAN, chunk=256, grid=grid,
                           schedule=schedule, tensor_cores=tensor_cores)
        eng.set_theta(pack_layers([tuple(t.float() for t in layer) for layer in layers]))
        eng.set_problem(spec)
        ps = eng.points(x)
        opt = adam(1e-3)
        losses = [eng.fused_step(ps, opt["learning_rate"]).item() for _ in range(3)]
        torch.cuda.synchronize()
        ps.check_status()
        results.append((losses, eng.theta.cpu().clone()))
    for losses, theta in results[1:]:
        assert losses == results[0][0]
        assert torch.equal(theta, results[0][1])


def test_pipelined_host_points_match_serial_steps(cuda):
    """Host-fed points: copying the next step's points in and building their
    lists on a second stream during the current step gives bit-identical
    parameters and losses to the serial host-point step (graph and eager)."""
    from fbpinns_gb300.trainers import FusedStep
    from fbpinns_gb300.optim import adam
    static = decomposition("poisson")
    layers = random_layers([2, 16, 16, 1], static["m"], seed=3)
    prob_static = PR.Poisson2D.init_params(n_freq=6, sd=0.1)[0]
    spec = PR.Poisson2D.fused_spec({"static": {"problem": prob_static}})
    g = torch.Generator().manual_seed(9)
    batches = [torch.rand((1 << 14, 2), generator=g).pin_memory() for _ in range(6)]
    results = []
    for pipeline, use_graph in ((False, True), (True, True), (True, False)):
        eng = _engine(static, layers, 3 | _lib.D2_LAPLACIAN, chunk=512)
        st = FusedStep(eng, spec, adam(1e-3), host_points=1 << 14, x_probe=batches[0], use_graph=use_graph,
                       pipeline=pipeline)
        losses = []
        for k in range(5):
            st.step(batches[k], batches[k + 1])
            torch.cuda.synchronize()
            losses.append(float(st.loss_host.item()))
        st.check()
        results.append((eng.theta.cpu().clone(), losses))
    ref = results[0]
    for theta, losses in results[1:]:
        assert losses == ref[1]
        assert torch.equal(theta, ref[0])


def test_resampled_steps_match_oracle_points(cuda):
    """The points drawn on the device are uniform in the box and each step's
    interaction lists equal the oracle's for those points."""
    from fbpinns_gb300.trainers import FusedStep
    from fbpinns_gb300.optim import adam
    static = decomposition("multilevel")
    layers = random_layers([2, 8, 8, 1], static["m"], seed=1)
    prob_static = PR.Poisson2D.init_params(n_freq=6, sd=0.1)[0]
    spec = PR.Poisson2D.fused_spec({"static": {"problem": prob_static}})
    eng = _engine(static, layers, 3)
    st = FusedStep(eng, spec, adam(1e-3), resample=(4096, [0., 0.], [1., 1.], 5), use_graph=False)
    for _ in range(2):
        st.step()
        torch.cuda.synchronize()
        x = st.ps.x.cpu().numpy()
        assert x.min() >= 0.0 and x.max() < 1.0
        ref = _oracle_takes_for(static, x)
        t = st.ps.takes
        s = int(t.pt_off[t.n].item())
        np.testing.assert_array_equal(t.n_take[:s].cpu().numpy(), ref[1])
        np.testing.assert_array_equal(t.m_take[:s].cpu().numpy(), ref[0])
    st.check()


def _oracle_takes_for(static, x):
    p = static["subdomain"]["params"]
    takes, _, _ = OT.get_inputs(x, np.ones(static["m"], dtype=int), p[0].numpy(), p[1].numpy(),
                                static["subdomain"]["pou"].numpy())
    return takes


def test_trainer_short_run_matches_oracle_training(cuda):
    """FBPINNTrainer (fused HO hard-BC, 15 subdomains, 1-32-32-1, 200 grid points)
    vs the oracle's Adam loop from the same initial parameters: parameters after
    5 steps agree, and the test L1 decreases over 300 steps."""
    from fbpinns_gb300.constants import Constants, get_subdomain_ws
    from fbpinns_gb300.trainers import FBPINNTrainer, init_subdomain_networks
    from fbpinns_gb300 import networks
    sx = [np.linspace(0, 1, 15)]
    c = Constants(problem=PR.HarmonicOscillator1DHardBC, problem_init_kwargs=dict(d=2, w0=80, sd=0.1),
                  decomposition_init_kwargs=dict(subdomain_xs=sx, subdomain_ws=get_subdomain_ws(sx, 2.0),
                                                 unnorm=(0., 1.)),
                  network_init_kwargs=dict(layer_sizes=[1, 32, 32, 1]), ns=((200,),), n_test=(1000,),
                  n_steps=5, summary_freq=5, test_freq=5, use_graph=False)
    tr = FBPINNTrainer(c)
    ap = tr.train()
    got = networks.pack_layers(ap["trainable"]["network"]["subdomain"]["layers"]).double()
    # oracle
    static = tr.all_params["static"]["decomposition"]
    m = static["m"]
    _, net = init_subdomain_networks(networks.FCN, c.network_init_kwargs, m, c.seed)
    layers = [(w.double(), b.double()) for w, b in net["layers"]]
    P = oracle_params(static, layers, {"sd": 0.1, "mu": 4, "k": 6400})
    x = np.linspace(0, 1, 200, dtype=np.float64).astype(np.float32).reshape(-1, 1)
    p = static["subdomain"]["params"]
    takes, all_ims, (active, a_ims, f_ims) = OT.get_inputs(x, np.ones(m, dtype=int), p[0].numpy(), p[1].numpy(),
                                                          static["subdomain"]["pou"].numpy())
    jm = OM.get_jmaps(((0, ()), (0, (0,)), (0, (0, 0))))
    mu = [torch.zeros_like(t) for wb in layers for t in wb]
    nu = [torch.zeros_like(t) for wb in layers for t in wb]
    ai = torch.as_tensor(a_ims)
    for it in range(5):
        _, grads, _ = OM.value_and_grad(P, a_ims, f_ims, [[torch.tensor(x, dtype=torch.float64)]], [takes], [jm],
                                        OP.HarmonicOscillator1DHardBC)
        flat = [t for gw in grads for t in gw]
        new = []
        for li, (w, b) in enumerate(P["layers"]):
            pair = []
            for k, t in enumerate((w, b)):
                idx = 2 * li + k
                g = torch.zeros_like(t)
                g[ai] = flat[idx]
                th, mu[idx], nu[idx], _ = OM.adam_update(t, g, mu[idx], nu[idx], it, 1e-3)
                pair.append(th)
            new.append(tuple(pair))
        P["layers"] = new
    ref = networks.pack_layers([(w, b) for w, b in P["layers"]])
    # Adam normalises the update, so compare the parameter change after 5 steps
    init = networks.pack_layers(layers)
    d_got, d_ref = (got - init).numpy(), (ref - init).numpy()
    assert rel_err(d_got, d_ref) < 1e-3
    # and a longer run reduces the test error
    c2 = Constants(**{k: v for k, v in vars(c).items() if k in ("problem", "problem_init_kwargs",
                                                                 "decomposition_init_kwargs", "network_init_kwargs",
                                                                 "ns", "n_test")},
                   n_steps=300, summary_freq=100, test_freq=300, use_graph=True)
    tr2 = FBPINNTrainer(c2)
    tr2.train()
    l1 = [r[1] for r in tr2.u_test_losses]
    assert l1[-1] < l1[0]


def test_fast_tanh_error(cuda):
    """The device tanh of the jet kernels vs torch's float64 tanh: absolute error
    below 2.5e-7 over [-20, 20] (the jets need absolute accuracy)."""
    from fbpinns_gb300 import _lib
    lib = _lib.load()
    x = torch.cat([torch.linspace(-20, 20, 2_000_001), torch.linspace(-1e-3, 1e-3, 100_001),
                   torch.tensor([0.0, -0.0, 1e-30, -1e-30, 80.0, -80.0])]).to(cuda)
    y = torch.empty_like(x)
    _lib.check(lib.fbp_tanh_probe(_lib.ptr(x), _lib.ptr(y), x.numel(), _lib.stream_ptr()), "fbp_tanh_probe")
    ref = torch.tanh(x.double())
    err = (y.double() - ref).abs().max().item()
    assert err < 2.5e-7, err
    assert torch.all(y.abs() <= 1.0)


def test_work_item_autotuner(cuda):
    """The autotuner times every candidate on the actual points, keeps the
    fastest on the engine, and the step then uses exactly those item sizes
    (and gives the same loss as an engine set to them by hand)."""
    from fbpinns_gb300.autotune import tune_work_items
    static = decomposition("poisson")
    layers = random_layers([2, 16, 16, 1], static["m"], seed=6)
    prob_static = PR.Poisson2D.init_params(n_freq=6, sd=0.1)[0]
    spec = PR.Poisson2D.fused_spec({"static": {"problem": prob_static}})
    x = torch.rand((1 << 14, 2), generator=torch.Generator().manual_seed(4))
    eng = _engine(static, layers, 3 | _lib.D2_LAPLACIAN, chunk=1024)
    eng.set_problem(spec)
    cands = [(256, 256), (256, 1024), (512, 2048)]
    tuned = tune_work_items(eng, x, candidates=cands, use_cache=False)
    sizes = {f"{a}/{f} dynamic/dynamic g0 fg0": (a, f) for a, f in cands}
    assert set(sizes) <= set(tuned["timings_ms"])
    best_size = min(sizes, key=lambda k: tuned["timings_ms"][k])
    ch = tuned["choice"]
    best = (ch["chunk"], ch["forward_chunk"])
    assert best == sizes[best_size]  # later stages tune the schedule and grids at these sizes
    assert tuned["best_ms"] == min(tuned["timings_ms"].values())
    assert (eng.chunk, eng.forward_chunk) == best
    ps = eng.points(x)
    assert (ps.chunk, ps.fwd_chunk) == best
    eng.forward_pairs(ps)
    loss = eng.pou_loss(ps).item()
    ref = FBPINNEngine(static, layer_sizes(layers), 3 | _lib.D2_LAPLACIAN, chunk=best[0], forward_chunk=best[1],
                       adaptive_items=False, schedule=ch["schedule"], grid=ch["grid"])
    ref.forward_grid, ref.forward_schedule = ch["forward_grid"], ch["forward_schedule"]
    ref.set_theta(eng.theta.clone())
    ref.set_problem(spec)
    ps2 = ref.points(x)
    ref.forward_pairs(ps2)
    assert ref.pou_loss(ps2).item() == loss


def test_scheduled_point_set_vs_oracle(cuda):
    """A scheduler mask applied on the device (fbp_train_mask, the kept-pair
    sort and the masked loss) over all global points, against the reference's
    own _get_update_inputs for that mask (golden inputs_burgers_sched: a line
    scheduler's mask on a 40 x 20 grid): the same subdomain states and
    training points (bit-exact), and the loss and gradients of the oracle on
    those training points (1e-5)."""
    g = golden("inputs_burgers_sched.npz")
    static = decomposition("burgers")
    m = static["m"]
    raw = np.asarray(g["active_in"]).astype(int)
    x_global = np.asarray(g["x_global"], dtype=np.float32)
    recipe, ls, pcls, pkw, ocls, opar, d2 = CASES["burgers"]
    layers32 = [(w.float().double(), b.float().double()) for w, b in random_layers(ls, m, seed=11)]
    eng = _engine(static, layers32, d2, chunk=256)
    prob_static = pcls.init_params(**pkw)[0]
    eng.set_problem(pcls.fused_spec({"static": {"problem": prob_static}}))
    eng.set_raw_state(raw)
    ps = eng.points(torch.tensor(x_global), scheduled=True)
    assert np.array_equal(eng.state.cpu().numpy(), np.asarray(g["active_out"]))
    keep = ps.pt_keep[:ps.n].cpu().numpy().astype(bool)
    assert np.array_equal(x_global[keep], np.asarray(g["x_batch"], dtype=np.float32))
    assert int(ps.n_keep.item()) == keep.sum()
    eng.forward_pairs(ps)
    loss = eng.pou_loss(ps).item()
    grad = eng.adjoint(ps).cpu().numpy()
    ps.check_status()
    # oracle on the reference's training points for this mask
    xb = x_global[keep]
    p = static["subdomain"]["params"]
    takes, all_ims, (active, a_ims, f_ims) = OT.get_inputs(xb, raw, p[0].numpy(), p[1].numpy(),
                                                          static["subdomain"]["pou"].numpy())
    assert np.array_equal(np.asarray(active), eng.state.cpu().numpy())
    P = oracle_params(static, layers32, opar)
    loss_ref, grads, _ = OM.value_and_grad(P, a_ims, f_ims, [[torch.tensor(xb, dtype=torch.float64)]], [takes],
                                           [OM.get_jmaps(_required("burgers"))], ocls)
    g_ref = torch.cat([t.reshape(len(a_ims), -1) for dw, db in grads for t in (dw, db)], 1).numpy()
    assert abs(loss - loss_ref.item()) <= JET_TOL * abs(loss_ref.item()), (loss, loss_ref.item())
    assert (e := rel_err(grad[a_ims], g_ref)) < GRAD_TOL, e
    assert np.all(grad[np.setdiff1d(np.arange(m), a_ims)] == 0)


@pytest.mark.parametrize("window", ["cosine", "sigmoid", "bump", "wendland", "rbf"])
@pytest.mark.parametrize("ls,tc", [([2, 8, 8, 1], False), ([2, 16, 16, 1], True)])
def test_window_kinds_vs_oracle(cuda, window, ls, tc):
    """Every window of fbpinns/windows.py in the jet kernels (the
    decompositions' window option): POU-combined jets (u, u_x, u_y, u_xx +
    u_yy), the fused Poisson loss and the gradients against the float64
    oracle, whose windows are pinned on the reference's values; FMA kernels
    (2-8-8-1) and the tensor-core forward and adjoint (2-16-16-1)."""
    static = decomposition("multilevel", window=window)
    m = static["m"]
    layers32 = [(w.float().double(), b.float().double()) for w, b in random_layers(ls, m, seed=17)]
    x = _points("poisson", 1500, 31)
    d2 = 3 | _lib.D2_LAPLACIAN
    eng = _engine(static, layers32, d2, chunk=256, tensor_cores=tc, tc_adjoint=tc)
    assert eng.tensor_cores == tc and eng.tc_adjoint == tc
    prob_static = PR.Poisson2D.init_params(n_freq=6, sd=0.1)[0]
    eng.set_problem(PR.Poisson2D.fused_spec({"static": {"problem": prob_static}}))
    ps = eng.points(torch.tensor(x))
    U = FBPINNJet.apply(eng.theta, eng, ps).double().cpu().numpy()
    eng.forward_pairs(ps)
    loss = eng.pou_loss(ps).item()
    grad = eng.adjoint(ps).cpu().numpy()
    ps.check_status()
    P = oracle_params(static, layers32, {"sd": 0.1, "n_freq": 6})
    assert P["window"] == window
    p = static["subdomain"]["params"]
    takes, all_ims, (active, a_ims, f_ims) = OT.get_inputs(x, np.ones(m, dtype=int), p[0].numpy(), p[1].numpy(),
                                                          static["subdomain"]["pou"].numpy())
    Pc = OM.cut_params(P, all_ims)
    req = ((0, ()), (0, (0,)), (0, (1,)), (0, (0, 0)), (0, (1, 1)))
    ujs = OM.fbpinn_forward(Pc, torch.tensor(x, dtype=torch.float64), takes, lambda P_, xb, u: u, OM.get_jmaps(req))
    for k in range(3):
        assert rel_err(U[:, k:k + 1], ujs[k].numpy()) < JET_TOL, (window, k)
    assert rel_err(U[:, 3:4], (ujs[3] + ujs[4]).numpy()) < JET_TOL, window
    loss_ref, grads, _ = OM.value_and_grad(P, a_ims, f_ims, [[torch.tensor(x, dtype=torch.float64)]], [takes],
                                           [OM.get_jmaps(_required("poisson"))], OP.Poisson2D)
    g_ref = torch.cat([t.reshape(len(a_ims), -1) for dw, db in grads for t in (dw, db)], 1).numpy()
    assert abs(loss - loss_ref.item()) <= JET_TOL * abs(loss_ref.item()), (window, loss, loss_ref.item())
    assert (e := rel_err(grad[a_ims], g_ref)) < GRAD_TOL, (window, e)


@pytest.mark.parametrize("name,lap,tc,act", [("poisson_bench", True, True, "tanh"), ("poisson_bench", True, False, "tanh"),
                                             ("poisson_bench", False, True, "tanh"),
                                             ("poisson_bench", False, False, "tanh"),
                                             ("wave_bench", True, False, "tanh"), ("poisson", True, False, "adaptive_tanh"),
                                             ("poisson", False, False, "sin")])
def test_stored_layer2_jets_match_recompute(cuda, name, lap, tc, act):
    """The adjoint reading the layer-2 z-jets stored by the forward
    (fbp_pairs.zs) against the same adjoint recomputing them: bitwise equal
    gradients after the FMA forward (the same sums in the same order), within
    1e-6 after the tensor-core forward (3xTF32 z-jets); a point set over the
    memory limit keeps no buffer and recomputes."""
    recipe, ls, pcls, pkw, ocls, opar, d2 = CASES[name]
    static = decomposition(recipe)
    scale = 1.0 if act in ("tanh", "adaptive_tanh") else math.sqrt(6.0)
    gen = torch.Generator().manual_seed(71)
    layers = [(w * scale, b * scale) + tuple(0.5 + torch.rand(b.shape, generator=gen, dtype=torch.float64)
                                             for _ in range(_lib.ACT_EXTRA[act]))
              for w, b in random_layers(ls, static["m"], seed=5)]
    theta = pack_layers([tuple(t.float() for t in layer) for layer in layers])
    x = _points(recipe if recipe != "multilevel" else "poisson", 2000, 23)
    prob_static = pcls.init_params(**pkw)[0]
    d2e = d2 | (0 if not lap else _lib.D2_LAPLACIAN if d2 == 3 else _lib.D2_GROUP(3))

    def run(limit=None):
        eng = FBPINNEngine(static, ls, d2e, chunk=1024, activation=act, tensor_cores=tc, store_z2=True)
        if limit is not None:
            eng.z2_limit = limit
        eng.set_theta(theta)
        eng.set_problem(pcls.fused_spec({"static": {"problem": prob_static}}))
        ps = eng.points(torch.tensor(x))
        eng.forward_pairs(ps)
        loss = eng.pou_loss(ps).item()
        g_store = eng.adjoint(ps).clone()
        g_recompute = eng.adjoint(ps, z2=False).clone()
        ps.check_status()
        return eng, ps, loss, g_store, g_recompute

    eng, ps, loss, gs, gr = run()
    assert ps.zs is not None and tuple(ps.zs.shape) == (eng.J * ls[2], ps.s_cap)
    assert eng.tensor_cores == tc
    if tc:
        assert (e := rel_err(gs.cpu().numpy(), gr.cpu().numpy())) < 1e-6, e
    else:
        assert torch.equal(gs, gr)
    _, ps0, loss0, gs0, gr0 = run(limit=0)
    assert ps0.zs is None and loss0 == loss
    assert torch.equal(gs0, gr0) and torch.equal(gr0, gr)


def test_host_point_order_follows_probe_extent(cuda):
    """Host batches enter the point set in cell order over the first batch's
    box, which gives the loss of the drawn order up to FP32 rounding (the same
    points, summed in another order); a first batch with no extent along a dim
    turns the ordering off, and the step still runs."""
    from fbpinns_gb300.trainers import FusedStep
    from fbpinns_gb300.optim import adam
    static = decomposition("poisson")
    layers = random_layers([2, 16, 16, 1], static["m"], seed=3)
    prob_static = PR.Poisson2D.init_params(n_freq=6, sd=0.1)[0]
    spec = PR.Poisson2D.fused_spec({"static": {"problem": prob_static}})
    g = torch.Generator().manual_seed(9)
    x = torch.rand((1 << 14, 2), generator=g).pin_memory()
    losses = {}
    for order in (True, False):
        eng = FBPINNEngine(static, layer_sizes(layers), 3 | _lib.D2_LAPLACIAN, chunk=512, cell_order=order)
        eng.set_theta(pack_layers([tuple(t.float() for t in layer) for layer in layers]))
        st = FusedStep(eng, spec, adam(1e-3), host_points=1 << 14, x_probe=x, use_graph=False, pipeline=False)
        assert st.order_host == order
        st.step(x)
        torch.cuda.synchronize()
        st.check()
        losses[order] = float(st.loss_host.item())
        if order:  # the point set holds the batch in cell order: the same points, sorted differently
            a, b = st.ps.x.cpu().numpy(), x.numpy()
            assert not np.array_equal(a, b)
            np.testing.assert_array_equal(a[np.lexsort((a[:, 1], a[:, 0]))], b[np.lexsort((b[:, 1], b[:, 0]))])
    # a slot's pairs are summed by a segmented scan whose shape follows their
    # lanes in a row of 32 pairs, so another order rounds each point's FP32 sums
    # differently: equal to FP32 rounding (measured 3.5e-11 relative)
    assert abs(losses[True] - losses[False]) <= 1e-6 * abs(losses[False])
    flat = x.clone()
    flat[:, 1] = 0.5  # no extent along y
    eng = FBPINNEngine(static, layer_sizes(layers), 3 | _lib.D2_LAPLACIAN, chunk=512)
    eng.set_theta(pack_layers([tuple(t.float() for t in layer) for layer in layers]))
    st = FusedStep(eng, spec, adam(1e-3), host_points=1 << 14, x_probe=flat.pin_memory(), use_graph=False,
                   pipeline=False)
    assert not st.order_host
    st.step(flat.pin_memory())
    torch.cuda.synchronize()
    st.check()
    assert np.isfinite(float(st.loss_host.item()))
