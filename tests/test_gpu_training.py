"""Training runs on the GPU: every workload configuration (reduced sizes)
through FBPINNTrainer, matched test error of the fused and plain steps, the
PINN trainer, and model save / load in the reference's pickle layout."""

import math
import os

import numpy as np
import pytest
import torch

from fbpinns_gb300 import configs
from fbpinns_gb300.trainers import FBPINNTrainer, PINNTrainer

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,steps", [("ho", 300), ("burgers", 300), ("poisson", 200), ("wave", 60),
                                        ("helmholtz", 60)])
def test_config_trains(cuda, name, steps):
    c = configs.CONFIGS[name](n_steps=steps, small=True)
    c.summary_freq = max(1, steps // 6)
    c.test_freq = steps
    tr = FBPINNTrainer(c)
    tr.train()
    losses = [h["loss"] for h in tr.history]
    assert all(math.isfinite(v) for v in losses)
    l1 = [r[1] for r in tr.u_test_losses]
    assert len(l1) == 2 and all(math.isfinite(v) for v in l1)
    if name in ("ho", "poisson", "burgers"):
        assert losses[-1] < losses[0]


def test_matched_test_error_fused_vs_plain(cuda):
    """Same initial parameters and the same per-step points (Philox stream keyed
    by the step count): the fused and the plain step reach the same test L1."""
    res = {}
    for engine in ("fused", "plain"):
        c = configs.poisson(n_steps=120, small=True)
        c.engine = engine
        c.summary_freq, c.test_freq = 40, 120
        tr = FBPINNTrainer(c)
        tr.train()
        res[engine] = (tr.u_test_losses[-1][1], [h["loss"] for h in tr.history])
    l1f, l1p = res["fused"][0], res["plain"][0]
    assert abs(l1f - l1p) <= 0.05 * l1p, (l1f, l1p)
    for a, b in zip(res["fused"][1], res["plain"][1]):
        assert abs(a - b) <= 0.05 * abs(b)


def test_pinn_trainer(cuda):
    c = configs.ho(n_steps=200)
    c.network_init_kwargs = dict(layer_sizes=[1, 32, 32, 1])
    c.summary_freq, c.test_freq = 50, 200
    tr = PINNTrainer(c)
    ap = tr.train()
    assert tr.engine.m == 1
    assert float(tr.engine.grid.flags[0]) == 0.0
    losses = [h["loss"] for h in tr.history]
    assert losses[-1] < losses[0]


def test_model_save_and_load(cuda, tmp_path, monkeypatch):
    from fbpinns_gb300.analysis import load_model, FBPINN_solution
    monkeypatch.chdir(tmp_path)
    c = configs.ho(n_steps=20)
    c.run = "saved"
    c.save_models = True
    c.model_save_freq = 20
    c.summary_freq, c.test_freq = 10, 20
    tr = FBPINNTrainer(c)
    tr.train()
    c2, model = load_model("saved", rootdir="results/")
    i, all_params, opt, active, losses = model
    assert i == 20 and opt["count"] == 20 and active.shape == (15,)
    x = torch.linspace(0, 1, 50).reshape(-1, 1)
    u_loaded = FBPINN_solution(c2, all_params, active, x)
    u_live = FBPINNTrainer.predict(tr.engine, tr.all_params, c.problem, x)
    assert torch.allclose(u_loaded, u_live, rtol=1e-6, atol=1e-6)


def test_siren_network_trains_fused(cuda):
    """A SIREN network (sin activations, networks.py:102-131) through the fused
    engine: the HO problem trains and the saved-model inference agrees."""
    from fbpinns_gb300.networks import SIREN
    c = configs.ho(n_steps=150)
    c.network = SIREN
    c.summary_freq, c.test_freq = 50, 150
    tr = FBPINNTrainer(c)
    tr.train()
    assert tr.engine.activation == "sin" and not tr.engine.tensor_cores
    losses = [h["loss"] for h in tr.history]
    assert all(math.isfinite(v) for v in losses) and losses[-1] < losses[0]


@pytest.mark.parametrize("netname", ["AdaptiveFCN", "AdaptiveSIREN"])
def test_adaptive_networks_train_fused(cuda, netname):
    """Adaptive networks through the fused engine: the HO problem trains, the
    activation parameters move, and the returned params keep the reference's
    per-layer tuples (W, b, a) / (W, b, c, o)."""
    from fbpinns_gb300 import networks
    c = configs.ho(n_steps=150)
    c.network = getattr(networks, netname)
    c.summary_freq, c.test_freq = 50, 150
    tr = FBPINNTrainer(c)
    ap = tr.train()
    losses = [h["loss"] for h in tr.history]
    assert all(math.isfinite(v) for v in losses) and losses[-1] < losses[0]
    layers = ap["trainable"]["network"]["subdomain"]["layers"]
    assert all(len(layer) == (3 if netname == "AdaptiveFCN" else 4) for layer in layers)
    assert not torch.allclose(layers[0][2], torch.ones_like(layers[0][2]))


def test_fourier_network_trains_fused_and_reloads(cuda, tmp_path, monkeypatch):
    """FourierFCN (networks.py:165-194; 8 features, one hidden layer of 32)
    through the fused engine: the HO problem trains, omega stays as it was
    drawn, the returned and saved params keep the reference's layout
    (static omega (m, F, xd), trainable [(W (m,32,16), b), (W (m,1,32), b)])
    and inference from the saved model agrees with the live engine."""
    from fbpinns_gb300.analysis import load_model, FBPINN_solution
    from fbpinns_gb300.networks import FourierFCN
    monkeypatch.chdir(tmp_path)
    c = configs.ho(n_steps=150)
    c.network = FourierFCN
    c.network_init_kwargs = dict(layer_sizes=[1, 32, 1], mu=0.0, sd=1.0, n_features=8)
    c.run = "fourier"
    c.save_models, c.model_save_freq = True, 150
    c.summary_freq, c.test_freq = 50, 150
    tr = FBPINNTrainer(c)
    ap = tr.train()
    assert tr.engine.activation == "fourier" and tr.engine.layer_sizes == [1, 16, 32, 1]
    losses = [h["loss"] for h in tr.history]
    assert all(math.isfinite(v) for v in losses) and losses[-1] < losses[0]
    omega = ap["static"]["network"]["subdomain"]["omega"]
    assert tuple(omega.shape) == (15, 8, 1)
    W1 = tr.engine.theta[:, :16].reshape(15, 16, 1).cpu()
    assert torch.equal(W1[:, :8], omega.float()) and torch.equal(W1[:, 8:], omega.float())
    layers = ap["trainable"]["network"]["subdomain"]["layers"]
    assert [tuple(layer[0].shape) for layer in layers] == [(15, 32, 16), (15, 1, 32)]
    c2, model = load_model("fourier", rootdir="results/")
    x = torch.linspace(0, 1, 50).reshape(-1, 1)
    u_loaded = FBPINN_solution(c2, model[1], model[3], x)
    u_live = FBPINNTrainer.predict(tr.engine, tr.all_params, c.problem, x)
    assert torch.allclose(u_loaded, u_live, rtol=1e-6, atol=1e-6)


@pytest.mark.parametrize("engine", ["fused", "plain"])
def test_list_overflow_raises_during_training(cuda, engine):
    """Pair and slot capacities too small for the resampled batches (0.3 x
    the first batch) stop training at the first status check -- the first
    summary step for the fused step, the first step for the plain one (it
    reads its sizes every step) -- not after the last step: the kernels skip
    what does not fit, so later steps would train on truncated lists."""
    from fbpinns_gb300._lib import FBPLibraryError
    c = configs.poisson(n_steps=40, small=True)
    c.engine = engine
    c.pair_headroom = 0.3
    c.summary_freq, c.test_freq = 4, 40
    tr = FBPINNTrainer(c)
    with pytest.raises(FBPLibraryError, match="capacity"):
        tr.train()
    assert tr.history == []  # raised before the first summary line was recorded
    assert int(tr.engine.count.item()) <= (4 if engine == "fused" else 0)


def test_scheduler_changes_replay_one_capture(cuda):
    """Burgers with the line scheduler (many mask changes): the fused step
    follows every change on the device -- one host-to-device copy of the
    mask, the training points, states and work queues rebuilt by kernels --
    with one graph capture in total, and gives the same losses and test
    error as the host path that builds a new point set (and capture) per
    change."""
    from fbpinns_gb300.trainers import FusedStep
    res = {}
    for dev_sched in (True, False):
        c = configs.burgers(n_steps=400, small=True)
        c.summary_freq, c.test_freq = 20, 400
        c.device_schedule = dev_sched
        c.autotune = False
        captures = []
        orig = FusedStep.capture

        def counted(self, *a, **k):
            captures.append(1)
            return orig(self, *a, **k)
        FusedStep.capture = counted
        try:
            tr = FBPINNTrainer(c)
            tr.train()
        finally:
            FusedStep.capture = orig
        res[dev_sched] = ([h["loss"] for h in tr.history], tr.u_test_losses[-1][1], len(captures))
    (l_dev, t_dev, n_dev), (l_host, t_host, n_host) = res[True], res[False]
    assert n_dev == 1 and n_host > 1, (n_dev, n_host)
    assert len(l_dev) == len(l_host) == 20
    for a, b in zip(l_dev, l_host):
        assert abs(a - b) <= 1e-4 * abs(b), (a, b)
    assert abs(t_dev - t_host) <= 1e-4 * t_host


def test_autotuner_searches_launches_and_caches(cuda, tmp_path, monkeypatch):
    """The launch autotuner searches item sizes, schedule and both CTA
    counts, keeps the fastest on the engine, and a second engine of the same
    configuration takes the choice from the on-disk cache without timing."""
    from fbpinns_gb300 import autotune
    from fbpinns_gb300.engine import FBPINNEngine
    from fbpinns_gb300.problems import Poisson2D
    monkeypatch.setenv(autotune.CACHE_ENV, str(tmp_path / "tune.json"))
    c = configs.poisson(n_steps=1, small=True)
    dec = c.decomposition.init_params(**c.decomposition_init_kwargs)[0]
    x = torch.rand((1 << 14, 2), generator=torch.Generator().manual_seed(3))
    spec = Poisson2D.fused_spec({"static": {"problem": Poisson2D.init_params(n_freq=4, sd=0.1)[0]}})
    out = []
    for _ in range(2):
        eng = FBPINNEngine(dec, [2, 16, 16, 1], 3 | 8)
        eng.set_problem(spec)
        out.append(autotune.tune_work_items(eng, x))
    first, second = out
    assert first["cache"] == "miss" and second["cache"] == "hit"
    assert second["choice"] == first["choice"]
    assert set(first["searched"]) == {"item_sizes", "schedule", "forward_schedule", "grid", "forward_grid"}
    assert len(first["timings_ms"]) >= len(first["searched"]["item_sizes"]) + 2
    ch = first["choice"]
    assert (eng.chunk, eng.forward_chunk, eng.schedule, eng.launch_grid, eng.forward_grid) == \
        (ch["chunk"], ch["forward_chunk"], ch["schedule"], ch["grid"], ch["forward_grid"])
    assert eng.fwd_schedule() == ch["forward_schedule"]


def test_pinn_trainer_matches_oracle(cuda):
    """PINNTrainer (the one-box case of the engine) against the oracle's own
    restatement of the reference PINN (fbpinns/trainers.py:120-124, 179-195,
    269-306: domain normalisation, one network, unnormalisation, hard
    constraint, no window and no partition of unity): the same initial
    network, points and Adam settings give the same loss at each of the
    first five steps (1e-5) and the same parameters after them (1e-6 of
    their scale)."""
    from fbpinns_gb300.networks import FCN, unpack_layers
    from fbpinns_gb300.trainers import init_subdomain_networks
    from oracle import model as OM
    from oracle import problems as OP
    c = configs.ho(n_steps=5)
    c.network_init_kwargs = dict(layer_sizes=[1, 32, 32, 1])
    c.summary_freq, c.test_freq = 1, 5
    tr = PINNTrainer(c)
    tr.train()
    losses = [h["loss"] for h in tr.history]
    assert len(losses) == 5
    # the oracle from the same initial network (init_subdomain_networks with m = 1)
    _, net = init_subdomain_networks(FCN, c.network_init_kwargs, 1, c.seed)
    layers = [tuple(t[0].double() for t in layer) for layer in net["layers"]]
    x = torch.linspace(0, 1, 200, dtype=torch.float64).reshape(-1, 1)
    P = {"domain_xmin": torch.tensor([0.0], dtype=torch.float64), "domain_xmax": torch.tensor([1.0], dtype=torch.float64),
         "unnorm": (0.0, 1.0), "layers": layers, "problem": {"sd": 0.1, "mu": 4.0, "k": 6400.0}}
    jm = [OM.get_jmaps(((0, ()), (0, (0,)), (0, (0, 0))))]
    mus = [tuple(torch.zeros_like(t) for t in layer) for layer in layers]
    nus = [tuple(torch.zeros_like(t) for t in layer) for layer in layers]
    for k in range(5):
        loss, grads = OM.pinn_value_and_grad(P, [[x]], jm, OP.HarmonicOscillator1DHardBC)
        assert abs(losses[k] - loss.item()) <= 1e-5 * abs(loss.item()), (k, losses[k], loss.item())
        new, nm, nn = [], [], []
        for layer, g, mu, nu in zip(P["layers"], grads, mus, nus):
            out = [OM.adam_update(t, gt, m1, m2, k, 1e-3) for t, gt, m1, m2 in zip(layer, g, mu, nu)]
            new.append(tuple(o[0] for o in out))
            nm.append(tuple(o[1] for o in out))
            nn.append(tuple(o[2] for o in out))
        P["layers"], mus, nus = new, nm, nn
    got = unpack_layers(tr.engine.theta, tr.engine.layer_sizes, tr.engine.extra)
    for lg, lo in zip(got, P["layers"]):
        for tg, to in zip(lg, lo):
            tg = tg[0].double().cpu()
            assert (tg - to).abs().max().item() <= 1e-6 * max(to.abs().max().item(), 1.0)


def test_ho_training_trajectory_matches_oracle():
    """The oscillator configuration (15 subdomains of width 2x spacing, FCN
    1-32-32-1, 200 grid points, Adam 1e-3) trained for 200 steps through
    FBPINNTrainer on the GPU and by the float64 oracle's Adam loop on the CPU
    from the same initial parameters: the test L1 on 1000 points after 0, 100
    and 200 steps agrees to 1e-4 relative (measured over 2000 steps: to
    4e-7 at step 2000)."""
    from helpers import oracle_params
    from oracle import model as OM, problems as OP, takes as OT
    from fbpinns_gb300 import configs, networks
    from fbpinns_gb300.decompositions import RectangularDecompositionND
    from fbpinns_gb300.problems import HarmonicOscillator1DHardBC
    from fbpinns_gb300.trainers import FBPINNTrainer, init_subdomain_networks
    steps = 200
    c = configs.ho(n_steps=steps)
    c.test_freq = 100
    tr = FBPINNTrainer(c)
    tr.train()
    got = [r[1] for r in tr.u_test_losses]
    static = RectangularDecompositionND.init_params(**c.decomposition_init_kwargs)[0]
    m = static["m"]
    _, net = init_subdomain_networks(networks.FCN, c.network_init_kwargs, m, c.seed)
    layers = [(w.double(), b.double()) for w, b in net["layers"]]
    P = oracle_params(static, layers, {"sd": 0.1, "mu": 4, "k": 6400})
    p = static["subdomain"]["params"]
    bounds = (p[0].numpy(), p[1].numpy(), static["subdomain"]["pou"].numpy())
    x = np.linspace(0, 1, 200).astype(np.float32).reshape(-1, 1)
    takes, _, (_, a_ims, f_ims) = OT.get_inputs(x, np.ones(m, dtype=int), *bounds)
    xt = np.linspace(0, 1, 1000).astype(np.float32).reshape(-1, 1)
    t_takes, t_all, _ = OT.get_inputs(xt, np.ones(m, dtype=int), *bounds)
    ps, _ = HarmonicOscillator1DHardBC.init_params(d=2, w0=80, sd=0.1)
    u_ex = HarmonicOscillator1DHardBC.exact_solution({"static": {"problem": ps}}, torch.tensor(xt)).double()
    jm = OM.get_jmaps(((0, ()), (0, (0,)), (0, (0, 0))))
    cfn = OP.HarmonicOscillator1DHardBC.constraining_fn
    mu = [torch.zeros_like(t) for wb in layers for t in wb]
    nu = [torch.zeros_like(t) for wb in layers for t in wb]
    ai = torch.as_tensor(a_ims)
    ref = []
    for it in range(steps + 1):
        if it % 100 == 0:
            with torch.no_grad():
                u = OM.fbpinn_model(OM.cut_params(P, t_all), torch.tensor(xt, dtype=torch.float64), t_takes, cfn)[0]
            ref.append(float(torch.mean(torch.abs(u.reshape(-1) - u_ex.reshape(-1)))))
        if it == steps:
            break
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
    assert len(got) == len(ref) == 3
    for a, b in zip(got, ref):
        assert abs(a - b) <= 1e-4 * b, (got, ref)


def test_resampled_training_on_benchmark_shapes_matches_oracle():
    """The benchmark's decomposition and network (m = 1365, 2-16-16-1,
    Laplacian jets) trained by the fused step on batches of 4096 points redrawn
    each step (in cell order), and by the float64 oracle's Adam loop on the
    same points: the losses agree to 1e-6 relative at each of 10 steps
    (measured over 50 steps: within 7.4e-8)."""
    from helpers import decomposition, oracle_params, random_layers
    from oracle import model as OM, problems as OP, takes as OT
    from fbpinns_gb300 import _lib, networks
    from fbpinns_gb300 import problems as PR
    from fbpinns_gb300.engine import FBPINNEngine
    from fbpinns_gb300.optim import adam
    from fbpinns_gb300.trainers import FusedStep
    static = decomposition("poisson")
    m = static["m"]
    layers = [(w.float().double(), b.float().double()) for w, b in random_layers([2, 16, 16, 1], m, seed=12)]
    prob_static = PR.Poisson2D.init_params(n_freq=6, sd=0.1)[0]
    spec = PR.Poisson2D.fused_spec({"static": {"problem": prob_static}})
    eng = FBPINNEngine(static, [2, 16, 16, 1], 3 | _lib.D2_LAPLACIAN)
    eng.set_theta(networks.pack_layers([tuple(t.float() for t in layer) for layer in layers]))
    st = FusedStep(eng, spec, adam(1e-3), resample=(4096, [0.0, 0.0], [1.0, 1.0], 11), use_graph=False)
    P = oracle_params(static, layers, {"sd": 0.1, "n_freq": 6})
    p = static["subdomain"]["params"]
    bounds = (p[0].numpy(), p[1].numpy(), static["subdomain"]["pou"].numpy())
    jm = OM.get_jmaps(((0, (0, 0)), (0, (1, 1))))
    mu = [torch.zeros_like(t) for wb in layers for t in wb]
    nu = [torch.zeros_like(t) for wb in layers for t in wb]
    for it in range(10):
        x = st.ps.x.detach().cpu().numpy().copy()
        lg = float(st.step().item())
        takes, _, (_, a_ims, f_ims) = OT.get_inputs(x, np.ones(m, dtype=int), *bounds)
        lo, grads, _ = OM.value_and_grad(P, a_ims, f_ims, [[torch.tensor(x, dtype=torch.float64)]], [takes], [jm],
                                         OP.Poisson2D)
        ai = torch.as_tensor(a_ims)
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
        assert abs(lg - float(lo)) <= 1e-6 * abs(float(lo)), (it, lg, float(lo))
    st.check()
