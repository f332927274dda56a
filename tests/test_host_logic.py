"""Host-side logic (no GPU): the product's decompositions, schedulers, windows,
networks, samplers and exact solutions against golden vectors from the
reference's own code, the cell grid's completeness property, and the C ABI
library's exported symbols."""

import math
import os

import numpy as np
import pytest
import torch

from conftest import golden
from fbpinns_gb300 import decompositions as D, schedulers as S, windows as Wn, networks as N
from fbpinns_gb300 import problems as PR, domains as DOM
from fbpinns_gb300.constants import Constants, get_subdomain_ws


def _static_recipe(recipe):
    if recipe == "poisson":
        sxs = [[np.array([0.5])] * 2] + [[np.linspace(0, 1, k)] * 2 for k in (2, 4, 8, 16, 32)]
        sws = [[np.array([1.0])] * 2] + [get_subdomain_ws(s, 2.9) for s in sxs[1:]]
        return D.MultilevelRectangularDecompositionND.init_params(sxs, sws, (0., 1.))[0]
    if recipe == "3d":
        sx = [np.linspace(-1, 1, 5), np.linspace(-1, 1, 4), np.linspace(0, 1, 3)]
        return D.RectangularDecompositionND.init_params(sx, get_subdomain_ws(sx, 2.0), (0.5, 2.0))[0]
    return D.RectangularDecompositionND.init_params([np.array([0.5])], [np.array([1.2])], (0., 1.))[0]


@pytest.mark.parametrize("name,recipe", [("level_params_poisson.npz", "poisson"), ("level_params_3d.npz", "3d"),
                                         ("level_params_single.npz", "single")])
def test_decomposition_params_match_reference(name, recipe):
    g = golden(name)
    st = _static_recipe(recipe)
    p = st["subdomain"]["params"]
    for k, nm in enumerate(["xmins", "xmaxs", "wmins", "wmaxs", "flags", "unnorms"]):
        np.testing.assert_array_equal(p[k].numpy(), g[nm].astype(np.float32), err_msg=nm)
    np.testing.assert_array_equal(st["subdomain"]["pou"].numpy(), g["pou"].astype(np.float32))
    if "xmins0" in g:
        np.testing.assert_array_equal(st["xmins0"], g["xmins0"])
        np.testing.assert_array_equal(st["xmaxs0"], g["xmaxs0"])


def test_non_overlapping_decomposition_rejected():
    with pytest.raises(ValueError, match="not overlapping"):
        D.RectangularDecompositionND.init_params([np.linspace(0, 1, 5)], [0.2 * np.ones(5)], (0., 1.))
    with pytest.raises(ValueError, match="not same"):
        D.RectangularDecompositionND.init_params([np.linspace(0, 1, 5)], [np.ones(4)], (0., 1.))


def _sched_all_params(sxx, width):
    st = D.RectangularDecompositionND.init_params(sxx, [width * np.ones_like(v) for v in sxx], (0, 1))[0]
    return {"static": {"decomposition": st}}


def _record(s):
    steps, ms = [], []
    for i, a in enumerate(s):
        if a is not None:
            steps.append(i)
            ms.append(np.array(a).copy())
    return np.array(steps), np.array(ms)


def test_schedulers_match_reference():
    g = golden("schedulers.npz")
    xs1 = [np.array([-6, -4, -2, 0, 2, 4, 6.])]
    for tag, sxx in [("1d", xs1), ("2d", xs1 * 2), ("3d", xs1 * 3)]:
        ap = _sched_all_params(sxx, 3)
        xd = len(sxx)
        st, ms = _record(S.PointSchedulerRectangularND(ap, 100, np.zeros(xd)))
        np.testing.assert_array_equal(st, g[f"point_{tag}_steps"])
        np.testing.assert_array_equal(ms, g[f"point_{tag}_masks"])
        if xd >= 2:
            st, ms = _record(S.LineSchedulerRectangularND(ap, 100, np.zeros(xd - 1), 0))
            np.testing.assert_array_equal(st, g[f"line_{tag}_steps"])
            np.testing.assert_array_equal(ms, g[f"line_{tag}_masks"])
        if xd >= 3:
            st, ms = _record(S.PlaneSchedulerRectangularND(ap, 100, np.zeros(xd - 2), [0, 1]))
            np.testing.assert_array_equal(st, g[f"plane_{tag}_steps"])
            np.testing.assert_array_equal(ms, g[f"plane_{tag}_masks"])
    sxb = [np.linspace(-1, 1, 16), np.linspace(0, 1, 8)]
    apb = {"static": {"decomposition": D.RectangularDecompositionND.init_params(
        sxb, get_subdomain_ws(sxb, 2.9), (0., 1.))[0]}}
    st, ms = _record(S.LineSchedulerRectangularND(apb, 1000, point=[0.], iaxis=0))
    np.testing.assert_array_equal(st, g["burgers_steps"])
    np.testing.assert_array_equal(ms, g["burgers_masks"])
    st, ms = _record(S.AllActiveSchedulerND(apb, 10))
    np.testing.assert_array_equal(st, g["allactive_steps"])
    np.testing.assert_array_equal(ms, g["allactive_masks"])


def test_scheduler_argument_validation():
    ap = _sched_all_params([np.array([-6, -4, -2, 0, 2, 4, 6.])] * 2, 3)
    with pytest.raises(Exception):
        S.PointSchedulerRectangularND(ap, 10, [0.])
    with pytest.raises(Exception):
        S.PlaneSchedulerRectangularND(ap, 10, [], [0, 1])
    with pytest.raises(Exception):
        S.LineSchedulerRectangularND(ap, 10, [0., 0.], 0)


def test_windows_and_networks_match_reference():
    g = golden("windows_networks.npz")
    x = torch.tensor(g["x"])
    lo, hi, wl, wh = (torch.tensor(g[k]) for k in ("lo", "hi", "wl", "wh"))
    np.testing.assert_allclose(Wn.sigmoid(lo, hi, wl, wh, x).numpy(), g["win_sigmoid"], rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(Wn.cosine(lo, hi, x).numpy(), g["win_cosine"], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(Wn.bump(lo, hi, x).numpy(), g["win_bump"], rtol=1e-12)
    np.testing.assert_allclose(Wn.wendland(lo, hi, x).numpy(), g["win_wendland"], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(Wn.rbf(lo, hi, x).numpy(), g["win_rbf"], rtol=1e-12)
    lay = [(torch.tensor(g[f"W{i}"]), torch.tensor(g[f"b{i}"])) for i in range(2)]
    mk = lambda L, st=None: {"static": {"network": {"subdomain": st or {}}},
                             "trainable": {"network": {"subdomain": {"layers": L}}}}
    np.testing.assert_allclose(N.FCN.network_fn(mk(lay), x).numpy(), g["net_FCN"], rtol=1e-12)
    layA = [(w, b, torch.tensor(g[f"A{i}"])) for i, (w, b) in enumerate(lay)]
    np.testing.assert_allclose(N.AdaptiveFCN.network_fn(mk(layA), x).numpy(), g["net_AdaptiveFCN"], rtol=1e-12)
    np.testing.assert_allclose(N.SIREN.network_fn(mk(lay), x).numpy(), g["net_SIREN"], rtol=1e-12)
    layS = [(w, b, torch.tensor(g[f"C{i}"]), torch.tensor(g[f"O{i}"])) for i, (w, b) in enumerate(lay)]
    np.testing.assert_allclose(N.AdaptiveSIREN.network_fn(mk(layS), x).numpy(), g["net_AdaptiveSIREN"], rtol=1e-12)
    layF = [(torch.tensor(g["WF0"]), torch.tensor(g["bF0"])), lay[1]]
    np.testing.assert_allclose(N.FourierFCN.network_fn(mk(layF, {"omega": torch.tensor(g["omega"])}), x).numpy(),
                               g["net_FourierFCN"], rtol=1e-12)


def test_network_init_distribution_and_packing():
    _, tp = N.FCN.init_params(3, [2, 16, 16, 1])
    for (w, b), fi in zip(tp["layers"], [2, 16, 16]):
        v = 1 / math.sqrt(fi)
        assert w.abs().max() <= v and b.abs().max() <= v
    m = 5
    layers = [(torch.randn(m, fo, fi), torch.randn(m, fo)) for fi, fo in [(2, 16), (16, 16), (16, 1)]]
    theta = N.pack_layers(layers)
    assert theta.shape == (m, N.fcn_param_count([2, 16, 16, 1])) == (m, 337)
    for (w, b), (w2, b2) in zip(layers, N.unpack_layers(theta, [2, 16, 16, 1])):
        assert torch.equal(w, w2) and torch.equal(b, b2)


def test_grid_sampler_matches_reference():
    """Grid order and values; values within one float32 ulp, since the fixture's
    linspace ran in numpy float32 (the reference's jnp.linspace rounds in float32
    its own way, this engine computes in float64 and rounds once)."""
    g = golden("grid_sampler.npz")
    s = DOM.RectangularDomainND._rectangle_samplerND
    ulp = dict(rtol=0, atol=1.2e-7)
    np.testing.assert_allclose(s(None, "grid", [0.], [1.], (200,)).numpy(), g["g1"], **ulp)
    np.testing.assert_allclose(s(None, "grid", [-1., 0.], [1., 1.], (20, 10)).numpy(), g["g2"], **ulp)
    np.testing.assert_allclose(s(None, "grid", [-1., -1., 0.], [1., 1., 1.], (5, 4, 3)).numpy(), g["g3"], **ulp)
    u = s(0, "uniform", [-1., 0.], [1., 2.], (1000, 3))
    assert u.shape == (3000, 2) and u[:, 0].min() >= -1 and u[:, 1].max() <= 2
    assert s(None, "sobol", [0., 0.], [1., 1.], (16, 4)).shape == (64, 2)
    assert s(None, "halton", [0.], [1.], (10,)).shape == (10, 1)
    with pytest.raises(ValueError):
        s(None, "bogus", [0.], [1.], (10,))


def test_sample_boundaries_layout():
    ps, _ = DOM.RectangularDomainND.init_params(np.array([0., 1.]), np.array([1., 2.]))
    xb = DOM.RectangularDomainND.sample_boundaries({"static": {"domain": ps}}, 0, "grid", ((3,), (4,), (5,), (6,)))
    assert [x.shape[0] for x in xb] == [3, 4, 5, 6]
    assert torch.all(xb[0][:, 0] == 0) and torch.all(xb[1][:, 0] == 1)
    assert torch.all(xb[2][:, 1] == 1) and torch.all(xb[3][:, 1] == 2)


def test_burgers_exact_solution_matches_reference():
    g = golden("burgers_exact.npz")
    ap = {"static": {"problem": PR.BurgersEquation2D.init_params()[0]}}
    u = PR.BurgersEquation2D.exact_solution(ap, torch.tensor(g["x"]), (64, 32)).double().numpy()
    np.testing.assert_allclose(u, g["u"].astype(np.float32), rtol=0, atol=2e-6)


def test_problem_functions_match_reference():
    g = golden("problems.npz")
    x, u = torch.tensor(g["x"]), torch.tensor(g["u"])
    j = [torch.tensor(g[f"j{i}"]) for i in range(4)]
    src = np.array([[0.1, -0.2, 0.3, 1.0], [-0.3, 0.2, 0.25, 0.5]])
    apw = {"static": {"problem": PR.WaveEquationConstantVelocity3D.init_params(c0=1.5, source=src)[0]}}
    apw["static"]["problem"]["source"] = torch.tensor(src)  # float64 table, as the fixture used
    np.testing.assert_allclose(PR.WaveEquationConstantVelocity3D.constraining_fn(apw, x, u).numpy(), g["wave_c"],
                               rtol=1e-12)
    np.testing.assert_allclose(PR.WaveEquationConstantVelocity3D.loss_fn(apw, [[x, j[0], j[1], j[2]]]).item(),
                               g["wave_loss"], rtol=1e-12)
    mix = np.array([[0.2, 0.1, 0.5, 0.3], [-0.4, -0.1, 0.3, -0.2]])
    apg = {"static": {"problem": PR.WaveEquationGaussianVelocity3D.init_params(c0=1.0, source=src, mixture=mix)[0]}}
    apg["static"]["problem"]["mixture"] = torch.tensor(mix)
    np.testing.assert_allclose(PR.WaveEquationGaussianVelocity3D.c_fn(apg, x).numpy(), g["wave_gauss_c_fn"],
                               rtol=1e-12)
    apb = {"static": {"problem": PR.BurgersEquation2D.init_params()[0]}}
    np.testing.assert_allclose(PR.BurgersEquation2D.constraining_fn(apb, x[:, :2], u).numpy(), g["burgers_c"],
                               rtol=1e-12)
    aph = {"static": {"problem": PR.HarmonicOscillator1DHardBC.init_params(d=2, w0=80, sd=0.1)[0]}}
    np.testing.assert_allclose(PR.HarmonicOscillator1DHardBC.constraining_fn(aph, x[:, :1], u).numpy(),
                               g["hohard_c"], rtol=1e-12)
    api = {"static": {"problem": PR.HarmonicOscillator1DInverse.init_params(d=2, w0=20)[0]}}
    np.testing.assert_allclose(
        PR.HarmonicOscillator1DInverse.exact_solution(api, torch.linspace(0, 1, 13, dtype=torch.float64)
                                                      .reshape(13, 1)).numpy(), g["ho_inv_data"], rtol=1e-12)


def test_poisson_manufactured_solution_consistent():
    """-lap of the manufactured u equals the source f (central differences)."""
    ap = {"static": {"problem": PR.Poisson2D.init_params()[0]}}
    x = torch.rand(50, 2, dtype=torch.float64) * 0.8 + 0.1
    h = 1e-4
    lap = 0
    for d in range(2):
        e = torch.zeros(1, 2, dtype=torch.float64)
        e[0, d] = h
        u = lambda z: PR.Poisson2D.exact_solution(ap, z).double()
        lap = lap + (u(x + e) - 2 * u(x) + u(x - e)) / h ** 2
    f = PR.Poisson2D.source(ap, x)
    assert torch.allclose(-lap, f, rtol=0, atol=1e-4 * f.abs().max().item())


def test_cell_grid_registers_every_containing_box():
    """Monotone cell lookup: every box containing a point is in the point's cell list."""
    rng = np.random.default_rng(0)
    xmin = rng.uniform(0, 1, (300, 2)).astype(np.float32)
    xmax = (xmin + rng.uniform(0.01, 0.3, (300, 2))).astype(np.float32)
    g = D.build_cell_grid(xmin, xmax)
    x = np.concatenate([rng.uniform(-0.1, 1.4, (5000, 2)), xmin, xmax]).astype(np.float32)
    cells = [D.cell_coord(x[:, d], g["lo"][d], g["inv_h"][d], g["ncell"][d]) for d in range(2)]
    cid = cells[0] + g["ncell"][0] * cells[1]
    inside = np.all((x[:, None, :] >= xmin[None]) & (x[:, None, :] <= xmax[None]), -1)
    for p in range(x.shape[0]):
        cand = set(g["cell_boxes"][g["cell_start"][cid[p]]:g["cell_start"][cid[p] + 1]].tolist())
        assert set(np.nonzero(inside[p])[0].tolist()) <= cand
    # boxes ascending within every cell
    for c in range(len(g["cell_start"]) - 1):
        seg = g["cell_boxes"][g["cell_start"][c]:g["cell_start"][c + 1]]
        assert np.all(np.diff(seg) > 0)


def test_jet_layout_with_second_derivative_groups():
    """Jet component layout for per-dim, Laplacian and grouped d2masks."""
    from fbpinns_gb300 import _lib
    from fbpinns_gb300.engine import jet_index, jet_size, laplacian_index
    assert jet_size(2, 3) == 5 and jet_index(2, 3, (1, 1)) == 4
    lap = 3 | _lib.D2_LAPLACIAN
    assert jet_size(2, lap) == 4 and laplacian_index(2, lap) == 3
    with pytest.raises(ValueError):
        jet_index(2, lap, (0, 0))
    wave = 7 | _lib.D2_GROUP(3)
    assert _lib.d2_group(wave) == 3 and jet_size(3, wave) == 6
    assert laplacian_index(3, wave) == 4 and jet_index(3, wave, (2, 2)) == 5
    assert jet_index(3, wave, (0,)) == 1 and jet_index(3, 7, (2, 2)) == 6


def test_constants_key_checking_and_defaults():
    c = Constants(n_steps=3)
    assert c.n_steps == 3 and c["sampler"] == "grid"
    with pytest.raises(KeyError):
        c["nonexistent"] = 1
    with pytest.raises(KeyError):
        Constants(nonexistent=1)
    assert [float(v) for v in get_subdomain_ws([np.linspace(0, 1, 5)], 2.0)[0]] == [0.5] * 5


def test_library_exports_every_declared_symbol():
    """libfbpgpu.so loads without a GPU and exports every entry point of include/fbpgpu.h."""
    from fbpinns_gb300 import _lib
    lib = _lib.load()
    declared = _lib.declared_symbols()
    assert len(declared) >= 20
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, missing
    assert set(declared) <= set(_lib._SIG), set(declared) - set(_lib._SIG)
    assert lib.fbp_abi_version() == 1


def test_required_ujs_mapping():
    from fbpinns_gb300.engine import d2mask_of, jet_index, jet_size
    assert d2mask_of([((0, ()), (0, (0,)), (0, (1,)), (0, (0, 0)))], 2) == 1
    assert d2mask_of([((0, (0, 0)), (0, (1, 1)), (0, (2, 2)))], 3) == 7
    assert jet_size(3, 7) == 7 and jet_index(3, 7, (2, 2)) == 6 and jet_index(2, 2, (1, 1)) == 3
    with pytest.raises(NotImplementedError):
        d2mask_of([((0, (0, 1)),)], 2)
    with pytest.raises(NotImplementedError):
        d2mask_of([((0, (0, 0, 0)),)], 1)


def test_work_item_sizes():
    """Adjoint/forward work-item sizes and the schedule choice: the requested
    1024/4096 pairs for the 2D Poisson bench (9.4e6 pairs on 152 SMs), powers
    of two cut for small steps, and the counter schedule only with more items
    than resident CTAs."""
    from fbpinns_gb300.engine import work_item_sizes
    assert work_item_sizes(11_711_911, 1365, 152, 1024, 4096) == (1024, 4096, True)
    adj, fwd, dyn = work_item_sizes(314_672, 128, 152, 1024, 4096)  # Burgers
    assert (adj, fwd, dyn) == (256, 512, True)
    assert work_item_sizes(398, 15, 152, 1024, 4096) == (128, 128, False)  # HO: 15 items
    assert work_item_sizes(314_672, 128, 152, 1024, 4096, adaptive=False) == (1024, 4096, False)
    for s in (10, 10_000, 10_000_000):
        adj, fwd, _ = work_item_sizes(s, 100, 152, 1024, 4096)
        assert adj & (adj - 1) == 0 and fwd & (fwd - 1) == 0 and 128 <= adj <= fwd <= 4096


def test_fourier_network_maps_to_a_frozen_sin_layer():
    """FourierFCN (fbpinns/networks.py:165-194) as the kernels see it: a first
    layer sin(W x + b) with W = [omega; omega], b = [0; pi/2] ahead of the
    reference's FCN layers; the oracle's "fourier" network (sin and cos of
    omega x) equals the reference network_fn restated in networks.py, and the
    packed layer equals it to FP32 rounding; more hidden layers are refused."""
    from oracle import model as OM
    g = torch.Generator().manual_seed(3)
    m, F, xd, h = 5, 4, 2, 8
    st, tr = N.FourierFCN.init_params(11, [xd, h, 1], 0.0, 1.0, F)
    omega = torch.stack([st["omega"]] * m)
    layers = [tuple(torch.stack([t] * m) for t in layer) for layer in tr["layers"]]
    ls, act, eng_layers, skip = N.engine_network(N.FourierFCN, {"omega": omega}, layers, [xd, h, 1])
    assert ls == [xd, 2 * F, h, 1] and act == "fourier" and skip == 1 and len(eng_layers) == 3
    W, b = eng_layers[0]
    assert torch.equal(W[:, :F], omega) and torch.equal(W[:, F:], omega)
    assert torch.equal(b[:, :F], torch.zeros(m, F)) and torch.allclose(b[:, F:], torch.full((m, F), math.pi / 2))
    x = torch.rand((m, xd), generator=g, dtype=torch.float64)
    L64 = [tuple(t.double() for t in layer) for layer in eng_layers]
    ref = torch.stack([N.FourierFCN.network_fn({"static": {"network": {"subdomain": {"omega": omega[i].double()}}},
                                                "trainable": {"network": {"subdomain": {"layers": [
                                                    tuple(t[i].double() for t in layer) for layer in layers]}}}},
                                               x[i]) for i in range(m)])
    assert torch.allclose(OM.fcn(L64, x, "fourier"), ref, rtol=0, atol=1e-12)
    # the packed form (sin(z + pi/2) for cos z) agrees to the rounding of the FP32 bias
    z = torch.einsum("sij,sj->si", L64[0][0], x) + L64[0][1]
    hh = torch.tanh(torch.einsum("sij,sj->si", L64[1][0], torch.sin(z)) + L64[1][1])
    packed = torch.einsum("sij,sj->si", L64[2][0], hh) + L64[2][1]
    assert torch.allclose(packed, ref, rtol=0, atol=1e-6)
    with pytest.raises(NotImplementedError):
        N.engine_network(N.FourierFCN, {"omega": omega}, layers, [xd, h, h, 1])


def test_autotune_candidates_follow_the_pair_count():
    from fbpinns_gb300.autotune import default_candidates
    assert default_candidates(9_368_709, 1365, 152) == [(a, a * k) for a in (512, 1024, 2048) for k in (1, 2, 4)]
    small = default_candidates(314_672, 128, 152)
    assert (256, 512) in small and min(a for a, _ in small) == 128
    assert all(f <= 8192 and f >= a for a, f in default_candidates(10 ** 9, 4096, 152))


def test_constrained_jets_identity_and_needed_components():
    """constrained_jets (the jets of constraining_fn(u) for the generic step):
    exact against closed forms for the HO hard-constraint ansatz
    u_c = 1 + tanh(t/sd)^2 u (value, first and second derivative, and the
    gradient with respect to the input jets); an identity constraining_fn
    returns the input jets themselves; ``need`` computes only the requested
    dims (others zero) with the same values."""
    from fbpinns_gb300.engine import constrained_jets
    g = torch.Generator().manual_seed(1)
    x = torch.rand((64, 1), generator=g, dtype=torch.float64)
    U = torch.randn((64, 3), generator=g, dtype=torch.float64, requires_grad=True)
    sp = PR.HarmonicOscillator1DHardBC.init_params(d=2, w0=80, sd=0.1)[0]
    ap = {"static": {"problem": sp}, "trainable": {}}
    cfn = PR.HarmonicOscillator1DHardBC.constraining_fn
    Uc = constrained_jets(cfn, ap, x, U, 1, 1)
    sd = 0.1
    th = torch.tanh(x / sd)
    s = th ** 2                                   # ansatz factor and its t-derivatives
    s1 = 2 * th * (1 - th ** 2) / sd
    s2 = (2 * (1 - th ** 2) ** 2 - 4 * th ** 2 * (1 - th ** 2)) / sd ** 2
    u, u1, u2 = U[:, 0:1], U[:, 1:2], U[:, 2:3]
    ref = torch.cat([1 + s * u, s1 * u + s * u1, s2 * u + 2 * s1 * u1 + s * u2], 1)
    assert torch.allclose(Uc, ref, rtol=1e-12, atol=1e-12)
    w = torch.randn((64, 3), generator=g, dtype=torch.float64)
    ga, = torch.autograd.grad((Uc * w).sum(), U)
    gb, = torch.autograd.grad((ref * w).sum(), U)
    assert torch.allclose(ga, gb, rtol=1e-12, atol=1e-12)
    # identity: the jets themselves
    ident = lambda all_params, x_batch, u: u
    assert constrained_jets(ident, ap, x, U, 1, 1) is U
    # only the value needed: no derivative work, zeros in the rest
    Uv = constrained_jets(cfn, ap, x, U, 1, 1, need=[0])
    assert torch.equal(Uv[:, 0:1], Uc[:, 0:1]) and torch.all(Uv[:, 1:] == 0)
    assert torch.equal(constrained_jets(cfn, ap, x, U, 1, 1, need=[0, 2]), Uc)


def test_integration_binding_matches_the_library_binding():
    """The ctypes stub shown for the reference side declares
    the same structures and argument types as the binding this package uses,
    so the document cannot drift from the ABI."""
    import ctypes as C
    import re
    from fbpinns_gb300 import _lib
    here = os.path.dirname(os.path.abspath(__file__))
    txt = open(os.path.join(here, "..", "INTEGRATION.md")).read()
    code = re.search(r"```python\n(.*?)```", txt, re.S).group(1)

    class _Fn:
        pass

    class _Lib:
        def __getattr__(self, name):
            f = _Fn()
            object.__setattr__(self, name, f)
            return f

    real_cdll = C.CDLL
    C.CDLL = lambda *a, **k: _Lib()
    try:
        ns = {}
        exec(code, ns)
    finally:
        C.CDLL = real_cdll
    for st in ("Boxes", "Net", "Pairs", "Problem"):
        doc = [(n, t.__name__) for n, t in ns[st]._fields_]
        ours = [(n, t.__name__) for n, t in getattr(_lib, st)._fields_]
        assert doc == ours, st
    lib = ns["lib"]
    checked = 0
    for name, (res, args) in _lib._SIG.items():
        f = lib.__dict__.get(name)
        if f is None or not hasattr(f, "argtypes"):
            continue
        norm = lambda ts: [t.__name__ if not hasattr(t, "_type_") or not isinstance(t._type_, type)
                           else "P:" + t._type_.__name__ for t in ts]
        assert norm(f.argtypes) == norm(args), name
        checked += 1
    assert checked >= 15


def test_header_constants_match_the_python_binding():
    """Activation codes, status bits, jet-mask flags and problem ids of
    include/fbpgpu.h equal the constants the Python side passes."""
    import re
    from fbpinns_gb300 import _lib
    here = os.path.dirname(os.path.abspath(__file__))
    hdr = open(os.path.join(here, "..", "include", "fbpgpu.h")).read()
    vals = {}
    for name, expr in re.findall(r"^#define (FBP_[A-Z0-9_]+) ([^/\n]+)", hdr, re.M):
        try:
            vals[name] = eval(expr.strip(), {})
        except Exception:
            pass
    assert vals["FBP_D2_LAPLACIAN"] == _lib.D2_LAPLACIAN
    assert all(_lib.D2_GROUP(d) == ((d & 7) << 4) for d in range(8))
    for key, code in _lib.ACTIVATIONS.items():
        assert vals["FBP_ACT_" + key.upper()] == code, key
    for bit in _lib.STATUS_BITS:
        assert bit in (vals["FBP_STATUS_PAIR_OVERFLOW"], vals["FBP_STATUS_SLOT_OVERFLOW"],
                       vals["FBP_STATUS_ITEM_OVERFLOW"], vals["FBP_STATUS_LEVEL_ORDER"],
                       vals["FBP_STATUS_BAD_INDEX"], vals["FBP_STATUS_TC_TIMEOUT"])
    ids = (_lib.PROBLEM_NONE, _lib.PROBLEM_HO_HARDBC, _lib.PROBLEM_BURGERS, _lib.PROBLEM_POISSON2D,
           _lib.PROBLEM_WAVE_C, _lib.PROBLEM_HELMHOLTZ2D)
    assert ids == tuple(vals[k] for k in ("FBP_PROBLEM_NONE", "FBP_PROBLEM_HO_HARDBC", "FBP_PROBLEM_BURGERS",
                                           "FBP_PROBLEM_POISSON2D", "FBP_PROBLEM_WAVE_C",
                                           "FBP_PROBLEM_HELMHOLTZ2D"))
    assert vals["FBP_OK"] == _lib.FBP_OK == 0


@pytest.mark.parametrize("name", ["ho", "burgers", "poisson", "wave", "helmholtz"])
def test_configurations_set_up_on_the_host(name):
    """Each workload configuration builds its Constants and, on the host, its
    decomposition (subdomain count as documented), problem parameters,
    collocation batch and the fused-loss description of its problem."""
    from fbpinns_gb300 import configs
    m_expected = {"ho": 15, "burgers": 128, "poisson": 1365, "wave": 900, "helmholtz": 4096}[name]
    c = configs.CONFIGS[name](n_steps=10)
    assert c["n_steps"] == 10 and c["network"] is N.FCN
    dec = c.decomposition.init_params(**c.decomposition_init_kwargs)[0]
    assert dec["m"] == m_expected
    ps, pt = c.problem.init_params(**c.problem_init_kwargs)
    dom = c.domain.init_params(**c.domain_init_kwargs)[0]
    all_params = {"static": {"domain": dom, "problem": ps, "decomposition": dec}, "trainable": {"problem": pt}}
    spec = c.problem.fused_spec(all_params)
    assert spec is not None and "kind" in spec
    small = configs.CONFIGS[name](n_steps=10, small=True)
    assert np.prod(small.ns[0]) <= np.prod(c.ns[0])


def test_wave_source_width_bound():
    """The wave workload's 12 sources keep their centres (same seed) when the
    lower bound of their widths changes; the ansatz's hand-over time t1 is the
    smallest width / c0."""
    from fbpinns_gb300 import configs
    a = np.asarray(configs.wave(n_steps=10).problem_init_kwargs["source"])
    b = np.asarray(configs.wave(n_steps=10, min_width=0.1).problem_init_kwargs["source"])
    assert a.shape == b.shape == (12, 4)
    np.testing.assert_array_equal(a[:, :2], b[:, :2])
    assert 0.02 <= a[:, 2].min() < 0.1 <= b[:, 2].min() and b[:, 2].max() <= 0.2


def test_constants_and_model_files_round_trip(tmp_path, monkeypatch):
    """Constants files and model pickles in the reference's layout
    (results/summaries/<run>/constants_<run>.pickle, results/models/<run>/
    model_XXXXXXXX.jax) load back through analysis.load_model, which picks
    the latest model when no step is given."""
    import pickle
    from fbpinns_gb300 import configs
    from fbpinns_gb300.analysis import load_model
    monkeypatch.chdir(tmp_path)
    c = configs.ho(n_steps=10)
    c.run = "roundtrip"
    c.get_outdirs()
    c.save_constants_file()
    for i in (5, 10):
        model = (i, {"static": {}, "trainable": {"network": {"subdomain": {"layers": [(np.ones((15, 32, 1)),)]}}}},
                 {"count": i}, np.ones(15, dtype=int), np.zeros((1, 3)))
        with open(c.model_out_dir + f"model_{i:08d}.jax", "wb") as f:
            pickle.dump(model, f)
    c2, model = load_model("roundtrip", rootdir="results/")
    assert model[0] == 10 and model[2]["count"] == 10
    assert c2.run == "roundtrip" and c2.network is N.FCN and c2.n_steps == 10
    c3, model5 = load_model("roundtrip", i=5, rootdir="results/")
    assert model5[0] == 5


def test_wave_field_matches_reference_cpml_solver():
    """The leapfrog wave field that feeds the wave test error (wave_fd.py)
    against the reference's own field (fbpinns/problems.py:408-474, its
    seismic CPML finite-difference solver, run by tests/golden/make_golden.py)
    on a 41 x 41 x 6 grid over [-1,1]^2 x [0,0.5] with two Gaussian sources:
    relative L1 below 1.2% at every output time and the largest difference
    below 2% of the field's peak (the leapfrog field is converged to 0.05%:
    the rest is the reference solver's discretisation)."""
    from fbpinns_gb300.problems import WaveEquationConstantVelocity3D as WV
    from fbpinns_gb300.wave_fd import wave_exact
    g = golden("wave_exact.npz")
    ap = {"static": {"problem": WV.init_params(c0=float(g["c0"]), source=g["source"])[0]}}
    bs = tuple(int(v) for v in g["batch_shape"])
    u = wave_exact(ap, torch.tensor(g["x"]), bs).numpy().reshape(bs)
    ur = g["u"].reshape(bs)
    for k in range(bs[2]):
        d = np.abs(u[..., k] - ur[..., k])
        assert d.mean() < 0.012 * np.abs(ur[..., k]).mean(), k
        assert d.max() < 0.02 * np.abs(ur).max(), k


def test_helmholtz_reference_field_convergence():
    """The finite-difference field of the Helmholtz problem (helmholtz_fd.py),
    grid n against 2n on interior points.  Off resonance (k = 3 pi) it
    converges at second order (the difference falls 4x per halving of h).
    At k = 40 pi -- a Dirichlet eigenvalue of the unit square, since
    24^2 + 32^2 = 40^2 -- it does not converge (differences of the order of
    the field): -lap u - k^2 u = f with u = 0 on the boundary has no solution
    for a generic f there, so no test error can be defined for that k."""
    from fbpinns_gb300.helmholtz_fd import helmholtz_grid
    from fbpinns_gb300.problems import seeded_gaussians
    from fbpinns_gb300.wave_fd import bilinear
    src = seeded_gaussians(8, 1, width=(0.05, 0.1))
    g = np.linspace(0.05, 0.95, 46)
    X, Y = np.meshgrid(g, g, indexing="ij")

    def diffs(k, ns):
        v = {}
        for n in ns:
            xs, U = helmholtz_grid(k, src, n)
            v[n] = bilinear(xs, xs, U, X.ravel(), Y.ravel())
        return [np.abs(v[a] - v[b]).mean() / np.abs(v[b]).mean() for a, b in zip(ns[:-1], ns[1:])]

    e = diffs(3 * math.pi, (100, 200, 400))
    assert e[1] < 1e-3 and 3.5 < e[0] / e[1] < 4.5, e
    r = diffs(40 * math.pi, (200, 400, 800))
    assert min(r) > 0.3, r
