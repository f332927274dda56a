"""Generate golden vectors by running the reference library's own source files.

Run where a checkout of the reference library is available (its path is
given by ``--ref`` or the ``FBPINNS_REFERENCE`` environment variable); JAX is
not needed::

    python tests/golden/make_golden.py --ref <path of the reference checkout>

``jaxshim`` replaces ``jax.numpy`` by numpy, so the reference functions run
unchanged: in float32 (JAX's default mode) for the integer interaction lists
and decomposition parameters, in float64 for the model values.  Derivative
jets are the reference model's own forward values differentiated by float64
Richardson-extrapolated central differences (the reference's ``jvp`` cannot
run without JAX).  Inputs are seeded numpy draws (JAX's PRNG is unavailable).

The ``.npz`` files written next to this script are small and committed; the
tests read them, never the reference checkout.
"""

import argparse
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.dont_write_bytecode = True
sys.path.insert(0, HERE)
import jaxshim  # noqa: E402


OUT = HERE


def save(name, **arrays):
    path = os.path.join(OUT, name)
    np.savez_compressed(path, **{k: np.asarray(v) for k, v in arrays.items()})
    print(f"wrote {name}: " + ", ".join(f"{k}{np.asarray(v).shape}" for k, v in arrays.items()))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("FBPINNS_REFERENCE"),
                    help="path of the reference checkout (default: $FBPINNS_REFERENCE)")
    ap.add_argument("--out", default=HERE, help="output folder (default: next to this script)")
    args = ap.parse_args()
    if not args.ref:
        ap.error("give the reference checkout with --ref or FBPINNS_REFERENCE")
    global OUT
    OUT = args.out
    jaxshim.install()
    sys.path.insert(0, args.ref)
    from fbpinns import decompositions_base, decompositions, windows, networks, schedulers
    from fbpinns import domains, problems, trainers
    from fbpinns.constants import get_subdomain_ws
    import jax.numpy as jnp

    D = decompositions.RectangularDecompositionND
    DM = decompositions.MultilevelRectangularDecompositionND

    # ------------------------------------------------------------------
    # 1. known-answer test of decompositions_base.py:87-128 with seeded points
    # ------------------------------------------------------------------
    jaxshim.X64 = False
    rng = np.random.default_rng(0)
    n, m = 10000, 1000
    x = rng.uniform(0, 2, (n, 2)).astype(np.float32)
    c = rng.uniform(1, 3, (m, 2)).astype(np.float32)
    xmin, xmax = c - np.float32(0.1), c + np.float32(0.1)
    aps = [jnp.array(xmin), jnp.array(xmax)]

    def inside_fn(all_params, x_batch, ims):
        xb = jnp.expand_dims(x_batch, 1)
        lo = jnp.expand_dims(all_params[0][ims], 0)
        hi = jnp.expand_dims(all_params[1][ims], 0)
        return jnp.all((xb >= lo) & (xb <= hi), -1)

    ims = jnp.arange(m)
    res = None
    for bs in [1, 9, 10, 128, n]:
        nt, mt, iims = decompositions_base.inside_points_batch(aps, jnp.array(x), ims, bs, inside_fn)
        ips, d = decompositions_base.inside_models_batch(aps, jnp.array(x), ims, bs, inside_fn)
        if res is None:
            res = (nt, mt, iims, ips, d)
        else:
            assert all(np.array_equal(a, b) for a, b in zip(res[:4], (nt, mt, iims, ips)))
    save("takes_kat.npz", x=x, xmin=xmin, xmax=xmax, n_take=res[0], m_take=res[1],
         inside_ims=res[2], inside_ips=res[3], d=np.float64(res[4]))

    # ------------------------------------------------------------------
    # 2. decomposition parameters (float32 mode, as the reference runs)
    # ------------------------------------------------------------------
    sxs = [[np.array([0.5])] * 2] + [[np.linspace(0, 1, k)] * 2 for k in (2, 4, 8, 16, 32)]
    sws = [[np.array([1.0])] * 2] + [get_subdomain_ws(s, 2.9) for s in sxs[1:]]
    sp, _ = DM.init_params(sxs, sws, (0., 1.))
    p = sp["subdomain"]["params"]
    save("level_params_poisson.npz", xmins=p[0], xmaxs=p[1], wmins=p[2], wmaxs=p[3], flags=p[4],
         unnorms=p[5], pou=sp["subdomain"]["pou"], xmins0=sp["xmins0"], xmaxs0=sp["xmaxs0"],
         m=sp["m"])
    sx3 = [np.linspace(-1, 1, 5), np.linspace(-1, 1, 4), np.linspace(0, 1, 3)]
    sp3, _ = D.init_params(sx3, get_subdomain_ws(sx3, 2.0), (0.5, 2.0))
    p = sp3["subdomain"]["params"]
    save("level_params_3d.npz", xmins=p[0], xmaxs=p[1], wmins=p[2], wmaxs=p[3], flags=p[4],
         unnorms=p[5], pou=sp3["subdomain"]["pou"], xmins0=sp3["xmins0"], xmaxs0=sp3["xmaxs0"])
    sp1, _ = D.init_params([np.array([0.5])], [np.array([1.2])], (0., 1.))
    p = sp1["subdomain"]["params"]
    save("level_params_single.npz", xmins=p[0], xmaxs=p[1], wmins=p[2], wmaxs=p[3], flags=p[4],
         unnorms=p[5], pou=sp1["subdomain"]["pou"])

    # ------------------------------------------------------------------
    # 3. grid sampler (domains.py:113-142)
    # ------------------------------------------------------------------
    g1 = domains.RectangularDomainND._rectangle_samplerND(None, "grid", jnp.array(np.array([0.])), jnp.array(np.array([1.])), (200,))
    g2 = domains.RectangularDomainND._rectangle_samplerND(None, "grid", jnp.array(np.array([-1., 0.])), jnp.array(np.array([1., 1.])), (20, 10))
    g3 = domains.RectangularDomainND._rectangle_samplerND(None, "grid", jnp.array(np.array([-1., -1., 0.])), jnp.array(np.array([1., 1., 1.])), (5, 4, 3))
    save("grid_sampler.npz", g1=g1, g2=g2, g3=g3)

    # ------------------------------------------------------------------
    # 4. get_inputs / _get_update_inputs (trainers.py:332-575), float32 mode
    # ------------------------------------------------------------------
    def run_update_inputs(tag, decomp, sp, x_global, constraint_fs, offsets, active, extra_cons=None):
        all_params = {"static": {"decomposition": sp}, "trainable": {}}
        tr = object.__new__(trainers.FBPINNTrainer)
        tr.c = types.SimpleNamespace(n_steps=1)
        cons_global = [[x_global[offsets[i]:(offsets[i + 1] if i + 1 < len(offsets) else None)]]
                       for i in range(len(offsets))]
        out = tr._get_update_inputs(0, active, all_params, {}, jnp.array(x_global), cons_global,
                                    jnp.array(constraint_fs), jnp.array(np.array(offsets)), decomp, None)
        act, _, _, _, _, _, takess, constraints, x_batch = out
        takes, all_ims, (act2, *_rest) = trainers.get_inputs(x_batch, active, all_params, decomp)
        arrays = dict(x_global=x_global, constraint_fs=constraint_fs, offsets=np.array(offsets),
                      active_in=np.asarray(active), active_out=np.asarray(act), x_batch=x_batch,
                      all_ims=all_ims, npou=takes[4])
        for k, nm in enumerate(["m_take", "n_take", "p_take", "np_take"]):
            arrays[nm] = takes[k]
        for ic, tk in enumerate(takess):
            for k, nm in enumerate(["m_take", "n_take", "p_take", "np_take"]):
                arrays[f"c{ic}_{nm}"] = tk[k]
        save(f"inputs_{tag}.npz", **arrays)

    # 4a. HO: 15 subdomains, width 2x spacing, 200 grid points, all active
    sx = [np.linspace(0, 1, 15)]
    sp, _ = D.init_params(sx, get_subdomain_ws(sx, 2.0), (0., 1.))
    xg = np.asarray(g1)
    run_update_inputs("ho", D, sp, xg, np.ones((200, 1), bool), [0], np.ones(15, dtype=int))

    # 4b. HO soft BC: two constraints (interior grid + boundary point), scheduled
    xg2 = np.concatenate([np.asarray(domains.RectangularDomainND._rectangle_samplerND(
        None, "grid", jnp.array(np.array([0.])), jnp.array(np.array([1.])), (60,))), np.zeros((1, 1), np.float32)])
    cf = np.zeros((61, 2), bool)
    cf[:60, 0] = True
    cf[60:, 1] = True
    act = np.zeros(15, dtype=int)
    act[:4] = 2
    act[4:7] = 1
    run_update_inputs("ho2c", D, sp, xg2, cf, [0, 60], act)

    # 4c. Burgers-like 16x8 width 2.9 on a 40x20 grid with a line-scheduler mask
    sxb = [np.linspace(-1, 1, 16), np.linspace(0, 1, 8)]
    spb, _ = D.init_params(sxb, get_subdomain_ws(sxb, 2.9), (0., 1.))
    gb = np.asarray(domains.RectangularDomainND._rectangle_samplerND(
        None, "grid", jnp.array(np.array([-1., 0.])), jnp.array(np.array([1., 1.])), (40, 20)))
    sch = schedulers.LineSchedulerRectangularND({"static": {"decomposition": spb}}, 100, point=[0.], iaxis=0)
    masks = [a.copy() for a in sch if a is not None]
    run_update_inputs("burgers_all", D, spb, gb, np.ones((gb.shape[0], 1), bool), [0], np.ones(128, dtype=int))
    run_update_inputs("burgers_sched", D, spb, gb, np.ones((gb.shape[0], 1), bool), [0], masks[len(masks) // 2])

    # 4d. multilevel 2D (levels 1,2,4,8), 3000 uniform points (and duplicates)
    sxs4 = sxs[:4]
    sws4 = sws[:4]
    spm, _ = DM.init_params(sxs4, sws4, (0., 1.))
    xu = rng.uniform(0, 1, (3000, 2)).astype(np.float32)
    xu[100:110] = xu[0]
    xu[200] = np.array([0.5, 0.5], np.float32)
    run_update_inputs("multilevel", DM, spm, xu, np.ones((3000, 1), bool), [0], np.ones(spm["m"], dtype=int))

    # 4e. 3D grid, some points outside every box
    x3 = np.asarray(domains.RectangularDomainND._rectangle_samplerND(
        None, "grid", jnp.array(np.array([-1.2, -1., 0.])), jnp.array(np.array([1.2, 1., 1.])), (9, 8, 5)))
    act3 = np.ones(sp3["m"], dtype=int)
    act3[::5] = 2
    act3[1] = 0
    run_update_inputs("wave3d", D, sp3, x3, np.ones((x3.shape[0], 1), bool), [0], act3)

    # ------------------------------------------------------------------
    # 5. model forward (trainers.py:126-177) in float64 + FD jets + losses
    # ------------------------------------------------------------------
    jaxshim.X64 = True
    # float64 copies of the decompositions for the model fixtures
    sp, _ = D.init_params(sx, get_subdomain_ws(sx, 2.0), (0., 1.))
    spb, _ = D.init_params(sxb, get_subdomain_ws(sxb, 2.9), (0., 1.))
    sp3, _ = D.init_params(sx3, get_subdomain_ws(sx3, 2.0), (0.5, 2.0))
    spm, _ = DM.init_params(sxs4, sws4, (0., 1.))

    def fd_jets(ufun, xb, dims, h1=2.5e-4, h2=5e-4):
        """Richardson-extrapolated central differences of ufun at xb."""
        out = {}
        for i in dims:
            e = np.zeros(xb.shape[1])
            e[i] = 1.0

            def d1(h):
                return (ufun(xb + h * e) - ufun(xb - h * e)) / (2 * h)

            def d2(h):
                return (ufun(xb + h * e) - 2 * ufun(xb) + ufun(xb - h * e)) / (h * h)
            out[(i,)] = (4 * d1(h1 / 2) - d1(h1)) / 3
            out[(i, i)] = (4 * d2(h2 / 2) - d2(h2)) / 3
        return out

    def far_from_edges(xb, xmins, xmaxs, margin):
        dmin = np.min(np.abs(xb[:, None, :] - xmins[None]), axis=(1, 2))
        dmax = np.min(np.abs(xb[:, None, :] - xmaxs[None]), axis=(1, 2))
        return (dmin > margin) & (dmax > margin)

    def model_case(tag, decomp, sp_params, problem, pkw, layer_sizes, xb, seed, dims, network="FCN", wscale=1.0,
                   n_features=0, margin=1e-2, slim=False):
        r = np.random.default_rng(seed)
        ps_prob = problem.init_params(**pkw)[0]
        m = sp_params["m"]
        layers = []
        net_static = {}
        if network == "FourierFCN":  # per-subdomain omega, 2 pi (mu + sd N(0,1)) with mu = 0, sd = 0.5
            omega = jnp.array(2 * np.pi * 0.5 * r.normal(size=(m, n_features, layer_sizes[0])))
            net_static = {"omega": omega}
            layer_sizes = [2 * n_features] + list(layer_sizes)[1:]
        for fi, fo in zip(layer_sizes[:-1], layer_sizes[1:]):
            v = wscale * np.sqrt(1 / fi)
            wb = [r.uniform(-v, v, (m, fo, fi)), r.uniform(-v, v, (m, fo))]
            if slim:  # multiples of 2^-12: exact in float32, so they are stored as float32
                wb = [np.round(t * 4096.0) / 4096.0 for t in wb]
            layer = (jnp.array(wb[0]), jnp.array(wb[1]))
            # adaptive activations: per-neuron parameters away from their initial 1
            nx = {"AdaptiveFCN": 1, "AdaptiveSIREN": 2}.get(network, 0)
            layer += tuple(jnp.array(r.uniform(0.5, 1.5, (m, fo))) for _ in range(nx))
            layers.append(layer)
        sub = sp_params["subdomain"]["params"]
        keep = far_from_edges(xb, np.asarray(sub[0]), np.asarray(sub[1]), margin)
        xb = xb[keep].astype(np.float64)
        all_params = {"static": {"decomposition": sp_params, "problem": ps_prob},
                      "trainable": {"network": {"subdomain": {"layers": layers}}}}
        if net_static:
            all_params["static"]["network"] = {"subdomain": net_static}
        active = np.ones(m, dtype=int)
        takes, all_ims, (_, _, _, cut_all, _) = trainers.get_inputs(jnp.array(xb), active, all_params, decomp)
        apc = {"static": cut_all(all_params["static"]), "trainable": cut_all(all_params["trainable"])}
        mf = (decomp.norm_fn, getattr(networks, network).network_fn, decomp.unnorm_fn, decomp.window_fn,
              problem.constraining_fn)
        u, wp, us, ws, ur = trainers.FBPINN_model(apc, jnp.array(xb), takes, mf, verbose=False)
        # POU-combined u before the constraining operator
        mf_id = mf[:4] + (lambda a, xb_, u_: u_,)
        ufun = lambda xx: np.asarray(trainers.FBPINN_model(apc, jnp.array(xx), takes, mf, verbose=False)[0])
        ufun_raw = lambda xx: np.asarray(trainers.FBPINN_model(apc, jnp.array(xx), takes, mf_id, verbose=False)[0])
        jets = fd_jets(ufun, xb, dims)
        jets_raw = fd_jets(ufun_raw, xb, dims)
        arrays = dict(x_batch=xb, m_take=takes[0], n_take=takes[1], p_take=takes[2], np_take=takes[3],
                      npou=takes[4], all_ims=all_ims, u=u, wp=wp, us=us, ws=ws, us_raw=ur,
                      u_raw=ufun_raw(xb))
        if net_static:
            arrays["omega"] = net_static["omega"]
        for i, layer in enumerate(layers):
            arrays[f"W{i}"] = layer[0]
            arrays[f"b{i}"] = layer[1]
            for k, t in zip("AO", layer[2:]):  # AdaptiveFCN: a; AdaptiveSIREN: c, o
                arrays[f"{k}{i}"] = t
        for k, v in jets.items():
            arrays["d" + "".join(map(str, k))] = v
        for k, v in jets_raw.items():
            arrays["raw_d" + "".join(map(str, k))] = v
        # reference loss on the FD jets
        cons = problem.sample_constraints  # noqa: F841  (constraint layout documented by the problem)
        arrays["loss"] = np.float64(loss_fns[tag](all_params, xb, u, jets))
        if slim:  # what the jet tests read: points, weights (float32-exact), POU output and its jets
            arrays = {k: (np.asarray(v, np.float32) if k[0] in "Wb" else v) for k, v in arrays.items()
                      if k in ("x_batch", "u_raw", "loss") or k.startswith(("raw_d", "W", "b"))}
        save(f"model_{tag}.npz", **arrays)

    loss_fns = {}
    HOH = problems.HarmonicOscillator1DHardBC
    loss_fns["ho_hardbc"] = lambda ap_, xb, u, j: HOH.loss_fn(ap_, [[xb, u, j[(0,)], j[(0, 0)]]])
    xho = np.asarray(g1).astype(np.float64)
    model_case("ho_hardbc", D, sp, HOH, dict(d=2, w0=80, sd=0.1), [1, 32, 32, 1], xho, 11, [0])

    BU = problems.BurgersEquation2D
    loss_fns["burgers"] = lambda ap_, xb, u, j: BU.loss_fn(ap_, [[xb, u, j[(0,)], j[(1,)], j[(0, 0)]]])
    xbu = np.asarray(gb).astype(np.float64)
    model_case("burgers", D, spb, BU, dict(), [2, 16, 16, 1], xbu, 12, [0, 1])

    WV = problems.WaveEquationConstantVelocity3D
    src = np.array([[0.1, -0.2, 0.3, 1.0], [-0.3, 0.2, 0.25, 0.5]])
    loss_fns["wave"] = lambda ap_, xb, u, j: WV.loss_fn(ap_, [[xb, j[(0, 0)], j[(1, 1)], j[(2, 2)]]])
    x3f = rng.uniform([-1, -1, 0], [1, 1, 1], (400, 3))
    model_case("wave", D, sp3, WV, dict(c0=1.0, source=src), [3, 8, 8, 1], x3f, 13, [0, 1, 2])

    loss_fns["multilevel"] = lambda ap_, xb, u, j: np.mean((j[(0, 0)] + j[(1, 1)]) ** 2)
    xml = rng.uniform(0, 1, (600, 2))
    model_case("multilevel", DM, spm, BU, dict(), [2, 8, 8, 1], xml, 14, [0, 1])
    # SIREN networks (networks.py:102-131, U(+-sqrt(6/fan_in)) weights); own
    # generator so the draws above are unchanged
    rng_s = np.random.default_rng(31)
    loss_fns["ho_hardbc_siren"] = loss_fns["ho_hardbc"]
    model_case("ho_hardbc_siren", D, sp, HOH, dict(d=2, w0=80, sd=0.1), [1, 8, 8, 1], xho, 15, [0],
               network="SIREN", wscale=np.sqrt(6.0))
    loss_fns["multilevel_siren"] = loss_fns["multilevel"]
    model_case("multilevel_siren", DM, spm, BU, dict(), [2, 8, 8, 1], rng_s.uniform(0, 1, (600, 2)), 16, [0, 1],
               network="SIREN", wscale=np.sqrt(6.0))
    # AdaptiveFCN (networks.py:70-100) and AdaptiveSIREN (networks.py:133-163)
    rng_a = np.random.default_rng(37)
    loss_fns["ho_hardbc_adafcn"] = loss_fns["ho_hardbc"]
    model_case("ho_hardbc_adafcn", D, sp, HOH, dict(d=2, w0=80, sd=0.1), [1, 8, 8, 1], xho, 17, [0],
               network="AdaptiveFCN")
    loss_fns["multilevel_adafcn"] = loss_fns["multilevel"]
    model_case("multilevel_adafcn", DM, spm, BU, dict(), [2, 8, 8, 1], rng_a.uniform(0, 1, (600, 2)), 18, [0, 1],
               network="AdaptiveFCN")
    loss_fns["ho_hardbc_adasiren"] = loss_fns["ho_hardbc"]
    model_case("ho_hardbc_adasiren", D, sp, HOH, dict(d=2, w0=80, sd=0.1), [1, 8, 8, 1], xho, 19, [0],
               network="AdaptiveSIREN", wscale=np.sqrt(6.0))
    loss_fns["multilevel_adasiren"] = loss_fns["multilevel"]
    model_case("multilevel_adasiren", DM, spm, BU, dict(), [2, 8, 8, 1], rng_a.uniform(0, 1, (600, 2)), 20,
               [0, 1], network="AdaptiveSIREN", wscale=np.sqrt(6.0))
    # FourierFCN (networks.py:165-194): 4 features, one hidden layer of 8
    rng_f = np.random.default_rng(93)
    loss_fns["ho_hardbc_fourier"] = loss_fns["ho_hardbc"]
    model_case("ho_hardbc_fourier", D, sp, HOH, dict(d=2, w0=80, sd=0.1), [1, 8, 1], xho, 21, [0],
               network="FourierFCN", n_features=4)
    loss_fns["multilevel_fourier"] = loss_fns["multilevel"]
    model_case("multilevel_fourier", DM, spm, BU, dict(), [2, 8, 1], rng_f.uniform(0, 1, (600, 2)), 22, [0, 1],
               network="FourierFCN", n_features=4)

    # 2-16-16-1 networks on the full six-level decomposition (levels 1, 2, 4,
    # 8, 16, 32 per dim, m = 1365): the benchmarked shape.  Box edges are
    # dense at the finest level, so the points keep a 2e-3 margin from every
    # edge (the difference stencils reach 5e-4).  Own generator: the draws
    # above are unchanged.
    rng_p = np.random.default_rng(41)
    spp, _ = DM.init_params(sxs, sws, (0., 1.))
    loss_fns["poisson16"] = loss_fns["multilevel"]
    model_case("poisson16", DM, spp, BU, dict(), [2, 16, 16, 1], rng_p.uniform(0, 1, (2000, 2)), 24, [0, 1],
               margin=2e-3, slim=True)

    # the reference's own wave field (problems.py:408-474: the seismic CPML
    # finite-difference solver) on a small grid, for the test of the
    # leapfrog field that stands in for it
    srcw = np.array([[0.1, -0.2, 0.15, 1.0], [-0.3, 0.25, 0.2, 0.5]])
    apw2 = {"static": {"problem": WV.init_params(c0=1.0, source=srcw)[0]}}
    bsw = (41, 41, 6)
    xw3 = np.asarray(domains.RectangularDomainND._rectangle_samplerND(
        None, "grid", jnp.array(np.array([-1., -1., 0.])), jnp.array(np.array([1., 1., 0.5])), bsw))
    uw3 = WV.exact_solution(apw2, xw3, bsw)
    save("wave_exact.npz", x=xw3, u=np.asarray(uw3), source=srcw, c0=np.float64(1.0), batch_shape=np.array(bsw))

    # constraining functions and losses on given jets
    xc = rng.uniform([-1, -1, 0], [1, 1, 1], (64, 3))
    uc = rng.normal(size=(64, 1))
    jc = [rng.normal(size=(64, 1)) for _ in range(4)]
    apw = {"static": {"problem": WV.init_params(c0=1.5, source=src)[0]}}
    mix = np.array([[0.2, 0.1, 0.5, 0.3], [-0.4, -0.1, 0.3, -0.2]])
    WG = problems.WaveEquationGaussianVelocity3D
    apg = {"static": {"problem": WG.init_params(c0=1.0, source=src, mixture=mix)[0]}}
    aph = {"static": {"problem": problems.HarmonicOscillator1D.init_params(d=2, w0=80)[0]}}
    api = {"static": {"problem": problems.HarmonicOscillator1DInverse.init_params(d=2, w0=20)[0]},
           "trainable": {"problem": {"mu": np.float64(3.3)}}}
    aphh = {"static": {"problem": HOH.init_params(d=2, w0=80, sd=0.1)[0]}}
    apb = {"static": {"problem": BU.init_params()[0]}}
    xdat = np.linspace(0, 1, 13).reshape((13, 1))
    save("problems.npz", x=xc, u=uc, j0=jc[0], j1=jc[1], j2=jc[2], j3=jc[3],
         wave_c=WV.constraining_fn(apw, xc, uc),
         wave_loss=WV.loss_fn(apw, [[xc, jc[0], jc[1], jc[2]]]),
         wave_gauss_c_fn=WG.c_fn(apg, xc),
         wave_gauss_loss=WG.loss_fn(apg, [[xc, jc[0], jc[1], jc[2]]]),
         burgers_c=BU.constraining_fn(apb, xc[:, :2], uc),
         burgers_loss=BU.loss_fn(apb, [[xc[:, :2], uc, jc[0], jc[1], jc[2]]]),
         hohard_c=HOH.constraining_fn(aphh, xc[:, :1], uc),
         ho_loss=problems.HarmonicOscillator1D.loss_fn(aph, [[xc[:, :1], uc, jc[0], jc[1]],
                                                              [xc[:2, :1], jc[2][:2], jc[3][:2], uc[:2], jc[0][:2]]]),
         ho_inv_loss=problems.HarmonicOscillator1DInverse.loss_fn(api, [[xc[:, :1], uc, jc[0], jc[1]],
                                                                        [xc[:3, :1], jc[2][:3], jc[3][:3]]]),
         ho_inv_data=problems.HarmonicOscillator1DInverse.exact_solution(api, xdat),
         ho_exact=problems.HarmonicOscillator1D.exact_solution(aph, np.linspace(0, 1, 1000).reshape(-1, 1)))

    # exact Burgers solution (problems.py:329-341 -> burgers_viscous_time_exact1)
    xt = np.asarray(domains.RectangularDomainND._rectangle_samplerND(
        None, "grid", np.array([-1., 0.]), np.array([1., 1.]), (64, 32)))
    ub = BU.exact_solution({"static": {"problem": BU.init_params()[0]}}, xt, (64, 32))
    save("burgers_exact.npz", x=xt, u=ub)

    # windows and networks (windows.py:11-70, networks.py:43-201)
    xw = rng.uniform(-1.2, 1.2, (50, 2))
    lo, hi = np.array([-1.0, -0.8]), np.array([1.0, 0.9])
    wl, wh = np.array([0.3, 0.2]), np.array([0.4, 0.25])
    win = {nm: np.stack([getattr(windows, nm)(*(a for a in (
        (lo, hi, wl, wh) if nm == "sigmoid" else (lo, hi))), xx) for xx in xw])
        for nm in ["sigmoid", "cosine", "bump", "wendland", "rbf"]}
    rr = np.random.default_rng(5)
    lay = [(rr.uniform(-1, 1, (8, 2)), rr.uniform(-1, 1, (8,))), (rr.uniform(-1, 1, (1, 8)), rr.uniform(-1, 1, (1,)))]
    layA = [(w, b, rr.uniform(0.5, 1.5, b.shape)) for w, b in lay]
    layS = [(w, b, rr.uniform(0.5, 1.5, b.shape), rr.uniform(0.5, 1.5, b.shape)) for w, b in lay]
    omega = rr.normal(size=(3, 2))
    layF = [(rr.uniform(-1, 1, (8, 6)), rr.uniform(-1, 1, (8,)))] + lay[1:]
    nets = {}
    for nm, L, st in [("FCN", lay, {}), ("AdaptiveFCN", layA, {}), ("SIREN", lay, {}),
                      ("AdaptiveSIREN", layS, {}), ("FourierFCN", layF, {"omega": omega})]:
        prm = {"static": {"network": {"subdomain": st}}, "trainable": {"network": {"subdomain": {"layers": L}}}}
        nets[nm] = np.stack([getattr(networks, nm).network_fn(prm, xx) for xx in xw])
    arrs = dict(x=xw, lo=lo, hi=hi, wl=wl, wh=wh, omega=omega)
    for i, (w, b) in enumerate(lay):
        arrs[f"W{i}"], arrs[f"b{i}"] = w, b
        arrs[f"A{i}"] = layA[i][2]
        arrs[f"C{i}"], arrs[f"O{i}"] = layS[i][2], layS[i][3]
    arrs["WF0"], arrs["bF0"] = layF[0]
    arrs.update({"win_" + k: v for k, v in win.items()})
    arrs.update({"net_" + k: v for k, v in nets.items()})
    save("windows_networks.npz", **arrs)

    # ------------------------------------------------------------------
    # 6. schedulers (schedulers.py, numpy-only: run as-is)
    # ------------------------------------------------------------------
    def sched_record(s):
        steps, ms = [], []
        for i, a in enumerate(s):
            if a is not None:
                steps.append(i)
                ms.append(np.array(a).copy())
        return np.array(steps), np.array(ms)

    xs1 = [np.array([-6, -4, -2, 0, 2, 4, 6.])]
    out = {}
    for tag, sxx in [("1d", xs1), ("2d", xs1 * 2), ("3d", xs1 * 3)]:
        spx, _ = D.init_params(sxx, [3 * np.ones_like(v) for v in sxx], (0, 1))
        apx = {"static": {"decomposition": spx}}
        xd = len(sxx)
        st, ms = sched_record(schedulers.PointSchedulerRectangularND(apx, 100, np.zeros(xd)))
        out[f"point_{tag}_steps"], out[f"point_{tag}_masks"] = st, ms
        if xd >= 2:
            st, ms = sched_record(schedulers.LineSchedulerRectangularND(apx, 100, np.zeros(xd - 1), 0))
            out[f"line_{tag}_steps"], out[f"line_{tag}_masks"] = st, ms
        if xd >= 3:
            st, ms = sched_record(schedulers.PlaneSchedulerRectangularND(apx, 100, np.zeros(xd - 2), [0, 1]))
            out[f"plane_{tag}_steps"], out[f"plane_{tag}_masks"] = st, ms
    st, ms = sched_record(schedulers.LineSchedulerRectangularND({"static": {"decomposition": spb}}, 1000, point=[0.], iaxis=0))
    out["burgers_steps"], out["burgers_masks"] = st, ms
    st, ms = sched_record(schedulers.AllActiveSchedulerND({"static": {"decomposition": spb}}, 10))
    out["allactive_steps"], out["allactive_masks"] = st, ms
    save("schedulers.npz", **out)


if __name__ == "__main__":
    main()
