"""Tensor-core (tcgen05, 3xTF32) forward jets vs the CUDA-core FMA kernel.

Both kernels write the same per-pair records (jets of u*w and of w); the
tensor-core one computes layer 2 with TF32 operands split hi + lo and three
products, so it agrees with the FP32 FMA path to FP32 rounding, not bitwise.
Tolerance: max |difference| per jet component below 2e-5 of that component's
largest magnitude.
"""

import ctypes as C
import math

import numpy as np
import pytest
import torch

from helpers import decomposition, random_layers, layer_sizes
from fbpinns_gb300 import _lib
from fbpinns_gb300.engine import FBPINNEngine
from fbpinns_gb300.networks import pack_layers

pytestmark = pytest.mark.gpu

TC_TOL = 2e-5


def _records(recipe, d2, n, seed, chunk=512):
    static = decomposition(recipe)
    m = static["subdomain"]["params"][0].shape[0]
    layers = random_layers([2, 16, 16, 1], m, seed)
    eng = FBPINNEngine(static, layer_sizes(layers), d2, chunk=chunk, tensor_cores=False)
    eng.set_theta(pack_layers([(w.float(), b.float()) for w, b in layers]))
    g = torch.Generator().manual_seed(seed)
    ps = eng.points(torch.rand((n, 2), generator=g))
    lib = _lib.load()
    net, pr = eng.net_struct(None), ps.pairs_struct(False)
    eng.forward_pairs(ps)
    ref = ps.pair_out[:ps.s].clone()
    ps.pair_out.fill_(float("nan"))
    status = torch.zeros(1, dtype=torch.int32, device=ps.x.device)
    _lib.check(lib.fbp_forward_pairs_tc(C.byref(net), _lib.ptr(ps.x), C.byref(pr), _lib.ptr(ps.pair_out),
                                        _lib.ptr(status), 0, _lib.stream_ptr()), "fbp_forward_pairs_tc")
    torch.cuda.synchronize()
    assert int(status.item()) == 0, _lib.decode_status(int(status.item()))
    return ref, ps.pair_out[:ps.s].clone(), eng.J


def _check(ref, tc, J):
    assert torch.isfinite(tc).all()
    for c in range(2 * J):
        scale = ref[:, c].abs().max().item()
        err = (tc[:, c] - ref[:, c]).abs().max().item()
        assert err <= TC_TOL * max(scale, 1e-30), (c, err, scale)


@pytest.mark.parametrize("d2", [3, 1, 0, 3 | 8])
def test_tensor_core_forward_matches_fma_small(cuda, d2):
    """Four-level decomposition (85 subdomains), 3000 points, all compiled jet
    masks (3 | 8: one Laplacian slot)."""
    ref, tc, J = _records("multilevel", d2, 3000, seed=5 + d2)
    _check(ref, tc, J)


def test_tensor_core_forward_matches_fma_poisson(cuda):
    """Six-level Poisson decomposition (1365 subdomains), 2^16 points: many
    full and partial 128-pair tiles per work item."""
    ref, tc, J = _records("poisson", 3, 1 << 16, seed=11)
    _check(ref, tc, J)


def test_tensor_core_forward_rejects_other_shapes(cuda):
    static = decomposition("multilevel")
    m = static["subdomain"]["params"][0].shape[0]
    layers = random_layers([2, 8, 8, 1], m, 1)
    eng = FBPINNEngine(static, layer_sizes(layers), 3)
    eng.set_theta(pack_layers([(w.float(), b.float()) for w, b in layers]))
    ps = eng.points(torch.rand((100, 2)))
    lib = _lib.load()
    status = torch.zeros(1, dtype=torch.int32, device=ps.x.device)
    rc = lib.fbp_forward_pairs_tc(C.byref(eng.net_struct(None)), _lib.ptr(ps.x), C.byref(ps.pairs_struct(False)),
                                  _lib.ptr(ps.pair_out), _lib.ptr(status), 0, _lib.stream_ptr())
    assert rc == -3  # FBP_ERR_UNSUPPORTED
    assert b"16-16" in lib.fbp_last_error()


def _net_layers(act, m, seed):
    """2-16-16-1 layers of each compiled activation (adaptive parameters and
    SIREN scales away from the defaults; FourierFCN: 8 features)."""
    from fbpinns_gb300.networks import fourier_feature_layer
    gen = torch.Generator().manual_seed(seed)
    base = random_layers([2, 16, 16, 1], m, seed)
    if act == "fourier":
        omega = 2 * math.pi * 0.5 * torch.randn((m, 8, 2), generator=gen, dtype=torch.float64)
        return [fourier_feature_layer(omega)] + [(w.float(), b.float()) for w, b in base[1:]]
    scale = math.sqrt(6.0) if act in ("sin", "adaptive_sin") else 1.0
    nx = {"sin": 0, "adaptive_tanh": 1, "adaptive_sin": 2}[act]
    return [tuple([(w * scale).float(), (b * scale).float()] +
                  [(0.5 + torch.rand(b.shape, generator=gen, dtype=torch.float64)).float() for _ in range(nx)])
            for w, b in base]


@pytest.mark.parametrize("act,d2", [("sin", 3 | 8), ("sin", 1), ("adaptive_tanh", 3 | 8), ("adaptive_tanh", 1),
                                    ("adaptive_sin", 3 | 8), ("adaptive_sin", 1), ("fourier", 1)])
def test_tensor_core_forward_other_activations(cuda, act, d2):
    """SIREN, AdaptiveFCN, AdaptiveSIREN and FourierFCN 2-16-16-1 networks on
    the tensor cores agree with the FMA kernel's records (four-level
    decomposition, 3000 points)."""
    static = decomposition("multilevel")
    m = static["subdomain"]["params"][0].shape[0]
    layers = _net_layers(act, m, seed=13)
    recs = []
    for tc in (False, True):
        eng = FBPINNEngine(static, [2, 16, 16, 1], d2, chunk=512, tensor_cores=tc, activation=act)
        eng.set_theta(pack_layers(layers))
        ps = eng.points(torch.rand((3000, 2), generator=torch.Generator().manual_seed(7)))
        ps.pair_out.fill_(float("nan"))
        eng.forward_pairs(ps)
        torch.cuda.synchronize()
        ps.check_status()
        recs.append(ps.pair_out[:ps.s].clone())
        J = eng.J
    _check(recs[0], recs[1], J)


def test_tensor_core_timeout_path_reports_and_recovers(cuda):
    """Failure detection without a fault: with FBP_STATUS_TC_TEST_NO_MMA the
    kernel issues no MMAs, its bounded waits (1 ms) run out, it reports
    FBP_STATUS_TC_TIMEOUT, frees its tensor memory and returns; the context
    stays usable and the next launch writes the same records as the FMA
    kernel."""
    static = decomposition("multilevel")
    m = static["subdomain"]["params"][0].shape[0]
    layers = random_layers([2, 16, 16, 1], m, 5)
    eng = FBPINNEngine(static, [2, 16, 16, 1], 3 | 8, chunk=512, tensor_cores=False)
    eng.set_theta(pack_layers([(w.float(), b.float()) for w, b in layers]))
    ps = eng.points(torch.rand((3000, 2), generator=torch.Generator().manual_seed(2)))
    eng.forward_pairs(ps)
    ref = ps.pair_out[:ps.s].clone()
    lib = _lib.load()
    net, pr = eng.net_struct(None), ps.pairs_struct(False)
    status = torch.full((1,), 1 << 30, dtype=torch.int32, device=ps.x.device)  # FBP_STATUS_TC_TEST_NO_MMA
    _lib.check(lib.fbp_forward_pairs_tc(C.byref(net), _lib.ptr(ps.x), C.byref(pr), _lib.ptr(ps.pair_out),
                                        _lib.ptr(status), 0, _lib.stream_ptr()), "fbp_forward_pairs_tc")
    torch.cuda.synchronize()
    assert int(status.item()) & 32  # FBP_STATUS_TC_TIMEOUT
    status.zero_()
    ps.pair_out.fill_(float("nan"))
    _lib.check(lib.fbp_forward_pairs_tc(C.byref(net), _lib.ptr(ps.x), C.byref(pr), _lib.ptr(ps.pair_out),
                                        _lib.ptr(status), 0, _lib.stream_ptr()), "fbp_forward_pairs_tc")
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    _check(ref, ps.pair_out[:ps.s].clone(), eng.J)


def _grads(recipe, d2, n, seed, tc_adjoint, problem="poisson", points=None):
    """Per-subdomain gradient of the fused loss with the FMA or the
    tensor-core adjoint (same forward, same seeds)."""
    from fbpinns_gb300 import problems as PR
    static = decomposition(recipe)
    m = static["subdomain"]["params"][0].shape[0]
    layers = random_layers([2, 16, 16, 1], m, seed)
    eng = FBPINNEngine(static, [2, 16, 16, 1], d2, chunk=512, tc_adjoint=tc_adjoint)
    assert eng.tc_adjoint == tc_adjoint
    eng.set_theta(pack_layers([(w.float(), b.float()) for w, b in layers]))
    if problem == "poisson":
        spec = PR.Poisson2D.fused_spec({"static": {"problem": PR.Poisson2D.init_params(n_freq=6, sd=0.1)[0]}})
    else:
        spec = PR.BurgersEquation2D.fused_spec({"static": {"problem": PR.BurgersEquation2D.init_params()[0]}})
    eng.set_problem(spec)
    ps = eng.points(points if points is not None else torch.rand((n, 2), generator=torch.Generator().manual_seed(seed)))
    eng.forward_pairs(ps)
    loss = eng.pou_loss(ps).item()
    ps.grad_part.fill_(float("nan"))
    g = eng.adjoint(ps).clone()
    torch.cuda.synchronize()
    ps.check_status()
    return loss, g


@pytest.mark.parametrize("recipe,d2,n,problem", [("multilevel", 3 | 8, 3000, "poisson"),
                                                 ("multilevel", 3, 3000, "poisson"),
                                                 ("poisson", 3 | 8, 1 << 16, "poisson"),
                                                 ("burgers", 1, 4000, "burgers")])
def test_tensor_core_adjoint_matches_fma(cuda, recipe, d2, n, problem):
    """The adjoint with the layer-2 recompute on the tensor cores gives the
    FMA adjoint's gradients (every subdomain's, 2e-5 of the largest): the
    benchmark's six-level Poisson shape with the Laplacian slot, per-dim
    slots, and the Burgers jet (u_xx)."""
    pts = None
    if problem == "burgers":
        g = torch.Generator().manual_seed(4)
        pts = torch.stack([torch.rand(n, generator=g) * 2 - 1, torch.rand(n, generator=g)], 1)
    l0, g0 = _grads(recipe, d2, n, 9, False, problem, pts)
    l1, g1 = _grads(recipe, d2, n, 9, True, problem, pts)
    assert l0 == l1  # the same forward and loss kernels
    assert torch.isfinite(g1).all()
    err = (g1 - g0).abs().max().item() / g0.abs().max().item()
    assert err < TC_TOL, err


def test_tensor_core_adjoint_timeout_path_reports_and_recovers(cuda):
    """The tensor-core adjoint's bounded waits: with FBP_STATUS_TC_TEST_NO_MMA
    no MMAs are issued, the waits (1 ms) run out, the kernel reports
    FBP_STATUS_TC_TIMEOUT, frees its tensor memory and returns; the next
    launch on the same context gives the FMA adjoint's gradient partials."""
    from fbpinns_gb300 import problems as PR
    static = decomposition("multilevel")
    m = static["subdomain"]["params"][0].shape[0]
    layers = random_layers([2, 16, 16, 1], m, 5)
    eng = FBPINNEngine(static, [2, 16, 16, 1], 3 | 8, chunk=512)
    eng.set_theta(pack_layers([(w.float(), b.float()) for w, b in layers]))
    eng.set_problem(PR.Poisson2D.fused_spec({"static": {"problem": PR.Poisson2D.init_params(n_freq=6, sd=0.1)[0]}}))
    ps = eng.points(torch.rand((3000, 2), generator=torch.Generator().manual_seed(2)))
    eng.forward_pairs(ps)
    eng.pou_loss(ps)
    eng.adjoint(ps, reduce=False)
    ref = ps.grad_part.clone()
    lib = _lib.load()
    net, pr = eng.net_struct(None), ps.pairs_struct(True)
    status = torch.full((1,), 1 << 30, dtype=torch.int32, device=ps.x.device)  # FBP_STATUS_TC_TEST_NO_MMA
    _lib.check(lib.fbp_adjoint_pairs_tc(C.byref(net), _lib.ptr(ps.x), C.byref(pr), _lib.ptr(ps.slot_out),
                                        _lib.ptr(ps.grad_part), _lib.ptr(status), 0, _lib.stream_ptr()),
               "fbp_adjoint_pairs_tc")
    torch.cuda.synchronize()
    assert int(status.item()) & 32  # FBP_STATUS_TC_TIMEOUT
    status.zero_()
    ps.grad_part.fill_(float("nan"))
    _lib.check(lib.fbp_adjoint_pairs_tc(C.byref(net), _lib.ptr(ps.x), C.byref(pr), _lib.ptr(ps.slot_out),
                                        _lib.ptr(ps.grad_part), _lib.ptr(status), 0, _lib.stream_ptr()),
               "fbp_adjoint_pairs_tc")
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    n_items = int(ps.n_items_act.item())
    a, b = ref[:n_items], ps.grad_part[:n_items]
    assert torch.isfinite(b).all()
    assert (a - b).abs().max().item() <= TC_TOL * a.abs().max().item()
