"""The fused step at the full bench size (2D multilevel Poisson, m = 1365,
FCN 2-16-16-1, 2^18 points, Laplacian jets), checked through properties that
do not need the oracle at that size:

* additivity: the loss is a mean of per-point terms and each point's jets
  depend only on that point, so loss(all) = (n_A loss(A) + n_B loss(B)) / n
  and the gradient sums the halves' gradients weighted the same way
  (FP32 sums in a different order: relative tolerance 1e-5 on the loss and
  on the gradient);
* the tensor-core and the CUDA-core forward give the same loss and gradient
  (tolerance as above);
* a second evaluation of the same step is bitwise identical (determinism).
"""

import numpy as np
import pytest
import torch

from helpers import decomposition, random_layers, layer_sizes, rel_err
from fbpinns_gb300 import _lib
from fbpinns_gb300 import problems as PR
from fbpinns_gb300.engine import FBPINNEngine
from fbpinns_gb300.networks import pack_layers

pytestmark = pytest.mark.gpu

N = 1 << 18
LOSS_TOL = 1e-5
GRAD_TOL = 1e-5


def _setup(tensor_cores):
    static = decomposition("poisson")
    layers = random_layers([2, 16, 16, 1], static["m"], seed=41)
    eng = FBPINNEngine(static, layer_sizes(layers), 3 | _lib.D2_LAPLACIAN, chunk=512, tensor_cores=tensor_cores)
    eng.set_theta(pack_layers([(w.float(), b.float()) for w, b in layers]))
    prob = PR.Poisson2D.init_params(n_freq=6, sd=0.1)[0]
    eng.set_problem(PR.Poisson2D.fused_spec({"static": {"problem": prob}}))
    return eng


def _loss_grad(eng, x):
    ps = eng.points(x)
    eng.forward_pairs(ps)
    loss = eng.pou_loss(ps).item()
    grad = eng.adjoint(ps).double().cpu().numpy()
    ps.check_status()
    return loss, grad


@pytest.fixture(scope="module")
def points():
    g = torch.Generator().manual_seed(5)
    return torch.rand((N, 2), generator=g)


def test_full_size_loss_and_gradient_are_additive_over_point_halves(cuda, points):
    eng = _setup(None)
    assert eng.tensor_cores
    loss, grad = _loss_grad(eng, points)
    h = N // 2
    la, ga = _loss_grad(eng, points[:h])
    lb, gb = _loss_grad(eng, points[h:])
    assert np.isfinite(loss) and loss > 0
    comb = (h * la + (N - h) * lb) / N
    assert abs(loss - comb) <= LOSS_TOL * abs(loss), (loss, comb)
    gcomb = (h * ga + (N - h) * gb) / N
    assert (e := rel_err(grad, gcomb)) < GRAD_TOL, e


def test_full_size_tensor_core_forward_matches_fma(cuda, points):
    lt, gt = _loss_grad(_setup(True), points)
    lf, gf = _loss_grad(_setup(False), points)
    assert abs(lt - lf) <= LOSS_TOL * abs(lf), (lt, lf)
    assert (e := rel_err(gt, gf)) < GRAD_TOL, e


def test_full_size_step_is_deterministic(cuda, points):
    eng = _setup(None)
    l1, g1 = _loss_grad(eng, points)
    l2, g2 = _loss_grad(eng, points)
    assert l1 == l2
    assert np.array_equal(g1, g2)
