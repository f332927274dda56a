"""Collocation points ordered by Morton cells (fbp_sort_points_cells) against
a numpy stable sort of the same cell keys, and the engine's ordered sampler
against the unordered one (the same batch of points)."""
import ctypes as C

import numpy as np
import pytest
import torch

from fbpinns_gb300 import _lib
from helpers import decomposition

pytestmark = pytest.mark.gpu


def _cell_bits(n, xd):
    """Bits per dim of the cell index: about n / 64 cells, rounded up to whole
    bits per dim, at most 2^16 cells."""
    total = 0
    while total < 16 and (64 << (total + 1)) <= n:
        total += 1
    b = (total + xd - 1) // xd
    while b * xd > 16:
        b -= 1
    return b


def _spread(v, xd):
    out = np.zeros_like(v, dtype=np.uint64)
    for bit in range(16):
        out |= ((v.astype(np.uint64) >> np.uint64(bit)) & np.uint64(1)) << np.uint64(bit * xd)
    return out


def _expected_order(x, lo, hi):
    n, xd = x.shape
    b = _cell_bits(n, xd)
    top = (1 << b) - 1
    key = np.zeros(n, dtype=np.uint64)
    for d in range(xd):
        scale = np.float32((1 << b) / (hi[d] - lo[d]))
        f = (x[:, d] - np.float32(lo[d])) * scale  # float32 arithmetic, as on the device
        c = np.where(f >= 0, f, 0).astype(np.int64).clip(0, top)
        key |= _spread(c, xd) << np.uint64(d)
    return np.argsort(key, kind="stable")


@pytest.mark.parametrize("xd,n,crowded", [(1, 100, False), (2, 5000, False), (2, 1 << 16, False),
                                           (2, 70001, False), (3, 40000, False), (2, 40000, True)])
def test_point_cell_order_matches_stable_sort(cuda, xd, n, crowded):
    """Bitwise the points in (Morton cell, input index) order; crowded: the
    points fill a small corner of the cell grid's box (cells of ~1000 points,
    ranked chunk by chunk), with some outside it (clamped to edge cells)."""
    rng = np.random.default_rng(n + xd)
    lo, hi = [-1.0, 0.0, 0.5][:xd], [1.0, 2.0, 1.5][:xd]
    x = (np.asarray(lo) + (np.asarray(hi) - np.asarray(lo)) * rng.uniform(0, 1, (n, xd))).astype(np.float32)
    x[:7] = np.asarray(hi, dtype=np.float32)  # points on the upper bounds: the last cell
    x[7:9] = np.asarray(lo, dtype=np.float32)
    if crowded:
        lo, hi = [-1.0, 0.0, 0.5][:xd], [7.0, 8.0, 8.5][:xd]
        x[9:20] = np.float32(-5.0)  # below the box
    lib = _lib.load()
    xin = torch.from_numpy(x).cuda()
    out = torch.full_like(xin, float("nan"))
    nb = int(lib.fbp_sort_points_scratch_bytes(n, xd))
    scratch = torch.empty(nb // 4 + 1, dtype=torch.int32, device="cuda")
    clo, chi = (C.c_double * 3)(*lo), (C.c_double * 3)(*hi)
    for _ in range(2):  # the same result every time
        _lib.check(lib.fbp_sort_points_cells(_lib.ptr(xin), n, xd, clo, chi, _lib.ptr(out), _lib.ptr(scratch), nb,
                                             None), "fbp_sort_points_cells")
        torch.cuda.synchronize()
        np.testing.assert_array_equal(out.cpu().numpy(), x[_expected_order(x, lo, hi)])
    # too little scratch and aliased buffers are refused
    assert lib.fbp_sort_points_cells(_lib.ptr(xin), n, xd, clo, chi, _lib.ptr(out), _lib.ptr(scratch), nb - 4,
                                     None) == -1  # FBP_ERR_INVALID
    assert lib.fbp_sort_points_cells(_lib.ptr(xin), n, xd, clo, chi, _lib.ptr(xin), _lib.ptr(scratch), nb,
                                     None) == -1  # FBP_ERR_INVALID


def test_ordered_sampler_draws_the_same_batch(cuda):
    """engine.sample with the cell order: the points of the unordered draw (as a
    set, bitwise), in cell order; the step count offsets the stream as before."""
    from fbpinns_gb300.engine import FBPINNEngine
    static = decomposition("multilevel")
    eng = FBPINNEngine(static, [2, 8, 8, 1], 3)
    n = 1 << 15
    a = torch.empty((n, 2), device="cuda")
    b = torch.empty((n, 2), device="cuda")
    eng.sample(a, 11, 3, [0.0, 0.0], [1.0, 1.0], counter=eng.count, order=False)
    eng.sample(b, 11, 3, [0.0, 0.0], [1.0, 1.0], counter=eng.count)
    torch.cuda.synchronize()
    xa, xb = a.cpu().numpy(), b.cpu().numpy()
    assert not np.array_equal(xa, xb)
    np.testing.assert_array_equal(xb, xa[_expected_order(xa, [0.0, 0.0], [1.0, 1.0])])
