"""Interaction lists on the GPU: bit-exact against the reference's golden
vectors and against the oracle, including edge cases and full-size runs."""

import numpy as np
import pytest
import torch

from conftest import golden
from helpers import decomposition, boxes_static
from oracle import takes as OT
from fbpinns_gb300 import takes as T
from fbpinns_gb300.engine import FBPINNEngine

pytestmark = pytest.mark.gpu


def _np(t):
    return t.cpu().numpy().astype(np.int64)


def test_kat_inside_points_and_models(cuda):
    """decompositions_base.py:87-128 known-answer configuration (seeded points)."""
    g = golden("takes_kat.npz")
    st = boxes_static(g["xmin"], g["xmax"])
    n_take, m_take, iims = T.inside_points(st, torch.tensor(g["x"]))
    np.testing.assert_array_equal(_np(n_take), g["n_take"])
    np.testing.assert_array_equal(_np(m_take), g["m_take"])
    np.testing.assert_array_equal(_np(iims), g["inside_ims"])
    ips, d = T.inside_models(st, torch.tensor(g["x"]), np.arange(1000))
    np.testing.assert_array_equal(_np(ips), g["inside_ips"])
    assert abs(d - float(g["d"])) <= 1e-6 * abs(float(g["d"]))


@pytest.mark.parametrize("tag", ["ho", "ho2c", "burgers_all", "burgers_sched", "multilevel", "wave3d"])
def test_get_inputs_bit_exact(cuda, tag):
    """get_inputs + _get_x_batch + per-constraint split (trainers.py:332-575)."""
    g = golden(f"inputs_{tag}.npz")
    static = decomposition(tag)
    all_params = {"static": {"decomposition": static}}
    ims = np.arange(static["m"])[g["active_in"] == 1]
    ips, _ = T.inside_models(static, torch.tensor(g["x_global"]), ims)
    x_batch = g["x_global"][_np(ips)]
    np.testing.assert_array_equal(x_batch, g["x_batch"])
    takes, all_ims, (active, _, _) = T.get_inputs(x_batch, g["active_in"], all_params)
    np.testing.assert_array_equal(active, g["active_out"])
    np.testing.assert_array_equal(_np(all_ims), g["all_ims"])
    for k, nm in enumerate(["m_take", "n_take", "p_take", "np_take"]):
        np.testing.assert_array_equal(_np(takes[k]), g[nm])
    assert takes[4] == int(g["npou"])
    cfs = g["constraint_fs"][_np(ips)]
    offsets = [int(cfs[:, :ic].any(1).sum()) if ic else 0 for ic in range(cfs.shape[1])]
    for ic, tk in enumerate(T.split_takes(takes, offsets, x_batch.shape[0])):
        for k, nm in enumerate(["m_take", "n_take", "p_take", "np_take"]):
            np.testing.assert_array_equal(_np(tk[k]), g[f"c{ic}_{nm}"])


def _oracle_takes(static, x):
    p = static["subdomain"]["params"]
    xmins, xmaxs = p[0].numpy(), p[1].numpy()
    pou = static["subdomain"]["pou"].numpy()
    takes, all_ims, _ = OT.get_inputs(x, np.ones(static["m"], dtype=int), xmins, xmaxs, pou)
    return takes


@pytest.mark.parametrize("n,seed", [(1, 0), (7, 1), (4097, 2), (60000, 3)])
def test_random_points_multilevel_vs_oracle(cuda, n, seed):
    static = decomposition("multilevel")
    rng = np.random.default_rng(seed)
    x = rng.uniform(-0.05, 1.05, (n, 2)).astype(np.float32)  # some points outside every box
    x[: min(n, 3)] = np.float32(0.5)                          # duplicates on box edges/centres
    ref = _oracle_takes(static, x)
    takes, _, _ = T.get_inputs(x, np.ones(static["m"], dtype=int), {"static": {"decomposition": static}})
    for k in range(4):
        np.testing.assert_array_equal(_np(takes[k]), ref[k])


@pytest.mark.parametrize("dense", [False, True])
def test_fill_hit_masks_match_testing_again(cuda, dense):
    """The fill pass takes its hits from the count pass's candidate masks
    (cells of <= 64 candidates) or tests the candidates again (denser cells, or
    no masks passed): the lists are identical either way and match the oracle.
    dense=True adds 80 boxes covering the whole domain, so every cell has more
    than 64 candidates."""
    rng = np.random.default_rng(9)
    lo = rng.uniform(0, 0.9, (150, 2)).astype(np.float32)
    hi = (lo + rng.uniform(0.05, 0.3, (150, 2))).astype(np.float32)
    if dense:
        lo = np.concatenate([lo, rng.uniform(-0.3, -0.06, (80, 2)).astype(np.float32)])
        hi = np.concatenate([hi, rng.uniform(1.3, 1.5, (80, 2)).astype(np.float32)])
    pou = (np.arange(lo.shape[0]) % 5).astype(np.float32)
    st = boxes_static(lo, hi, pou)
    x = rng.uniform(-0.05, 1.25, (5000, 2)).astype(np.float32)
    g = T.grid_of(st)
    xd = torch.tensor(x, device=g.device)
    out = []
    for masks in (True, False):
        t = T.PointTakes(g, x.shape[0])
        t.use_hit_masks = masks
        s, u = t.build(xd)
        t.check_status()
        out.append([_np(a[:k]) for a, k in ((t.n_take, s), (t.m_take, s), (t.p_take, s), (t.np_take, u))])
        if masks:
            cand = _np(t.pt_cand)
            assert (cand < 0).all() if dense else (cand >= 0).all()
    for a, b in zip(out[0], out[1]):
        np.testing.assert_array_equal(a, b)
    ref = OT.get_inputs(x, np.ones(lo.shape[0], dtype=int), lo, hi, pou.astype(np.int64))[0]
    np.testing.assert_array_equal(out[0][1], ref[0])  # m_take
    np.testing.assert_array_equal(out[0][0], ref[1])  # n_take
    np.testing.assert_array_equal(out[0][2], ref[2])  # p_take
    np.testing.assert_array_equal(out[0][3], ref[3])  # np_take


def test_points_on_box_boundaries_3d(cuda):
    """Points exactly on box faces (closed boxes) and outside the decomposition."""
    static = decomposition("wave")
    p = static["subdomain"]["params"]
    corners = torch.cat([p[0], p[1]]).numpy()
    x = np.concatenate([corners, corners + np.float32(1e-7), corners - np.float32(1e-7),
                        np.array([[5., 5., 5.], [-5., 0., 0.5]], np.float32)]).astype(np.float32)
    ref = _oracle_takes(static, x)
    takes, _, _ = T.get_inputs(x, np.ones(static["m"], dtype=int), {"static": {"decomposition": static}})
    for k in range(4):
        np.testing.assert_array_equal(_np(takes[k]), ref[k])


def test_sort_and_work_queue(cuda):
    """The subdomain-major order is a stable sort of the pairs by subdomain and the
    work items tile each subdomain's run."""
    static = decomposition("poisson")
    eng = FBPINNEngine(static, [2, 16, 16, 1], d2mask=3, chunk=256)
    rng = np.random.default_rng(7)
    x = torch.tensor(rng.uniform(0, 1, (20000, 2)).astype(np.float32))
    ps = eng.points(x)
    s = ps.s
    m_take = _np(ps.takes.m_take[:s])
    order = np.argsort(m_take, kind="stable")
    np.testing.assert_array_equal(_np(ps.sd_pair[:s]), order)
    np.testing.assert_array_equal(_np(ps.sd_point[:s]), _np(ps.takes.n_take[:s])[order])
    np.testing.assert_array_equal(_np(ps.sd_slot[:s]), _np(ps.takes.p_take[:s])[order])
    counts = np.bincount(m_take, minlength=static["m"])
    np.testing.assert_array_equal(_np(ps.sd_start), np.concatenate([[0], np.cumsum(counts)]))
    # forward items of up to 4 x 256 pairs (the engine's default), adjoint items of up to 256
    assert ps.fwd_chunk == 1024 and ps.chunk == 256
    for n_items, queue, chunk in ((ps.n_items_all, ps.items_all, 1024), (ps.n_items_act, ps.items_act, 256)):
        nit = int(n_items.item())
        items = _np(queue[: 3 * nit]).reshape(-1, 3)
        cover = np.zeros(s, dtype=np.int64)
        for j, b, c in items:
            assert 0 < c <= chunk
            assert m_take[order[b:b + c]].tolist() == [j] * c
            cover[b:b + c] += 1
        assert (cover == 1).all()


@pytest.mark.slow
def test_full_size_poisson_takes(cuda):
    """2D multilevel Poisson at full size (2^18 uniform points, 1365 boxes):
    bit-exact against the oracle's dense point-in-box test."""
    static = decomposition("poisson")
    rng = np.random.default_rng(11)
    x = rng.uniform(0, 1, (1 << 18, 2)).astype(np.float32)
    takes, _, _ = T.get_inputs(x, np.ones(static["m"], dtype=int), {"static": {"decomposition": static}})
    p = static["subdomain"]["params"]
    xmins, xmaxs = p[0].numpy(), p[1].numpy()
    n_ref, m_ref = [], []
    for i in range(0, x.shape[0], 8192):
        a, b = np.nonzero(OT.inside_rectangle(xmins, xmaxs, x[i:i + 8192], np.arange(static["m"])))
        n_ref.append(a + i)
        m_ref.append(b)
    np.testing.assert_array_equal(_np(takes[1]), np.concatenate(n_ref))
    np.testing.assert_array_equal(_np(takes[0]), np.concatenate(m_ref))
    # slots: np_take sorted, p_take consistent with (point, level)
    pou = static["subdomain"]["pou"].numpy().reshape(-1).astype(np.int64)
    key = np.concatenate(n_ref) * 64 + pou[np.concatenate(m_ref)]
    u, inv = np.unique(key, return_inverse=True)
    np.testing.assert_array_equal(_np(takes[2]), inv)
    np.testing.assert_array_equal(_np(takes[3]), u // 64)


@pytest.mark.parametrize("n", [1, 2047, 2048, 2049, 5_000_000, 9_000_000])
def test_exclusive_scan_matches_cumsum(cuda, n):
    """fbp_scan_i32 against numpy: out[i] = sum in[:i], out[n] = the total --
    up to 4096 tiles of 2048 (the down-sweep adds the earlier tiles' sums
    itself) and beyond (a scan of the tile sums in between)."""
    from fbpinns_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(n)
    x = rng.integers(0, 200, n).astype(np.int32)
    xin = torch.from_numpy(x).cuda()
    out = torch.full((n + 1,), -1, dtype=torch.int32, device="cuda")
    nb = int(lib.fbp_scan_scratch_bytes(n))
    scratch = torch.empty(nb // 4 + 1, dtype=torch.int32, device="cuda")
    _lib.check(lib.fbp_scan_i32(_lib.ptr(xin), _lib.ptr(out), n, _lib.ptr(scratch), nb, _lib.stream_ptr()),
               "fbp_scan_i32")
    ref = np.concatenate([[0], np.cumsum(x, dtype=np.int64)]).astype(np.int32)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)
