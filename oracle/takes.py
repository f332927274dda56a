"""numpy restatement of the reference's interaction-list ("takes") construction.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Every function follows the reference algorithm step by step, including the
memory-bounded point batching with its shifted, masked last batch, so that the
outputs can be compared bit-exactly with the CUDA kernels.  Indices are int64
here; the reference uses int32 (``dtype=int`` without x64) and the values are
identical.
"""

import numpy as np


def inside_rectangle(xmins, xmaxs, x_batch, ims):
    """Closed-box test ``xmin <= x <= xmax`` on all dims, (n, len(ims)) bool.

    Follows ``fbpinns/decompositions.py:218-227`` (``_inside_rectangleND``).
    Inputs are float32 arrays, compared in float32 like the reference.
    """
    x = x_batch[:, None, :]
    lo = xmins[ims][None]
    hi = xmaxs[ims][None]
    return np.all((x >= lo) & (x <= hi), axis=-1)


def _batches(n, batch_size):
    """Start indices and masks of the fully-populated point batches.

    ``fbpinns/decompositions_base.py:33-39``: the last batch is shifted back so
    that it is full, and its leading ``shift`` rows (already covered by the
    previous batch) are masked out.
    """
    r = n % batch_size
    shift = batch_size - r if r else 0
    starts = np.arange(0, n, batch_size)
    mask = np.ones((len(starts), batch_size), dtype=bool)
    starts[-1] -= shift
    mask[-1, :shift] = False
    return starts, mask, shift


def inside_sum_batch(xmins, xmaxs, x_batch, ims, batch_size):
    """``fbpinns/decompositions_base.py:24-48`` (``_inside_sum_batch``).

    Returns (s, inside_ips (n,) bool, inside_ims (len(ims),) bool, d).
    """
    n, xd = x_batch.shape
    starts, mask, shift = _batches(n, batch_size)
    s1, s2 = [], []
    for i, mk in zip(starts, mask):
        ins = mk[:, None] & inside_rectangle(xmins, xmaxs, x_batch[i:i + batch_size], ims)
        s1.append(ins.any(axis=1))
        s2.append(ins.sum(axis=0))
    s1, s2 = np.stack(s1), np.stack(s2)
    inside_ips = np.concatenate([s1[:-1].ravel(), s1[-1][shift:]], axis=0)
    counts = s2.sum(axis=0)
    d = counts.mean() ** (1.0 / xd)
    s = int(counts.sum())
    return s, inside_ips, counts.astype(bool), d


def inside_take_batch(xmins, xmaxs, x_batch, ims, batch_size, s):
    """``fbpinns/decompositions_base.py:51-68`` (``_inside_take_batch``).

    Cumulative-sum compaction of each batch's (point, model) mask into the
    global (s, 2) take array, accumulated with scatter-add semantics exactly as
    ``take.at[s+itake].add(ii_)`` (masked entries add zeros).
    """
    n = x_batch.shape[0]
    starts, mask, _ = _batches(n, batch_size)
    mc = len(ims)
    ix, iy = np.meshgrid(np.arange(batch_size), np.arange(mc), indexing="ij")
    ii = np.stack([ix.ravel(), iy.ravel()], axis=1)
    take = np.zeros((s, 2), dtype=np.int64)
    off = 0
    for i, mk in zip(starts, mask):
        ins = (mk[:, None] & inside_rectangle(xmins, xmaxs, x_batch[i:i + batch_size], ims)).ravel()
        itake = np.cumsum(ins) - 1
        ii_ = ins[:, None].astype(np.int64) * (ii + np.array([i, 0]))
        if s > 0:
            np.add.at(take, off + itake, ii_)
        off = off + int(itake[-1]) + 1
    return take


def default_batch_size(n, mc):
    """``fbpinns/decompositions.py:205,212``: ``min(int(1e9/(4*mc)), n)``."""
    return min(int(1e9 / (4 * mc)), n)


def inside_points(xmins, xmaxs, x_batch, batch_size=None):
    """``RectangularDecompositionND.inside_points`` -> ``inside_points_batch``.

    ``fbpinns/decompositions.py:202-208`` and ``decompositions_base.py:70-76``.
    Returns (n_take, m_take, inside_ims) in point-major, model-minor order.
    """
    m = xmins.shape[0]
    ims = np.arange(m)
    if batch_size is None:
        batch_size = default_batch_size(x_batch.shape[0], m)
    assert batch_size <= x_batch.shape[0]
    s, _, inside_ims, _ = inside_sum_batch(xmins, xmaxs, x_batch, ims, batch_size)
    inside_ims = np.arange(m)[inside_ims]
    take = inside_take_batch(xmins, xmaxs, x_batch, ims, batch_size, s)
    return take[:, 0], take[:, 1], inside_ims


def inside_models(xmins, xmaxs, x_batch, ims, batch_size=None):
    """``RectangularDecompositionND.inside_models`` -> ``inside_models_batch``.

    ``fbpinns/decompositions.py:211-215`` and ``decompositions_base.py:78-82``.
    Returns (inside_ips, d): the points inside at least one model of ``ims``.
    """
    ims = np.asarray(ims)
    if batch_size is None:
        batch_size = default_batch_size(x_batch.shape[0], ims.shape[0])
    assert batch_size <= x_batch.shape[0]
    _, inside_ips, _, d = inside_sum_batch(xmins, xmaxs, x_batch, ims, batch_size)
    return np.arange(x_batch.shape[0])[inside_ips], d


def get_inputs(x_batch, active, xmins, xmaxs, pou, batch_size=None):
    """``fbpinns/trainers.py:332-419`` (``get_inputs``), integer part.

    Returns ``takes=(m_take, n_take, p_take, np_take, npou)``, ``all_ims`` and
    (updated active, active_ims, fixed_ims).
    """
    m = xmins.shape[0]
    n_take, m_take, training_ims = inside_points(xmins, xmaxs, x_batch, batch_size)
    active = np.array(active).copy()
    assert np.isin(active, np.array([0, 1, 2])).all()
    assert active.shape == (m,)
    active[active == 0] = 1
    mask = np.zeros_like(active)
    mask[training_ims] = 1
    active = active * mask
    ims_ = np.arange(m)
    active_ims = ims_[active == 1]
    fixed_ims = ims_[active == 2]
    all_ims = np.concatenate([active_ims, fixed_ims])
    inv = np.zeros(m, dtype=np.int64)
    inv[all_ims] = np.arange(len(all_ims))
    m_take = inv[m_take]
    pou = np.asarray(pou).reshape(m, -1)
    pous = pou[all_ims].astype(int)
    np_ = np.stack([n_take, pous[m_take, 0]], axis=-1).astype(int)
    if np_.shape[0]:
        npu, p_take = np.unique(np_, axis=0, return_inverse=True)
    else:
        npu, p_take = np.zeros((0, 2), dtype=int), np.zeros((0,), dtype=int)
    p_take = p_take.reshape(-1)
    np_take = npu[:, 0]
    npou = len(np.unique(pou.astype(int)))
    takes = (m_take, n_take, p_take, np_take, npou)
    return takes, all_ims, (active, active_ims, fixed_ims)


def split_takes(takes, constraint_fs, n_points):
    """``fbpinns/trainers.py:544-571``: re-index the takes per constraint.

    ``constraint_fs`` is the (n, c) bool filter of training points per
    constraint.  Returns the list of per-constraint takes.
    """
    m_take, n_take, p_take, np_take, npou = takes
    ix_ = np.arange(n_points)
    iu_ = np.arange(np_take.shape[0])
    takess = []
    for f in constraint_fs.T:
        ips = ix_[f]
        f1 = f
        f2 = f[np_take]
        ius = iu_[f2]
        f3 = f1[n_take]
        f4 = f2[p_take]
        inv = np.zeros(n_points, dtype=np.int64)
        inv[ips] = np.arange(len(ips))
        inv2 = np.zeros(np_take.shape[0], dtype=np.int64)
        inv2[ius] = np.arange(len(ius))
        takess.append((m_take[f3], inv[n_take[f3]], inv2[p_take[f4]], inv[np_take[f2]], npou))
    return takess


def get_x_batch(active, xmins, xmaxs, x_batch_global, constraint_fs_global, batch_size=None):
    """``fbpinns/trainers.py:482-507`` (``FBPINNTrainer._get_x_batch``), index part.

    Returns (training_ips, constraint_fs, constraint_ips): the global indices of
    the training points (inside any model with raw state 1), their constraint
    filter and the per-constraint point indices.
    """
    m = xmins.shape[0]
    ims = np.arange(m)[np.asarray(active) == 1]
    training_ips, _ = inside_models(xmins, xmaxs, x_batch_global, ims, batch_size)
    constraint_fs = constraint_fs_global[training_ips]
    ix_ = np.arange(training_ips.shape[0])
    constraint_ips = [ix_[f] for f in constraint_fs.T]
    return training_ips, constraint_fs, constraint_ips
