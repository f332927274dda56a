"""torch restatement of the reference FBPINN model, jets, loss, gradient and Adam.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Everything runs on the CPU in the dtype of its inputs (float64 for parity
checks, float32 for the timed CPU baseline).  JAX's ``vmap``/``jvp``/
``value_and_grad`` are replaced by per-pair batched torch ops,
``torch.func.jvp`` and ``torch.autograd.grad``; the algorithm (gathers per
pair, two segment sums, nested forward-mode jets, reverse-mode gradient of the
loss with respect to the active subdomain parameters only) is the reference's.

Parameter container used here (a flat dict instead of the reference pytree)::

    P = {"xmins": (m,xd), "xmaxs": (m,xd), "flags": (m,1), "unnorms": (m,2),
         "pou": (m,1) int, "layers": [(W (m,fo,fi), b (m,fo)), ...],
         "problem": {static problem params}, "problem_trainable": {...}}
"""

import math

import numpy as np
import torch


# ---------------------------------------------------------------------------
# decomposition parameters (numpy float64, like the reference)
# ---------------------------------------------------------------------------

def level_params(il, xd, subdomain_xs, subdomain_ws, unnorm):
    """``fbpinns/decompositions.py:136-181`` (``_get_level_params``).

    Returns [xmins, xmaxs, wmins, wmaxs, flags, unnorms, pous], numpy float64.
    """
    xs = np.stack(np.meshgrid(*subdomain_xs, indexing="ij"), 0)
    ws = np.stack(np.meshgrid(*subdomain_ws, indexing="ij"), 0)
    if xs.shape != ws.shape:
        raise ValueError("shape of subdomain_ws not same as subdomain_xs")
    xmins, xmaxs = xs - (ws / 2), xs + (ws / 2)
    wmins, wmaxs = 0.5 * (xmaxs - xmins), 0.5 * (xmaxs - xmins)
    for i in range(xd):
        sl0, sl1 = [slice(None)] * xd, [slice(None)] * xd
        sl0[i] = slice(None, -1)
        sl1[i] = slice(1, None)
        sl0, sl1 = (i,) + tuple(sl0), (i,) + tuple(sl1)
        wmaxs[sl0] = wmins[sl1] = xmaxs[sl0] - xmins[sl1]
        sl0, sl1 = [slice(None)] * xd, [slice(None)] * xd
        sl0[i] = 0
        sl1[i] = -1
        sl0, sl1 = (i,) + tuple(sl0), (i,) + tuple(sl1)
        wmins[sl0] = wmaxs[sl0]
        wmaxs[sl1] = wmins[sl1]
    if (wmins <= 0).any() or (wmaxs <= 0).any():
        raise ValueError("some subdomains are not overlapping!")
    f = lambda a: (a.reshape(xd, -1)).T
    xmins, xmaxs, wmins, wmaxs = f(xmins), f(xmaxs), f(wmins), f(wmaxs)
    s = (xmins.shape[0], 1)
    flags = np.zeros(s) if xmins.shape[0] == 1 else np.ones(s)
    unnorms = np.concatenate([unnorm[0] * np.ones(s), unnorm[1] * np.ones(s)], axis=1)
    pous = il * np.ones(s)
    return [xmins, xmaxs, wmins, wmaxs, flags, unnorms, pous]


def multilevel_params(subdomain_xss, subdomain_wss, unnorm):
    """``fbpinns/decompositions.py:342-375`` (levels concatenated, pou = level)."""
    xd = len(subdomain_xss[0])
    ps = [[] for _ in range(7)]
    for il, (sx, sw) in enumerate(zip(subdomain_xss, subdomain_wss)):
        for i, p_ in enumerate(level_params(il, xd, sx, sw, unnorm)):
            ps[i].append(p_)
    return [np.concatenate(p) for p in ps]


def scheduler_bounds(ps):
    """``fbpinns/decompositions.py:120,362``: centre lines of the overlaps."""
    return ps[0] + ps[2] / 2, ps[1] - ps[3] / 2


# ---------------------------------------------------------------------------
# per-pair model pieces (batched over pairs; the reference vmaps single points)
# ---------------------------------------------------------------------------

def norm(mu, sd, x):
    """``fbpinns/networks.py:197-198``."""
    return (x - mu) / sd


def unnorm(mu, sd, x):
    """``fbpinns/networks.py:200-201``."""
    return x * sd + mu


def heaviside1(v):
    """``jnp.heaviside(v, 1)`` with JAX's zero derivative."""
    return (v >= 0).to(v.dtype)


def cosine_window(xmin, xmax, x):
    """``fbpinns/windows.py:25-35`` batched: (s,xd) -> (s,1)."""
    mu, sd = (xmin + xmax) / 2, (xmax - xmin) / 2
    ws = ((1 + torch.cos(math.pi * (x - mu) / sd)) / 2) ** 2
    ws = heaviside1(x - xmin) * heaviside1(xmax - x) * ws
    return torch.prod(ws, dim=1, keepdim=True)


def sigmoid_window(xmin, xmax, wmin, wmax, x, tol=1e-8):
    """``fbpinns/windows.py:11-22`` batched: logistic ramps over the overlaps."""
    t = math.log((1 - tol) / tol)
    mu_min, sd_min = xmin + wmin / 2, wmin / (2 * t)
    mu_max, sd_max = xmax - wmax / 2, wmax / (2 * t)
    ws = torch.sigmoid((x - mu_min) / sd_min) * torch.sigmoid((mu_max - x) / sd_max)
    return torch.prod(ws, dim=1, keepdim=True)


def bump_window(xmin, xmax, x):
    """``fbpinns/windows.py:38-46`` batched."""
    mu, sd = (xmin + xmax) / 2, (xmax - xmin) / 2
    ws = torch.exp(3 / (((x - mu) / sd) ** 2 - 1.001)) / math.exp(-3)
    return torch.prod(ws, dim=1, keepdim=True)


def wendland_window(xmin, xmax, x):
    """``fbpinns/windows.py:49-59`` batched."""
    mu, sd = (xmin + xmax) / 2, (xmax - xmin) / 2
    r = torch.abs((x - mu) / sd)
    ws = ((1 - r) ** 4) * (4 * r + 1)
    ws = heaviside1(x - xmin) * heaviside1(xmax - x) * ws
    return torch.prod(ws, dim=1, keepdim=True)


def rbf_window(xmin, xmax, x):
    """``fbpinns/windows.py:62-68`` batched."""
    mu, sd = (xmin + xmax) / 2, (xmax - xmin) / 2
    return torch.exp(-0.5 * torch.sum(((x - mu) / (0.25 * sd)) ** 2, dim=1, keepdim=True))


def window(P, m_take, x_take):
    """The subdomain window named by P["window"] (default the decompositions'
    cosine, ``decompositions.py:197-199``) at the pairs' points."""
    name = P.get("window", "cosine")
    xmin, xmax = P["xmins"][m_take], P["xmaxs"][m_take]
    if name == "cosine":
        return cosine_window(xmin, xmax, x_take)
    if name == "sigmoid":
        return sigmoid_window(xmin, xmax, P["wmins"][m_take], P["wmaxs"][m_take], x_take)
    return {"bump": bump_window, "wendland": wendland_window, "rbf": rbf_window}[name](xmin, xmax, x_take)


def fcn(layers, x, activation="tanh"):
    """The reference's networks batched over pairs: W (s,fo,fi), b (s,fo) and the
    layer's activation parameters (s,fo): FCN tanh (``fbpinns/networks.py:61-68``),
    SIREN sin (``:102-131``), AdaptiveFCN a tanh(x/a) (``:70-100``), AdaptiveSIREN
    c sin(o x) (``:133-163``).  FourierFCN (``:165-194``, activation "fourier"):
    the first layer holds its features as W = [omega; omega] (the engine's
    packing); the oracle reads omega from the first half of the rows and
    computes [sin(omega x), cos(omega x)] as the reference does, then tanh layers."""
    for li, layer in enumerate(layers[:-1]):
        w, b = layer[0], layer[1]
        if activation == "fourier" and li == 0:
            F = w.shape[1] // 2
            z = torch.einsum("sij,sj->si", w[:, :F], x)
            x = torch.cat([torch.sin(z), torch.cos(z)], dim=1)
            continue
        x = torch.einsum("sij,sj->si", w, x) + b
        if activation == "tanh" or activation == "fourier":
            x = torch.tanh(x)
        elif activation == "sin":
            x = torch.sin(x)
        elif activation == "adaptive_tanh":
            x = layer[2] * torch.tanh(x / layer[2])
        elif activation == "adaptive_sin":
            x = layer[2] * torch.sin(layer[3] * x)
        else:
            raise ValueError(activation)
    w, b = layers[-1][0], layers[-1][1]
    return torch.einsum("sij,sj->si", w, x) + b


def segment_sum(data, ids, num):
    """``jax.ops.segment_sum`` with unsorted ids."""
    out = torch.zeros((num,) + tuple(data.shape[1:]), dtype=data.dtype)
    return out.index_add(0, ids, data)


def fbpinn_model(P, x_batch, takes, constraining_fn):
    """``fbpinns/trainers.py:113-118,126-177`` (``FBPINN_model``).

    ``P`` holds the parameters already cut to ``all_ims`` order (m_take indexes
    them).  Returns (u, wp, us, ws, us_raw).
    """
    m_take, n_take, p_take, np_take, npou = takes
    m_take = torch.as_tensor(m_take, dtype=torch.long)
    n_take = torch.as_tensor(n_take, dtype=torch.long)
    p_take = torch.as_tensor(p_take, dtype=torch.long)
    np_take = torch.as_tensor(np_take, dtype=torch.long)
    x_take = x_batch[n_take]
    xmin, xmax = P["xmins"][m_take], P["xmaxs"][m_take]
    # norm_fn  (decompositions.py:184-188)
    x_norm = norm((xmax + xmin) / 2, (xmax - xmin) / 2, x_take)
    # network_fn  (networks.py:61-68)
    layers = [tuple(t[m_take] for t in layer) for layer in P["layers"]]
    u_raw = fcn(layers, x_norm, P.get("activation", "tanh"))
    # unnorm_fn  (decompositions.py:191-194)
    un = P["unnorms"][m_take]
    u = unnorm(un[:, 0:1], un[:, 1:2], u_raw)
    # window_fn  (decompositions.py:197-199)
    flag = P["flags"][m_take]
    w = flag * window(P, m_take, x_take) + (1 - flag)
    us, ws = u * w, w
    # POU  (trainers.py:163-170)
    uu = torch.cat([us, ws], dim=1)
    uu = segment_sum(uu, p_take, len(np_take))
    wp = uu[:, -1:]
    uu = uu[:, :-1] / wp
    uu = segment_sum(uu, np_take, x_batch.shape[0])
    uu = uu / npou
    uu = constraining_fn(P, x_batch, uu)
    return uu, wp, us, ws, u_raw


# ---------------------------------------------------------------------------
# nested forward-mode jets (trainers.py:63-107, 197-247)
# ---------------------------------------------------------------------------

def get_jmaps(required_ujs):
    """``fbpinns/trainers.py:63-107`` (``get_jmaps``)."""
    tree = {}
    for iu, ixs in required_ujs:
        t = tree
        for ix in ixs:
            if ix not in t:
                t[ix] = {}
            t = t[ix]

    def get_nodes(t, n=(), ks=()):
        ni = len(n) - 1 + 1
        for k in t:
            ks_ = ks + (k,)
            if t[k]:
                n += (((ni, k), ks_, 0),)
                n = get_nodes(t[k], n, ks_)
            else:
                n += (((ni, k), ks_, 1),)
        return n

    nodes = get_nodes(tree)
    leaves = tuple((i + 1, node[1]) for i, node in enumerate(nodes) if node[2])
    if not leaves:
        leaves = ((0, ()),)
    jac_is = ()
    for iu, ixs in required_ujs:
        io = len(ixs)
        il = [leaf[1][:io] for leaf in leaves].index(ixs)
        jac_is += ((il, io, iu),)
    return nodes, leaves, jac_is


def _jacfwd(f, v):
    """``fbpinns/trainers.py:241-247``."""
    def jacfun(x):
        y, j, aux = torch.func.jvp(f, (x,), (v,), has_aux=True)
        return j, aux + (y,)
    return jacfun


def get_ujs(x_batch, jmaps, u):
    """``fbpinns/trainers.py:213-239`` (``_get_ujs``)."""
    nodes, leaves, jac_is = jmaps
    xd = x_batch.shape[1]
    vs = torch.eye(xd, dtype=x_batch.dtype).expand(x_batch.shape[0], xd, xd)
    fs = [u]
    for (ni, ix), _, _ in nodes:
        fs.append(_jacfwd(fs[ni], vs[:, ix].contiguous()))
    jacs = []
    for ie, _ in leaves:
        fin, jac = fs[ie](x_batch)
        jacs.append(jac + (fin,))
    return [jacs[il][io][:, iu:iu + 1] for il, io, iu in jac_is]


def fbpinn_forward(P, x_batch, takes, constraining_fn, jmaps):
    """``fbpinns/trainers.py:197-203`` (``FBPINN_forward``)."""
    def u(xb):
        return fbpinn_model(P, xb, takes, constraining_fn)[0], ()
    return get_ujs(x_batch, jmaps, u)


# ---------------------------------------------------------------------------
# loss, gradient, Adam
# ---------------------------------------------------------------------------

def cut_params(P, ims):
    """The ``cut_all`` / ``cut_active`` slicing of subdomain params (trainers.py:394-408)."""
    ims = torch.as_tensor(np.asarray(ims), dtype=torch.long)
    Q = dict(P)
    for k in ("xmins", "xmaxs", "flags", "unnorms", "pou", "wmins", "wmaxs"):
        if k in P:
            Q[k] = P[k][ims]
    Q["layers"] = [tuple(t[ims] for t in layer) for layer in P["layers"]]
    return Q


def fbpinn_loss(P, constraints, takess, jmapss, problem):
    """``fbpinns/trainers.py:249-267`` (``FBPINN_loss``) with params pre-cut."""
    constraints_ = []
    for takes, jmaps, constraint in zip(takess, jmapss, constraints):
        ujs = fbpinn_forward(P, constraint[0], takes, problem.constraining_fn, jmaps)
        constraints_.append(list(constraint) + ujs)
    return problem.loss_fn(P, constraints_)


def value_and_grad(P_all, active_ims, fixed_ims, constraints, takess, jmapss, problem,
                   trainable_problem_keys=()):
    """``fbpinns/trainers.py:285-293``: loss and d loss / d (active params).

    ``P_all`` holds all m subdomains.  The active rows get gradients, the fixed
    rows are constants, and the params are concatenated [active; fixed] as in
    ``FBPINN_loss`` (trainers.py:252-256).  Returns (loss, grads) where grads
    is a list of (dW, db) for the active rows plus a dict for trainable problem
    params.
    """
    all_ims = np.concatenate([active_ims, fixed_ims])
    Q = cut_params(P_all, all_ims)
    na = len(active_ims)
    leaves = []
    layers = []
    sizes = []
    for layer in Q["layers"]:
        act_t = [t[:na].detach().clone().requires_grad_(True) for t in layer]
        leaves += act_t
        sizes.append(len(layer))
        layers.append(tuple(torch.cat([ta, t[na:].detach()]) for ta, t in zip(act_t, layer)))
    Q["layers"] = layers
    pt = {}
    for k in trainable_problem_keys:
        pt[k] = torch.as_tensor(P_all["problem_trainable"][k]).detach().clone().requires_grad_(True)
        leaves.append(pt[k])
    Q["problem_trainable"] = pt
    loss = fbpinn_loss(Q, constraints, takess, jmapss, problem)
    g = torch.autograd.grad(loss, leaves, allow_unused=True)
    g = [torch.zeros_like(l) if gi is None else gi for gi, l in zip(g, leaves)]
    grads, o = [], 0
    for k in sizes:
        grads.append(tuple(g[o:o + k]))
        o += k
    gprob = {k: g[o + j] for j, k in enumerate(trainable_problem_keys)}
    return loss.detach(), grads, gprob


def pinn_model(P, x_batch, constraining_fn):
    """``fbpinns/trainers.py:120-124,179-195`` (``PINN_model``): one network
    over the whole domain -- the domain's norm_fn (``domains.py:106-110``),
    the network, the unnorm of ``decomposition_init_kwargs["unnorm"]``, then
    the constraining operator.  P: "domain_xmin", "domain_xmax" (xd,),
    "unnorm" (mu, sd), "layers" [(W (fo,fi), b (fo)), ...]."""
    lo, hi = P["domain_xmin"], P["domain_xmax"]
    n = x_batch.shape[0]
    x_norm = norm((hi + lo) / 2, (hi - lo) / 2, x_batch)
    layers = [tuple(t.expand((n,) + tuple(t.shape)) for t in layer) for layer in P["layers"]]
    u_raw = fcn(layers, x_norm, P.get("activation", "tanh"))
    u = unnorm(P["unnorm"][0], P["unnorm"][1], u_raw)
    return constraining_fn(P, x_batch, u), u_raw


def pinn_value_and_grad(P, constraints, jmapss, problem):
    """``fbpinns/trainers.py:269-306`` (``PINN_loss`` under ``value_and_grad``):
    the loss and its gradient with respect to every layer tensor."""
    leaves = []
    layers = []
    for layer in P["layers"]:
        ts = [t.detach().clone().requires_grad_(True) for t in layer]
        leaves += ts
        layers.append(tuple(ts))
    Q = dict(P, layers=layers)
    constraints_ = []
    for jmaps, constraint in zip(jmapss, constraints):
        def u(xb):
            return pinn_model(Q, xb, problem.constraining_fn)[0], ()
        constraints_.append(list(constraint) + get_ujs(constraint[0], jmaps, u))
    loss = problem.loss_fn(Q, constraints_)
    g = torch.autograd.grad(loss, leaves)
    grads, o = [], 0
    for layer in P["layers"]:
        grads.append(tuple(g[o:o + len(layer)]))
        o += len(layer)
    return loss.detach(), grads


def adam_update(params, grads, mu, nu, count, lr, b1=0.9, b2=0.999, eps=1e-8, eps_root=0.0):
    """optax ``adam`` = ``scale_by_adam`` + ``scale(-lr)``, then ``apply_updates``.

    Published Adam (Kingma & Ba 2015) with optax's defaults and ordering: the
    shared step ``count`` is incremented before the bias correction.  Returns
    (params, mu, nu, count) as new tensors.
    """
    mu = (1 - b1) * grads + b1 * mu
    nu = (1 - b2) * grads * grads + b2 * nu
    count = count + 1
    mu_hat = mu / (1 - b1 ** count)
    nu_hat = nu / (1 - b2 ** count)
    upd = mu_hat / (torch.sqrt(nu_hat + eps_root) + eps)
    return params - lr * upd, mu, nu, count
