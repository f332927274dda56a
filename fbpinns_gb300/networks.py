"""Subdomain networks (the reference's ``fbpinns/networks.py`` API), in torch.

``network_fn(params, x)`` evaluates one network on x (..., fan_in) — a single
point or a batch; per-pair parameter batches (leading dim s) are supported by
``batched_linear``.  Initialisation draws W, b ~ U(-1/sqrt(fan_in),
+1/sqrt(fan_in)) like ``FCN._random_layer_params`` (fbpinns/networks.py:51-58);
the reference uses JAX's PRNG, this engine a seeded torch generator, so the
draws differ but the distribution is the same.
"""

import math

import torch


def _gen(key):
    if isinstance(key, torch.Generator):
        return key
    g = torch.Generator()
    g.manual_seed(int(key))
    return g


def _uniform(g, shape, v):
    return (torch.rand(shape, generator=g, dtype=torch.float64) * 2 - 1).mul_(v).float()


def batched_linear(w, b, x):
    """x @ w^T + b for w (..., fo, fi) and x (..., fi)."""
    return torch.einsum("...ij,...j->...i", w, x) + b


class Network:
    """Base class (fbpinns/networks.py:14-34)."""

    @staticmethod
    def init_params(*args):
        raise NotImplementedError

    @staticmethod
    def network_fn(params, x):
        raise NotImplementedError


class FCN(Network):
    """tanh hidden layers, linear output (fbpinns/networks.py:39-68)."""

    @staticmethod
    def init_params(key, layer_sizes):
        g = _gen(key)
        layers = []
        for fi, fo in zip(layer_sizes[:-1], layer_sizes[1:]):
            v = math.sqrt(1.0 / fi)
            layers.append((_uniform(g, (fo, fi), v), _uniform(g, (fo,), v)))
        return {}, {"layers": layers}

    @staticmethod
    def network_fn(params, x):
        layers = params["trainable"]["network"]["subdomain"]["layers"]
        for w, b in layers[:-1]:
            x = torch.tanh(batched_linear(w, b, x))
        w, b = layers[-1]
        return batched_linear(w, b, x)


class AdaptiveFCN(Network):
    """a tanh(x / a) activations (fbpinns/networks.py:70-100)."""

    @staticmethod
    def init_params(key, layer_sizes):
        _, tp = FCN.init_params(key, layer_sizes)
        return {}, {"layers": [(w, b, torch.ones_like(b)) for w, b in tp["layers"]]}

    @staticmethod
    def network_fn(params, x):
        layers = params["trainable"]["network"]["subdomain"]["layers"]
        for w, b, a in layers[:-1]:
            x = a * torch.tanh(batched_linear(w, b, x) / a)
        w, b, _ = layers[-1]
        return batched_linear(w, b, x)


class SIREN(Network):
    """sin activations, U(+-sqrt(6/fan_in)) init (fbpinns/networks.py:102-131)."""

    @staticmethod
    def init_params(key, layer_sizes):
        g = _gen(key)
        layers = []
        for fi, fo in zip(layer_sizes[:-1], layer_sizes[1:]):
            v = math.sqrt(6.0 / fi)
            layers.append((_uniform(g, (fo, fi), v), _uniform(g, (fo,), v)))
        return {}, {"layers": layers}

    @staticmethod
    def network_fn(params, x):
        layers = params["trainable"]["network"]["subdomain"]["layers"]
        for w, b in layers[:-1]:
            x = torch.sin(batched_linear(w, b, x))
        w, b = layers[-1]
        return batched_linear(w, b, x)


class AdaptiveSIREN(Network):
    """c sin(o x) activations (fbpinns/networks.py:133-163)."""

    @staticmethod
    def init_params(key, layer_sizes):
        _, tp = SIREN.init_params(key, layer_sizes)
        return {}, {"layers": [(w, b, torch.ones_like(b), torch.ones_like(b)) for w, b in tp["layers"]]}

    @staticmethod
    def network_fn(params, x):
        layers = params["trainable"]["network"]["subdomain"]["layers"]
        for w, b, c, o in layers[:-1]:
            x = c * torch.sin(o * batched_linear(w, b, x))
        w, b, _, _ = layers[-1]
        return batched_linear(w, b, x)


class FourierFCN(FCN):
    """Fourier features [sin(omega x), cos(omega x)] then an FCN (fbpinns/networks.py:165-194)."""

    @staticmethod
    def init_params(key, layer_sizes, mu, sd, n_features):
        g = _gen(key)
        omega = (2 * math.pi * (mu + sd * torch.randn((n_features, layer_sizes[0]), generator=g,
                                                      dtype=torch.float64))).float()
        _, tp = FCN.init_params(g, [2 * n_features] + list(layer_sizes)[1:])
        return {"omega": omega}, tp

    @staticmethod
    def network_fn(params, x):
        omega = params["static"]["network"]["subdomain"]["omega"]
        x = torch.einsum("...ij,...j->...i", omega, x)
        x = torch.cat([torch.sin(x), torch.cos(x)], dim=-1)
        return FCN.network_fn(params, x)


# Network classes with compiled jet kernels, by activation code of the kernels
NETWORK_ACTIVATIONS = {FCN: "tanh", SIREN: "sin", AdaptiveFCN: "adaptive_tanh", AdaptiveSIREN: "adaptive_sin",
                       FourierFCN: "fourier"}


def fourier_feature_layer(omega):
    """FourierFCN's feature map as a first layer sin(W x + b) of the kernels:
    W = [omega; omega], b = [0; pi/2], i.e. [sin(omega x), cos(omega x)]
    (fbpinns/networks.py:186-188); omega (m, F, xd) -> (W (m, 2F, xd), b (m, 2F))."""
    omega = torch.as_tensor(omega, dtype=torch.float32)
    m, F = omega.shape[0], omega.shape[1]
    W = torch.cat([omega, omega], dim=1)
    b = torch.cat([torch.zeros((m, F)), torch.full((m, F), math.pi / 2)], dim=1).to(omega.device)
    return W, b


def engine_network(network, static, layers, layer_sizes):
    """The compiled kernels' view of a network: (layer sizes, activation,
    layers as packed tuples, leading engine layers that are not trainable).
    FourierFCN with layer_sizes [xd, h, 1] becomes [xd, 2F, h, 1] with the frozen
    feature layer first; FourierFCN with more hidden layers has no kernel."""
    if network not in NETWORK_ACTIVATIONS:
        raise NotImplementedError("the compiled jet kernels implement the FCN, SIREN, AdaptiveFCN, AdaptiveSIREN "
                                  "and FourierFCN networks")
    act = NETWORK_ACTIVATIONS[network]
    ls = list(layer_sizes)
    if network is FourierFCN:
        if len(ls) != 3:
            raise NotImplementedError("FourierFCN runs in the compiled kernels with one hidden layer after its "
                                      f"features (layer_sizes [xd, h, 1]), not {ls}")
        omega = static["omega"]
        feat = fourier_feature_layer(omega)
        return [ls[0], 2 * omega.shape[1]] + ls[1:], act, [feat] + list(layers), 1
    return ls, act, list(layers), 0


def norm(mu, sd, x):
    """fbpinns/networks.py:197-198."""
    return (x - mu) / sd


def unnorm(mu, sd, x):
    """fbpinns/networks.py:200-201."""
    return x * sd + mu


# ---------------------------------------------------------------------------
# packed parameter layout used by the CUDA kernels
# ---------------------------------------------------------------------------

def fcn_param_count(layer_sizes, extra=0):
    """P = sum over layers of fan_out * (fan_in + 1 + extra): W, b and
    ``extra`` per-neuron activation parameters (AdaptiveFCN 1, AdaptiveSIREN 2)."""
    return sum(fo * (fi + 1 + extra) for fi, fo in zip(layer_sizes[:-1], layer_sizes[1:]))


def pack_layers(layers):
    """[(W (m,fo,fi), b (m,fo), *params (m,fo)), ...] -> theta (m, P): per layer
    W row-major, b, then the activation parameters in tuple order."""
    m = layers[0][0].shape[0]
    return torch.cat([t.reshape(m, -1) for layer in layers for t in layer], dim=1).contiguous()


def unpack_layers(theta, layer_sizes, extra=0):
    """theta (m, P) -> [(W, b, *params), ...] as views into theta."""
    out, o = [], 0
    m = theta.shape[0]
    for fi, fo in zip(layer_sizes[:-1], layer_sizes[1:]):
        w = theta[:, o:o + fo * fi].view(m, fo, fi)
        o += fo * fi
        layer = [w]
        for _ in range(1 + extra):
            layer.append(theta[:, o:o + fo])
            o += fo
        out.append(tuple(layer))
    return out
