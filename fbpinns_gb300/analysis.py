"""Loading saved models and running them (the reference's ``fbpinns/analysis.py``).

Model files are pickles of ``(i, all_params, all_opt_states, active,
u_test_losses)`` with numpy arrays, the layout the reference writes
(fbpinns/trainers.py:721, trainers_base.py:64-69), under
``results/models/<run>/model_XXXXXXXX.jax``; constants under
``results/summaries/<run>/constants_<run>.pickle``.
"""

import os
import pickle

import numpy as np
import torch


class DictToObj:
    """Attribute access to a dict of constants."""

    def __init__(self, **kw):
        self.__dict__.update(kw)


def load_model(run, i=None, rootdir="results/"):
    """(constants object, model tuple) of a saved run (fbpinns/analysis.py:18-46)."""
    model_dir = os.path.join(rootdir, "models", run)
    summary_dir = os.path.join(rootdir, "summaries", run)
    with open(os.path.join(summary_dir, f"constants_{run}.pickle"), "rb") as f:
        c = DictToObj(**pickle.load(f))
    if i is None:
        last = sorted(f for f in os.listdir(model_dir) if f.startswith("model_"))[-1]
        i = int(os.path.splitext(last)[0].split("_")[1])
    with open(os.path.join(model_dir, f"model_{i:08d}.jax"), "rb") as f:
        model = pickle.load(f)
    return c, model


def _torch_tree(d):
    if isinstance(d, dict):
        return {k: _torch_tree(v) for k, v in d.items()}
    if isinstance(d, (list, tuple)):
        return type(d)(_torch_tree(v) for v in d)
    if isinstance(d, np.ndarray) and d.dtype.kind == "f":
        return torch.as_tensor(d)
    return d


def FBPINN_solution(c, all_params, active, x_batch):
    """The FBPINN at points x_batch with all subdomains (fbpinns/analysis.py:49-55), on the GPU engine."""
    from .engine import FBPINNEngine, inference_d2mask
    from .networks import pack_layers, engine_network
    from .trainers import FBPINNTrainer
    ap = _torch_tree(all_params)
    layers = [tuple(torch.as_tensor(t) for t in layer) for layer in ap["trainable"]["network"]["subdomain"]["layers"]]
    static = ap["static"].get("network", {}).get("subdomain", {})
    in_dim = static["omega"].shape[2] if "omega" in static else layers[0][0].shape[2]
    sizes = [in_dim] + [layer[0].shape[1] for layer in layers]
    sizes, act, layers, _ = engine_network(c.network, static, layers, sizes)
    eng = FBPINNEngine(ap["static"]["decomposition"], sizes, inference_d2mask(sizes, act), activation=act)
    eng.set_theta(pack_layers(layers))
    dev = eng.device
    ap["static"]["problem"] = {k: (v.to(dev) if torch.is_tensor(v) else v) for k, v in ap["static"]["problem"].items()}
    return FBPINNTrainer.predict(eng, ap, c.problem, torch.as_tensor(x_batch, dtype=torch.float32))
