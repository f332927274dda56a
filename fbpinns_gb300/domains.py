"""Problem domains (the reference's ``fbpinns/domains.py`` API).

``key`` arguments are an int seed or a ``torch.Generator`` (the reference takes
a JAX PRNG key).  Points are float32, like the reference's default dtype.
"""

import numpy as np
import scipy.stats
import torch

from . import networks


def _gen(key):
    if isinstance(key, torch.Generator):
        return key
    g = torch.Generator()
    g.manual_seed(0 if key is None else int(key))
    return g


class Domain:
    """Base class (fbpinns/domains.py:18-55)."""

    @staticmethod
    def init_params(*args):
        raise NotImplementedError

    @staticmethod
    def sample_interior(all_params, key, sampler, batch_shape):
        raise NotImplementedError

    @staticmethod
    def sample_boundaries(all_params, key, sampler, batch_shapes):
        raise NotImplementedError

    @staticmethod
    def norm_fn(all_params, x):
        raise NotImplementedError


class RectangularDomainND(Domain):
    """Axis-aligned box [xmin, xmax] (fbpinns/domains.py:60-142)."""

    @staticmethod
    def init_params(xmin, xmax):
        xmin, xmax = np.asarray(xmin, dtype=np.float64), np.asarray(xmax, dtype=np.float64)
        assert xmin.shape == xmax.shape and xmin.ndim == 1
        return {"xd": len(xmin), "xmin": torch.as_tensor(xmin, dtype=torch.float32),
                "xmax": torch.as_tensor(xmax, dtype=torch.float32)}, {}

    @staticmethod
    def sample_interior(all_params, key, sampler, batch_shape):
        d = all_params["static"]["domain"]
        return RectangularDomainND._rectangle_samplerND(key, sampler, d["xmin"], d["xmax"], batch_shape)

    @staticmethod
    def sample_boundaries(all_params, key, sampler, batch_shapes):
        """Points on each of the 2*xd faces, in the order (dim 0 min, dim 0 max, dim 1 min, ...)."""
        d = all_params["static"]["domain"]
        xmin, xmax, xd = d["xmin"], d["xmax"], d["xd"]
        assert len(batch_shapes) == 2 * xd
        g = _gen(key)
        out = []
        for i in range(xd):
            ic = [k for k in range(xd) if k != i]
            for j, v in enumerate([xmin[i], xmax[i]]):
                bs = batch_shapes[2 * i + j]
                if ic:
                    xb_ = RectangularDomainND._rectangle_samplerND(g, sampler, xmin[ic], xmax[ic], bs)
                    xb = torch.full((xb_.shape[0], xd), float(v), dtype=torch.float32)
                    xb[:, ic] = xb_
                else:
                    assert len(bs) == 1
                    xb = torch.full(tuple(bs) + (1,), float(v), dtype=torch.float32)
                out.append(xb)
        return out

    @staticmethod
    def norm_fn(all_params, x):
        d = all_params["static"]["domain"]
        return networks.norm((d["xmax"] + d["xmin"]) / 2, (d["xmax"] - d["xmin"]) / 2, x)

    @staticmethod
    def _rectangle_samplerND(key, sampler, xmin, xmax, batch_shape):
        """Flattened grid (ij order, last dim fastest) or random samples in a box."""
        xmin = torch.as_tensor(xmin, dtype=torch.float32).reshape(-1)
        xmax = torch.as_tensor(xmax, dtype=torch.float32).reshape(-1)
        xd = xmin.numel()
        assert len(batch_shape) == xd
        if sampler not in ("grid", "uniform", "sobol", "halton"):
            raise ValueError("ERROR: unexpected sampler")
        n = int(np.prod(batch_shape))
        if sampler == "grid":
            axes = [torch.linspace(float(a), float(b), int(k), dtype=torch.float64)
                    for a, b, k in zip(xmin.tolist(), xmax.tolist(), batch_shape)]
            xx = torch.stack(torch.meshgrid(*axes, indexing="ij"), -1).reshape(-1, xd)
            return xx.float()
        if sampler == "uniform":
            s = torch.rand((n, xd), generator=_gen(key), dtype=torch.float32)
        elif sampler == "halton":
            s = torch.as_tensor(scipy.stats.qmc.Halton(xd).random(n), dtype=torch.float32)
        else:
            s = torch.as_tensor(scipy.stats.qmc.Sobol(xd).random(n), dtype=torch.float32)
        return xmin.reshape(1, -1) + (xmax - xmin).reshape(1, -1) * s
