"""Active-subdomain schedulers (the reference's ``fbpinns/schedulers.py`` API).

Each scheduler is an iterable of length n_steps that yields, per training
step, either ``None`` (mask unchanged) or an int array of length m with
0 = inactive (still trained if it overlaps active ones), 1 = active,
2 = fixed.  Host-side numpy; the engine turns each mask change into device
masks without recompiling anything.
"""

import numpy as np


class ActiveScheduler:
    """Base class (fbpinns/schedulers.py:16-38)."""

    def __init__(self, all_params, n_steps):
        self.n_steps = n_steps
        self.m = all_params["static"]["decomposition"]["m"]
        self.xd = all_params["static"]["decomposition"]["xd"]

    def __len__(self):
        return self.n_steps

    def __iter__(self):
        raise NotImplementedError


class AllActiveSchedulerND(ActiveScheduler):
    """Every subdomain active from the first step (fbpinns/schedulers.py:41-49)."""

    def __iter__(self):
        for i in range(self.n_steps):
            yield np.ones(self.m, dtype=int) if i == 0 else None


class _SubspacePointSchedulerRectangularND(ActiveScheduler):
    """A radius grows linearly over the steps from a point of the constrained
    axes; a subdomain becomes active while the radius lies between its
    nearest and farthest distance to that point, and fixed afterwards
    (fbpinns/schedulers.py:52-135).  Distances use the centre lines of the
    overlap regions (``xmins0``/``xmaxs0``) restricted to the constrained axes.
    """

    def __init__(self, all_params, n_steps, point, iaxes):
        super().__init__(all_params, n_steps)
        point = np.array(point)
        iaxes = list(iaxes)
        if point.ndim != 1:
            raise Exception("ERROR: point.ndim != 1")
        if len(point) > self.xd:
            raise Exception("ERROR: len(point) > self.xd")
        if len(iaxes) + len(point) != self.xd:
            raise Exception("ERROR: len(iaxes) + len(point) != self.xd")
        self.point = point
        self.iaxes = iaxes
        self.xmins0 = np.array(all_params["static"]["decomposition"]["xmins0"], dtype=np.float64)
        self.xmaxs0 = np.array(all_params["static"]["decomposition"]["xmaxs0"], dtype=np.float64)

    @staticmethod
    def _get_radii(point, xmins, xmaxs):
        """(rmin, rmax): distance from ``point`` to each box and to its farthest corner."""
        assert xmins.shape[1] == xmaxs.shape[1] == point.shape[0]
        p = point[None, :]
        near = np.clip(p, xmins, xmaxs)
        lo_off, hi_off = p - xmins, p - xmaxs
        far = p - np.where(np.abs(lo_off) >= np.abs(hi_off), lo_off, hi_off)
        rmin = np.sqrt(np.sum((near - p) ** 2, axis=1))
        rmax = np.sqrt(np.sum((far - p) ** 2, axis=1))
        inside = np.all((p >= xmins) & (p <= xmaxs), axis=1)
        rmin[inside] = 0.0
        return rmin, rmax

    def __iter__(self):
        ic = [i for i in range(self.xd) if i not in self.iaxes]
        rmin, rmax = self._get_radii(self.point, self.xmins0[:, ic], self.xmaxs0[:, ic])
        r_lo, r_hi = rmin.min(), rmax.max()
        state = np.zeros(self.m, dtype=int)
        for i in range(self.n_steps):
            rt = r_lo + (r_hi - r_lo) * (i / self.n_steps)
            in_band = (rt >= rmin) & (rt < rmax)
            to_active = (state == 0) & in_band
            to_fixed = (state == 1) & ~in_band
            if to_active.any() or to_fixed.any():
                state[to_active] = 1
                state[to_fixed] = 2
                yield state
            else:
                yield None


class PointSchedulerRectangularND(_SubspacePointSchedulerRectangularND):
    """Expands from a point of the domain (fbpinns/schedulers.py:137-143)."""

    def __init__(self, all_params, n_steps, point):
        xd = all_params["static"]["decomposition"]["xd"]
        if len(point) != xd:
            raise Exception(f"ERROR: point incorrect shape {np.shape(point)}")
        super().__init__(all_params, n_steps, point, iaxes=[])


class LineSchedulerRectangularND(_SubspacePointSchedulerRectangularND):
    """Expands from a line along axis ``iaxis`` (fbpinns/schedulers.py:145-152)."""

    def __init__(self, all_params, n_steps, point, iaxis):
        xd = all_params["static"]["decomposition"]["xd"]
        if xd < 2:
            raise Exception("ERROR: requires nd >=2")
        if len(point) != xd - 1:
            raise Exception(f"ERROR: point incorrect shape {np.shape(point)}")
        super().__init__(all_params, n_steps, point, iaxes=[iaxis])


class PlaneSchedulerRectangularND(_SubspacePointSchedulerRectangularND):
    """Expands from a plane spanned by ``iaxes`` (fbpinns/schedulers.py:154-160)."""

    def __init__(self, all_params, n_steps, point, iaxes):
        xd = all_params["static"]["decomposition"]["xd"]
        if xd < 3:
            raise Exception("ERROR: requires nd >=3")
        if len(point) != xd - 2:
            raise Exception(f"ERROR: point incorrect shape {np.shape(point)}")
        super().__init__(all_params, n_steps, point, iaxes=iaxes)
