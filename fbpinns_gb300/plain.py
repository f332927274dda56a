"""Plain GPU drop-in step: the baseline of the fused engine.

Same point sampling, interaction lists and subdomain-major order as the fused
step (the same CUDA kernels), but the model is expressed in torch: the pairs
of each group of subdomains (one group per POU level) are padded into a
(G, max_count, xd) batch, the FCN runs as batched matmuls, the derivative jets
come from torch's own double backward with respect to the input points, the
POU combination is an index_add, and the gradient is torch autograd.  Adam is
the same masked kernel.  This is what a direct GPU port of the reference step
(fbpinns/trainers.py:126-177, 213-247, 285-296) looks like in PyTorch.
"""


import numpy as np
import torch

from . import windows
from .decompositions import WINDOWS as _WINDOWS
from .engine import constrained_jets, jet_index
from .networks import unpack_layers


class PlainStep:
    def __init__(self, engine, problem, all_params, required_ujs, opt, x=None, resample=None, headroom=1.25):
        self.eng, self.problem, self.all_params, self.opt = engine, problem, all_params, opt
        self.required = required_ujs
        self.resample = resample
        g = engine.grid
        self.pou = g.pou.long()
        levels = torch.unique(self.pou).tolist()
        self.groups = [torch.nonzero(self.pou == lv).reshape(-1) for lv in levels]
        if resample is not None:
            n, xmin, xmax, seed = resample
            self.xmin, self.xmax, self.seed = list(xmin), list(xmax), int(seed)
            x0 = torch.empty((n, engine.xd), dtype=torch.float32, device=engine.device)
            engine.sample(x0, self.seed, 1 << 32, self.xmin, self.xmax)
            probe = engine.points(x0)
            caps = (int(probe.s * headroom) + 1024, int(probe.u * headroom) + 1024)
            del probe
            self.ps = engine.points(x0, caps=caps)
        else:
            self.ps = engine.points(torch.as_tensor(x, dtype=torch.float32).to(engine.device))

    def _pair_jets(self, theta, ids, start, counts, maxc):
        """Per-pair jets (uw, w) of the subdomains ``ids`` by double backward."""
        eng, ps = self.eng, self.ps
        g = eng.grid
        G = ids.numel()
        ar = torch.arange(maxc, device=eng.device)
        valid = ar[None, :] < counts[:, None]
        pos = torch.where(valid, start[:, None] + ar[None, :], start[:, None].clamp(max=max(ps.s_cap - 1, 0)))
        pos = pos.clamp(0, max(ps.s_cap - 1, 0))
        point = ps.sd_point[pos].long()
        slot = ps.sd_slot[pos].long()
        xg = ps.x[point].detach().requires_grad_(True)
        lo, hi = g.xmins[ids][:, None, :], g.xmaxs[ids][:, None, :]
        mu, sd = (hi + lo) / 2, (hi - lo) / 2
        xn = (xg - mu) / sd
        rows = theta[ids]
        layers = unpack_layers(rows, eng.layer_sizes, eng.extra)
        h = xn
        for li, layer in enumerate(layers[:-1]):
            z = torch.baddbmm(layer[1][:, None, :], h, layer[0].transpose(1, 2))
            if eng.activation == "fourier":  # the frozen feature layer, then tanh
                h = torch.sin(z) if li == 0 else torch.tanh(z)
            elif eng.activation == "tanh":
                h = torch.tanh(z)
            elif eng.activation == "sin":
                h = torch.sin(z)
            elif eng.activation == "adaptive_tanh":  # a tanh(z / a)
                a = layer[2][:, None, :]
                h = a * torch.tanh(z / a)
            else:  # c sin(o z)
                h = layer[2][:, None, :] * torch.sin(layer[3][:, None, :] * z)
        w, b = layers[-1][:2]
        u = torch.baddbmm(b[:, None, :], h, w.transpose(1, 2))
        un = g.unnorms[ids]
        u = u * un[:, None, 1:2] + un[:, None, 0:1]
        flag = g.flags[ids][:, None, None]
        wname = _WINDOWS[g.window]
        if wname == "sigmoid":
            win = windows.sigmoid(lo, hi, g.wmins[ids][:, None, :], g.wmaxs[ids][:, None, :], xg)
        else:
            win = getattr(windows, wname)(lo, hi, xg)
        win = flag * win + (1 - flag)
        f = u * win
        xd, d2 = eng.xd, eng.d2mask
        J = eng.J
        uw = [f]
        ww = [win]
        gf = torch.autograd.grad(f.sum(), xg, create_graph=True)[0]
        gw = torch.autograd.grad(win.sum(), xg, create_graph=True)[0]
        uw += [gf[..., d:d + 1] for d in range(xd)]
        ww += [gw[..., d:d + 1] for d in range(xd)]
        for d in range(xd):
            if (d2 >> d) & 1:
                uw.append(torch.autograd.grad(gf[..., d].sum(), xg, create_graph=True)[0][..., d:d + 1])
                ww.append(torch.autograd.grad(gw[..., d].sum(), xg, retain_graph=True)[0][..., d:d + 1])
        m = valid[..., None].to(f.dtype)
        UW = torch.cat(uw, -1) * m
        WW = torch.cat(ww, -1).detach() * m
        return UW.reshape(-1, J), WW.reshape(-1, J), slot.reshape(-1)

    def loss(self, theta):
        eng, ps = self.eng, self.ps
        J, xd, d2 = eng.J, eng.xd, eng.d2mask
        sd_start = ps.sd_start.long()
        counts_all = (sd_start[1:] - sd_start[:-1])
        # one host read per step: the slot count, the lists' status word and
        # each group's largest pair count (the padded batch shapes)
        head = torch.stack([ps.takes.np_off[ps.n].long(), ps.takes.status[0].long()] +
                           [counts_all[ids].max() for ids in self.groups]).tolist()
        u_total, status, maxcs = head[0], head[1], head[2:]
        if status:
            ps.check_status()  # raises: a fixed-capacity list overflowed
        N = torch.zeros((u_total, J), dtype=torch.float32, device=eng.device)
        Wn = torch.zeros((u_total, J), dtype=torch.float32, device=eng.device)
        for ids, maxc in zip(self.groups, maxcs):
            counts = counts_all[ids]
            if maxc == 0:
                continue
            UW, WW, slot = self._pair_jets(theta, ids, sd_start[ids], counts, maxc)
            N = N.index_add(0, slot, UW)
            Wn = Wn.index_add(0, slot, WW)
        # quotient-rule POU per (point, level), then the level sum / npou
        r = 1.0 / Wn[:, 0:1]
        U0 = N[:, 0:1] * r
        comps = [U0]
        Ud = [(N[:, 1 + d:2 + d] - U0 * Wn[:, 1 + d:2 + d]) * r for d in range(xd)]
        comps += Ud
        for d in range(xd):
            if (d2 >> d) & 1:
                k = jet_index(xd, d2, (d, d))
                comps.append((N[:, k:k + 1] - 2 * Ud[d] * Wn[:, 1 + d:2 + d] - U0 * Wn[:, k:k + 1]) * r)
        Ul = torch.cat(comps, 1)
        np_take = ps.takes.np_take[:u_total].long()
        U = torch.zeros((ps.n, J), dtype=torch.float32, device=eng.device).index_add(0, np_take, Ul) / eng.npou
        Uc = constrained_jets(self.problem.constraining_fn, self.all_params, ps.x, U, xd, d2)
        ujs = [Uc[:, jet_index(xd, d2, ixs):jet_index(xd, d2, ixs) + 1] for _, ixs in self.required]
        return self.problem.loss_fn(self.all_params, [[ps.x] + ujs])

    def step(self):
        eng, o = self.eng, self.opt
        if self.resample is not None:
            eng.sample(self.ps.x, self.seed, 0, self.xmin, self.xmax, counter=eng.count)
            self.ps.rebuild()
        theta = eng.theta.detach().clone().requires_grad_(True)
        loss = self.loss(theta)
        (g,) = torch.autograd.grad(loss, [theta])
        eng.adam(o["learning_rate"], o["b1"], o["b2"], o["eps"], o["eps_root"], grad=g.contiguous())
        return loss.detach()

    def check(self):
        """Raise if the interaction lists of this step overflowed their fixed
        capacities (the sticky status word of the point set)."""
        self.ps.check_status()
