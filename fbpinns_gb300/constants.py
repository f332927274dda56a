"""Run configuration (the reference's ``fbpinns/constants.py`` API).

``Constants`` keeps the reference's keys and defaults (fbpinns/constants.py:27-97)
and its key-checked ``__setitem__`` (fbpinns/constants_base.py:12-20); engine
keys are added at the end.
"""

import os
import pickle
import socket

import numpy as np

from . import domains, problems, decompositions, networks, schedulers, optim


def get_subdomain_ws(subdomain_xs, width):
    """Widths = width x the minimum centre spacing, per dim (fbpinns/constants.py:21-22)."""
    return [width * np.min(np.diff(x)) * np.ones_like(x) for x in subdomain_xs]


class ConstantsBase:
    """Attribute bag whose item access is restricted to existing keys."""

    def __getitem__(self, key):
        if key not in vars(self):
            raise KeyError(f'key "{key}" not defined in class')
        return getattr(self, key)

    def __setitem__(self, key, item):
        if key not in vars(self):
            raise KeyError(f'key "{key}" not defined in class')
        setattr(self, key, item)

    def __str__(self):
        s = repr(self) + "\n"
        for k in vars(self):
            s += f"{k}: {self[k]}\n"
        return s

    @property
    def summary_out_dir(self):
        return f"results/summaries/{self.run}/"

    @property
    def model_out_dir(self):
        return f"results/models/{self.run}/"

    def get_outdirs(self):
        for d in (self.summary_out_dir, self.model_out_dir):
            os.makedirs(d, exist_ok=True)
            for f in os.listdir(d):
                p = os.path.join(d, f)
                if os.path.isfile(p):
                    os.remove(p)

    def save_constants_file(self):
        with open(self.summary_out_dir + f"constants_{self.run}.txt", "w") as f:
            for k in vars(self):
                f.write(f"{k}: {self[k]}\n")
        with open(self.summary_out_dir + f"constants_{self.run}.pickle", "wb") as f:
            pickle.dump(vars(self), f)

    @property
    def constants_file(self):
        return self.summary_out_dir + f"constants_{self.run}.pickle"


class Constants(ConstantsBase):

    def __init__(self, **kwargs):
        self.run = "test"
        self.domain = domains.RectangularDomainND
        self.domain_init_kwargs = dict(xmin=np.array([0.]), xmax=np.array([1.]))
        self.problem = problems.HarmonicOscillator1D
        self.problem_init_kwargs = dict(d=2, w0=20)
        subdomain_xs = [np.linspace(0, 1, 5)]
        self.decomposition = decompositions.RectangularDecompositionND
        self.decomposition_init_kwargs = dict(subdomain_xs=subdomain_xs,
                                              subdomain_ws=get_subdomain_ws(subdomain_xs, 2.99),
                                              unnorm=(0., 1.))
        self.network = networks.FCN
        self.network_init_kwargs = dict(layer_sizes=[1, 32, 1])
        self.n_steps = 15000
        self.scheduler = schedulers.AllActiveSchedulerND
        self.scheduler_kwargs = dict()
        self.ns = ((60,),)
        self.n_test = (200,)
        self.sampler = "grid"
        self.optimiser = optim.adam
        self.optimiser_kwargs = dict(learning_rate=1e-3)
        self.seed = 0
        self.summary_freq = 1000
        self.test_freq = 1000
        self.model_save_freq = 10000
        self.show_figures = True
        self.save_figures = False
        self.clear_output = False
        self.hostname = socket.gethostname().lower()
        # engine keys
        self.engine = "fused"          # "fused" (CUDA adjoint + fused loss) or "plain" (torch autograd)
        self.resample = False          # redraw uniform collocation points every step on the device
        self.device = "cuda"
        self.chunk = 1024              # pairs per adjoint work item
        self.forward_chunk = None      # pairs per forward work item (None: 4 x chunk)
        self.autotune = True           # measure the work-item sizes on the first batch (fused step)
        self.launch_grid = 0           # CTAs of the persistent jet kernels (0 = 4 per SM)
        self.use_graph = True          # capture the step in a CUDA graph
        self.tensor_cores = None       # forward jets on tcgen05 (3xTF32): None = where compiled, True, False
        self.store_z2 = None           # forward stores the layer-2 z-jets for the adjoint: None = hidden >= 32
        self.pair_headroom = 1.25      # pair-buffer capacity factor for resampled steps
        self.device_schedule = True    # fused step: follow scheduler changes on the device (no re-capture)
        self.save_models = False       # write model pickles at model_save_freq
        for key in kwargs:
            self[key] = kwargs[key]
