"""ctypes binding of ``cstep.c``: the C restatement of one reference training
step of the 2D multilevel Poisson workload on the host cores.

TEST AND BENCHMARK INFRASTRUCTURE ONLY (see ``oracle/__init__.py``): the CPU
baseline of ``bench.py`` (its reference arm) and a CPU test against the
float64 torch oracle.  ``build()`` compiles ``liboraclestep.so`` next to this
file with the host C compiler (no CUDA).
"""

import ctypes as C
import os
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cstep.c")
LIB = os.path.join(HERE, "_build", "liboraclestep.so")


def build(force=False):
    """Compile the C restatement (gcc -O3, pthreads); returns the library path."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC),
                                                                            os.path.getmtime(__file__)):
        return LIB
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("no C compiler for the oracle's C restatement")
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    tmp = LIB + ".tmp"
    r = subprocess.run([cc, "-O3", "-std=gnu11", "-shared", "-fPIC", "-pthread", SRC, "-o", tmp, "-lm"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"building {SRC} failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


class _Problem(C.Structure):
    _fields_ = [("m", C.c_int), ("h", C.c_int), ("npou", C.c_int),
                ("xmins", C.c_void_p), ("xmaxs", C.c_void_p), ("flags", C.c_void_p), ("unnorms", C.c_void_p),
                ("pou", C.c_void_p), ("sd", C.c_float), ("n_freq", C.c_int)]


_lib = None


def load():
    global _lib
    if _lib is None:
        lib = C.CDLL(build())
        lib.cs_loss_grad.restype = C.c_int
        lib.cs_loss_grad.argtypes = [C.POINTER(_Problem), C.c_void_p, C.c_void_p, C.c_int64, C.c_int,
                                     C.POINTER(C.c_double), C.c_void_p, C.c_void_p, C.POINTER(C.c_int64)]
        lib.cs_step.restype = C.c_int
        lib.cs_step.argtypes = [C.POINTER(_Problem), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                C.c_void_p, C.c_int64, C.c_float, C.c_int, C.POINTER(C.c_double), C.c_void_p,
                                C.POINTER(C.c_int64)]
        lib.cs_n_params.restype = C.c_int
        lib.cs_n_params.argtypes = [C.c_int]
        _lib = lib
    return _lib


def _ptr(a):
    return C.c_void_p(a.ctypes.data)


class PoissonStep:
    """The reference step of the Poisson workload on ``threads`` host threads.

    ``params``: the decomposition's [xmins, xmaxs, wmins, wmaxs, flags,
    unnorms] (m rows each) and ``pou`` (m); ``theta`` (m, P) float32 in the
    layout W1 b1 W2 b2 W3 b3 per subdomain; ``sd`` and ``n_freq`` of the
    Poisson problem.  Arrays are kept as contiguous float32 / int32 copies."""

    def __init__(self, params, pou, theta, hidden, sd=0.1, n_freq=6, threads=1, lr=1e-3):
        lib = load()
        f32 = lambda a: np.ascontiguousarray(np.asarray(a, dtype=np.float32))
        self.xmins, self.xmaxs = f32(params[0]), f32(params[1])
        self.flags = f32(np.asarray(params[4]).reshape(-1))
        self.unnorms = f32(params[5])
        self.pou = np.ascontiguousarray(np.asarray(pou).reshape(-1).astype(np.int32))
        m = self.xmins.shape[0]
        self.P = lib.cs_n_params(hidden)
        self.theta = f32(theta).reshape(m, self.P).copy()
        self.m1 = np.zeros_like(self.theta)
        self.m2 = np.zeros_like(self.theta)
        self.grad = np.zeros_like(self.theta)
        self.count = np.zeros(1, dtype=np.int32)
        self.pb = _Problem(m, hidden, int(self.pou.max()) + 1, _ptr(self.xmins).value, _ptr(self.xmaxs).value,
                           _ptr(self.flags).value, _ptr(self.unnorms).value, _ptr(self.pou).value, sd, n_freq)
        self.threads, self.lr = int(threads), float(lr)
        self.times = np.zeros(5)
        self.pairs = 0

    def loss_grad(self, x):
        """(loss, grad (m, P)) at points x (n, 2) with the current theta."""
        x = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
        loss, s = C.c_double(), C.c_int64()
        rc = load().cs_loss_grad(C.byref(self.pb), _ptr(self.theta), _ptr(x), x.shape[0], self.threads,
                                 C.byref(loss), _ptr(self.grad), _ptr(self.times), C.byref(s))
        if rc:
            raise RuntimeError(f"cs_loss_grad failed ({rc})")
        self.pairs = s.value
        return loss.value, self.grad.copy()

    def step(self, x):
        """One training step (lists, forward, loss, gradient, Adam); returns the loss."""
        x = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
        loss, s = C.c_double(), C.c_int64()
        rc = load().cs_step(C.byref(self.pb), _ptr(self.theta), _ptr(self.m1), _ptr(self.m2), _ptr(self.grad),
                            _ptr(self.count), _ptr(x), x.shape[0], self.lr, self.threads, C.byref(loss),
                            _ptr(self.times), C.byref(s))
        if rc:
            raise RuntimeError(f"cs_step failed ({rc})")
        self.pairs = s.value
        return loss.value
