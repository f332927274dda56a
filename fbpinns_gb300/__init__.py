"""fbpinns_gb300: a GB300-native FBPINN training engine.

The reference library's API (benmoseley/FBPINNs, fbpinns v0.2.0) is kept —
domains, problems, decompositions, networks, schedulers, constants and the
FBPINN trainer — and the training step runs as hand-written sm_103a CUDA
kernels behind the C ABI of include/fbpgpu.h (libfbpgpu.so, loaded with
ctypes).  There is no CPU or PyTorch fallback for the step.
"""

__version__ = "0.1.0"
