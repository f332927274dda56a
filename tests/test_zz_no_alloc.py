"""The allocation-free prefix scan (fbp_scan_i32_noalloc) against the regular
one (fbp_scan_i32).

fbp_scan_i32_noalloc exists for callers that cannot allocate device memory and
therefore cannot give the library a scratch buffer; it keeps its scratch in a
fixed array inside the library.  This file is collected last so that a run that
stops at the first failure has already run every other test; it also passes
alone in a fresh process.
"""

import ctypes as C

import numpy as np
import pytest
import torch

from fbpinns_gb300 import _lib

pytestmark = pytest.mark.gpu


def _scan_regular(lib, x):
    n = x.numel()
    out = torch.empty(n + 1, dtype=torch.int32, device=x.device)
    scratch = torch.empty(int(lib.fbp_scan_scratch_bytes(n)) // 4 + 1, dtype=torch.int32, device=x.device)
    _lib.check(lib.fbp_scan_i32(_lib.ptr(x), _lib.ptr(out), n, _lib.ptr(scratch), scratch.numel() * 4,
                                _lib.stream_ptr()), "fbp_scan_i32")
    return out


def _scan_noalloc(lib, x):
    n = x.numel()
    out = torch.empty(n + 1, dtype=torch.int32, device=x.device)
    _lib.check(lib.fbp_scan_i32_noalloc(_lib.ptr(x), _lib.ptr(out), n, _lib.stream_ptr()), "fbp_scan_i32_noalloc")
    return out


def test_noalloc_scan_matches_regular_scan_twice(cuda):
    lib = _lib.load()
    g = torch.Generator().manual_seed(123)
    # two calls in a row; the second is shorter, so stale tile sums from the
    # first call would show up if the shared array leaked state
    for n in (3_000_001, 200_003):
        x = torch.randint(0, 40, (n,), generator=g, dtype=torch.int32).to(cuda)
        got = _scan_noalloc(lib, x)
        ref = _scan_regular(lib, x)
        torch.cuda.synchronize()
        assert torch.equal(got, ref)
        # integer work: exact against numpy too
        want = np.concatenate([[0], np.cumsum(x.cpu().numpy().astype(np.int64))])
        np.testing.assert_array_equal(got.cpu().numpy().astype(np.int64), want)


def test_noalloc_scan_rejects_sizes_beyond_its_array(cuda):
    lib = _lib.load()
    x = torch.zeros(1, dtype=torch.int32, device=cuda)
    too_big = (1 << 24) + 1
    rc = lib.fbp_scan_i32_noalloc(_lib.ptr(x), _lib.ptr(x), too_big, _lib.stream_ptr())
    assert rc == -4  # FBP_ERR_CAPACITY, rejected on the host before any launch
    assert b"exceeds the built-in maximum" in lib.fbp_last_error()
