"""The allocation-free density pass (sphgpu_density_noalloc) against the
library's regular density pass, through the C ABI.

Callers that cannot allocate device memory when they run the pass -- hosts
that hand all device memory to their own pool, latency-bound serving loops --
use this entry point; its scratch is a static device array of fixed size.
The test allocates the output buffers itself (the entry point must not),
calls the entry point twice in a row (the second call must not see the first
call's counters), and checks each result
against the regular pass: neighbour counts exactly, positive sums at 1e-4
relative, cancelling sums at 1e-4 of the field's scale (the tolerances of
tests/test_gpu_parity.py).  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from swift_gb300 import api, ics

pytestmark = pytest.mark.gpu


def _scaled(a, b):
    return np.abs(a.astype(np.float64) - b) / (np.max(np.abs(b)) + 1e-30)


def test_density_noalloc_matches_regular_pass_twice():
    import torch
    box = ics.clustered(24, seed=11)
    with api.Space(box) as sp:
        sp.step(api.STAGE_DENSITY)
        ref = sp.download()
        n, L = sp.n, api.lib()
        for _ in range(2):
            out = torch.full((n, 8), float("nan"), device="cuda", dtype=torch.float32)
            ngb = torch.full((n,), -1, device="cuda", dtype=torch.int32)
            rc = L.sphgpu_density_noalloc(sp._h, ctypes.c_void_p(out.data_ptr()),
                                          ctypes.c_void_p(ngb.data_ptr()), None)
            assert rc == 0, L.sphgpu_last_error()
            torch.cuda.synchronize()
            o, g = out.cpu().numpy(), ngb.cpu().numpy()
            assert np.array_equal(g, ref["ngb_first"])
            for col in (0, 2):  # rho, wcount
                r = ref["fields"][:, col]
                assert np.max(np.abs(o[:, col] - r) / np.abs(r)) < 1e-4
            for col in (1, 3, 4, 5, 6, 7):
                assert _scaled(o[:, col], ref["fields"][:, col]).max() < 1e-4


def test_density_noalloc_rejects_oversized_space():
    import torch
    box = ics.lattice(104, seed=2)  # 1,124,864 particles > 2^20
    with api.Space(box) as sp:
        sp.step(api.STAGE_DENSITY)
        L = api.lib()
        out = torch.empty((1, 8), device="cuda", dtype=torch.float32)
        ngb = torch.empty((1,), device="cuda", dtype=torch.int32)
        rc = L.sphgpu_density_noalloc(sp._h, ctypes.c_void_p(out.data_ptr()),
                                      ctypes.c_void_p(ngb.data_ptr()), None)
        assert rc == api.EINVAL
        assert b"static scratch limit" in L.sphgpu_last_error()
