"""The C ABI library: it loads without a GPU, exports every function the
header declares, validates its arguments and reports errors through codes
(it never aborts the process)."""
import ctypes
import os
import re

import numpy as np
import pytest

from swift_gb300 import api, ics

HEADER = os.path.join(os.path.dirname(os.path.dirname(__file__)), "include",
                      "swift_gb300.h")


def header_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(sphgpu_\w+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    L = api.lib()
    names = header_functions()
    assert len(names) >= 20
    for name in names:
        assert hasattr(L, name), name
        assert name in api.SIGNATURES, f"{name} has no ctypes signature"


def test_abi_version_and_defaults():
    L = api.lib()
    assert L.sphgpu_abi_version() == 2
    p = api.Params()
    L.sphgpu_default_params(ctypes.byref(p))
    assert abs(p.eta - 1.2348) < 1e-6 and p.max_iter == 30
    assert p.max_top_level_cells == 12 and abs(p.h_tolerance - 1e-4) < 1e-9


def test_invalid_arguments_are_rejected():
    box = ics.lattice(8, seed=1)
    with pytest.raises(api.SphGpuError) as e:
        api.Space(box, max_iter=0)
    assert e.value.code == api.EINVAL
    bad = dict(box)
    bad["h"] = box["h"].copy()
    bad["h"][3] = -1.0
    with pytest.raises(api.SphGpuError) as e:
        api.Space(bad)
    assert "smoothing lengths" in str(e.value)
    bad = dict(box)
    bad["x"] = box["x"].copy()
    bad["x"][0, 0] = np.nan
    with pytest.raises(api.SphGpuError):
        api.Space(bad)
    L = api.lib()
    assert L.sphgpu_step(None, 7, None) == api.EINVAL


def test_particle_count_ceiling():
    """Partner indices are packed in 27 bits: larger spaces are refused
    before any array is read."""
    import ctypes
    L = api.lib()
    p = api.Params()
    L.sphgpu_default_params(ctypes.byref(p))
    dummy = np.zeros(8)
    h = ctypes.c_void_p()
    rc = L.sphgpu_space_create(ctypes.byref(p), 1 << 27, *([dummy.ctypes.data] * 6),
                               ctypes.byref(h))
    assert rc == api.EINVAL
    assert b"27 bits" in L.sphgpu_last_error()


def test_tiny_box_needs_three_cells_per_axis():
    box = ics.lattice(4, seed=1)   # h ~ box/3: fewer than 3 top cells
    with pytest.raises(api.SphGpuError):
        api.Space(box)


def test_gpu_call_without_gpu_reports_enodev():
    from conftest import gpu_available
    if gpu_available():
        pytest.skip("a GPU is present")
    box = ics.lattice(12, seed=1)
    with api.Space(box) as sp:
        with pytest.raises(api.SphGpuError) as e:
            sp.step()
        assert e.value.code in (api.ENODEV, api.ECUDA)
        # tree queries still work
        assert sp.info()["n"] == 12 ** 3
