"""Failure handling without faulting anything: forced non-convergence of the
ghost (one round, a tolerance nothing meets) must come back as a status, not
an abort -- in the oracle on the CPU and through the C ABI on the GPU."""
import numpy as np
import pytest

from swift_gb300 import api, ics


def test_oracle_reports_nonconvergence(oracle_lib):
    box = ics.lattice(12, seed=5)
    out = oracle_lib.run(box, max_iter=1, h_tolerance=1e-12)
    assert out["status"] == 1
    out = oracle_lib.run(box)
    assert out["status"] == 0


@pytest.mark.gpu
def test_gpu_reports_nonconvergence_and_recovers():
    box = ics.lattice(12, seed=5)
    with api.Space(box, max_iter=1, h_tolerance=1e-12) as sp:
        with pytest.raises(api.SphGpuError) as e:
            sp.step()
        assert e.value.code == api.ENOCONV
    with api.Space(box) as sp:  # the context stays usable
        sp.step()
        assert np.isfinite(sp.download()["h"]).all()
