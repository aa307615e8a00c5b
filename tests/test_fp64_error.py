"""Errors against an FP64 brute force (oracle/sph_oracle.c,
sph_oracle_exact64: double-precision sums over every minimum-image pair
within gamma*h, at the state the tested code converged to).  The reference's
own FP32 loops (through the bit-identical oracle) and the GPU path are both
held to the same bounds, and their errors are printed side by side (run with
-s to see them)."""
import numpy as np
import pytest

from swift_gb300 import ics

CASES = ["lattice:16", "clustered:20", "clustered:32"]
RHO_BOUND = 1e-5        # relative, per particle
SCALED_BOUND = 5e-5     # of the field's largest magnitude (cancelling sums)


def fp64_errors(box, out, oracle_lib):
    ex = oracle_lib.exact64(box, out)
    err = {"rho": float(np.max(np.abs(out["rho"] - ex[:, 0]) / ex[:, 0]))}
    for k, c in (("ax", 3), ("ay", 4), ("az", 5), ("u_dt", 6)):
        err[k] = float(np.max(np.abs(out[k] - ex[:, c])) / (np.max(np.abs(ex[:, c])) + 1e-300))
    return err


def check(err):
    assert err["rho"] < RHO_BOUND, err
    for k in ("ax", "ay", "az", "u_dt"):
        assert err[k] < SCALED_BOUND, err


@pytest.mark.parametrize("cfg", CASES)
def test_reference_loops_against_fp64(cfg, oracle_lib):
    box = ics.make(cfg, seed=7)
    err = fp64_errors(box, oracle_lib.run(box), oracle_lib)
    print(f"\n{cfg} reference loops (FP32) vs FP64:", {k: f"{v:.2e}" for k, v in err.items()})
    check(err)


@pytest.mark.gpu
@pytest.mark.parametrize("cfg", CASES)
def test_gpu_against_fp64(cfg, oracle_lib):
    from swift_gb300 import api
    box = ics.make(cfg, seed=7)
    with api.Space(box) as sp:
        sp.step()
        out = sp.download()
    err = fp64_errors(box, out, oracle_lib)
    ref = fp64_errors(box, oracle_lib.run(box), oracle_lib)
    print(f"\n{cfg} GPU vs FP64:", {k: f"{v:.2e}" for k, v in err.items()},
          " reference loops vs FP64:", {k: f"{v:.2e}" for k, v in ref.items()})
    check(err)
