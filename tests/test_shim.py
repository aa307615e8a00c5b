"""The reference-side shim (swift_gb300/shim/runner_gb300.c) compiled against
the reference's own headers with the oracle recipe's build configuration,
linked with the reference's objects (oracle/build_ref.sh) and
libswiftgb300.so, and driven through the reference's runner symbols by
tests/shim/shim_driver.c.

Each replaced symbol must reach the library, and a failing library call must
come back through the reference's error() convention (error.h:60: message,
exit status 1).  Without a GPU the first GPU call of each symbol reports
SPHGPU_ENODEV; the rebuild hook, which plans on the host, succeeds.  The
reference's own hydro loop objects must not be linked in: the binary defines
the replaced symbols, and no other symbol of runner_doiact_hydro.o.

Needs the reference tree (SWIFT_REFERENCE_ROOT, or a `reference` directory
beside the repository) and the recipe's parity build under oracle/_ref/.
"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("SWIFT_REFERENCE_ROOT", os.path.join(ROOT, "..", "reference"))
OUT = os.path.join(ROOT, "oracle", "_ref", "parity")

SYMBOLS = ["runner_dosub_self1_density", "runner_dosub_pair1_density", "runner_do_ghost",
           "runner_dosub_self2_force", "runner_dosub_pair2_force",
           "runner_do_end_hydro_force", "runner_do_hydro_sort"]


def _gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    if not os.path.isdir(os.path.join(REF, "src")):
        pytest.skip("reference tree not present")
    if not os.path.exists(os.path.join(OUT, "libswiftref.a")):
        r = subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_ref.sh"), REF],
                           capture_output=True, text=True)
        if r.returncode != 0:
            pytest.skip("reference recipe did not build: " + r.stderr[-300:])
    from swift_gb300 import build
    lib = build.build()
    d = tmp_path_factory.mktemp("shim")
    cf = ["-std=gnu11", "-O2", "-fcommon", "-w", "-I" + os.path.join(OUT, "include"),
          "-I" + os.path.join(REF, "src"), "-I" + os.path.join(REF, "src", "lightcone"),
          "-include", "float.h", "-include", "swift.h", "-include", "mhd.h"]
    objs = []
    for src in (os.path.join(ROOT, "swift_gb300", "shim", "runner_gb300.c"),
                os.path.join(ROOT, "tests", "shim", "shim_driver.c")):
        o = str(d / (os.path.basename(src) + ".o"))
        subprocess.run(["gcc"] + cf + ["-c", src, "-o", o], check=True)
        objs.append(o)
    exe = str(d / "shim_driver")
    libdir = os.path.dirname(lib)
    subprocess.run(["gcc"] + objs + [os.path.join(OUT, "libswiftref.a"),
                                     os.path.join(OUT, "ref_stubs.o"),
                                     "-L" + libdir, "-lswiftgb300", "-Wl,-rpath," + libdir,
                                     "-lm", "-lpthread", "-Wl,--gc-sections", "-o", exe],
                   check=True)
    return exe


def _run(exe, call):
    return subprocess.run([exe, call], capture_output=True, text=True, timeout=120)


def test_replaced_symbols_come_from_the_shim(driver):
    nm = subprocess.run(["nm", driver], capture_output=True, text=True, check=True).stdout
    defined = {line.split()[-1] for line in nm.splitlines() if " T " in line}
    for sym in SYMBOLS + ["gb300_rebuild", "gb300_start_step", "gb300_fetch"]:
        assert sym in defined, sym
    # no other symbol of the reference's loop objects came along
    for sym in ("runner_doself1_branch_density", "runner_dopair1_branch_density",
                "runner_dosub_self_subset_density", "runner_do_extra_ghost"):
        assert sym not in defined, sym


def test_rebuild_plans_on_the_host(driver):
    r = _run(driver, "rebuild")
    assert r.returncode == 0, r.stderr
    assert "rebuild ok" in r.stdout and "returned" in r.stdout


@pytest.mark.parametrize("call", SYMBOLS + ["gb300_start_step"])
def test_each_symbol_reaches_the_library(driver, call):
    r = _run(driver, call)
    assert "rebuild ok" in r.stdout
    if _gpu():
        assert r.returncode == 0 and "returned" in r.stdout, r.stderr
    else:
        # SPHGPU_ENODEV through the reference's error(): message, exit(1)
        assert r.returncode == 1, (r.returncode, r.stderr)
        assert "returned" not in r.stdout
        assert "runner_gb300.c" in r.stderr and "no CUDA device" in r.stderr
        assert "code -6" in r.stderr


def test_fetch_before_any_step_is_an_error(driver):
    r = _run(driver, "gb300_fetch")
    assert r.returncode == 1 and "no step has run" in r.stderr


def test_task_below_the_top_level_is_refused(driver):
    r = _run(driver, "deep_cell")
    assert r.returncode == 1 and "below the top level" in r.stderr
