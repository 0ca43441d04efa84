"""The in-process binding (include/gbfwi_reference_shim.h) against the
reference's own classes.

GbSolver and GbFilter implement the virtual members of the reference's
Solver (solver/solver.h:158-267) and Filter (filter/filter.h:9-14) with
`override`, so compiling them together with the reference's headers checks
every signature, and linking the A/B driver (oracle/ab_main.cu: the
reference's mode-2 main with the solver and filter chosen by id) against
libgbfwi.so checks that every C-ABI call the shim makes is exported. Needs a
checkout of the reference sources: GBFWI_REF_SRC, or the one the oracle's
`make ref` recorded in oracle/_ref/refsrc; skipped without one.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE = os.path.join(ROOT, "oracle")


def reference_checkout():
    cand = os.environ.get("GBFWI_REF_SRC", "")
    rec = os.path.join(ORACLE, "_ref", "refsrc")
    if not cand and os.path.exists(rec):
        cand = open(rec).read().strip()
    return cand if cand and os.path.exists(os.path.join(cand, "lib", "index.h")) else None


def test_shim_compiles_against_reference_and_links_with_library(pkg):
    ref = reference_checkout()
    if ref is None:
        pytest.skip("no reference checkout (GBFWI_REF_SRC or oracle/_ref/refsrc)")
    if shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"):
        pytest.skip("nvcc not available")
    pkg.lib()  # libgbfwi.so is built
    r = subprocess.run(["make", "-s", "-B", "-C", ORACLE, "ab", "REFSRC=" + ref], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    exe = os.path.join(ORACLE, "_ref", "ab_harness")
    assert os.path.exists(exe)
    # the shim's overrides are in the binary and its C-ABI calls resolve in libgbfwi.so
    nm = subprocess.run(["nm", "-C", exe], capture_output=True, text=True).stdout
    for sym in ("GbSolver::runForward", "GbSolver::runAdjoint", "GbSolver::init", "GbFilter::apply"):
        assert sym in nm, sym
    for sym in ("gb_run_forward", "gb_run_adjoint", "gb_solver_ptr", "gb_filter_apply", "gb_config_load"):
        assert (" U " + sym) in nm, sym
    ldd = subprocess.run(["ldd", exe], capture_output=True, text=True).stdout
    assert "libgbfwi.so" in ldd and "not found" not in ldd.split("libgbfwi.so")[1].split("\n")[0]
    # without arguments it prints its usage and touches no device
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr
