"""The C ABI without a GPU: the library loads, exports every symbol the
header declares, and its configuration parser agrees with the oracle's
restatement of lib/config.h on the reference's own example files."""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gbfwi.h")
GOLD = os.path.join(os.path.dirname(__file__), "golden", "checker_golden.npz")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(gb_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(pkg):
    lib = pkg.lib()
    names = declared_functions()
    assert len(names) > 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_exported_symbols_listed_by_nm(pkg):
    nm = shutil.which("nm")
    if not nm:
        pytest.skip("nm not available")
    out = subprocess.run([nm, "-D", "--defined-only", pkg.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (gb_[a-z0-9_]+)", out))
    assert set(declared_functions()) <= exported


def test_version_and_error_string(pkg):
    assert pkg.lib().gb_version() == 1
    assert isinstance(pkg.last_error(), str)


def write_example(tmp, orc, extra_ini=""):
    g = np.load(GOLD)
    d = os.path.join(tmp, "ex")
    os.makedirs(os.path.join(d, "model_true"))
    os.makedirs(os.path.join(d, "model_init"))
    keys = [str(k) for k in g["cfg_keys"]]
    with open(os.path.join(d, "config.ini"), "w") as fh:
        fh.write("[global]\n# a comment = 5\n")
        for k, v in zip(keys, g["cfg_vals"]):
            fh.write("%s = %r    # note\n" % (k, float(v)))
        fh.write(extra_ini)
    with open(os.path.join(d, "sources.dat"), "w") as fh:
        fh.write("# x | z | type | f0 | t0 | angle | amp\n")
        for s in g["src"]:
            fh.write(" ".join("%.6e" % v for v in s) + "\n")
        fh.write("1 2 3 4 5 6 7 \n")  # trailing blank: the reference skips it
        fh.write("1 2 3 4 5 6\n")  # six numbers: skipped
    with open(os.path.join(d, "stations.dat"), "w") as fh:
        fh.write("# x | z\n")
        for r in g["rec"]:
            fh.write("%.6e %.6e\n" % tuple(r))
    for c in ("x", "z", "vp", "vs", "rho"):
        orc.write_bin(os.path.join(d, "model_true", "proc000000_%s.bin" % c), g["true_" + c])
        orc.write_bin(os.path.join(d, "model_init", "proc000000_%s.bin" % c), g["init_" + c])
    return d


def test_config_parser_agrees_with_oracle(pkg, orc, tmp_path):
    d = write_example(str(tmp_path), orc, extra_ini="nt = 123\nbatch = 4\n")
    ref = orc.Config.load(d, overrides={"dt": "0.05"})
    c = pkg.Config.load(d, overrides={"dt": "0.05"})
    for k in ref.f:
        assert c.f(k) == pytest.approx(ref.f[k], rel=0, abs=0), k
        assert c.i(k) == ref.i[k], k
    assert c.f("dt") == np.float32(0.05)      # command line wins
    assert c.i("nt") == 5000                   # first definition in the file wins
    assert len(c.src) == len(ref.src) == 25    # the two malformed lines are skipped
    np.testing.assert_array_equal(np.array(c.src, np.float32), np.array(ref.src, np.float32))
    np.testing.assert_array_equal(np.array(c.rec, np.float32), np.array(ref.rec, np.float32))
    assert os.path.isdir(os.path.join(d, "output"))


def test_config_inherit_is_one_level(pkg, orc, tmp_path):
    base = tmp_path / "base.ini"
    base.write_text("nt = 10\ndt = 0.5\nsfe = 2\n")
    d = tmp_path / "child"
    d.mkdir()
    (d / "config.ini").write_text("inherit = %s\nnt = 20\n" % base)
    c = pkg.Config.load(str(d))
    ref = orc.Config.load(str(d))
    assert c.i("nt") == ref.i["nt"] == 20
    assert c.f("dt") == ref.f["dt"] == 0.5
    assert c.i("sfe") == 2 and not c.has("inherit")


def test_solver_calls_fail_loudly_without_gpu(pkg):
    if pkg.device_count() > 0:
        pytest.skip("a GPU is present")
    c = pkg.Config.new(".", {"nt": 10, "dt": 0.001, "sh": 1, "mode": 3})
    with pytest.raises(pkg.GbError):
        pkg.FdmSolver(c, grid=(10, 10, 90.0, 90.0))
