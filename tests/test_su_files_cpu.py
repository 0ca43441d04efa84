"""The library's host-side file handling on the CPU, against the
reference's example/checker data (tests/golden/checker_golden.npz): its SU
files (gb_su_write / gb_su_read, the host code of gb_export_traces and of
the trace_file import; 240-byte headers byte for byte, samples, read-back)
and the grid it infers from model_true (gb_infer_grid, the host code of
gb_solver_create)."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "checker_golden.npz")


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLD)


def _cfg(g, key):
    return float(g["cfg_vals"][list(g["cfg_keys"]).index(key)])


def test_su_headers_and_samples_match_golden(pkg, golden, tmp_path):
    src, rec = golden["src"], golden["rec"]
    nt, dt = int(_cfg(golden, "nt")), np.float32(_cfg(golden, "dt"))
    nrec = len(rec)
    for k, shot in enumerate(golden["golden_shots"]):
        traces = np.zeros((nrec, nt), np.float32)
        traces[golden["golden_recs"]] = golden["golden_vy"][k]
        path = str(tmp_path / ("vy_%06d.su" % shot))
        pkg.su_write(path, traces, dt, src[shot, 0], src[shot, 1], rec[:, 0], rec[:, 1])
        raw = open(path, "rb").read()
        assert len(raw) == nrec * (240 + 4 * nt)
        for q, r in enumerate(golden["golden_recs"]):
            off = r * (240 + 4 * nt)
            assert raw[off:off + 240] == golden["golden_heads"][k, q].tobytes(), (shot, r)
            samples = np.frombuffer(raw[off + 240:off + 240 + 4 * nt], np.float32)
            np.testing.assert_array_equal(samples, golden["golden_vy"][k, q])
        np.testing.assert_array_equal(pkg.su_read(path, nrec, nt), traces)


def test_su_read_rejects_short_file(pkg, tmp_path):
    path = str(tmp_path / "short.su")
    pkg.su_write(path, np.ones((2, 10), np.float32), 1e-3, 0, 0, [0.0, 1.0], [0.0, 0.0])
    with pytest.raises(pkg.GbError):
        pkg.su_read(path, 3, 10)


def test_grid_inference_matches_oracle(pkg, orc, golden, tmp_path):
    """gb_infer_grid (the host code of gb_solver_create) on the checker's own
    model points, and on a rectangular grid of points, against the oracle."""
    d = tmp_path / "model_true"
    d.mkdir()
    orc.write_bin(str(d / "proc000000_x.bin"), golden["true_x"])
    orc.write_bin(str(d / "proc000000_z.bin"), golden["true_z"])
    nx, nz, xmax, zmax, npt = pkg.infer_grid(str(tmp_path))
    ref = orc.infer_grid(golden["true_x"], golden["true_z"])
    assert (nx, nz) == (ref[0], ref[1]) and npt == golden["true_x"].size
    assert np.float32(xmax) == np.float32(ref[4]) and np.float32(zmax) == np.float32(ref[5])
    ii, jj = np.meshgrid(np.arange(137), np.arange(61), indexing="ij")
    x = (ii * 12.5).astype(np.float32).ravel()
    z = (jj * 12.5).astype(np.float32).ravel()
    orc.write_bin(str(d / "proc000000_x.bin"), x)
    orc.write_bin(str(d / "proc000000_z.bin"), z)
    nx, nz, xmax, zmax, npt = pkg.infer_grid(str(tmp_path))
    assert (nx, nz, npt) == (137, 61, 137 * 61)
    assert (nx, nz) == tuple(orc.infer_grid(x, z)[:2])
