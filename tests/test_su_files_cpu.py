"""The library's SU files (gb_su_write / gb_su_read, host code of
gb_export_traces and of the trace_file import) against the reference's
golden SU files of example/checker (tests/golden/checker_golden.npz): the
240-byte headers byte for byte, the samples, and the read-back."""
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
