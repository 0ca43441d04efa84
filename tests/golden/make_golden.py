"""Builds tests/golden/checker_golden.npz from the reference's example/checker.

The reference ships no tests; its only known-answer data are the SH velocity
seismograms example/checker/traces/vy_0000NN.su (25 shots x 132 receivers x
5000 steps). This script keeps what the golden test needs, small enough to
commit: the checker model (vs, rho on the 201 x 201 grid; vp is 0), the
config values, the source/station lists, and the golden traces of shots 0, 12
and 24 at every 11th receiver, with their 240-byte SU headers.

Run from the repository root, where the reference checkout is available:
    python tests/golden/make_golden.py /path/to/reference
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import oracle as O  # noqa: E402

SHOTS = (0, 12, 24)
REC_STRIDE = 11


def main(ref):
    ex = os.path.join(ref, "example", "checker")
    cfg = O.Config.load(ex, cwd=ref)
    arrays = {}
    for c in ("x", "z", "vp", "vs", "rho"):
        arrays["true_" + c] = O.read_bin(os.path.join(ex, "model_true", "proc000000_%s.bin" % c))
        arrays["init_" + c] = O.read_bin(os.path.join(ex, "model_init", "proc000000_%s.bin" % c))
    arrays["src"] = np.array(cfg.src, np.float32)
    arrays["rec"] = np.array(cfg.rec, np.float32)
    keys = sorted(cfg.f)
    arrays["cfg_keys"] = np.array(keys)
    arrays["cfg_vals"] = np.array([cfg.f[k] for k in keys], np.float64)
    recs = np.arange(0, len(cfg.rec), REC_STRIDE)
    arrays["golden_shots"] = np.array(SHOTS, np.int32)
    arrays["golden_recs"] = recs.astype(np.int32)
    traces, heads = [], []
    for s in SHOTS:
        tr, hd = O.read_su(os.path.join(ex, "traces", "vy_%06d.su" % s))
        traces.append(tr[recs])
        heads.append(np.stack([hd[r] for r in recs]))
    arrays["golden_vy"] = np.stack(traces)
    arrays["golden_heads"] = np.stack(heads)
    out = os.path.join(HERE, "checker_golden.npz")
    np.savez_compressed(out, **arrays)
    print("wrote", out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <reference checkout>")
    main(sys.argv[1])
