"""Checkpoint precision: gradients with FP32, BF16 and FP16 forward
checkpoints (per-snapshot power-of-two scaling) against an FP64 oracle run.

The FP64 reference is the oracle's double-precision forward and adjoint with
the waveform adjoint source computed in double. Tolerances follow the
precision pattern: FP32 checkpoints match the FP64 gradient to 1e-4; 16-bit
checkpoints stay within 1e-3 (the bar for batched/served gradients).
"""
import numpy as np
import pytest

from tests import cases

pytestmark = pytest.mark.gpu


def fp64_gradient(orc, pb, obs, tw, dt, wave):
    comps = "xz" if wave == "psv" else "y"
    kern = None
    for s in range(pb.nsrc):
        ox, oy, oz, ck = orc.forward(pb, s, adj=True, precision="f64")
        syn = {"x": ox, "y": oy, "z": oz}
        ad = {}
        for c in "xyz":
            if c in comps:
                r = (syn[c] - obs[c][s].astype(np.float64)) * tw
                ad[c] = np.ascontiguousarray((2 * r * tw)[:, ::-1])
            else:
                ad[c] = np.zeros((pb.nrec, pb.nt))
        kern = orc.adjoint(pb, [ad["x"], ad["y"], ad["z"]], ck, kern, precision="f64")
    return kern


@pytest.mark.parametrize("wave", ["psv", "sh"])
def test_checkpoint_precision_vs_fp64_oracle(gpu, orc, wave):
    case = cases.make_case(wave=wave, nx=120, nz=90, nt=600, nsrc=2, nrec=40, sfe=10, seed=41)
    pb = cases.oracle_problem(orc, case)
    pert = dict(case, vs=(case["vs"] * 1.04).astype(np.float32), vp=(case["vp"] * 1.03).astype(np.float32))
    pbo = cases.oracle_problem(orc, pert)
    obs = {c: np.stack([orc.forward(pbo, s, adj=True)["xyz".index(c)] for s in range(case["nsrc"])])
           for c in "xyz"}
    tw = orc.taper(case["nt"], case["dt"]).astype(np.float64)
    ref = fp64_gradient(orc, pb, obs, tw, case["dt"], wave)
    names = ("k_lambda", "k_mu", "k_rho") if wave == "psv" else ("k_mu", "k_rho")
    errs = {}
    for prec in (0, 1, 2):
        cfg, sol = cases.gpu_solver(gpu, case)
        sol.set_option("ckpt", prec)
        m = gpu.Misfit.from_obs(0, sol, {c: obs[c] for c in ("xz" if wave == "psv" else "y")})
        m.run(kernel=True)
        k = sol.kernels()
        errs[prec] = max(cases.rel(k[n], ref[("k_lambda", "k_mu", "k_rho").index(n)]) for n in names)
        m.close()
        sol.close()
    print("gradient rel. error vs FP64 (fp32, bf16, fp16):", errs)
    assert errs[0] < 1e-4
    assert errs[2] < 1e-3
    assert errs[1] < 1e-2
