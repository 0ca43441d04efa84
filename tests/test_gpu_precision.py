"""Checkpoint precision: gradients with FP32, BF16 and FP16 forward
checkpoints against an FP64 oracle run.

The FP32 checkpoints hold the reference's fields (displacement, velocity);
the 16-bit forms hold the displacement's differences that the kernel
accumulation reads, and the velocity, each with a power-of-two scale per
snapshot and field. The FP64 reference is the oracle's double-precision
forward and adjoint with the waveform adjoint source formed in double.
Tolerances: FP32 checkpoints match the FP64 gradient to 1e-4 and FP16
checkpoints to 1e-3, the precision pattern's bar. BF16 keeps 8 significant
bits, so each stored value carries a relative rounding error of about
1.6e-3 rms, and the kernels' sums over checkpoints (which cancel) do not
average it down: BF16 gradients sit at 0.6-1.3e-3 on these cases (and at
1.6-3.6e-3 for 64 shots of the 2048x1024 study against FP32 checkpoints),
so BF16 is held to 2e-3 here and FP16 is the 16-bit form that meets the bar.
"""
import numpy as np
import pytest

from tests import cases

pytestmark = pytest.mark.gpu

NAMES = ("k_lambda", "k_mu", "k_rho")


def gradient_errors(gpu, orc, case, obs, wave, names):
    pb = cases.oracle_problem(orc, case)
    tw = orc.taper(case["nt"], case["dt"]).astype(np.float64)
    ref = cases.fp64_gradient(orc, pb, obs, tw, wave)
    errs = {}
    for prec in (0, 1, 2):
        cfg, sol = cases.gpu_solver(gpu, case)
        sol.set_option("ckpt", prec)
        m = gpu.Misfit.from_obs(0, sol, {c: obs[c] for c in ("xz" if wave == "psv" else "y")})
        m.run(kernel=True)
        k = sol.kernels()
        errs[("fp32", "bf16", "fp16")[prec]] = {n: cases.rel(k[n], ref[NAMES.index(n)]) for n in names}
        m.close()
        sol.close()
    return errs


@pytest.mark.parametrize("wave", ["psv", "sh"])
def test_checkpoint_precision_vs_fp64_oracle(gpu, orc, wave):
    case = cases.make_case(wave=wave, nx=120, nz=90, nt=600, nsrc=2, nrec=40, sfe=10, seed=41)
    pert = dict(case, vs=(case["vs"] * 1.04).astype(np.float32), vp=(case["vp"] * 1.03).astype(np.float32))
    pbo = cases.oracle_problem(orc, pert)
    obs = {c: np.stack([orc.forward(pbo, s, adj=True)["xyz".index(c)] for s in range(case["nsrc"])])
           for c in "xyz"}
    names = ("k_lambda", "k_mu", "k_rho") if wave == "psv" else ("k_mu", "k_rho")
    errs = gradient_errors(gpu, orc, case, obs, wave, names)
    print("gradient rel. error vs FP64:", errs)
    assert max(errs["fp32"].values()) < 1e-4
    assert max(errs["fp16"].values()) < 1e-3
    assert max(errs["bf16"].values()) < 2e-3


def test_precision_study_grid_vs_fp64_oracle(gpu, orc):
    """The precision study's grid and model (P-SV 2048x1024 at 5 m, dt
    0.4 ms, smooth random vp 2000-4500 and vp/vs 1.7-2.0, checkpoints every
    50 steps, f0 15 Hz) with one shot and 2000 of its 6000 steps, so that
    the FP64 oracle finishes in about a minute: each checkpoint precision's
    gradient against the FP64 oracle's: FP32 within 1e-4, FP16 within
    1e-3, BF16 within 2e-3."""
    case = cases.random_smooth_case(nt=2000, nsrc=1)
    pert = dict(case, vs=(case["vs"] * 1.02).astype(np.float32), vp=(case["vp"] * 1.02).astype(np.float32))
    cfg, sol = cases.gpu_solver(gpu, pert)
    sol.run_forward_batch([0])
    obs = {c: sol.out(c, slot=0)[None] for c in "xz"}
    sol.close()
    errs = gradient_errors(gpu, orc, case, obs, "psv", NAMES)
    print("precision study grid, gradient rel. error vs FP64:", errs)
    bars = {"fp32": 1e-4, "fp16": 1e-3, "bf16": 2e-3}
    for prec, e in errs.items():
        assert max(e.values()) < bars[prec], (prec, e)
