"""Parity with the reference's own device code.

The reference's kernels (solver/fdm.h, filter/gaussian.h), compiled from its
sources into oracle/_ref/inv_ref.cubin, run under oracle/ref_harness.cu's
restatement of its host loops (runForward, runAdjoint, GaussianFilter). The
GB300 path and the C oracle are compared with what they compute, on the
same inputs: seismograms within relative L2 1e-5 after the full time loop,
kernels and misfits within 1e-4, filter and absorbing profile within 1e-6.

The reference divides where the GB300 kernels multiply by reciprocals and
contracts its own expressions into FMAs, so results agree to rounding, not
bit for bit.
"""
import numpy as np
import pytest

from tests import cases

pytestmark = pytest.mark.gpu

TRACE_TOL = 1e-5
KERNEL_TOL = 1e-4


@pytest.fixture(scope="module")
def ref(orc):
    if not orc.ref_available():
        pytest.skip("the reference's kernels were not built (no reference checkout where the oracle was built)")
    orc.ref_lib()
    return orc


def comps(wave):
    return "xz" if wave == "psv" else "y"


def kernel_names(wave):
    return ("k_lambda", "k_mu", "k_rho") if wave == "psv" else ("k_mu", "k_rho")


def test_absorbing_profile_matches_reference(ref):
    for args in ((150, 110, 20, 0.015, 1, 1, 1, 0), (64, 48, 12, 0.02, 1, 1, 1, 1), (40, 90, 30, 0.01, 0, 1, 0, 1)):
        a = ref.ref_absbound(*args)
        b = ref.absbound(*args)
        assert np.abs(a - b).max() <= 1e-6, args


@pytest.mark.parametrize("wave", ["psv", "sh"])
def test_forward_matches_reference_kernels(gpu, ref, wave):
    """Displacement seismograms of every shot (adjoint mode) and velocity
    seismograms (trace mode): the GB300 cluster and per-step paths and the C
    oracle against the reference's kernels, 600 steps."""
    case = cases.make_case(wave=wave, nx=140, nz=100, nt=600, nsrc=2, nrec=45, seed=13)
    pb = cases.oracle_problem(ref, case)
    ab = ref.ref_absbound(case["nx"], case["nz"], case["values"]["abs_width"], case["values"]["abs_alpha"],
                          1, 1, 1, 0)
    for cluster in (1, 0):
        cfg, sol = cases.gpu_solver(gpu, case)
        sol.set_option("cluster", cluster)
        for s in range(case["nsrc"]):
            sol.runForward(s)
            r = ref.ref_forward(pb, s, adj=True, ab=ab)
            for c in comps(wave):
                q = "xyz".index(c)
                assert cases.rel(sol.out(c), r[q]) < TRACE_TOL, (cluster, s, c)
        sol.close()
    o = ref.forward(pb, 0, adj=True)
    r = ref.ref_forward(pb, 0, adj=True, ab=ab)
    for c in comps(wave):
        q = "xyz".index(c)
        assert cases.rel(o[q], r[q]) < TRACE_TOL, c
    # checkpoints: the same one-step offset and reversed slots
    assert cases.rel(o[3], r[3]) < TRACE_TOL
    # velocity recording (trace_type 0, no checkpoints)
    case["values"]["mode"] = 3
    cfg, sol = cases.gpu_solver(gpu, case)
    sol.runForward(1)
    r = ref.ref_forward(pb, 1, adj=False, record_u=False, ab=ab)
    for c in comps(wave):
        assert cases.rel(sol.out(c), r["xyz".index(c)]) < TRACE_TOL, c


@pytest.mark.parametrize("wave", ["psv", "sh"])
def test_adjoint_kernels_match_reference_kernels(gpu, ref, wave):
    """Sensitivity kernels of two shots, each adjoint driven by random
    adjoint sources at every receiver, against the reference's runAdjoint on
    its own forward checkpoints."""
    case = cases.make_case(wave=wave, nx=120, nz=96, nt=500, nsrc=2, nrec=40, sfe=10, seed=17)
    pb = cases.oracle_problem(ref, case)
    ab = ref.ref_absbound(case["nx"], case["nz"], case["values"]["abs_width"], case["values"]["abs_alpha"],
                          1, 1, 1, 0)
    rng = np.random.default_rng(4)
    ads = [{c: (rng.standard_normal((pb.nrec, pb.nt)) * 1e-3).astype(np.float32) for c in "xyz"} for _ in range(2)]
    kern = None
    for s in range(2):
        r = ref.ref_forward(pb, s, adj=True, ab=ab)
        kern = ref.ref_adjoint(pb, [ads[s]["x"], ads[s]["y"], ads[s]["z"]], r[3], kern, ab=ab)
    for cluster in (1, 0):
        cfg, sol = cases.gpu_solver(gpu, case)
        sol.set_option("cluster", cluster)
        sol.run_forward_batch([0, 1])
        for b in range(2):
            for c in comps(wave):
                sol.set_adstf(c, ads[b][c], slot=b)
        sol.initKernels()
        sol.run_adjoint_batch([0, 1])
        k = sol.kernels()
        for name in kernel_names(wave):
            q = ("k_lambda", "k_mu", "k_rho").index(name)
            assert cases.rel(k[name], kern[q]) < KERNEL_TOL, (cluster, name)
        sol.close()
    # and the C oracle
    ko = None
    for s in range(2):
        o = ref.forward(pb, s, adj=True)
        ko = ref.adjoint(pb, [ads[s]["x"], ads[s]["y"], ads[s]["z"]], o[3], ko)
    for name in kernel_names(wave):
        q = ("k_lambda", "k_mu", "k_rho").index(name)
        assert cases.rel(ko[q], kern[q]) < KERNEL_TOL, name


@pytest.mark.parametrize("nx,nz,sigma", [(120, 80, 5), (200, 141, 10), (64, 300, 3)])
def test_gaussian_filter_matches_reference_kernels(gpu, ref, nx, nz, sigma):
    rng = np.random.default_rng(nx + sigma)
    data = rng.standard_normal(nx * nz).astype(np.float32)
    r = ref.ref_gaussian(nx, nz, sigma, data)
    g = gpu.GaussianFilter(nx, nz, sigma).apply_host(data)
    assert cases.rel(g, r) < 1e-6
    assert cases.rel(ref.gaussian_filter(nx, nz, sigma, data), r) < 1e-6


@pytest.mark.parametrize("kind,wave", [(0, "sh"), (0, "psv"), (1, "sh"), (1, "psv")])
def test_misfit_matches_reference_kernels(gpu, ref, kind, wave):
    """Waveform (0) and envelope (1) misfits: per-trace values and adjoint
    sources of the C oracle, and the GB300 misfit's total and adjoint
    sources, against the reference's per-trace run (its kernels, cuFFT and
    cuBLAS); the GB300 total is an FP64 sum of the per-trace values."""
    case = cases.make_case(wave=wave, nx=100, nz=80, nt=512 if kind else 400, nsrc=2, nrec=24, seed=31)
    cfg, sol = cases.gpu_solver(gpu, case)
    pb = cases.oracle_problem(ref, case)
    pert = dict(case)
    pert["vs"] = (case["vs"] * 1.03).astype(np.float32)
    pert["vp"] = (case["vp"] * 1.02).astype(np.float32)
    pbo = cases.oracle_problem(ref, pert)
    obs, syn = {c: [] for c in "xyz"}, {c: [] for c in "xyz"}
    for s in range(case["nsrc"]):
        o = ref.forward(pbo, s, adj=True)
        y = ref.forward(pb, s, adj=True)
        for q, c in enumerate("xyz"):
            obs[c].append(o[q])
            syn[c].append(y[q])
    total = 0.0
    last = {}
    tw = ref.taper(case["nt"], case["dt"])
    for s in range(case["nsrc"]):
        for c in comps(wave):
            v, ad = ref.ref_misfit(kind, syn[c][s], obs[c][s], case["dt"])
            total += float(np.sum(v.astype(np.float64)))
            for r in range(pb.nrec):
                if kind == 0:
                    ov, oad = ref.waveform_misfit(syn[c][s][r:r + 1], obs[c][s][r:r + 1], tw, case["dt"])
                else:
                    ov, oad = ref.envelope_misfit(syn[c][s][r:r + 1], obs[c][s][r:r + 1], case["dt"])
                assert abs(ov - v[r]) <= 1e-4 * abs(v[r]) + 1e-12, (s, c, r)
                assert cases.rel(oad[0], ad[r]) < 1e-4, (s, c, r)
            last[c] = ad
    m = gpu.Misfit.from_obs(kind, sol, {c: np.stack(obs[c]) for c in comps(wave)})
    val = m.run(kernel=False)
    assert abs(val - total) / abs(total) < 1e-4
    slot = (case["nsrc"] - 1) % sol.capacity
    for c in comps(wave):
        assert cases.rel(sol.adstf(c, slot=slot), last[c]) < 1e-4, c
