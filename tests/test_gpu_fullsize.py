"""Parity at the benchmark configurations' full sizes.

The oracle finishes a full P-SV shot of the 200x200 configuration in
seconds, so that one is compared directly. At the larger sizes the checks
are properties that do not depend on the size: the cluster-resident pass
and the per-step kernels, and the marching kernel's two load paths, compute
every cell with the same operations, so their seismograms must agree bit for
bit over the whole time loop."""
import numpy as np
import pytest

from tests import cases

pytestmark = pytest.mark.gpu


def surface_receivers(case, h):
    """One receiver per column, two cells deep (distinct cells)."""
    case["rec"] = [[i * h, 2 * h] for i in range(case["nx"])]
    case["nrec"] = case["nx"]
    return case


@pytest.mark.parametrize("cluster", [1, 0])
def test_c1_full_psv_forward_matches_oracle(gpu, orc, cluster):
    """The 200x200 P-SV checkerboard (vp 3000, vs 1732, rho 2600, +-5 % in
    20-cell squares), 4 shots, dt 1 ms, all 2000 steps, a receiver in every
    column two cells deep, through the cluster pass and through the per-step
    kernels: the displacement seismograms of every shot match the FP32 oracle
    within relative L2 1e-5 over the whole time loop. On this model the
    scheme is well conditioned: the oracle's own FP32 and FP64 builds stay
    about 1.5e-6 apart over the 2000 steps."""
    case = cases.checkerboard_case()
    cfg, sol = cases.gpu_solver(gpu, case)
    sol.set_option("cluster", cluster)
    sol.run_forward_batch([0, 1, 2, 3])
    assert (sol.stats().tile_tz < 0) == (cluster == 1), "unexpected kernel form"
    pb = cases.oracle_problem(orc, case)
    for s in range(4):
        o32 = orc.forward(pb, s, adj=True)
        for q, c in ((0, "x"), (2, "z")):
            g = sol.out(c, slot=s)
            assert np.abs(g).max() > 0, (s, c)
            assert cases.rel(g, o32[q]) < 1e-5, (s, c)


def test_jittered_layered_psv_short_run_matches_oracle(gpu, orc):
    """P-SV 200x200 on a layered, faulted model with 3 % per-cell jitter,
    800 steps. Over longer runs this model carries a mode of the reference
    scheme that grows by about 0.75 % per step (shot 2's FP64 trace norm per
    1000 steps: ~1e2 at steps 2000-3000, ~2e18 at steps 7000-8000), and the
    oracle's FP32 and FP64 builds part from step ~1500 on (7.7e-4 over steps
    1000-2000, 0.55 after), so no FP32 code holds a 1e-5 bar there. The
    first 800 steps are well conditioned (FP32 to FP64: 7.9e-7)."""
    h = 10.0
    case = surface_receivers(cases.make_case(wave="psv", nx=200, nz=200, nt=800, nsrc=4, dx=h, dt=1e-3, f0=10.0,
                                             abs_width=20, sfe=10, seed=1), h)
    cfg, sol = cases.gpu_solver(gpu, case)
    sol.run_forward_batch([0, 1, 2, 3])
    assert sol.stats().tile_tz < 0, "the cluster path did not run"
    pb = cases.oracle_problem(orc, case)
    o32 = orc.forward(pb, 2, adj=True)
    for q, c in ((0, "x"), (2, "z")):
        assert cases.rel(sol.out(c, slot=2), o32[q]) < 1e-5, c


def test_c2_full_cluster_equals_step_kernels(gpu, orc):
    """SH 681x141 at 12.5 m, 4000 steps, 16 shots, 681 receivers, FP32
    checkpoints every 10 steps: forward seismograms of the cluster pass and
    of the per-step kernels are identical and match the oracle; the kernels
    differ only by the order the shots are summed."""
    h = 12.5
    case = surface_receivers(cases.make_case(wave="sh", nx=681, nz=141, nt=4000, nsrc=16, dx=h, dt=1e-3, f0=8.0,
                                             abs_width=20, sfe=10, seed=2), h)
    rng = np.random.default_rng(4)
    ad = [(rng.standard_normal((681, 4000)) * 1e-3).astype(np.float32) for _ in range(16)]
    shots = list(range(16))
    res = []
    for cluster in (1, 0):
        cfg, sol = cases.gpu_solver(gpu, case)
        sol.set_option("cluster", cluster)
        sol.run_forward_batch(shots)
        tr = [sol.out("y", slot=b) for b in shots]
        assert (sol.stats().tile_tz < 0) == (cluster == 1)
        for b in shots:
            sol.set_adstf("y", ad[b], slot=b)
        sol.initKernels()
        sol.run_adjoint_batch(shots)
        res.append((tr, sol.kernels()))
        sol.close()
    for b in shots:
        np.testing.assert_array_equal(res[0][0][b], res[1][0][b])
    for n in ("k_mu", "k_rho"):
        assert cases.rel(res[0][1][n], res[1][1][n]) < 1e-6, n
    # and the full 4000-step seismogram of one shot against the oracle (this
    # SH configuration is well conditioned: FP32 and FP64 oracles agree to 2e-6)
    o = orc.forward(cases.oracle_problem(orc, case), 0, adj=True)
    assert cases.rel(res[0][0][0], o[1]) < 1e-5


def test_c5_grid_bulk_loads_equal_cp_async(gpu, orc):
    """P-SV 4096x1024 (the full-inversion grid), 2 shots, 40 steps: the
    marching kernel with bulk tensor loads and with per-row cp.async."""
    case = cases.make_case(wave="psv", nx=4096, nz=1024, nt=40, nsrc=2, nrec=256, dx=5.0, dt=4e-4, f0=12.0,
                           abs_width=20, sfe=10, seed=5)
    rng = np.random.default_rng(6)
    ad = {c: (rng.standard_normal((256, 40)) * 1e-3).astype(np.float32) for c in "xz"}
    res = []
    for tma in (1, 0):
        cfg, sol = cases.gpu_solver(gpu, case)
        sol.set_option("cluster", 0)
        sol.set_option("tile", 19)
        sol.set_option("tma", tma)
        sol.run_forward_batch([0, 1])
        assert sol.stats().march_bulk == tma
        tr = {c: sol.out(c, slot=1) for c in "xz"}
        for b in (0, 1):
            for c in "xz":
                sol.set_adstf(c, ad[c], slot=b)
        sol.initKernels()
        sol.run_adjoint_batch([0, 1])
        res.append((tr, sol.kernels()))
        sol.close()
    for c in "xz":
        np.testing.assert_array_equal(res[0][0][c], res[1][0][c])
    for n in ("k_lambda", "k_mu", "k_rho"):
        np.testing.assert_array_equal(res[0][1][n], res[1][1][n])


@pytest.mark.parametrize("kind,wave", [(1, "sh"), (0, "sh"), (1, "psv")])
def test_c2_pipelined_gradient_identical(gpu, orc, kind, wave):
    """The C2 shapes with 16 shots take more than one round of resident
    clusters, SH and P-SV alike: the pipelined gradient (each round's misfit
    overlapping the next forward round and the previous adjoint round) gives
    the same misfit value and kernels, bit for bit, as forward, misfit and
    adjoint run one after another."""
    h = 12.5
    nt = 400 if wave == "sh" else 200
    case = surface_receivers(cases.make_case(wave=wave, nx=681, nz=141, nt=nt, nsrc=16, dx=h, dt=1e-3, f0=8.0,
                                             abs_width=20, sfe=10, seed=2), h)
    comps = "y" if wave == "sh" else "xz"
    names = ("k_mu", "k_rho") if wave == "sh" else ("k_lambda", "k_mu", "k_rho")
    pert = dict(case)
    pert["vs"] = (case["vs"] * 1.02).astype(np.float32)
    cfg, sol = cases.gpu_solver(gpu, pert)
    sol.set_option("batch", 16)
    sol.run_forward_batch(list(range(16)))
    obs = {c: np.stack([sol.out(c, slot=b) for b in range(16)]) for c in comps}
    sol.close()
    out = []
    for pipe in (1, 0):
        cfg, sol = cases.gpu_solver(gpu, case)
        sol.set_option("pipeline", pipe)
        sol.set_option("batch", 16)
        m = gpu.Misfit.from_obs(kind, sol, obs)
        val = m.run(kernel=True)
        assert sol.stats().tile_tz < 0, "the cluster path did not run"
        out.append((val, sol.kernels()))
        sol.close()
    assert out[0][0] == out[1][0]
    for n in names:
        np.testing.assert_array_equal(out[0][1][n], out[1][1][n])


@pytest.mark.parametrize("wave", ["sh", "psv"])
def test_observed_traces_queued_during_the_forward_identical(gpu, orc, wave):
    """gb_misfit_set_obs_async queues the observed traces' upload on a stream
    of its own, overlapping the next run's forward pass (only the misfit
    stages wait for it): on the C2 shapes (pipelined rounds) the misfit and
    kernels are bit-identical to those of a run after gb_misfit_set_obs, and
    the same holds on a grid that runs the per-step kernels."""
    h = 12.5
    for nx, nz, cluster in ((681, 141, 1), (200, 120, 0)):
        case = surface_receivers(cases.make_case(wave=wave, nx=nx, nz=nz, nt=200, nsrc=16, dx=h, dt=1e-3, f0=8.0,
                                                 abs_width=20, sfe=10, seed=3), h)
        comps = "y" if wave == "sh" else "xz"
        pert = dict(case)
        pert["vs"] = (case["vs"] * 1.02).astype(np.float32)
        cfg, sol = cases.gpu_solver(gpu, pert)
        sol.set_option("batch", 16)
        sol.run_forward_batch(list(range(16)))
        obs = {c: np.stack([sol.out(c, slot=b) for b in range(16)]) for c in comps}
        sol.close()
        zeros = {c: np.zeros_like(v) for c, v in obs.items()}
        out = []
        for queued in (0, 1):
            cfg, sol = cases.gpu_solver(gpu, case)
            sol.set_option("batch", 16)
            sol.set_option("cluster", cluster)
            m = gpu.Misfit.from_obs(1, sol, zeros)
            if queued:
                m.set_obs_async(obs)
            else:
                m.set_obs(obs)
            val = m.run(kernel=True)
            out.append((val, sol.kernels()))
            if cluster:
                assert sol.stats().tile_tz < 0, "the cluster path did not run"
            sol.close()
        assert out[0][0] == out[1][0] and out[0][0] > 0
        for n in out[0][1]:
            np.testing.assert_array_equal(out[0][1][n], out[1][1][n])
