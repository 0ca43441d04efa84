"""GPU parity of the Gaussian filter, the misfits, the FP64 reductions and
the model intake against the CPU oracle, through the C ABI."""
import numpy as np
import pytest

from tests import cases

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nx,nz,sigma", [(64, 48, 3), (181, 97, 5), (300, 40, 10)])
def test_gaussian_filter_matches_oracle(gpu, orc, nx, nz, sigma):
    rng = np.random.default_rng(nx + nz + sigma)
    data = rng.standard_normal(nx * nz).astype(np.float32)
    f = gpu.GaussianFilter(nx, nz, sigma)
    got = f.apply_host(data)
    ref = orc.gaussian_filter(nx, nz, sigma, data)
    assert cases.rel(got, ref) < 1e-5


def test_gaussian_filter_is_one_sided(gpu):
    # a spike at (i0, j0) only spreads to i >= i0, j >= j0 (filter/gaussian.h:4-8)
    nx, nz, i0, j0 = 60, 50, 30, 20
    d = np.zeros(nx * nz, np.float32)
    d[i0 * nz + j0] = 1.0
    out = gpu.GaussianFilter(nx, nz, 4).apply_host(d).reshape(nx, nz)
    assert np.all(out[:i0, :] == 0) and np.all(out[:, :j0] == 0)
    assert out[i0, j0] > 0 and out[i0 + 3, j0 + 3] > 0


def _misfit_case(gpu, orc, kind, wave):
    case = cases.make_case(wave=wave, nx=100, nz=80, nt=512 if kind else 400, nsrc=3, nrec=24, seed=29)
    cfg, sol = cases.gpu_solver(gpu, case)
    pb = cases.oracle_problem(orc, case)
    # observed data: the same problem with a perturbed model
    pert = dict(case)
    pert["vs"] = (case["vs"] * 1.03).astype(np.float32)
    pert["vp"] = (case["vp"] * 1.02).astype(np.float32)
    pbo = cases.oracle_problem(orc, pert)
    obs = {c: [] for c in "xyz"}
    syn = {c: [] for c in "xyz"}
    for s in range(case["nsrc"]):
        o = orc.forward(pbo, s, adj=True)
        y = orc.forward(pb, s, adj=True)
        for q, c in enumerate("xyz"):
            obs[c].append(o[q])
            syn[c].append(y[q])
    obs = {c: np.stack(v) for c, v in obs.items()}
    syn = {c: np.stack(v) for c, v in syn.items()}
    m = gpu.Misfit.from_obs(kind, sol, {c: obs[c] for c in cases_comps(wave)})
    return case, sol, pb, m, obs, syn


def cases_comps(wave):
    return "xz" if wave == "psv" else "y"


@pytest.mark.parametrize("kind,wave", [(0, "psv"), (0, "sh"), (1, "sh"), (1, "psv")])
def test_misfit_value_and_adjoint_source(gpu, orc, kind, wave):
    case, sol, pb, m, obs, syn = _misfit_case(gpu, orc, kind, wave)
    val = m.run(kernel=False)
    tw = orc.taper(case["nt"], case["dt"])
    ref_total = 0.0
    for s in range(case["nsrc"]):
        for c in cases_comps(wave):
            if kind == 0:
                v, ad = orc.waveform_misfit(syn[c][s], obs[c][s], tw, case["dt"])
            else:
                v, ad = orc.envelope_misfit(syn[c][s], obs[c][s], case["dt"])
            ref_total += v
    assert abs(val - ref_total) / abs(ref_total) < 1e-4
    # adjoint sources of the last batch slot hold the last shot
    last = case["nsrc"] - 1
    slot = last % sol.capacity
    for c in cases_comps(wave):
        if kind == 0:
            _, ad = orc.waveform_misfit(syn[c][last], obs[c][last], tw, case["dt"])
        else:
            _, ad = orc.envelope_misfit(syn[c][last], obs[c][last], case["dt"])
        assert cases.rel(sol.adstf(c, slot=slot), ad) < 1e-4


@pytest.mark.parametrize("wave", ["psv", "sh"])
def test_gradient_pipeline_matches_oracle(gpu, orc, wave):
    """Misfit::run(kernel=true): batched forward, waveform misfit, batched
    adjoint, then the filter on all three kernels."""
    case, sol, pb, m0, obs, syn = _misfit_case(gpu, orc, 0, wave)
    sigma = 3
    filt = gpu.GaussianFilter(case["nx"], case["nz"], sigma)
    m = gpu.Misfit.from_obs(0, sol, {c: obs[c] for c in cases_comps(wave)}, filt)
    val = m.run(kernel=True)
    k = sol.kernels()
    tw = orc.taper(case["nt"], case["dt"])
    kern = None
    total = 0.0
    for s in range(case["nsrc"]):
        o = orc.forward(pb, s, adj=True)
        ad = {}
        for c in "xyz":
            if c in cases_comps(wave):
                v, ad[c] = orc.waveform_misfit(o["xyz".index(c)], obs[c][s], tw, case["dt"])
                total += v
            else:
                ad[c] = np.zeros((pb.nrec, pb.nt), np.float32)
        kern = orc.adjoint(pb, [ad["x"], ad["y"], ad["z"]], o[3], kern)
    kern = [orc.gaussian_filter(case["nx"], case["nz"], sigma, kk) for kk in kern]
    assert abs(val - total) / total < 1e-4
    names = ("k_lambda", "k_mu", "k_rho")
    for q, name in enumerate(names):
        if wave == "sh" and name == "k_lambda":
            continue
        assert cases.rel(k[name], kern[q]) < 1e-4, name


def test_fp64_reductions(gpu):
    rng = np.random.default_rng(3)
    a = rng.standard_normal(1_000_003).astype(np.float32)
    b = rng.standard_normal(1_000_003).astype(np.float32)
    da, db = gpu.DeviceArray(a), gpu.DeviceArray(b)
    ref = float(np.dot(a.astype(np.float64), b.astype(np.float64)))
    assert abs(gpu.dot64(da.ptr, db.ptr, a.size) - ref) <= 1e-9 * np.abs(a).sum()
    assert gpu.amax64(da.ptr, a.size) == float(np.abs(a).max())


def test_mesh2grid_brute_force_matches_oracle(gpu, orc):
    # irregular points force the nearest-point search (no exact grid match)
    rng = np.random.default_rng(4)
    nx, nz, npt = 40, 30, 700
    case = cases.make_case(wave="sh", nx=nx, nz=nz, nt=10, nsrc=1, nrec=4)
    case["values"]["model_type"] = 1
    cfg, sol = cases.gpu_solver(gpu, case)
    px = rng.uniform(0, case["xmax"], npt).astype(np.float32)
    pz = rng.uniform(0, case["zmax"], npt).astype(np.float32)
    px[:2] = [0, case["xmax"]]
    pz[:2] = [0, case["zmax"]]
    a, b, r = (rng.uniform(1, 2, npt).astype(np.float32) for _ in range(3))
    sol.set_model_points(px, pz, a, b, r)
    got = sol.model()
    lam, mu, rho = orc.mesh2grid(nx, nz, sol.dx, sol.dz, px, pz, a, b, r, case["xmax"], case["zmax"])
    # cells whose two nearest points are within rounding of each other may
    # resolve either way (contracted vs plain float distance); skip those
    gx = (np.arange(nx, dtype=np.float32) * np.float32(sol.dx)).astype(np.float64)
    gz = (np.arange(nz, dtype=np.float32) * np.float32(sol.dz)).astype(np.float64)
    d = (gx[:, None, None] - px[None, None, :]) ** 2 + (gz[None, :, None] - pz[None, None, :]) ** 2
    d2 = np.sort(d.reshape(nx * nz, npt), axis=1)[:, :2]
    clear = (d2[:, 1] - d2[:, 0]) > 1e-5 * d2[:, 1]
    assert clear.mean() > 0.95
    for name, ref in (("lambda", lam), ("mu", mu), ("rho", rho)):
        np.testing.assert_array_equal(got[name][clear], ref[clear])


def test_mesh2grid_fast_path_matches_brute_force(gpu, orc):
    nx, nz = 37, 23
    case = cases.make_case(wave="sh", nx=nx, nz=nz, nt=10, nsrc=1, nrec=4)
    cfg, sol = cases.gpu_solver(gpu, case)
    ii, jj = np.meshgrid(np.arange(nx), np.arange(nz), indexing="xy")
    px = (ii.ravel() * np.float32(sol.dx)).astype(np.float32)
    pz = (jj.ravel() * np.float32(sol.dz)).astype(np.float32)
    rng = np.random.default_rng(6)
    vp = rng.uniform(3000, 4000, px.size).astype(np.float32)
    vs = (vp / 1.8).astype(np.float32)
    rho = rng.uniform(2000, 2600, px.size).astype(np.float32)
    sol.set_model_points(px, pz, vp, vs, rho)
    got = sol.model()
    lam, mu, r = orc.mesh2grid(nx, nz, sol.dx, sol.dz, px, pz, vp, vs, rho, case["xmax"], case["zmax"])
    lam, mu = orc.vps2lm(lam, mu, r)
    np.testing.assert_array_equal(got["rho"], r)
    assert cases.rel(got["lambda"], lam) < 1e-6 and cases.rel(got["mu"], mu) < 1e-6


def test_lbfgs_without_memory_is_rejected(gpu, tmp_path):
    """optimizer = 1 with lbfgs_mem 0 (the reference indexes lbfgs_S[-1])
    fails at creation instead of running a search with no history buffers."""
    case = cases.make_case(wave="sh", nx=40, nz=30, nt=20, nsrc=1, nrec=4)
    cfg, sol = cases.gpu_solver(gpu, case, directory=str(tmp_path))
    cfg.set("optimizer", 1)
    cfg.set("lbfgs_mem", 0)
    mis = gpu.Misfit.from_obs(0, sol, {"y": np.zeros((1, 4, 20), np.float32)})
    with pytest.raises(gpu.GbError, match="lbfgs_mem"):
        gpu.Optimizer(cfg, sol, mis)
    mis.close()
    sol.close()


def test_misfit_and_optimizer_may_outlive_their_solver(gpu, orc):
    """Destroying a solver before the misfit and the optimizer built on it
    is allowed: their destruction does not touch the solver."""
    case = cases.make_case(wave="sh", nx=64, nz=48, nt=100, nsrc=2, nrec=16, sfe=10, seed=3)
    case["values"].update({"optimizer": 1, "inv_iteration": 1, "lbfgs_mem": 2, "ls_step": 2, "ls_step_max": 0.5,
                           "ls_step_init": 0.05, "ls_thresh": 1.2})
    cfg, sol = cases.gpu_solver(gpu, case)
    obs = {"y": np.zeros((2, 16, 100), np.float32)}
    m = gpu.Misfit.from_obs(0, sol, obs)
    opt = gpu.Optimizer(cfg, sol, m)
    m.run(kernel=True)
    sol.close()
    opt.close()
    m.close()
