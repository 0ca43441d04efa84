"""GPU parity of the solver against the CPU oracle, through the C ABI.

Tolerances: seismograms relative L2 <= 1e-5 after the full time loop;
sensitivity kernels and misfits <= 1e-4 (FP32 arithmetic, the kernels
replace divisions by reciprocal multiplies and contract into FMAs).
Batching, tile shape and graph capture must not change any bit.
"""
import numpy as np
import pytest

from tests import cases

pytestmark = pytest.mark.gpu

TRACE_TOL = 1e-5
KERNEL_TOL = 1e-4


def comps(wave):
    return "xz" if wave == "psv" else "y"


def kernel_names(wave):
    return ("k_lambda", "k_mu", "k_rho") if wave == "psv" else ("k_mu", "k_rho")


@pytest.mark.parametrize("wave", ["psv", "sh"])
def test_forward_traces_match_oracle(gpu, orc, wave):
    case = cases.make_case(wave=wave, nx=150, nz=110, nt=700, nsrc=2, nrec=50, seed=3)
    cfg, sol = cases.gpu_solver(gpu, case)
    pb = cases.oracle_problem(orc, case)
    for s in range(case["nsrc"]):
        sol.runForward(s)
        o = orc.forward(pb, s, adj=True)
        for c in comps(wave):
            assert cases.rel(sol.out(c), o["xyz".index(c)]) < TRACE_TOL


@pytest.mark.parametrize("wave", ["psv", "sh"])
def test_velocity_recording_without_adjoint(gpu, orc, wave):
    # mode 3: no checkpoints, velocity recorded (trace_type 0)
    case = cases.make_case(wave=wave, nx=90, nz=70, nt=400, nsrc=1, nrec=20, seed=5)
    case["values"]["mode"] = 3
    cfg, sol = cases.gpu_solver(gpu, case)
    pb = cases.oracle_problem(orc, case)
    sol.runForward(0)
    o = orc.forward(pb, 0, adj=False, record_u=False)
    for c in comps(wave):
        assert cases.rel(sol.out(c), o["xyz".index(c)]) < TRACE_TOL


def test_supershot_fires_every_source(gpu, orc):
    case = cases.make_case(wave="psv", nx=100, nz=80, nt=400, nsrc=3, nrec=30, seed=9)
    cfg, sol = cases.gpu_solver(gpu, case)
    pb = cases.oracle_problem(orc, case)
    sol.runForward(-1)
    o = orc.forward(pb, -1, adj=True)
    for c in "xz":
        assert cases.rel(sol.out(c), o["xyz".index(c)]) < TRACE_TOL


@pytest.mark.parametrize("wave", ["psv", "sh"])
def test_adjoint_kernels_match_oracle(gpu, orc, wave):
    case = cases.make_case(wave=wave, nx=120, nz=96, nt=500, nsrc=2, nrec=40, sfe=10, seed=11)
    cfg, sol = cases.gpu_solver(gpu, case)
    pb = cases.oracle_problem(orc, case)
    rng = np.random.default_rng(2)
    sol.initKernels()
    kern = None
    for s in range(case["nsrc"]):
        sol.runForward(s)
        o = orc.forward(pb, s, adj=True)
        ad = {c: (rng.standard_normal((pb.nrec, pb.nt)) * 1e-3).astype(np.float32) for c in "xyz"}
        for c in comps(wave):
            sol.set_adstf(c, ad[c])
        sol.runAdjoint(s)
        kern = orc.adjoint(pb, [ad["x"], ad["y"], ad["z"]], o[3], kern)
    k = sol.kernels()
    for name in kernel_names(wave):
        ref = kern[("k_lambda", "k_mu", "k_rho").index(name)]
        assert cases.rel(k[name], ref) < KERNEL_TOL, name


@pytest.mark.parametrize("wave", ["psv", "sh"])
def test_batch_equals_one_shot_at_a_time(gpu, orc, wave):
    case = cases.make_case(wave=wave, nx=110, nz=90, nt=300, nsrc=4, nrec=30, seed=13)
    cfg, sol = cases.gpu_solver(gpu, case)
    single = []
    for s in range(4):
        sol.runForward(s)
        single.append({c: sol.out(c) for c in comps(wave)})
    sol.run_forward_batch([0, 1, 2, 3])
    for s in range(4):
        for c in comps(wave):
            np.testing.assert_array_equal(sol.out(c, slot=s), single[s][c])


@pytest.mark.parametrize("wave", ["psv", "sh"])
@pytest.mark.parametrize("tile", list(range(2, 21)))
def test_kernel_configurations_give_identical_results(gpu, orc, tile, wave):
    """2-D tiles (ids 1-5) and marching strips/chunks (ids 6-20) compute every
    cell with the same operations in the same order."""
    case = cases.make_case(wave=wave, nx=133, nz=77, nt=250, nsrc=2, nrec=25, seed=17)
    rng = np.random.default_rng(5)
    ad = {c: (rng.standard_normal((case["nrec"], case["nt"])) * 1e-3).astype(np.float32) for c in "xyz"}

    def run(t):
        cfg, sol = cases.gpu_solver(gpu, case)
        sol.set_option("cluster", 0)
        sol.set_option("tile", t)
        sol.run_forward_batch([0, 1])
        tr = {c: sol.out(c, slot=1) for c in comps(wave)}
        for c in comps(wave):
            sol.set_adstf(c, ad[c], slot=0)
            sol.set_adstf(c, ad[c], slot=1)
        sol.initKernels()
        sol.run_adjoint_batch([0, 1])
        return tr, sol.kernels()

    ref_tr, ref_k = run(1)
    tr, k = run(tile)
    for c in comps(wave):
        np.testing.assert_array_equal(tr[c], ref_tr[c])
    for name in kernel_names(wave):
        np.testing.assert_array_equal(k[name], ref_k[name])


@pytest.mark.parametrize("wave", ["psv", "sh"])
@pytest.mark.parametrize("tile", [6, 8, 10, 13, 15, 17, 19, 20])
def test_march_bulk_loads_identical_to_cp_async(gpu, orc, tile, wave):
    """The marching kernel's bulk tensor loads (nz % 4 == 0) and its per-row
    cp.async staging give the same bits, and match the 2-D tile kernel."""
    case = cases.make_case(wave=wave, nx=133, nz=76, nt=250, nsrc=2, nrec=25, seed=29)
    rng = np.random.default_rng(7)
    ad = {c: (rng.standard_normal((case["nrec"], case["nt"])) * 1e-3).astype(np.float32) for c in "xyz"}

    def run(t, tma):
        cfg, sol = cases.gpu_solver(gpu, case)
        sol.set_option("cluster", 0)
        sol.set_option("tma", tma)
        sol.set_option("tile", t)
        sol.run_forward_batch([0, 1])
        bulk = sol.stats().march_bulk
        tr = {c: sol.out(c, slot=1) for c in comps(wave)}
        for c in comps(wave):
            sol.set_adstf(c, ad[c], slot=0)
            sol.set_adstf(c, ad[c], slot=1)
        sol.initKernels()
        sol.run_adjoint_batch([0, 1])
        return tr, sol.kernels(), bulk

    tr_b, k_b, bulk_b = run(tile, 1)
    tr_c, k_c, bulk_c = run(tile, 0)
    tr_t, k_t, _ = run(1, 1)
    assert bulk_b == 1 and bulk_c == 0
    for c in comps(wave):
        np.testing.assert_array_equal(tr_b[c], tr_c[c])
        np.testing.assert_array_equal(tr_b[c], tr_t[c])
    for name in kernel_names(wave):
        np.testing.assert_array_equal(k_b[name], k_c[name])
        np.testing.assert_array_equal(k_b[name], k_t[name])


@pytest.mark.parametrize("wave", ["psv", "sh"])
@pytest.mark.parametrize("tile", [13, 19])
def test_march_dense_and_duplicate_receivers_identical(gpu, orc, tile, wave):
    """A block of 20x20 receivers (more entries than a tile copies into
    shared memory, so those tiles walk their lists in global memory), sparse
    surface receivers (copied lists, samples gathered in shared memory) and
    duplicated receiver cells (several traces per cell): the marching kernel
    gives the 2-D tile kernel's bits."""
    h = 10.0
    case = cases.make_case(wave=wave, nx=133, nz=76, nt=120, nsrc=2, nrec=1, seed=31, dx=h)
    rec = [[(10 + a) * h, (5 + b) * h] for a in range(20) for b in range(20)]
    rec += [[(40 + 2 * a) * h, 2 * h] for a in range(40)]
    rec += [[(40 + 2 * a) * h, 2 * h] for a in range(0, 40, 7)] + [[12 * h, 7 * h]]
    case["rec"] = rec
    case["nrec"] = len(rec)
    rng = np.random.default_rng(8)
    ad = {c: (rng.standard_normal((case["nrec"], case["nt"])) * 1e-3).astype(np.float32) for c in "xyz"}

    def run(t):
        cfg, sol = cases.gpu_solver(gpu, case)
        sol.set_option("cluster", 0)
        sol.set_option("tile", t)
        sol.run_forward_batch([0, 1])
        tr = {c: sol.out(c, slot=1) for c in comps(wave)}
        for c in comps(wave):
            sol.set_adstf(c, ad[c], slot=0)
            sol.set_adstf(c, ad[c], slot=1)
        sol.initKernels()
        sol.run_adjoint_batch([0, 1])
        return tr, sol.kernels()

    tr_m, k_m = run(tile)
    tr_t, k_t = run(1)
    for c in comps(wave):
        assert np.abs(tr_m[c]).max() > 0
        np.testing.assert_array_equal(tr_m[c], tr_t[c])
    for name in kernel_names(wave):
        np.testing.assert_array_equal(k_m[name], k_t[name])


def test_graphs_and_eager_identical(gpu, orc):
    case = cases.make_case(wave="sh", nx=100, nz=64, nt=300, nsrc=2, nrec=20, seed=19)
    cfg, a = cases.gpu_solver(gpu, case)
    a.set_option("graphs", 0)
    a.set_option("cluster", 0)
    cfg2, b = cases.gpu_solver(gpu, case)
    b.set_option("graphs", 1)
    b.set_option("cluster", 0)
    for s in range(2):
        a.runForward(s)
        b.runForward(s)
        np.testing.assert_array_equal(a.out("y"), b.out("y"))
    rng = np.random.default_rng(0)
    ad = (rng.standard_normal((case["nrec"], case["nt"])) * 1e-3).astype(np.float32)
    for sol in (a, b):
        sol.initKernels()
        sol.set_adstf("y", ad)
        sol.runAdjoint(1)
    np.testing.assert_array_equal(a.kernels()["k_mu"], b.kernels()["k_mu"])


def test_both_wave_systems_in_one_solver(gpu, orc):
    case = cases.make_case(wave="psv", both=True, nx=90, nz=70, nt=300, nsrc=1, nrec=20, seed=23)
    cfg, sol = cases.gpu_solver(gpu, case)
    pb = cases.oracle_problem(orc, case)
    sol.runForward(0)
    o = orc.forward(pb, 0, adj=True)
    for c in "xyz":
        assert cases.rel(sol.out(c), o["xyz".index(c)]) < TRACE_TOL


@pytest.mark.parametrize("wave", ["psv", "sh"])
def test_adjoint_rejects_nt_not_a_multiple_of_sfe(gpu, wave):
    """With nt % sfe != 0 the reference's adjoint pairs its steps with the
    wrong checkpoints and reads slot nsfe, one past its array
    (solver/fdm.h:391,583-584). The library's adjoint refuses such a
    configuration with an error that says why, and the solver stays usable.
    The forward pass runs, and its checkpoint slots stay inside the array."""
    case = cases.make_case(wave=wave, nx=64, nz=48, nt=205, nsrc=1, nrec=8, sfe=10, seed=5)
    cfg, sol = cases.gpu_solver(gpu, case)
    sol.run_forward_batch([0])
    assert np.isfinite(sol.out(comps(wave)[0])).all()
    sol.initKernels()
    with pytest.raises(gpu.GbError, match="multiple of sfe"):
        sol.run_adjoint_batch([0])
    sol.run_forward_batch([0])  # still usable
