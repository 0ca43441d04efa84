"""Cluster-resident passes (a whole forward or adjoint pass per shot inside
one thread-block cluster, state in distributed shared memory) against the
per-step kernels and the CPU oracle."""
import numpy as np
import pytest

from tests import cases

pytestmark = pytest.mark.gpu


def comps(wave):
    return "xz" if wave == "psv" else "y"


def names(wave):
    return ("k_lambda", "k_mu", "k_rho") if wave == "psv" else ("k_mu", "k_rho")


def run(gpu, case, cluster, ad):
    cfg, sol = cases.gpu_solver(gpu, case)
    sol.set_option("cluster", cluster)
    shots = list(range(case["nsrc"]))
    sol.run_forward_batch(shots)
    tr = [{c: sol.out(c, slot=b) for c in comps(case["wave"])} for b in shots]
    st = sol.stats()
    for b in shots:
        for c in comps(case["wave"]):
            sol.set_adstf(c, ad[b][c], slot=b)
    sol.initKernels()
    sol.run_adjoint_batch(shots)
    return tr, sol.kernels(), st


@pytest.mark.parametrize("wave,nx,nz,nt", [("sh", 681, 141, 400), ("psv", 200, 200, 300), ("sh", 97, 61, 300),
                                           ("psv", 150, 110, 300)])
def test_cluster_pass_matches_step_kernels(gpu, orc, wave, nx, nz, nt):
    case = cases.make_case(wave=wave, nx=nx, nz=nz, nt=nt, nsrc=3, nrec=min(nx - 4, 60), sfe=10, seed=nx)
    rng = np.random.default_rng(nz)
    ad = [{c: (rng.standard_normal((case["nrec"], nt)) * 1e-3).astype(np.float32) for c in "xyz"}
          for _ in range(3)]
    tr_c, k_c, st_c = run(gpu, case, 1, ad)
    tr_t, k_t, st_t = run(gpu, case, 0, ad)
    assert st_c.tile_tz < 0, "the cluster path did not run"
    assert st_t.tile_tz > 0
    for b in range(3):
        for c in comps(wave):
            np.testing.assert_array_equal(tr_c[b][c], tr_t[b][c])
    for n in names(wave):
        # the cluster pass sums each shot's contribution separately
        assert cases.rel(k_c[n], k_t[n]) < 1e-6, n


@pytest.mark.parametrize("wave,nx,size", [("psv", 94, 1), ("psv", 94, 2), ("psv", 94, 3), ("psv", 94, 5),
                                          ("psv", 94, 8), ("psv", 94, 12), ("psv", 50, 4), ("sh", 94, 1),
                                          ("sh", 94, 4), ("sh", 94, 12), ("sh", 50, 4)])
def test_cluster_sizes_match_step_kernels(gpu, orc, wave, nx, size):
    """Cluster sizes (1 = automatic); 94 columns at 12 CTAs leave the last CTA
    6 columns, 50 at 4 CTAs (16 columns each) leave it 2. Receivers are
    scattered over the grid: several per thread, per CTA and at CTA edges."""
    nz, nt = 40, 150
    case = cases.make_case(wave=wave, nx=nx, nz=nz, nt=nt, nsrc=2, nrec=60, sfe=10, seed=size)
    rng = np.random.default_rng(size)
    cells = rng.choice(nx * nz, 60, replace=False)
    case["rec"] = [[float(c // nz) * 10.0, float(c % nz) * 10.0] for c in cells]
    ad = [{c: (rng.standard_normal((60, nt)) * 1e-3).astype(np.float32) for c in "xyz"} for _ in range(2)]
    tr_c, k_c, st_c = run(gpu, case, size, ad)
    tr_t, k_t, st_t = run(gpu, case, 0, ad)
    if size == 1:  # automatic size
        assert st_c.tile_tz < 0, "the cluster path did not run"
    else:
        assert st_c.tile_tz == -size, "the cluster path did not run with this size"
    for b in range(2):
        for c in comps(wave):
            np.testing.assert_array_equal(tr_c[b][c], tr_t[b][c])
    for n in names(wave):
        assert cases.rel(k_c[n], k_t[n]) < 1e-6, n


@pytest.mark.parametrize("wave,nx,nz", [("sh", 681, 141), ("psv", 150, 110)])
def test_cluster_adjoint_shared_memory_options_identical(gpu, orc, wave, nx, nz):
    """The adjoint's kernel accumulation gives the same bits whether each
    checkpoint is staged in shared memory or read from HBM, and whether the
    shot's kernels are accumulated in shared memory or in an HBM buffer."""
    case = cases.make_case(wave=wave, nx=nx, nz=nz, nt=200, nsrc=2, nrec=min(nx - 4, 60), sfe=10, seed=nz)
    rng = np.random.default_rng(3)
    ad = [{c: (rng.standard_normal((case["nrec"], 200)) * 1e-3).astype(np.float32) for c in "xyz"}
          for _ in range(2)]
    out, used = [], set()
    for stage, kacc in ((1, 1), (1, 0), (0, 1), (0, 0)):
        cfg, sol = cases.gpu_solver(gpu, case)
        sol.set_option("cluster_snap", 0)  # the in-pass accumulation's options
        sol.set_option("cluster_stage", stage)
        sol.set_option("cluster_kacc", kacc)
        shots = [0, 1]
        sol.run_forward_batch(shots)
        for b in shots:
            for c in comps(wave):
                sol.set_adstf(c, ad[b][c], slot=b)
        sol.initKernels()
        sol.run_adjoint_batch(shots)
        st = sol.stats()
        assert st.tile_tz < 0
        assert st.cluster_adj & ~(stage | 2 * kacc) == 0
        used.add(st.cluster_adj)
        out.append(sol.kernels())
        sol.close()
    assert 2 in used or 3 in used, "no pass accumulated its kernels in shared memory"
    assert 0 in used
    for o in out[1:]:
        for n in names(wave):
            np.testing.assert_array_equal(o[n], out[0][n])


@pytest.mark.parametrize("wave,nx,nz", [("sh", 681, 141), ("psv", 200, 200), ("sh", 94, 40)])
def test_cluster_row_shift_identical(gpu, orc, wave, nx, nz):
    """The row-shifted shared-memory layout (no bank conflicts) gives the same
    seismograms and kernels, bit for bit, as the unshifted one, with the
    kernels accumulated in shared memory or in HBM."""
    case = cases.make_case(wave=wave, nx=nx, nz=nz, nt=200, nsrc=2, nrec=min(nx - 4, 60), sfe=10, seed=nx + nz)
    rng = np.random.default_rng(5)
    ad = [{c: (rng.standard_normal((case["nrec"], 200)) * 1e-3).astype(np.float32) for c in "xyz"}
          for _ in range(2)]
    out, shifts = [], []
    for shift, kacc in ((1, 1), (1, 0), (0, 1)):
        cfg, sol = cases.gpu_solver(gpu, case)
        sol.set_option("cluster_shift", shift)
        sol.set_option("cluster_snap", 0)
        sol.set_option("cluster_kacc", kacc)
        shots = [0, 1]
        sol.run_forward_batch(shots)
        st = sol.stats()
        assert st.tile_tz < 0
        shifts.append(st.cluster_shift)
        tr = [{c: sol.out(c, slot=b) for c in comps(wave)} for b in shots]
        for b in shots:
            for c in comps(wave):
                sol.set_adstf(c, ad[b][c], slot=b)
        sol.initKernels()
        sol.run_adjoint_batch(shots)
        out.append((tr, sol.kernels()))
        sol.close()
    # 94x40 may get a geometry whose groups need no shift
    assert (shifts[0] != 0 or (nx, nz) == (94, 40)) and shifts[2] == 0
    for tr, k in out[1:]:
        for b in range(2):
            for c in comps(wave):
                np.testing.assert_array_equal(tr[b][c], out[0][0][b][c])
        for n in names(wave):
            np.testing.assert_array_equal(k[n], out[0][1][n])


@pytest.mark.parametrize("wave,nx,nz", [("sh", 681, 141), ("psv", 200, 200), ("psv", 94, 40)])
def test_cluster_adjoint_after_pass_identical(gpu, orc, wave, nx, nz):
    """Kernels accumulated after the pass from the stored adjoint state equal,
    bit for bit, those accumulated inside the pass (in shared memory or in
    HBM), and the forward seismograms are unchanged."""
    case = cases.make_case(wave=wave, nx=nx, nz=nz, nt=210, nsrc=3, nrec=min(nx - 4, 60), sfe=10, seed=nx - nz)
    rng = np.random.default_rng(9)
    ad = [{c: (rng.standard_normal((case["nrec"], 210)) * 1e-3).astype(np.float32) for c in "xyz"}
          for _ in range(3)]
    out, flags = [], []
    for snap, kacc in ((1, 1), (0, 1), (0, 0)):
        cfg, sol = cases.gpu_solver(gpu, case)
        sol.set_option("cluster_snap", snap)
        sol.set_option("cluster_kacc", kacc)
        shots = [0, 1, 2]
        sol.run_forward_batch(shots)
        tr = [{c: sol.out(c, slot=b) for c in comps(wave)} for b in shots]
        for b in shots:
            for c in comps(wave):
                sol.set_adstf(c, ad[b][c], slot=b)
        sol.initKernels()
        sol.run_adjoint_batch(shots)
        st = sol.stats()
        assert st.tile_tz < 0
        flags.append(st.cluster_adj)
        out.append((tr, sol.kernels()))
        sol.close()
    assert flags[0] & 4 and not flags[1] & 4 and not flags[2] & 4
    for tr, k in out[1:]:
        for b in range(3):
            for c in comps(wave):
                np.testing.assert_array_equal(tr[b][c], out[0][0][b][c])
        for n in names(wave):
            np.testing.assert_array_equal(k[n], out[0][1][n])


def test_cluster_adjoint_matches_oracle(gpu, orc):
    case = cases.make_case(wave="psv", nx=120, nz=96, nt=400, nsrc=2, nrec=40, sfe=10, seed=11)
    pb = cases.oracle_problem(orc, case)
    rng = np.random.default_rng(2)
    ad = [{c: (rng.standard_normal((pb.nrec, pb.nt)) * 1e-3).astype(np.float32) for c in "xyz"} for _ in range(2)]
    tr, k, st = run(gpu, case, 1, ad)
    assert st.tile_tz < 0
    kern = None
    for s in range(2):
        o = orc.forward(pb, s, adj=True)
        for c in "xz":
            assert cases.rel(tr[s][c], o["xyz".index(c)]) < 1e-5
        kern = orc.adjoint(pb, [ad[s]["x"], ad[s]["y"], ad[s]["z"]], o[3], kern)
    for q, n in enumerate(("k_lambda", "k_mu", "k_rho")):
        assert cases.rel(k[n], kern[q]) < 1e-4, n


def test_cluster_falls_back_for_16bit_checkpoints(gpu, orc):
    case = cases.make_case(wave="sh", nx=100, nz=60, nt=200, nsrc=1, nrec=20, seed=3)
    cfg, sol = cases.gpu_solver(gpu, case)
    sol.set_option("ckpt", 2)
    sol.run_forward_batch([0])
    assert sol.stats().tile_tz > 0
