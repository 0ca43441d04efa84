"""Serving engine: continuous batching of forward+adjoint requests with
different grids, step counts and wave systems. Each result must be the same
alone and in the mix (bit-identical: the same operations in the same order),
match the CPU oracle, and admission must respect the HBM budget."""
import numpy as np
import pytest

from tests import cases

pytestmark = pytest.mark.gpu


def request(psv, nx, nz, nt, seed, nrec=24):
    case = cases.make_case(wave="psv" if psv else "sh", nx=nx, nz=nz, nt=nt, nsrc=1, nrec=nrec, sfe=10,
                           seed=seed, abs_width=10)
    vp, vs, rho = case["vp"], case["vs"], case["rho"]
    f32 = np.float32
    lam = np.where(vp > vs, (rho * (vp * vp - f32(2) * vs * vs)).astype(f32), f32(0)).astype(f32)
    mu = (rho * vs * vs).astype(f32)
    req = dict(psv=int(psv), nx=nx, nz=nz, dx=10.0, dt=case["dt"], nt=nt, lam=lam, mu=mu, rho=rho,
               src=case["src"][0], rec=np.array(case["rec"], np.float32), abs_width=10)
    return case, req


MIX = [(1, 90, 70, 300, 1), (0, 120, 64, 200, 2), (1, 64, 96, 400, 3), (0, 80, 80, 300, 4),
       (1, 110, 50, 200, 5), (0, 70, 100, 400, 6)]


def test_results_same_alone_and_in_the_mix(gpu):
    reqs = [request(*m)[1] for m in MIX]
    srv = gpu.Server(sfe=10)
    ids = [srv.submit(arrival=0.002 * q, **r) for q, r in enumerate(reqs)]
    srv.run()
    st = srv.stats()
    assert st.completed == len(MIX)
    assert st.max_concurrent >= 3  # requests overlapped on the device
    mix = [srv.result(i) for i in ids]
    for q, r in enumerate(reqs):
        alone = gpu.Server(sfe=10)
        rid = alone.submit(**r)
        alone.run()
        res = alone.result(rid)
        for name in ("k_lambda", "k_mu", "k_rho"):
            np.testing.assert_array_equal(res[name], mix[q][name])
        assert res["misfit"] == mix[q]["misfit"]
        assert np.abs(mix[q]["k_mu"]).max() > 0


@pytest.mark.parametrize("psv", [1, 0])
def test_served_request_matches_oracle(gpu, orc, psv):
    case, req = request(psv, 96, 72, 300, 11)
    pb = cases.oracle_problem(orc, case)
    rng = np.random.default_rng(5)
    comps = "xz" if psv else "y"
    obs = {c: (rng.standard_normal((pb.nrec, pb.nt)) * 1e-9).astype(np.float32) for c in comps}
    srv = gpu.Server(sfe=10)
    rid = srv.submit(obs=np.stack([obs[c] for c in comps]), **req)
    srv.run()
    res = srv.result(rid)
    o = orc.forward(pb, 0, adj=True)
    tw = orc.taper(pb.nt, case["dt"])
    ad = {c: np.zeros((pb.nrec, pb.nt), np.float32) for c in "xyz"}
    total = 0.0
    for c in comps:
        v, ad[c] = orc.waveform_misfit(o["xyz".index(c)], obs[c], tw, case["dt"])
        total += v
    kern = orc.adjoint(pb, [ad["x"], ad["y"], ad["z"]], o[3])
    assert abs(res["misfit"] - total) / total < 1e-4
    names = ("k_lambda", "k_mu", "k_rho") if psv else ("k_mu", "k_rho")
    for name in names:
        ref = kern[("k_lambda", "k_mu", "k_rho").index(name)]
        assert cases.rel(res[name], ref) < 1e-4, name


def test_admission_waits_for_memory(gpu):
    reqs = [request(1, 100, 80, 300, 20 + q)[1] for q in range(4)]
    # each request needs about 5 MB (mostly checkpoints); 7 MB admits one at a time
    srv = gpu.Server(sfe=10, hbm_budget_gb=0.007)
    ids = [srv.submit(**r) for r in reqs]
    srv.run()
    st = srv.stats()
    assert st.completed == 4 and st.max_concurrent == 1
    free = gpu.Server(sfe=10)
    fid = [free.submit(**r) for r in reqs]
    free.run()
    assert free.stats().max_concurrent == 4
    for a, b in zip(ids, fid):
        np.testing.assert_array_equal(srv.result(a)["k_mu"], free.result(b)["k_mu"])


def test_bulk_loads_and_pitch_identical_to_per_row_loads(gpu):
    """Requests of any nz are stored at a pitch of nz rounded up to a
    multiple of 4 so that the marching kernel can load their columns with
    bulk tensor copies: the kernels and misfits are bit-identical to those
    of per-row cp.async loads (pitch unchanged there as well), to the 2-D
    tile kernel's, which keeps the reference layout, to runs with all
    steps on one stream and with the SH steps on one stream beside the P-SV
    ones (the default splits each system's requests over two streams), and
    to a run that launches the largest
    request's tile count for every request instead of a block map of the
    requests' own tiles."""
    mix = MIX + [(1, 77, 61, 200, 7), (0, 95, 33, 200, 8)]
    reqs = [request(*m)[1] for m in mix]
    out = []
    for opts in ({}, {"tma": 0}, {"tile": 3}, {"streams": 1}, {"streams": 2}, {"compact": 0}):
        srv = gpu.Server(sfe=10)
        for k, v in opts.items():
            srv.set_option(k, v)
        ids = [srv.submit(arrival=0.0, **r) for r in reqs]
        srv.run()
        out.append([srv.result(i) for i in ids])
    for other in out[1:]:
        for a, b in zip(out[0], other):
            for name in ("k_lambda", "k_mu", "k_rho"):
                np.testing.assert_array_equal(a[name], b[name])
            assert a["misfit"] == b["misfit"]


def test_served_request_with_odd_nz_matches_oracle(gpu, orc):
    case, req = request(1, 83, 69, 200, 13)
    pb = cases.oracle_problem(orc, case)
    rng = np.random.default_rng(6)
    obs = {c: (rng.standard_normal((pb.nrec, pb.nt)) * 1e-9).astype(np.float32) for c in "xz"}
    srv = gpu.Server(sfe=10)
    rid = srv.submit(obs=np.stack([obs[c] for c in "xz"]), **req)
    srv.run()
    res = srv.result(rid)
    o = orc.forward(pb, 0, adj=True)
    tw = orc.taper(pb.nt, case["dt"])
    ad = {c: np.zeros((pb.nrec, pb.nt), np.float32) for c in "xyz"}
    for c in "xz":
        _, ad[c] = orc.waveform_misfit(o["xyz".index(c)], obs[c], tw, case["dt"])
    kern = orc.adjoint(pb, [ad["x"], ad["y"], ad["z"]], o[3])
    for q, name in enumerate(("k_lambda", "k_mu", "k_rho")):
        assert cases.rel(res[name], kern[q]) < 1e-4, name


def test_many_completions_share_the_pinned_result_buffers(gpu):
    """Finished requests' kernels are copied out through a pool of eight
    pinned buffers and finalised when their copies complete; with twenty
    requests of different lengths in flight, completions outnumber the
    buffers and some wait for a buffer to be finalised. Every result is
    bit-identical to the same request served one at a time, and latencies
    (completion time from the copies' event) are ordered with the requests'
    lengths at equal arrival."""
    mix = [(q % 2, 48 + 8 * (q % 5), 40 + 4 * (q % 3), 100 + 20 * (q % 4), 40 + q) for q in range(20)]
    reqs = [request(*m, nrec=8)[1] for m in mix]
    srv = gpu.Server(sfe=10)
    ids = [srv.submit(arrival=0.0, **r) for r in reqs]
    srv.run()
    st = srv.stats()
    assert st.completed == len(reqs) and st.max_concurrent == len(reqs)
    together = [srv.result(i) for i in ids]
    one = gpu.Server(sfe=10, max_slots=1)
    ids1 = [one.submit(arrival=0.0, **r) for r in reqs]
    one.run()
    for q, i in enumerate(ids1):
        res = one.result(i)
        for name in ("k_lambda", "k_mu", "k_rho"):
            np.testing.assert_array_equal(res[name], together[q][name])
        assert res["misfit"] == together[q]["misfit"]
    # all admitted at t = 0 and advanced in lockstep: a request with fewer
    # steps never finishes after one with more
    lat = [r["latency"] for r in together]
    nts = [r["nt"] for r in reqs]
    for a in range(len(reqs)):
        for b in range(len(reqs)):
            if nts[a] < nts[b]:
                assert lat[a] <= lat[b]
