"""The CPU oracle against the reference's only known-answer data: the SH
velocity seismograms of example/checker (tests/golden/checker_golden.npz,
made by tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "checker_golden.npz")


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLD)


def checker_problem(orc, g):
    cfg = orc.Config(path="")
    for k, v in zip(g["cfg_keys"], g["cfg_vals"]):
        cfg.f[str(k)] = float(v)
        cfg.i[str(k)] = int(np.floor(abs(v) + 0.5)) * (1 if v >= 0 else -1)
    nx, nz, dx, dz, xmax, zmax = orc.infer_grid(g["true_x"], g["true_z"])
    lam, mu, rho = orc.mesh2grid(nx, nz, dx, dz, g["true_x"], g["true_z"], g["true_vp"], g["true_vs"],
                                 g["true_rho"], xmax, zmax)
    lam, mu = orc.vps2lm(lam, mu, rho)
    src, rec = g["src"], g["rec"]
    nt, dt = cfg.iv("nt"), cfg.fv("dt")
    stf = [np.zeros(len(src) * nt, np.float32) for _ in range(3)]
    for s in range(len(src)):
        c = orc.ricker(nt, dt, *src[s, 3:7])
        for q in range(3):
            stf[q][s * nt:(s + 1) * nt] = c[q]
    ab = orc.absbound(nx, nz, cfg.iv("abs_width"), cfg.fv("abs_alpha"), cfg.iv("abs_left"),
                      cfg.iv("abs_right"), cfg.iv("abs_bottom"), cfg.iv("abs_top"))
    return cfg, orc.Problem(nx=nx, nz=nz, nt=nt, dx=dx, dz=dz, dt=dt, sh=True, psv=False, sfe=cfg.iv("sfe"),
                            lam=lam, mu=mu, rho=rho, ab=ab, stf=tuple(stf),
                            src_id=(orc.calc_idx(src[:, 0], xmax, nx), orc.calc_idx(src[:, 1], zmax, nz)),
                            rec_id=(orc.calc_idx(rec[:, 0], xmax, nx), orc.calc_idx(rec[:, 1], zmax, nz)))


def test_grid_inference(orc, golden):
    nx, nz, dx, dz, xmax, zmax = orc.infer_grid(golden["true_x"], golden["true_z"])
    assert (nx, nz, dx, dz) == (201, 201, 2400.0, 2400.0)


@pytest.mark.parametrize("k", [0, 1, 2])
def test_forward_sh_matches_golden(orc, golden, k):
    cfg, pb = checker_problem(orc, golden)
    shot = int(golden["golden_shots"][k])
    pb.rec_id = tuple(a[golden["golden_recs"]] for a in pb.rec_id)
    _, vy, _, _ = orc.forward(pb, shot, adj=False)
    ref = golden["golden_vy"][k]
    err = np.linalg.norm(vy - ref) / np.linalg.norm(ref)
    # FP32 round-off between the reference's GPU build and the C oracle
    assert err < 1e-5, err
    per_trace = np.linalg.norm(vy - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert per_trace.max() < 1e-5


def test_su_headers_match_golden(orc, golden):
    cfg, pb = checker_problem(orc, golden)
    src, rec = golden["src"], golden["rec"]
    for k, shot in enumerate(golden["golden_shots"]):
        heads = orc.su_headers(len(rec), cfg.iv("nt"), cfg.fv("dt"), src[shot, 0], src[shot, 1], rec[:, 0],
                               rec[:, 1])
        for q, r in enumerate(golden["golden_recs"]):
            assert heads[r] == golden["golden_heads"][k, q].tobytes()


def test_fp64_oracle_close_to_golden(orc, golden):
    cfg, pb = checker_problem(orc, golden)
    pb.rec_id = tuple(a[golden["golden_recs"]] for a in pb.rec_id)
    _, vy, _, _ = orc.forward(pb, 0, adj=False, precision="f64")
    ref = golden["golden_vy"][0]
    assert np.linalg.norm(vy - ref) / np.linalg.norm(ref) < 1e-5
