"""The drop-in command line (gbinv) on the reference's checker example.

The example directory is rebuilt from tests/golden/checker_golden.npz
(config values, sources, stations, model_true/model_init point files), so the
tests need no reference checkout. Mode 3 must reproduce the reference's
golden seismograms; modes 0, 1, 2 and 5 must write the reference's output
files with the reference's stdout lines.
"""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "checker_golden.npz")


def write_checker(d, orc, nsrc=None, extra=None):
    g = np.load(GOLD)
    os.makedirs(os.path.join(d, "model_true"), exist_ok=True)
    os.makedirs(os.path.join(d, "model_init"), exist_ok=True)
    vals = {str(k): float(v) for k, v in zip(g["cfg_keys"], g["cfg_vals"])}
    vals.update(extra or {})
    with open(os.path.join(d, "config.ini"), "w") as fh:
        for k, v in vals.items():
            fh.write("%s = %s\n" % (k, repr(v)))
    src = g["src"] if nsrc is None else g["src"][:nsrc]
    with open(os.path.join(d, "sources.dat"), "w") as fh:
        fh.write("# x | z | type | f0 | t0 | angle | amp\n")
        for s in src:
            fh.write(" ".join(repr(float(v)) for v in s) + "\n")
    with open(os.path.join(d, "stations.dat"), "w") as fh:
        for r in g["rec"]:
            fh.write("%r %r\n" % (float(r[0]), float(r[1])))
    for c in ("x", "z", "vp", "vs", "rho"):
        orc.write_bin(os.path.join(d, "model_true", "proc000000_%s.bin" % c), g["true_" + c])
        orc.write_bin(os.path.join(d, "model_init", "proc000000_%s.bin" % c), g["init_" + c])
    return g


def gbinv(pkg, d, *args, timeout=600):
    r = subprocess.run([pkg.GBINV_PATH, d] + list(args), capture_output=True, text=True, timeout=timeout)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def test_mode3_reproduces_golden_seismograms(gpu, orc, tmp_path):
    d = str(tmp_path / "checker")
    g = write_checker(d, orc)
    gbinv(gpu, d, "-mode=3")
    recs = g["golden_recs"]
    for k, shot in enumerate(g["golden_shots"]):
        tr, heads = orc.read_su(os.path.join(d, "output", "vy_%06d.su" % shot))
        assert tr.shape == (132, 5000)
        ref = g["golden_vy"][k]
        got = tr[recs]
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-5
        for q, r in enumerate(recs):
            assert heads[r].tobytes() == g["golden_heads"][k, q].tobytes()


def test_mode5_exports_model_and_axis(gpu, orc, tmp_path):
    d = str(tmp_path / "checker")
    g = write_checker(d, orc)
    gbinv(gpu, d, "-mode=5")
    out = os.path.join(d, "output")
    x = orc.read_bin(os.path.join(out, "proc000000_x.bin"))
    z = orc.read_bin(os.path.join(out, "proc000000_z.bin"))
    assert x.size == z.size == 201 * 201
    assert x[201 * 5] == 5 * 2400.0 and z[7] == 7 * 2400.0
    vs = orc.read_bin(os.path.join(out, "proc000000_vs.bin")).reshape(201, 201)
    ref = g["true_vs"].reshape(201, 201).T  # model points are x-fastest, the grid z-fastest
    assert np.abs(vs - ref).max() / ref.max() < 1e-6
    # vp is exported only when both lambda and mu are inverted (solver/fdm.h:484)
    assert not os.path.exists(os.path.join(out, "proc000000_vp.bin"))


def test_mode2_kernel_matches_oracle(gpu, orc, tmp_path):
    d = str(tmp_path / "checker")
    write_checker(d, orc, nsrc=3, extra={"nt": 600.0})
    gbinv(gpu, d, "-mode=2")
    k_mu = orc.read_bin(os.path.join(d, "output", "proc000000_k_mu.bin"))
    cfg = orc.Config.load(d)
    true = orc.problem_from_config(cfg, "model_true")
    init = orc.problem_from_config(cfg, "model_init")
    kern = None
    for s in range(3):
        obs = orc.forward(true, s, adj=True)[1]
        syn, ck = orc.forward(init, s, adj=True)[1], orc.forward(init, s, adj=True)[3]
        _, ad = orc.envelope_misfit(syn, obs, cfg.fv("dt"))
        z = np.zeros_like(ad)
        kern = orc.adjoint(init, [z, ad, z], ck, kern)
    ref = orc.gaussian_filter(init.nx, init.nz, cfg.iv("filter_sigma"), kern[1])
    assert np.linalg.norm(k_mu - ref) / np.linalg.norm(ref) < 1e-4


def test_mode0_inversion_writes_iterations(gpu, orc, tmp_path):
    d = str(tmp_path / "checker")
    write_checker(d, orc, nsrc=3, extra={"nt": 600.0, "inv_iteration": 2.0})
    out = gbinv(gpu, d, "-mode=0")
    assert "Generating traces" in out
    assert "Starting iteration 1 / 2" in out and "Starting iteration 2 / 2" in out
    assert "  step 00  misfit = 1" in out
    assert "Final misfit: " in out and "Elapsed time: " in out
    final = float(out.split("Final misfit: ")[1].split()[0])
    assert 0 < final < 1
    for n in (1, 2):
        assert os.path.exists(os.path.join(d, "output", "proc%06d_vs.bin" % n))
        assert os.path.exists(os.path.join(d, "output", "proc%06d_k_mu.bin" % n))


def test_mode0_lbfgs_and_nlcg_both_reduce_misfit(gpu, orc, tmp_path):
    for opt in (0, 1):
        d = str(tmp_path / ("opt%d" % opt))
        write_checker(d, orc, nsrc=3, extra={"nt": 600.0, "inv_iteration": 3.0, "optimizer": float(opt),
                                             "misfit": 0.0})
        out = gbinv(gpu, d, "-mode=0")
        final = float(out.split("Final misfit: ")[1].split()[0])
        assert 0 < final < 1, out


def test_mode1_writes_snapshots_and_supershot_traces(gpu, orc, tmp_path):
    d = str(tmp_path / "checker")
    write_checker(d, orc, nsrc=3, extra={"nt": 400.0, "wfe": 200.0})
    gbinv(gpu, d, "-mode=1")
    out = os.path.join(d, "output")
    for it in (200, 400):
        snap = orc.read_bin(os.path.join(out, "proc%06d_vy.bin" % it))
        assert snap.size == 201 * 201 and np.isfinite(snap).all() and np.abs(snap).max() > 0
    tr, _ = orc.read_su(os.path.join(out, "vy_000000.su"))
    assert tr.shape == (132, 400)


@pytest.mark.parametrize("mode,key", [(1, "wfe"), (2, "wae")])
def test_async_snapshots_equal_blocking_ones(gpu, orc, tmp_path, mode, key):
    """Wavefield snapshots through the asynchronous writer (default) and
    through a blocking copy per field (snap_async = 0) give the same files,
    byte for byte, and all of them exist when the command returns: mode 1
    (forward, every wfe steps) and mode 2 (adjoint, every wae steps)."""
    files = {}
    for snap_async in (1, 0):
        d = str(tmp_path / ("m%d_a%d" % (mode, snap_async)))
        write_checker(d, orc, nsrc=2, extra={"nt": 400.0, key: 50.0})
        gbinv(gpu, d, "-mode=%d" % mode, "-snap_async=%d" % snap_async)
        out = os.path.join(d, "output")
        names = sorted(f for f in os.listdir(out) if f.startswith("proc") and f.endswith(".bin")
                       and f.split("_", 1)[1][:2] in ("vx", "vy", "vz", "ux", "uy", "uz"))
        files[snap_async] = {f: open(os.path.join(out, f), "rb").read() for f in names}
    assert len(files[1]) >= 8, sorted(files[1])
    assert files[1].keys() == files[0].keys()
    for f in files[1]:
        assert files[1][f] == files[0][f], f
