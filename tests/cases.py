"""Seeded synthetic problems shared by the GPU parity tests, the smoke check
and the benchmark's small cases.

A case is a plain dict (grid, time axis, config values, sources, stations
and the model on the grid). `gpu_solver` builds the library's solver from
it through the C ABI; `oracle_problem` builds the CPU oracle's problem from
the same numbers, so both sides see identical inputs.
"""
from __future__ import annotations

import math

import numpy as np


def layered_model(nx, nz, seed, vs_top=1700.0, vs_bottom=2300.0, nlayer=6, faults=1, jitter=0.03):
    """vp, vs, rho (float32, reference layout k = i*nz + j) of a layered model
    with dipping faults and a small random perturbation; vp = 1.73 vs,
    rho = 310 vp^0.25 (Gardner)."""
    rng = np.random.default_rng(seed)
    ii, jj = np.meshgrid(np.arange(nx), np.arange(nz), indexing="ij")
    depth = jj.astype(np.float64)
    for _ in range(faults):
        x0 = rng.uniform(0.2, 0.8) * nx
        dip = rng.uniform(0.3, 1.0)
        throw = rng.uniform(0.05, 0.15) * nz
        depth = depth + np.where(ii + (jj - nz / 2) * dip > x0, throw, 0.0)
    layer = np.clip((depth / nz * nlayer).astype(int), 0, nlayer - 1)
    vs_l = np.linspace(vs_top, vs_bottom, nlayer)
    vs = vs_l[layer] * (1 + jitter * rng.standard_normal((nx, nz)))
    vp = 1.73 * vs
    rho = 310.0 * vp ** 0.25
    f = lambda a: np.ascontiguousarray(a.astype(np.float32).ravel())
    return f(vp), f(vs), f(rho)


def make_case(wave="psv", nx=120, nz=100, nt=600, nsrc=2, nrec=40, sfe=10, seed=0, dx=10.0, dt=1e-3,
              f0=12.0, angle=math.pi / 4, amp=1e9, abs_width=12, model=None, both=False):
    xmax = (nx - 1) * dx
    zmax = (nz - 1) * dx
    if model is None:
        vp, vs, rho = layered_model(nx, nz, seed)
    else:
        vp, vs, rho = model
    src = [[xmax * (0.2 + 0.6 * (s + 0.5) / nsrc), 3 * dx, 0, f0, 1.2 / f0, angle, amp] for s in range(nsrc)]
    rec = [[xmax * (0.05 + 0.9 * r / max(nrec - 1, 1)), 2 * dx] for r in range(nrec)]
    values = {
        "mode": 2, "sh": int(wave == "sh" or both), "psv": int(wave == "psv" or both), "nt": nt, "dt": dt,
        "sfe": sfe, "model_type": 0, "trace_type": 0,
        "abs_left": 1, "abs_right": 1, "abs_bottom": 1, "abs_top": 0, "abs_width": abs_width,
        "abs_alpha": 0.015, "inv_lambda": 1, "inv_mu": 1, "inv_rho": 1,
    }
    return dict(wave=wave, nx=nx, nz=nz, nt=nt, nsrc=nsrc, nrec=nrec, sfe=sfe, xmax=xmax, zmax=zmax,
                values=values, src=src, rec=rec, vp=vp, vs=vs, rho=rho, dt=dt)


def checkerboard_case(nt=2000, nsrc=4):
    """The 200 x 200 P-SV checkerboard at 10 m, dt 1 ms: vp 3000, vs 1732,
    rho 2600 with a +-5 % checkerboard of 20-cell squares on vp and vs, four
    vertical-force Ricker sources (f0 10 Hz, t0 0.12 s) evenly spaced at 20 m
    depth, one receiver per column. Sources and receivers sit two cells deep:
    the reference's derivative guards (solver/fdm.h:76-136) leave row 0
    uncoupled, so a receiver at z = 0 records exact zeros."""
    nx = nz = 200
    h = 10.0
    ii, jj = np.meshgrid(np.arange(nx), np.arange(nz), indexing="ij")
    sign = np.where(((ii // 20) + (jj // 20)) % 2 == 0, 1.0, -1.0)
    f = lambda a: np.ascontiguousarray(a.astype(np.float32).ravel())
    vp, vs = f(3000.0 * (1 + 0.05 * sign)), f(1732.0 * (1 + 0.05 * sign))
    rho = np.full(nx * nz, 2600.0, np.float32)
    case = make_case(wave="psv", nx=nx, nz=nz, nt=nt, nsrc=nsrc, dx=h, dt=1e-3, f0=10.0, abs_width=20, sfe=10,
                     model=(vp, vs, rho), angle=math.pi / 2, amp=1e10)
    xmax = case["xmax"]
    case["src"] = [[xmax * (s + 0.5) / nsrc, 2 * h, 0, 10.0, 0.12, math.pi / 2, 1e10] for s in range(nsrc)]
    case["rec"] = [[i * h, 2 * h] for i in range(nx)]
    case["nrec"] = nx
    return case


def smooth_field(nx, nz, cells, rng):
    """A seeded random field smoothed by a separable Gaussian of `cells`
    cells, scaled to [0, 1] (float32, reference layout)."""
    a = rng.standard_normal((nx, nz))
    r = int(3 * cells)
    w = np.exp(-0.5 * (np.arange(-r, r + 1) / cells) ** 2)
    w /= w.sum()
    pad = np.pad(a, r, mode="wrap")
    t = sum(w[q] * pad[q:q + nx, :] for q in range(2 * r + 1))
    t = sum(w[q] * t[:, q:q + nz] for q in range(2 * r + 1))
    t = (t - t.min()) / (t.max() - t.min())
    return np.ascontiguousarray(t.astype(np.float32).ravel())


def random_smooth_case(nx=2048, nz=1024, nt=6000, nsrc=64, seed=7, cells=30.0):
    """The P-SV precision-study configuration: 5 m cells, dt 0.4 ms,
    checkpoints every 50 steps, a smooth random model with vp 2000-4500 m/s
    and vp/vs 1.7-2.0 (Gardner density), f0 15 Hz vertical-force sources at
    20 m depth, a receiver every 4th column at 10 m depth."""
    rng = np.random.default_rng(seed)
    vp = (2000.0 + 2500.0 * smooth_field(nx, nz, cells, rng)).astype(np.float32)
    vs = (vp / (1.7 + 0.3 * smooth_field(nx, nz, cells, rng))).astype(np.float32)
    rho = (310.0 * vp ** 0.25).astype(np.float32)
    h = 5.0
    case = make_case(wave="psv", nx=nx, nz=nz, nt=nt, nsrc=nsrc, dx=h, dt=4e-4, f0=15.0, abs_width=20, sfe=50,
                     model=(vp, vs, rho), angle=math.pi / 2, amp=1e10)
    xmax = case["xmax"]
    case["src"] = [[xmax * (s + 0.5) / nsrc, 4 * h, 0, 15.0, 0.08, math.pi / 2, 1e10] for s in range(nsrc)]
    case["rec"] = [[i * 4 * h, 2 * h] for i in range(nx // 4)]
    case["nrec"] = len(case["rec"])
    return case


def fp64_gradient(orc, pb, obs, tw, wave):
    """Kernels of the waveform misfit from the oracle's FP64 forward and
    adjoint, the adjoint source 2 r tw (r = (syn - obs) tw, time-reversed,
    misfit/waveform.h:4-40) formed in double."""
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


def lame(orc, case):
    """lambda, mu from vp, vs, rho with the oracle's vps2lm (float)."""
    lam, mu = orc.vps2lm(case["vp"], case["vs"], case["rho"])
    return lam, mu, case["rho"]


def gpu_solver(pkg, case, directory=".", extra=None):
    values = dict(case["values"])
    values.update(extra or {})
    cfg = pkg.Config.new(directory, values, case["src"], case["rec"])
    sol = pkg.FdmSolver(cfg, grid=(case["nx"], case["nz"], case["xmax"], case["zmax"]))
    vp, vs, rho = case["vp"], case["vs"], case["rho"]
    # the same float arithmetic as vps2lm (solver/fdm.h:25-36)
    lam = (rho * (vp * vp - np.float32(2) * vs * vs)).astype(np.float32)
    lam = np.where(vp > vs, lam, np.float32(0)).astype(np.float32)
    mu = (rho * vs * vs).astype(np.float32)
    sol.set_model_grid(lam, mu, rho)
    return cfg, sol


def oracle_problem(orc, case, lam_mu_rho=None):
    f32 = np.float32
    nx, nz, nt = case["nx"], case["nz"], case["nt"]
    xmax, zmax = f32(case["xmax"]), f32(case["zmax"])
    dx = float(xmax / f32(nx - 1))
    dz = float(zmax / f32(nz - 1))
    v = case["values"]
    if lam_mu_rho is None:
        vp, vs, rho = case["vp"], case["vs"], case["rho"]
        lam = (rho * (vp * vp - f32(2) * vs * vs)).astype(f32)
        lam = np.where(vp > vs, lam, f32(0)).astype(f32)
        mu = (rho * vs * vs).astype(f32)
    else:
        lam, mu, rho = lam_mu_rho
    src = np.array(case["src"], f32).reshape(-1, 7)
    rec = np.array(case["rec"], f32).reshape(-1, 2)
    stf = [np.zeros(len(src) * nt, f32) for _ in range(3)]
    for s in range(len(src)):
        c = orc.ricker(nt, v["dt"], src[s, 3], src[s, 4], src[s, 5], src[s, 6])
        for q in range(3):
            stf[q][s * nt:(s + 1) * nt] = c[q]
    ab = orc.absbound(nx, nz, v["abs_width"], v["abs_alpha"], v["abs_left"], v["abs_right"], v["abs_bottom"],
                      v["abs_top"])
    return orc.Problem(nx=nx, nz=nz, nt=nt, dx=dx, dz=dz, dt=float(f32(v["dt"])), sh=bool(v["sh"]),
                       psv=bool(v["psv"]), sfe=v["sfe"], lam=lam, mu=mu, rho=rho, ab=ab, stf=tuple(stf),
                       src_id=(orc.calc_idx(src[:, 0], float(xmax), nx), orc.calc_idx(src[:, 1], float(zmax), nz)),
                       rec_id=(orc.calc_idx(rec[:, 0], float(xmax), nx), orc.calc_idx(rec[:, 1], float(zmax), nz)),
                       inv_lambda=bool(v["inv_lambda"]), inv_mu=bool(v["inv_mu"]), inv_rho=bool(v["inv_rho"]))


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))
