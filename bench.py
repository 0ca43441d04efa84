"""Benchmark: batched forward+adjoint gradients of the inv.cu hot path on GB300.

Workload (the configuration the headline metric is quoted on): SH on a
681 x 141 grid at 12.5 m, dt = 1 ms, 4000 steps, 12 layers with vs from 1200
to 3500 m/s, 3 dipping normal faults with seeded throws, Gardner density,
16 shots at f0 = 8 Hz, 681 surface receivers, envelope misfit, Gaussian
smoothing sigma = 5 cells, forward checkpoints every 10 steps. One bench step
is one gradient (Misfit::run(kernel=true)): all 16 forward solves, the
envelope misfit and adjoint sources, all 16 adjoint solves with kernel
accumulation, and the smoothing of the three kernels.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`value` is shots/s (forward+adjoint pairs) with inputs resident in HBM,
timed with CUDA events on the solver's stream; `e2e` is the same metric
through the C ABI from pinned host buffers (model and observed traces in,
kernels and misfit out, copies inside the timed region). The reference arm
times the CPU port of the reference algorithm (oracle/, OpenMP on all host
cores), one full shot per step, and beside it one full gradient through the
reference's own CUDA kernels on the GPU (`reference_gpu`, also in the main
line). Both arms print the same `config`.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "shots/s fwd+adj & cell-updates/s (% HBM peak) vs plain path; p50/p99 solve latency"

# ----------------------------------------------------------------------------
# Workload
# ----------------------------------------------------------------------------
NX, NZ, H, DT, NT, NSHOT, F0, SFE, SIGMA = 681, 141, 12.5, 1e-3, 4000, 16, 8.0, 10, 5
SEED = 2024


def faulted_model(nx=NX, nz=NZ, h=H, seed=SEED, nlayer=12, vs_top=1200.0, vs_bottom=3500.0, nfault=3):
    """vs, vp, rho (float32, reference layout) of a layered model cut by
    dipping normal faults with seeded throws; vp = 1.73 vs, rho Gardner."""
    rng = np.random.default_rng(seed)
    x = (np.arange(nx) * h)[:, None]
    z = (np.arange(nz) * h)[None, :]
    zmax = (nz - 1) * h
    shift = np.zeros((nx, nz))
    for f in range(nfault):
        x0 = (0.2 + 0.6 * (f + rng.uniform(0.2, 0.8)) / nfault) * (nx - 1) * h
        dip = math.radians(rng.uniform(50, 70))
        throw = rng.uniform(0.03, 0.08) * zmax
        shift += np.where(x > x0 + z / math.tan(dip), throw, 0.0)
    thick = zmax / nlayer
    layer = np.clip(np.floor((z - shift) / thick), 0, nlayer - 1).astype(int)
    vs = np.linspace(vs_top, vs_bottom, nlayer)[layer]
    vp = 1.73 * vs
    rho = 310.0 * vp ** 0.25
    f32 = lambda a: np.ascontiguousarray(a.astype(np.float32).ravel())
    return f32(vs), f32(vp), f32(rho)


def smooth(a, nx, nz, cells):
    """Separable Gaussian blur (initial model), plain numpy."""
    a = a.reshape(nx, nz).astype(np.float64)
    r = int(3 * cells)
    w = np.exp(-0.5 * (np.arange(-r, r + 1) / cells) ** 2)
    w /= w.sum()
    pad = np.pad(a, r, mode="edge")
    t = sum(w[q] * pad[q:q + nx, :] for q in range(2 * r + 1))
    t = sum(w[q] * t[:, q:q + nz] for q in range(2 * r + 1))
    return np.ascontiguousarray(t.astype(np.float32).ravel())


def lame(vs, vp, rho):
    f32 = np.float32
    lam = np.where(vp > vs, (rho * (vp * vp - f32(2) * vs * vs)).astype(f32), f32(0)).astype(f32)
    mu = (rho * vs * vs).astype(f32)
    return lam, mu, rho


def workload():
    xmax, zmax = (NX - 1) * H, (NZ - 1) * H
    src = [[xmax * (s + 0.5) / NSHOT, 2 * H, 0, F0, 1.2 / F0, 0.0, 1e10] for s in range(NSHOT)]
    # receivers 2 cells deep: the reference's derivative guards leave the two
    # top rows without any coupling to the interior (they record zeros)
    rec = [[i * H, 2 * H] for i in range(NX)]
    values = {"mode": 2, "sh": 1, "psv": 0, "nt": NT, "dt": DT, "sfe": SFE, "model_type": 0, "trace_type": 0,
              "abs_left": 1, "abs_right": 1, "abs_bottom": 1, "abs_top": 0, "abs_width": 20, "abs_alpha": 0.015,
              "inv_lambda": 0, "inv_mu": 1, "inv_rho": 1, "misfit": 1, "filter": 0, "filter_sigma": SIGMA}
    vs, vp, rho = faulted_model()
    init = [smooth(a, NX, NZ, 250.0 / H / 2) for a in (vs, vp, rho)]
    return dict(xmax=xmax, zmax=zmax, src=src, rec=rec, values=values, true=lame(vs, vp, rho),
                init=lame(*init))


CONFIG_DESC = {
    "workload": "SH gradient, 681x141 grid at 12.5 m, dt 1 ms, 4000 steps, 16 shots f0 8 Hz, 681 receivers, "
                "envelope misfit, Gaussian smoothing sigma 5, checkpoints every 10 steps",
    "grid": [NX, NZ], "nt": NT, "shots": NSHOT, "receivers": NX, "source_receiver_depth_m": 2 * H,
    "sfe": SFE, "misfit": "envelope",
    "filter_sigma": SIGMA,
    "l2": "flushed (256 MB write) between timed steps; each step also streams 3.1 GB of checkpoints",
}


# ----------------------------------------------------------------------------
# Helpers
# ----------------------------------------------------------------------------
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """Samples nvidia-smi every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.out = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        self.out.flush()
        self.out.seek(0)
        rows = [r.split(",") for r in self.out.read().strip().splitlines() if r.strip()]
        os.unlink(self.out.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in rows if len(r) > 2 and r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) > 2 and r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for q, nm in enumerate(names):
                if len(r) > 5 + q and r[5 + q].strip().lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(kernel_tag):
    """DRAM bytes per time step of the dominant kernel from the committed ncu
    summary (profiles/dram_traffic.txt: `<tag> <bytes per step> <note>`)."""
    p = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        parts = line.split()
        if len(parts) >= 2 and parts[0] == kernel_tag and not line.startswith("#"):
            try:
                return float(parts[1])
            except ValueError:
                return None
    return None


# ----------------------------------------------------------------------------
# Baseline legs: the CPU port of the reference (oracle/, OpenMP) and the
# reference's own CUDA kernels (oracle/_ref, driven by oracle/ref_harness.cu
# in the reference's launch shapes and host loop). Checkers and baselines
# only: neither is on the product path.
# ----------------------------------------------------------------------------
def _oracle_problem(wl):
    from oracle import oracle as orc

    lam, mu, rho = wl["init"]
    v = wl["values"]
    src = np.array(wl["src"], np.float32)
    rec = np.array(wl["rec"], np.float32)
    stf = [np.zeros(len(src) * NT, np.float32) for _ in range(3)]
    for s in range(len(src)):
        c = orc.ricker(NT, DT, *src[s, 3:7])
        for q in range(3):
            stf[q][s * NT:(s + 1) * NT] = c[q]
    ab = orc.absbound(NX, NZ, v["abs_width"], v["abs_alpha"], 1, 1, 1, 0)
    dx = float(np.float32(wl["xmax"]) / np.float32(NX - 1))
    return orc.Problem(nx=NX, nz=NZ, nt=NT, dx=dx, dz=dx, dt=DT, sh=True, psv=False, sfe=SFE, lam=lam, mu=mu,
                       rho=rho, ab=ab, stf=tuple(stf),
                       src_id=(orc.calc_idx(src[:, 0], wl["xmax"], NX), orc.calc_idx(src[:, 1], wl["zmax"], NZ)),
                       rec_id=(orc.calc_idx(rec[:, 0], wl["xmax"], NX), orc.calc_idx(rec[:, 1], wl["zmax"], NZ)),
                       inv_lambda=False, inv_mu=True, inv_rho=True)


class CpuPort:
    """The oracle (C restatement of the reference, OpenMP over all host cores)
    on the workload. One step of it is one full shot: forward with
    checkpoints, envelope misfit against 0.9 x the synthetics, adjoint with
    kernel accumulation. The smoothing of the three kernels (once per
    gradient) is timed on its own; a gradient is 16 shots + one smoothing."""

    def __init__(self, wl):
        from oracle import oracle as orc

        self.orc = orc
        orc.set_threads(os.cpu_count() or 1)
        self.threads = orc.num_threads()
        self.pb = _oracle_problem(wl)
        self.kern = None

    def shot(self, s):
        orc = self.orc
        t0 = time.perf_counter()
        _, oy, _, ck = orc.forward(self.pb, s % NSHOT, adj=True)
        _, ad = orc.envelope_misfit(oy, oy * np.float32(0.9), DT)
        self.kern = orc.adjoint(self.pb, [np.zeros_like(ad), ad, np.zeros_like(ad)], ck, self.kern)
        return time.perf_counter() - t0

    def smoothing(self):
        t0 = time.perf_counter()
        for k in self.kern:
            self.orc.gaussian_filter(NX, NZ, SIGMA, k)
        return time.perf_counter() - t0


def cpu_sample(wl, nshots=1):
    """Bounded CPU sample beside the GPU number: `nshots` full shots and one
    smoothing. Returns (seconds per 16-shot gradient, threads, description)."""
    port = CpuPort(wl)
    t_shot = sum(port.shot(s) for s in range(nshots)) / nshots
    t_filter = port.smoothing()
    desc = ("%d of %d shots at full size (forward %d steps with checkpoints, envelope misfit, adjoint) plus "
            "one smoothing of 3 kernels; per-gradient time = 16 x shot + smoothing" % (nshots, NSHOT, NT))
    return NSHOT * t_shot + t_filter, port.threads, desc


def reference_gpu_sample(wl):
    """One full 16-shot gradient through the reference's own CUDA kernels
    (compiled from its sources for sm_103a), in its launch shapes (nx blocks
    of nz threads, six launches per time step, one-thread-block source and
    receiver launches) and host loop (solver/fdm.h:515-612: checkpoints
    copied to pageable host memory and back with blocking copies; per-trace
    envelope misfit with cuFFT and cuBLAS, misfit/envelope.h:58-90), plus the
    smoothing of the three kernels with its filter kernels. Wall time around
    the whole gradient (the reference's host loop is synchronous). Returns a
    dict for the JSON line, or one that says why it did not run."""
    from oracle import oracle as orc

    if not orc.ref_available():
        return {"unavailable": "the reference's kernels were not built (oracle/_ref/inv_ref.cubin absent)"}
    pb = _oracle_problem(wl)
    # warm-up: module load, cuFFT/cuBLAS handles, first launches (one short shot)
    short = _oracle_problem(wl)
    short.nt = 200
    short.stf = tuple(np.ascontiguousarray(a.reshape(NSHOT, NT)[:, :200]).ravel() for a in pb.stf)
    _, oy, _, ck = orc.ref_forward(short, 0, adj=True)
    _, ad = orc.ref_misfit(1, oy, oy * np.float32(0.9), DT)
    orc.ref_adjoint(short, [np.zeros_like(ad), ad, np.zeros_like(ad)], ck)
    t0 = time.perf_counter()
    kern = None
    for s in range(NSHOT):
        _, oy, _, ck = orc.ref_forward(pb, s, adj=True)
        _, ad = orc.ref_misfit(1, oy, oy * np.float32(0.9), DT)
        kern = orc.ref_adjoint(pb, [np.zeros_like(ad), ad, np.zeros_like(ad)], ck, kern)
    for k in kern:
        orc.ref_gaussian(NX, NZ, SIGMA, k)
    t = time.perf_counter() - t0
    return {"value": round(NSHOT / t, 3), "unit": "shots/s", "ms_per_gradient": round(1e3 * t, 1),
            "sample": "one full 16-shot gradient, wall time (no extrapolation)",
            "what": "the reference's own kernels compiled from its sources for sm_103a, run in its launch shapes "
                    "and host loop: six launches per step, checkpoints to pageable host memory by blocking "
                    "copies, per-trace cuFFT/cuBLAS envelope misfit, its Gaussian filter"}


# ----------------------------------------------------------------------------
# GPU arm
# ----------------------------------------------------------------------------
def run_ours(args, ws, rank, local):
    import __graft_entry__ as ge

    pkg = ge.load_package()
    if pkg.device_count() < 1:
        raise RuntimeError("no CUDA device")
    pkg.select_device(local)
    wl = workload()
    tmp = tempfile.mkdtemp(prefix="gbfwi_bench_")
    cfg = pkg.Config.new(tmp, wl["values"], wl["src"], wl["rec"])
    sol = pkg.FdmSolver(cfg, grid=(NX, NZ, wl["xmax"], wl["zmax"]))
    sol.set_option("batch", NSHOT)
    # observed data on the true model (setup, not timed)
    sol.set_model_grid(*wl["true"])
    sol.run_forward_batch(list(range(NSHOT)))
    obs = np.stack([sol.out("y", slot=b) for b in range(NSHOT)])
    sol.set_model_grid(*wl["init"])
    filt = pkg.GaussianFilter(NX, NZ, SIGMA)
    mis = pkg.Misfit.from_obs(1, sol, {"y": obs}, filt)
    flush = pkg.DeviceArray(np.zeros(64 << 20, np.float32))  # 256 MB
    zeros = np.zeros(64 << 20, np.float32)

    def l2_flush():
        pkg.h2d(flush.ptr, zeros)

    for _ in range(args.warmup):
        mis.run(kernel=True)
    sol.stats(reset=True)
    step_ms = []
    barrier(ws)
    with Clocks(local) as clk:
        for _ in range(args.steps):
            l2_flush()
            pkg.lib().gb_device_sync()
            sol.timer_begin()
            mis.run(kernel=True)
            step_ms.append(sol.timer_end())
    st = sol.stats()
    barrier(ws)
    total_ms = max_over_ranks(sum(step_ms), ws)
    value = NSHOT * args.steps * ws / (total_ms / 1e3)
    cells = NX * NZ

    # Roofline of the dominant kernel. The algorithmic bytes of one SH time
    # step are those of the per-step formulation: 40 bytes per cell (v, u,
    # two stresses read and written, mu and 1/rho read) for every shot.
    # step_ms / step_launches is the time per step (a cluster-resident pass
    # books its duration as nt steps).
    per_launch_ms = st.step_ms / max(st.step_launches, 1)
    algo_bytes = 40.0 * cells * NSHOT
    achieved = algo_bytes / (per_launch_ms * 1e-3) / 1e9
    peak, peak_kind = peaks()
    clustered = st.tile_tz < 0
    if clustered:
        kname = "k_cluster<SH> (whole forward/adjoint pass per shot in a %d-CTA cluster, state in shared memory)" % (
            -st.tile_tz)
        tag = "cluster_sh_c2"
        note = ("the wavefield stays in shared memory for the whole pass: DRAM traffic per step (traffic) is the "
                "checkpoints and traces only, far below the algorithmic bytes; achieved/peak compares the step "
                "time with an HBM-bound per-step kernel at the measured copy bandwidth")
    else:
        kname = "k_step<SH> (fused velocity+stress step, 16 shots per launch)"
        tag = "step_sh_c2"
        note = "state (16 shots x 4 fields + model) is L2-resident at this size"
    roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 3), "traffic": profiled_traffic(tag),
            "kernel": kname, "algorithmic_bytes_per_step": algo_bytes, "avg_step_us": round(per_launch_ms * 1e3, 2),
            "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
            "note": note}

    # end to end through the C ABI with pinned host buffers
    n_obs = obs.size
    h_obs = pkg.PinnedArray(n_obs)
    h_obs.array[:] = obs.ravel()
    h_model = [pkg.PinnedArray(cells) for _ in range(3)]
    for q in range(3):
        h_model[q].array[:] = wl["init"][q]
    h_k = [pkg.PinnedArray(cells) for _ in range(2)]
    e2e_ms = []
    mis_val = None
    for _ in range(args.steps):
        l2_flush()
        pkg.lib().gb_device_sync()
        t0 = time.perf_counter()
        pkg.check(pkg.lib().gb_set_model_grid(sol._h, *[pkg._ptr(m.array) for m in h_model]))
        # the observed traces' upload overlaps the forward pass (the misfit
        # stages wait for it); it completes inside mis.run
        pkg.check(pkg.lib().gb_misfit_set_obs_async(mis._h, None, pkg._ptr(h_obs.array), None))
        mis_val = mis.run(kernel=True)
        for q, which in enumerate((pkg.GB_K_MU, pkg.GB_K_RHO)):
            pkg.check(pkg.lib().gb_memcpy_d2h(h_k[q].ptr, sol.ptr(which), cells * 4))
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_total = max_over_ranks(sum(e2e_ms), ws)
    e2e = {"value": round(NSHOT * args.steps * ws / (e2e_total / 1e3), 3), "unit": "shots/s",
           "h2d_bytes_per_step": int(3 * cells * 4 + n_obs * 4), "d2h_bytes_per_step": int(2 * cells * 4 + 8),
           "ms_per_step": round(e2e_total / args.steps, 3)}

    # plain path: one shot per launch sequence, no graphs (same GPU, one gradient)
    plain = None
    if rank == 0 and not args.no_plain:
        cfgp = pkg.Config.new(tmp, dict(wl["values"], batch=1, graphs=0, cluster=0), wl["src"], wl["rec"])
        sp = pkg.FdmSolver(cfgp, grid=(NX, NZ, wl["xmax"], wl["zmax"]))
        sp.set_option("batch", 1)
        sp.set_option("graphs", 0)
        sp.set_option("cluster", 0)
        sp.set_model_grid(*wl["init"])
        mp = pkg.Misfit.from_obs(1, sp, {"y": obs}, pkg.GaussianFilter(NX, NZ, SIGMA))
        mp.run(kernel=True)
        sp.timer_begin()
        mp.run(kernel=True)
        plain_ms = sp.timer_end()
        plain = {"value": round(NSHOT / (plain_ms / 1e3), 3), "unit": "shots/s", "ms_per_step": round(plain_ms, 2),
                 "what": "one shot per call, one fused step kernel launch per time step, no CUDA graphs"}
        mp.close()
        sp.close()

    hbm = None
    if rank == 0 and not args.no_hbm_step:
        hbm = [hbm_step(pkg, wave) for wave in ("psv", "sh")]
    ref_gpu = None
    if rank == 0 and ws == 1 and not args.no_ref_gpu:
        ref_gpu = _reference_gpu_leg(wl)
        if "value" in ref_gpu:
            ref_gpu["ours_over_reference"] = round(value / ref_gpu["value"], 2)
            ref_gpu["ours_e2e_over_reference"] = round(e2e["value"] / ref_gpu["value"], 2)
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        t_grad, threads, desc = cpu_sample(wl)
        cpu = {"value": round(NSHOT / t_grad, 4), "unit": "shots/s", "cores": threads, "kind": "port",
               "sample": desc}
    clocks = clk.summary()
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "shots/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded faulted layered model with the workload's shapes; no dataset)",
        "config": dict(CONFIG_DESC),
        "run": {"step": "one gradient: 16 forward + envelope misfit + 16 adjoint + smoothing",
                "batch": st.batch_capacity, "tile": [st.tile_tz, st.tile_tx], "ckpt": "fp32",
                "parallelism": "shots sharded over %d rank(s), replicas" % ws},
        "cell_updates_per_s": round(2.0 * cells * NT * NSHOT * args.steps * ws / (total_ms / 1e3), 1),
        "misfit": mis_val, "plain_path": plain, "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
        "reference_gpu": ref_gpu, "hbm_step": hbm,
        "breakdown_ms_per_gradient": {k: round(getattr(st, k) / args.steps, 3)
                                      for k in ("forward_ms", "adjoint_ms", "misfit_ms", "filter_ms")},
        "gpu_launches": int(st.launches), "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def hbm_step(pkg, wave, nx=4096, nz=1024, nshot=16, nt=40):
    """The per-step marching kernel where the HBM roofline applies: a 16-shot
    batch on the full-inversion grid (4096 x 1024 at 5 m, dt 0.4 ms, 256
    receivers), forward, no checkpoints. The kernel configuration is tuned on
    a first pass (the solver's autotuner), then three passes of `nt` steps are
    timed with CUDA events in the solver's step windows (step kernels only).
    achieved = algorithmic bytes per step (68 B P-SV / 40 B SH per cell and
    shot: the state read and written once, the model read once) / time per
    step. The state (16 x 12 or 7 fields of 16.8 MB) is far larger than L2."""
    from tests import cases

    case = cases.make_case(wave=wave, nx=nx, nz=nz, nt=nt, nsrc=nshot, nrec=256, dx=5.0, dt=4e-4, f0=12.0,
                           abs_width=20, sfe=10, seed=5)
    case["values"]["mode"] = 3
    cfg, sol = cases.gpu_solver(pkg, case, extra={"cluster": 0})
    sol.set_option("cluster", 0)
    sol.set_option("batch", nshot)
    shots = list(range(nshot))
    sol.run_forward_batch(shots)  # tunes the configuration, warms up
    sol.stats(reset=True)
    for _ in range(3):
        sol.run_forward_batch(shots)
    st = sol.stats()
    sol.close()
    us = 1e3 * st.step_ms / max(st.step_launches, 1)
    per_cell = 68.0 if wave == "psv" else 40.0
    algo = per_cell * nx * nz * nshot
    gbs = algo / (us * 1e-6) / 1e9
    peak, kind = peaks()
    return {"wave": wave, "grid": [nx, nz], "shots": nshot, "steps_timed": int(st.step_launches),
            "kernel": "k_march (z-strip marching step, %d-row strips, %d-column chunks, bulk loads %d)" % (
                st.tile_tz, st.tile_tx, st.march_bulk),
            "us_per_step": round(us, 2), "algorithmic_bytes_per_step": algo, "achieved_gbs": round(gbs, 1),
            "peak_gbs": peak, "frac": round(gbs / peak, 3), "peak_source": kind,
            "cell_updates_per_s": round(nx * nz * nshot / (us * 1e-6), 1),
            "traffic_bytes_per_step": profiled_traffic("march_%s_4096x1024x16" % wave)}


# ----------------------------------------------------------------------------
# Other configurations (reported beside the headline, one JSON line each)
# ----------------------------------------------------------------------------
def _solver_for(pkg, tmp, values, src, rec, nx, nz, h, model):
    cfg = pkg.Config.new(tmp, values, src, rec)
    sol = pkg.FdmSolver(cfg, grid=(nx, nz, (nx - 1) * h, (nz - 1) * h))
    sol.set_model_grid(*model)
    return cfg, sol


def _line(metric, value, unit, config, **extra):
    d = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "higher_is_better": True,
         "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)", "config": config}
    d.update(extra)
    print(json.dumps(d), flush=True)


def run_c1(args):
    """P-SV checkerboard 200x200, 4 shots, nt 2000: one gradient, then 5 NLCG
    iterations through the optimizer."""
    import __graft_entry__ as ge

    pkg = ge.load_package()
    nx = nz = 200
    h, dt, nt = 10.0, 1e-3, 2000
    ii, jj = np.meshgrid(np.arange(nx), np.arange(nz), indexing="ij")
    sign = np.where(((ii // 20) + (jj // 20)) % 2 == 0, 1.0, -1.0)
    bg = (3000.0, 1732.0, 2600.0)
    true = [np.ascontiguousarray((v * (1 + 0.05 * sign)).astype(np.float32).ravel()) for v in bg[:2]]
    true.append(np.full(nx * nz, bg[2], np.float32))
    init = [np.full(nx * nz, v, np.float32) for v in bg]
    xmax = (nx - 1) * h
    src = [[xmax * (s + 0.5) / 4, 2 * h, 0, 10.0, 0.12, math.pi / 2, 1e10] for s in range(4)]
    rec = [[i * h, 2 * h] for i in range(nx)]
    values = {"mode": 0, "sh": 0, "psv": 1, "nt": nt, "dt": dt, "sfe": 10, "model_type": 0, "trace_type": 0,
              "abs_left": 1, "abs_right": 1, "abs_bottom": 1, "abs_top": 0, "abs_width": 20, "abs_alpha": 0.015,
              "inv_lambda": 1, "inv_mu": 1, "inv_rho": 0, "misfit": 0, "filter": 0, "filter_sigma": 5,
              "optimizer": 0, "inv_iteration": 5, "inv_cycle": 0, "nlcg_type": 1, "nlcg_thresh": 0.0,
              "ls_step": 10, "ls_step_max": 0.5, "ls_step_init": 0.05, "ls_thresh": 1.2}
    tmp = tempfile.mkdtemp(prefix="gbfwi_c1_")
    os.makedirs(os.path.join(tmp, "output"))
    cfg, sol = _solver_for(pkg, tmp, values, src, rec, nx, nz, h, lame(true[1], true[0], true[2]))
    sol.run_forward_batch(list(range(4)))
    obs = {c: np.stack([sol.out(c, slot=b) for b in range(4)]) for c in "xz"}
    sol.set_model_grid(*lame(init[1], init[0], init[2]))
    filt = pkg.GaussianFilter(nx, nz, 5)
    mis = pkg.Misfit.from_obs(0, sol, obs, filt)
    for _ in range(args.warmup):
        mis.run(kernel=True)
    ms = []
    for _ in range(args.steps):
        sol.timer_begin()
        mis.run(kernel=True)
        ms.append(sol.timer_end())
    grad_ms = sum(ms) / len(ms)
    init_model = lame(init[1], init[0], init[2])
    # the same gradient through the plain path (one shot per call, one fused
    # step launch per time step, no CUDA graphs, no cluster pass)
    plain = None
    if not args.no_plain:
        cfgp, sp = _solver_for(pkg, tmp, dict(values, batch=1, graphs=0, cluster=0), src, rec, nx, nz, h, init_model)
        sp.set_option("batch", 1)
        sp.set_option("graphs", 0)
        sp.set_option("cluster", 0)
        mp = pkg.Misfit.from_obs(0, sp, obs, pkg.GaussianFilter(nx, nz, 5))
        mp.run(kernel=True)
        sp.timer_begin()
        mp.run(kernel=True)
        plain_ms = sp.timer_end()
        plain = {"value": round(4 / (plain_ms / 1e3), 2), "unit": "shots/s", "ms_per_step": round(plain_ms, 2)}
        mp.close()
        sp.close()
    ref_gpu = None
    if not args.no_ref_gpu:
        ref_gpu = _c1_reference_gpu(values, src, rec, nx, nz, h, init_model, obs)
        if "value" in ref_gpu:
            ref_gpu["ours_over_reference"] = round((4 / (grad_ms / 1e3)) / ref_gpu["value"], 2)
    opt = pkg.Optimizer(cfg, sol, mis)
    t0 = time.perf_counter()
    opt.run()
    inv_s = time.perf_counter() - t0
    hist = opt.history()
    _line("shots/s fwd+adj (P-SV checkerboard gradient)", round(4 / (grad_ms / 1e3), 2), "shots/s",
          {"workload": "P-SV 200x200 checkerboard +-5% in 20-cell squares, nt 2000, 4 shots, waveform misfit, "
                       "then 5 NLCG iterations", "receivers_depth_m": 2 * h},
          ms_per_step=round(grad_ms, 3), steps=args.steps, warmup=args.warmup,
          plain_path=plain, reference_gpu=ref_gpu,
          inversion={"iterations": 5, "wall_s": round(inv_s, 3), "misfit_history": [round(v, 6) for v in hist],
                     "final_over_initial": round(hist[-1] / hist[0], 6) if len(hist) else None})


def _c1_reference_gpu(values, src, rec, nx, nz, h, model, obs):
    """One C1 gradient (4 P-SV shots, waveform misfit, smoothing of the
    lambda and mu kernels) through the reference's own CUDA kernels in its
    launch shapes and host loop (solver/fdm.h:515-612, misfit/waveform.h,
    filter/gaussian.h), after one warm-up shot; wall time, no extrapolation."""
    from oracle import oracle as orc

    if not orc.ref_available():
        return {"unavailable": "the reference's kernels were not built (oracle/_ref/inv_ref.cubin absent)"}
    f32 = np.float32
    nt, dt = values["nt"], values["dt"]
    xmax = zmax = (nx - 1) * h
    srca, reca = np.array(src, f32), np.array(rec, f32)
    stf = [np.zeros(len(srca) * nt, f32) for _ in range(3)]
    for s in range(len(srca)):
        c = orc.ricker(nt, dt, *srca[s, 3:7])
        for q in range(3):
            stf[q][s * nt:(s + 1) * nt] = c[q]
    ab = orc.absbound(nx, nz, values["abs_width"], values["abs_alpha"], values["abs_left"], values["abs_right"],
                      values["abs_bottom"], values["abs_top"])
    dx = float(f32(xmax) / f32(nx - 1))
    lam, mu, rho = model
    pb = orc.Problem(nx=nx, nz=nz, nt=nt, dx=dx, dz=dx, dt=float(f32(dt)), sh=False, psv=True, sfe=values["sfe"],
                     lam=lam, mu=mu, rho=rho, ab=ab, stf=tuple(stf),
                     src_id=(orc.calc_idx(srca[:, 0], float(xmax), nx), orc.calc_idx(srca[:, 1], float(zmax), nz)),
                     rec_id=(orc.calc_idx(reca[:, 0], float(xmax), nx), orc.calc_idx(reca[:, 1], float(zmax), nz)),
                     inv_lambda=True, inv_mu=True, inv_rho=False)
    nrec = len(reca)

    def shot(s, kern):
        ox, _, oz, ck = orc.ref_forward(pb, s, adj=True)
        _, adx = orc.ref_misfit(0, ox.reshape(nrec, nt), obs["x"][s], dt)
        _, adz = orc.ref_misfit(0, oz.reshape(nrec, nt), obs["z"][s], dt)
        return orc.ref_adjoint(pb, [adx, np.zeros_like(adx), adz], ck, kern)

    shot(0, None)  # warm-up: module load, cuFFT/cuBLAS handles, first launches
    t0 = time.perf_counter()
    kern = None
    for s in range(len(srca)):
        kern = shot(s, kern)
    for q in (0, 1):
        orc.ref_gaussian(nx, nz, 5, kern[q])
    t = time.perf_counter() - t0
    return {"value": round(len(srca) / t, 3), "unit": "shots/s", "ms_per_gradient": round(1e3 * t, 1),
            "sample": "one full 4-shot gradient, wall time (no extrapolation)",
            "what": "the reference's own kernels compiled from its sources for sm_103a, run in its launch shapes "
                    "and host loop: six launches per step, checkpoints to pageable host memory by blocking "
                    "copies, per-trace waveform misfit with cuBLAS, its Gaussian filter"}


def run_c3(args):
    """P-SV 2048x1024, nt 6000: one gradient with FP32, BF16 and FP16
    checkpoints; gradient differences against the FP32-checkpoint gradient.
    Each precision's error against an FP64 oracle run on this grid and model
    (one shot, 2000 steps) is a GPU test (tests/test_gpu_precision.py)."""
    import __graft_entry__ as ge
    from tests import cases

    pkg = ge.load_package()
    nshot = args.shots or 64
    case = cases.random_smooth_case(nt=6000, nsrc=nshot)
    nx, nz, h = case["nx"], case["nz"], 5.0
    tmp = tempfile.mkdtemp(prefix="gbfwi_c3_")
    values = dict(case["values"], mode=2)
    model = lame(case["vs"], case["vp"], case["rho"])
    obs = None
    res = {}
    grads = {}
    for prec in (0, 1, 2):
        cfg, sol = _solver_for(pkg, tmp, values, case["src"], case["rec"], nx, nz, h, model)
        sol.set_option("ckpt", prec)
        if obs is None:
            obs = {"x": [], "z": []}
            shots = list(range(nshot))
            cap = sol.capacity
            for a in range(0, nshot, cap):
                b = shots[a:a + cap]
                sol.run_forward_batch(b)
                for q in range(len(b)):
                    obs["x"].append(sol.out("x", slot=q) * np.float32(0.98))
                    obs["z"].append(sol.out("z", slot=q) * np.float32(0.98))
            obs = {c: np.stack(v) for c, v in obs.items()}
        mis = pkg.Misfit.from_obs(0, sol, obs)
        sol.timer_begin()
        mis.run(kernel=True)
        ms = sol.timer_end()
        st = sol.stats()
        grads[prec] = sol.kernels()
        res[("fp32", "bf16", "fp16")[prec]] = {"shots_per_s": round(nshot / (ms / 1e3), 3), "ms": round(ms, 1),
                                               "batch": st.batch_capacity, "tile": [st.tile_tz, st.tile_tx]}
        mis.close()
        sol.close()
    for prec in (1, 2):
        res[("fp32", "bf16", "fp16")[prec]]["grad_rel_diff_vs_fp32_ckpt"] = {
            n: float(np.linalg.norm(grads[prec][n] - grads[0][n]) / np.linalg.norm(grads[0][n]))
            for n in ("k_lambda", "k_mu", "k_rho")}
    _line("shots/s fwd+adj by checkpoint precision (P-SV 2048x1024)", res["bf16"]["shots_per_s"], "shots/s",
          {"workload": "P-SV 2048x1024 at 5 m, dt 0.4 ms, 6000 steps, %d shots f0 15 Hz, checkpoints every 50 "
                       "steps; smooth random vp 2000-4500, vp/vs 1.7-2.0" % nshot},
          precision=res, note="16-bit checkpoints hold the displacement differences the kernel accumulation "
                              "reads; each precision's error against an FP64 oracle run on this grid and "
                              "model is tests/test_gpu_precision.py::test_precision_study_grid_vs_fp64_oracle")


def run_c4(args):
    """Serving: forward+adjoint requests, mixed P-SV/SH, grid sides
    U[128,1024], 1000-5000 steps. Three runs of the same seeded requests:
    all queued at once (the engine's capacity: requests/s and
    cell-updates/s), Poisson arrivals at --load x that capacity (p50/p99
    latency), and the first --sequential of them solved one at a time (the
    plain comparator)."""
    import __graft_entry__ as ge

    pkg = ge.load_package()
    nreq = args.requests
    rng = np.random.default_rng(11)
    # eight seeded layered, faulted models of 1024 x 1024; a request takes the
    # top-left nx x nz window of one of them
    bases = [[a.reshape(1024, 1024) for a in lame(*faulted_model(nx=1024, nz=1024, h=10.0, seed=100 + b,
                                                                vs_bottom=3000.0))] for b in range(8)]
    reqs = []
    for q in range(nreq):
        nx, nz = int(rng.integers(128, 1025)), int(rng.integers(128, 1025))
        nt = int(round(rng.integers(1000, 5001) / 10.0)) * 10
        psv = int(q % 2 == 0)
        lam, mu, rho = (np.ascontiguousarray(a[:nx, :nz]).ravel() for a in bases[q % 8])
        xmax = (nx - 1) * 10.0
        src = [xmax * rng.uniform(0.2, 0.8), 30.0, 0, 10.0, 0.12, math.pi / 4, 1e10]
        rec = np.array([[i * 40.0, 20.0] for i in range(nx // 4)], np.float32)
        reqs.append(dict(psv=psv, nx=nx, nz=nz, dx=10.0, dt=8e-4, nt=nt, lam=lam, mu=mu, rho=rho, src=src,
                         rec=rec))
    cells = [2 * r["nx"] * r["nz"] * r["nt"] for r in reqs]

    def serve(arrivals, max_slots=0, tile=0):
        srv = pkg.Server(sfe=10, ckpt=2, max_slots=max_slots)
        if tile:
            srv.set_option("tile", tile)
        if args.server_streams:
            srv.set_option("streams", args.server_streams)
        if args.server_compact >= 0:
            srv.set_option("compact", args.server_compact)
        for q, r in enumerate(reqs[:len(arrivals)]):
            srv.submit(arrival=float(arrivals[q]), **r)
        srv.run()
        st = srv.stats()
        srv.close()
        return st

    # capacity: every request queued at t = 0
    sat = serve(np.zeros(nreq), tile=args.server_tile)
    cap = sat.completed / sat.wall_s
    # latency under load: Poisson arrivals at a fraction of that capacity
    # (--load 0 skips this run)
    rate = args.rate if args.rate > 0 else args.load * cap
    live = None
    if rate > 0:
        arrivals = np.cumsum(np.random.default_rng(12).exponential(1.0 / rate, nreq))
        live = serve(arrivals, tile=args.server_tile)
    # the plain comparator: the first `seq` requests one at a time, with the
    # 2-D tile kernel (configuration 3, the faster choice for a lone grid of
    # these sizes; the marching strips pay off with many requests in flight)
    # (--sequential 0 skips it)
    seq = min(nreq, args.sequential)
    one = serve(np.zeros(seq), max_slots=1, tile=3) if seq > 0 else None
    cu_sat = sat.cell_updates / sat.wall_s
    cu_seq = sum(cells[:seq]) / one.wall_s if one else None
    # the plain path: each request through its own solver, one shot per call,
    # one fused step launch per time step, FP32 checkpoints, no CUDA graphs,
    # no cluster pass (solver created, model uploaded and gradient run per
    # request, as a caller without the engine would)
    plain = None
    npl = min(nreq, args.sequential)
    if npl > 0:
        tmp = tempfile.mkdtemp(prefix="gbfwi_c4_")
        t0 = time.perf_counter()
        for r in reqs[:npl]:
            vals = {"mode": 2, "sh": 1 - r["psv"], "psv": r["psv"], "nt": r["nt"], "dt": r["dt"], "sfe": 10,
                    "model_type": 0, "trace_type": 0, "abs_left": 1, "abs_right": 1, "abs_bottom": 1, "abs_top": 0,
                    "abs_width": 20, "abs_alpha": 0.015, "inv_lambda": 1, "inv_mu": 1, "inv_rho": 1,
                    "batch": 1, "graphs": 0, "cluster": 0, "ckpt_precision": 0}
            cfg = pkg.Config.new(tmp, vals, [r["src"]], r["rec"].tolist())
            sol = pkg.FdmSolver(cfg, grid=(r["nx"], r["nz"], (r["nx"] - 1) * r["dx"], (r["nz"] - 1) * r["dx"]))
            sol.set_model_grid(r["lam"], r["mu"], r["rho"])
            comps = "xz" if r["psv"] else "y"
            mis = pkg.Misfit.from_obs(0, sol, {c: np.zeros((1, len(r["rec"]), r["nt"]), np.float32) for c in comps})
            mis.run(kernel=True)
            mis.close()
            sol.close()
            del cfg
        wall = time.perf_counter() - t0
        plain = {"requests": npl, "wall_s": round(wall, 2), "requests_per_s": round(npl / wall, 3),
                 "cell_updates_per_s": round(sum(cells[:npl]) / wall, 1),
                 "what": "each request through its own solver: one shot per call, one fused step launch per "
                         "time step, FP32 checkpoints, no CUDA graphs, no cluster pass"}
    _line("served forward+adjoint requests/s", round(cap, 3), "requests/s",
          {"workload": "%d requests, 50/50 P-SV/SH, sides U[128,1024] at 10 m, 1000-5000 steps (dt 0.8 ms), "
                       "layered faulted models, FP16 checkpoints" % nreq},
          capacity={"requests_per_s": round(cap, 3), "cell_updates_per_s": round(cu_sat, 1),
                    "wall_s": round(sat.wall_s, 2), "max_concurrent": sat.max_concurrent,
                    "over_sequential_cell_updates": round(cu_sat / cu_seq, 2) if cu_seq else None,
                    "over_plain_path_cell_updates": round(cu_sat / plain["cell_updates_per_s"], 2) if plain else None,
                    "launches": int(sat.launches), "rounds": int(sat.rounds)},
          under_load=None if live is None else {
              "arrival_rate_per_s": round(rate, 3), "fraction_of_capacity": round(rate / cap, 3),
              "requests_per_s": round(live.completed / live.wall_s, 3),
              "p50_latency_s": round(live.p50_s, 3), "p99_latency_s": round(live.p99_s, 3),
              "max_concurrent": live.max_concurrent, "wall_s": round(live.wall_s, 2)},
          sequential=None if one is None else {
              "requests": seq, "wall_s": round(one.wall_s, 2), "requests_per_s": round(seq / one.wall_s, 3),
              "cell_updates_per_s": round(cu_seq, 1), "p50_latency_s_one_at_a_time": round(one.p50_s, 3)},
          plain_path=plain,
          gpu_launches=int(sat.launches))


def run_c5(args):
    """P-SV 4096x1024 at 5 m, dt 0.4 ms, 8000 steps, 4096 receivers, on the
    faulted model of the headline workload generated at this grid. Without
    --iterations: one gradient of --shots shots (default 16) with FP16
    checkpoints. With --iterations N: the full inversion's setting (--shots,
    default 128; L-BFGS with memory 10; smoothing sigma 10 cells; lambda and
    mu inverted; initial model the true one smoothed by a Gaussian of 500 m)
    for N iterations, with BF16 and with FP32 checkpoints (--precisions),
    reporting the time per iteration, the misfit history, each final model's
    error against the true model and, with both precisions, the difference
    between the two final models."""
    import __graft_entry__ as ge

    pkg = ge.load_package()
    nx, nz, h, dt, nt = 4096, 1024, 5.0, 4e-4, 8000
    inversion = args.iterations > 0
    nshot = args.shots or (128 if inversion else 16)
    vs, vp, rho = faulted_model(nx=nx, nz=nz, h=h, seed=SEED, vs_bottom=3500.0)
    xmax = (nx - 1) * h
    src = [[xmax * (s + 0.5) / nshot, 4 * h, 0, 12.0, 0.1, math.pi / 2, 1e10] for s in range(nshot)]
    rec = [[i * h, 2 * h] for i in range(nx)]
    values = {"mode": 2, "sh": 0, "psv": 1, "nt": nt, "dt": dt, "sfe": 50, "model_type": 0, "trace_type": 0,
              "abs_left": 1, "abs_right": 1, "abs_bottom": 1, "abs_top": 0, "abs_width": 20, "abs_alpha": 0.015,
              "inv_lambda": 1, "inv_mu": 1, "inv_rho": 1 if not inversion else 0, "misfit": 0, "filter": 0,
              "filter_sigma": 10, "optimizer": 1, "lbfgs_mem": 10, "lbfgs_thresh": 0.0,
              "inv_iteration": max(args.iterations, 1), "inv_cycle": 0, "ls_step": 10, "ls_step_max": 0.5,
              "ls_step_init": 0.05, "ls_thresh": 1.2}
    tmp = tempfile.mkdtemp(prefix="gbfwi_c5_")
    os.makedirs(os.path.join(tmp, "output"), exist_ok=True)
    true = lame(vs, vp, rho)
    desc = ("P-SV 4096x1024 at 5 m, dt 0.4 ms, 8000 steps, %d shots f0 12 Hz, 4096 receivers, checkpoints every "
            "50 steps, smoothing sigma 10" % nshot)
    if not inversion:
        cfg, sol = _solver_for(pkg, tmp, values, src, rec, nx, nz, h, true)
        sol.set_option("ckpt", 2)
        obs = {"x": np.zeros((nshot, nx, nt), np.float32), "z": np.zeros((nshot, nx, nt), np.float32)}
        mis = pkg.Misfit.from_obs(0, sol, obs, pkg.GaussianFilter(nx, nz, 10))
        sol.timer_begin()
        mis.run(kernel=True)
        ms = sol.timer_end()
        st = sol.stats()
        per_launch = st.step_ms / max(st.step_launches, 1)
        cells = nx * nz * min(nshot, st.batch_capacity)
        _line("shots/s fwd+adj (P-SV 4096x1024 gradient)", round(nshot / (ms / 1e3), 3), "shots/s",
              {"workload": desc + ", FP16 checkpoints"},
              ms_per_step=round(ms, 1), batch=st.batch_capacity, tile=[st.tile_tz, st.tile_tx],
              step_kernel={"avg_launch_us": round(per_launch * 1e3, 2),
                           "achieved_gbs": round(68.0 * cells / (per_launch * 1e-3) / 1e9, 1)})
        return
    from scipy.ndimage import gaussian_filter

    init_v = [np.ascontiguousarray(gaussian_filter(a.reshape(nx, nz).astype(np.float64), 500.0 / h,
                                                   mode="nearest").astype(np.float32).ravel())
              for a in (vs, vp, rho)]
    init = lame(*init_v)
    # observed data on the true model (setup)
    cfg, sol = _solver_for(pkg, tmp, values, src, rec, nx, nz, h, true)
    obs = {"x": np.empty((nshot, nx, nt), np.float32), "z": np.empty((nshot, nx, nt), np.float32)}
    cap = sol.capacity
    for a0 in range(0, nshot, cap):
        shots = list(range(a0, min(nshot, a0 + cap)))
        sol.run_forward_batch(shots)
        for q, s_ in enumerate(shots):
            obs["x"][s_] = sol.out("x", slot=q)
            obs["z"][s_] = sol.out("z", slot=q)
    sol.close()
    res = {}
    models = {}
    names = [p.strip() for p in args.precisions.split(",") if p.strip()]
    if not names or any(p not in ("bf16", "fp32") for p in names):
        raise SystemExit("--precisions: bf16 and/or fp32")
    for prec, name in ((1, "bf16"), (0, "fp32")):
        if name not in names:
            continue
        cfg, sol = _solver_for(pkg, tmp, values, src, rec, nx, nz, h, init)
        sol.set_option("ckpt", prec)
        mis = pkg.Misfit.from_obs(0, sol, obs, pkg.GaussianFilter(nx, nz, 10))
        opt = pkg.Optimizer(cfg, sol, mis)
        t0 = time.perf_counter()
        opt.run()
        wall = time.perf_counter() - t0
        hist = opt.history()
        ev = opt.evaluations()
        models[name] = sol.model()
        st = sol.stats()
        # the history holds the misfit at the start of every iteration begun
        # and the final one; the optimizer stops before --iterations when a
        # line search fails (the reference's rule)
        begun = max(len(hist) - 1, 1)
        res[name] = {"wall_s": round(wall, 1), "iterations_begun": len(hist) - 1,
                     "s_per_iteration": round(wall / begun, 1),
                     "misfit_history": [float("%.6g" % v) for v in hist],
                     "evaluations": len(ev), "batch": st.batch_capacity}
        opt.close()
        mis.close()
        sol.close()

    def rel(a, b):
        return float(np.linalg.norm(a.astype(np.float64) - b) / np.linalg.norm(b.astype(np.float64)))

    for name in names:
        res[name]["model_error_vs_true"] = {k: rel(models[name][k], true[q]) for q, k in enumerate(("lambda", "mu"))}
    if len(names) == 2:
        res["bf16_vs_fp32_model"] = {k: rel(models["bf16"][k], models["fp32"][k]) for k in ("lambda", "mu")}
        res["bf16_vs_fp32_update"] = {
            k: float(np.linalg.norm(models["bf16"][k].astype(np.float64) - models["fp32"][k]) /
                     np.linalg.norm(models["fp32"][k].astype(np.float64) - init[q]))
            for q, k in enumerate(("lambda", "mu"))}
    res["initial_model_error_vs_true"] = {k: rel(init[q], true[q]) for q, k in enumerate(("lambda", "mu"))}
    _line("full inversion, s per L-BFGS iteration (P-SV 4096x1024, %d shots)" % nshot,
          res[names[0]]["s_per_iteration"], "s/iteration",
          {"workload": desc + ", L-BFGS memory 10, %d of 20 iterations requested, %s checkpoints, initial "
                       "model smoothed by a 500 m Gaussian" % (args.iterations, " and ".join(n.upper() for n in names))},
          higher_is_better=False, inversion=res)


def run_profile_case(args):
    """Small forward batch for ncu captures of the step kernel (eager launches)."""
    import __graft_entry__ as ge
    from tests import cases

    pkg = ge.load_package()
    name = args.profile_case
    if name == "sh-c2-nt200":
        # the headline workload's shapes (16 shots, 681 receivers, checkpoints
        # every 10 steps) over 200 steps: one forward and one adjoint pass
        wl = workload()
        cfg = pkg.Config.new(tempfile.mkdtemp(prefix="gbfwi_prof_"), dict(wl["values"], nt=200), wl["src"], wl["rec"])
        sol = pkg.FdmSolver(cfg, grid=(NX, NZ, wl["xmax"], wl["zmax"]))
        sol.set_option("batch", NSHOT)
        sol.set_option("graphs", 0)
        sol.set_option("cluster", args.cluster)
        sol.set_model_grid(*wl["init"])
        shots = list(range(NSHOT))
        sol.run_forward_batch(shots)
        rng = np.random.default_rng(0)
        for b in shots:
            sol.set_adstf("y", (rng.standard_normal((NX, 200)) * 1e-3).astype(np.float32), slot=b)
        sol.initKernels()
        sol.run_adjoint_batch(shots)
        st = sol.stats()
        print("profile case", name, "cluster", args.cluster, "forward_ms %.3f adjoint_ms %.3f" % (st.forward_ms,
                                                                                            st.adjoint_ms))
        return
    # "<psv|sh>-<nx>x<nz>x<shots>": a 12-step forward batch (the launches an
    # ncu capture selects), then three more timed with the solver's CUDA
    # events: time per step and algorithmic bandwidth (68 / 40 B per cell)
    try:
        wave, dims = name.split("-")
        nx, nz, nshot = (int(v) for v in dims.split("x"))
        assert wave in ("psv", "sh")
    except (ValueError, AssertionError):
        raise SystemExit("unknown profile case " + name)
    case = cases.make_case(wave=wave, nx=nx, nz=nz, nt=12, nsrc=nshot, nrec=min(nx - 4, 256), seed=1, abs_width=20)
    case["values"]["mode"] = 3
    cfg, sol = cases.gpu_solver(pkg, case)
    sol.set_option("tile", args.tile)
    sol.set_option("graphs", 0)
    sol.set_option("cluster", args.cluster)
    sol.set_option("tma", args.tma)
    shots = list(range(nshot))
    sol.run_forward_batch(shots)
    sol.stats(reset=True)
    for _ in range(3):
        sol.run_forward_batch(shots)
    st = sol.stats()
    us = 1e3 * st.step_ms / max(st.step_launches, 1)
    gbs = (68.0 if wave == "psv" else 40.0) * nx * nz * nshot / (us * 1e-6) / 1e9
    print("profile case %s tile %d cluster %d: %.2f us per step, %.1f GB/s algorithmic, bulk loads %d" %
          (name, args.tile, args.cluster, us, gbs, st.march_bulk))


def run_reference(args, ws, rank):
    """The reference arm. The reference's path is CUDA only; its CPU
    restatement (oracle/, pinned against the reference's golden seismograms)
    is the CPU implementation timed here, on all host cores: --warmup shots,
    then --steps timed shots (one shot per step, shots 0..15 in turn), and
    one smoothing of the three kernels timed on its own; shots/s counts a
    gradient as 16 shots + one smoothing. Beside it, when a GPU and the
    reference's compiled kernels are present, one full gradient through
    those kernels (`reference_gpu`)."""
    if rank != 0:
        return
    wl = workload()
    port = CpuPort(wl)
    for q in range(args.warmup):
        port.shot(q)
    shots = [port.shot(args.warmup + q) for q in range(args.steps)]
    t_smooth = port.smoothing()
    t_shot = sum(shots) / len(shots)
    value = NSHOT / (NSHOT * t_shot + t_smooth)
    ms_step = 1e3 * (t_shot + t_smooth / NSHOT)
    desc = ("one full shot per step (forward %d steps with checkpoints, envelope misfit, adjoint), %d steps; "
            "smoothing of 3 kernels timed once and shared over 16 shots" % (NT, args.steps))
    line = {
        "metric": METRIC, "value": round(value, 4), "unit": "shots/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_step, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded faulted layered model with the workload's shapes; no dataset)",
        "config": dict(CONFIG_DESC), "impl": "reference",
        "cpu_baseline": {"value": round(value, 4), "unit": "shots/s", "cores": port.threads, "kind": "port",
                         "sample": desc},
        "e2e": {"value": round(value, 4), "unit": "shots/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "run": {"parallelism": "host cores (OpenMP over columns)", "step": "one shot"},
        "note": "the reference's path is CUDA only; its CPU restatement (oracle/, pinned against the "
                "reference's golden seismograms) is the CPU implementation timed here",
    }
    if not args.no_ref_gpu:
        line["reference_gpu"] = _reference_gpu_leg(wl)
    print(json.dumps(line), flush=True)


def _reference_gpu_leg(wl):
    try:
        import __graft_entry__ as ge

        if ge.load_package().device_count() < 1:
            return {"unavailable": "no CUDA device"}
        return reference_gpu_sample(wl)
    except Exception as e:  # reported in the line, never fatal to the arm
        return {"unavailable": "%s: %s" % (type(e).__name__, e)}


# ----------------------------------------------------------------------------
_PG = None


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(v, ws):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(v)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain-path leg")
    ap.add_argument("--no-ref-gpu", action="store_true", help="skip the reference-kernels-on-GPU leg")
    ap.add_argument("--no-hbm-step", action="store_true", help="skip the per-step marching-kernel records")
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c3", "c4", "c5"],
                    help="c2 is the headline; the others print their own line")
    ap.add_argument("--shots", type=int, default=0,
                    help="shot count for c3/c5 (default 64; c5 16, or 128 with --iterations)")
    ap.add_argument("--iterations", type=int, default=0, help="c5: run that many L-BFGS iterations of the inversion")
    ap.add_argument("--precisions", default="bf16,fp32", help="c5 inversion: checkpoint precisions to run")
    ap.add_argument("--requests", type=int, default=512, help="c4 request count")
    ap.add_argument("--rate", type=float, default=0.0,
                    help="c4 Poisson arrival rate (requests/s); 0: --load x the measured capacity")
    ap.add_argument("--load", type=float, default=0.8, help="c4 arrival rate as a fraction of capacity")
    ap.add_argument("--sequential", type=int, default=64, help="c4 requests also solved one at a time")
    ap.add_argument("--server-tile", type=int, default=0,
                    help="c4 step kernel configuration (0: the engine's default)")
    ap.add_argument("--server-streams", type=int, default=0,
                    help="c4 engine streams, 1, 2 or 4 (0: the engine's default)")
    ap.add_argument("--server-compact", type=int, default=-1,
                    help="c4: 1 launches the requests' own tiles through a block map, 0 the largest request's "
                         "tile count for every request (default: the engine's choice)")
    ap.add_argument("--profile-case", default="", help="run one small case for an ncu capture")
    ap.add_argument("--tile", type=int, default=3, help="kernel configuration for --profile-case")
    ap.add_argument("--tma", type=int, default=1, help="--profile-case: marching kernel bulk loads (1) or cp.async (0)")
    ap.add_argument("--cluster", type=int, default=0,
                    help="--profile-case: 0 per-step kernels, 1 cluster-resident (automatic size), 2..16 that size")
    args = ap.parse_args()
    if args.profile_case:
        run_profile_case(args)
        return
    if args.workload != "c2":
        {"c1": run_c1, "c3": run_c3, "c4": run_c4, "c5": run_c5}[args.workload](args)
        return
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    try:
        if args.impl == "reference":
            run_reference(args, ws, rank)
        else:
            run_ours(args, ws, rank, local)
    finally:
        if ws > 1:
            import torch.distributed as dist

            dist.destroy_process_group()


if __name__ == "__main__":
    main()
