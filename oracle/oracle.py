"""CPU oracle for the inv.cu hot path — TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` import this module, as the checker (or the timed CPU baseline).
The product path never imports it.

It restates the reference algorithm:
  * heavy loops in C (``fdm_oracle.c``: solver/fdm.h, filter/gaussian.h,
    source/ricker.h, misfit/waveform.h taper), loaded with ctypes;
  * setup, file formats and misfits in numpy:
      - Config parsing ............ lib/config.h:9-108
      - grid inference ............ solver/fdm.h:354-391
      - model files (.bin) ........ solver/solver.h:225-252
      - SU traces ................. solver/solver.h:38-108, misfit/misfit.h:52-90
      - v->u integration .......... misfit/misfit.h:110-120
      - waveform misfit ........... misfit/waveform.h:4-40
      - envelope misfit ........... misfit/envelope.h:4-90 (Hilbert mask quirks)

Pinning: the forward SH path is pinned against the reference's golden
seismograms (example/checker/traces/*.su, see tests/golden/). On a GPU, the
reference's own kernels (compiled from its sources into _ref/inv_ref.cubin)
run under ref_harness.cu's restatement of its host loops (the ``ref_*``
functions below): forward P-SV/SH, adjoint kernels, absorbing boundary and
Gaussian filter as the reference computes them.
"""
from __future__ import annotations

import ctypes
import math
import os
import re
import subprocess
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


class OrcParams(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("nz", ctypes.c_int), ("nt", ctypes.c_int), ("sfe", ctypes.c_int),
        ("sh", ctypes.c_int), ("psv", ctypes.c_int), ("nsrc", ctypes.c_int), ("nrec", ctypes.c_int),
        ("dx", ctypes.c_double), ("dz", ctypes.c_double), ("dt", ctypes.c_double),
        ("record_u", ctypes.c_int), ("adj", ctypes.c_int),
        ("inv_lambda", ctypes.c_int), ("inv_mu", ctypes.c_int), ("inv_rho", ctypes.c_int),
    ]


# checkout of the reference sources, named by the environment (GBFWI_REF_SRC)
REF_SRC = os.environ.get("GBFWI_REF_SRC", "")
REF_CUBIN = os.path.join(_HERE, "_ref", "inv_ref.cubin")
_REF = None


def build() -> str:
    """Compile the C oracle (gcc) and the reference-kernel harness (nvcc) with
    the Makefile, and the reference's kernels when GBFWI_REF_SRC names a
    checkout of its sources (the cubin built earlier is kept otherwise)."""
    subprocess.run(["make", "-s", "-C", _HERE, "all", "harness"], check=True)
    if REF_SRC and os.path.exists(os.path.join(REF_SRC, "inv.cu")):
        subprocess.run(["make", "-s", "-C", _HERE, "ref", "REFSRC=" + REF_SRC], check=True)
    return os.path.join(_HERE, "_build", "liboracle.so")


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "_build", "liboracle.so")
        if not os.path.exists(path) or os.path.getmtime(path) < max(
                os.path.getmtime(os.path.join(_HERE, f)) for f in ("fdm_oracle.c", "fdm_oracle_body.h")):
            build()
        _LIB = ctypes.CDLL(path)
    return _LIB


def _p(a):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.c_void_p)


def set_threads(n: int) -> None:
    lib().orc_set_threads(ctypes.c_int(n))


def num_threads() -> int:
    return lib().orc_num_threads()


# ----------------------------------------------------------------------------
# Config (lib/config.h)
# ----------------------------------------------------------------------------
_FLOAT_TOKEN = r"[+-]?(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?"
_FLOAT_RE = re.compile(r"^" + _FLOAT_TOKEN + r"$")


def _parse_float_token(tok: str):
    """istringstream >> float accepted only when the whole token is consumed."""
    if _FLOAT_RE.match(tok):
        v = np.float32(float(tok))
        if np.isfinite(v):
            return float(v)
    return None


def _load_config_file(path: str, cfg: dict) -> None:
    """Config::loadConfig (lib/config.h:22-44): first definition of a key wins."""
    try:
        with open(path, "r", newline="\n") as fh:
            lines = fh.read().split("\n")
    except OSError:
        return
    for data in lines:
        data = data.lstrip(" \t")
        pos = data.find("=")
        if pos < 0:
            continue
        ktoks = data[:pos].split()
        vtoks = data[pos + 1:].split()
        key = ktoks[0] if ktoks else ""
        value = vtoks[0] if vtoks else ""
        if key and value and key[0] != "#" and not cfg.get(key):
            cfg[key] = value


def _load_rows(path: str, ncol: int) -> list:
    """Config::loadSource / loadStation (lib/config.h:45-84): a line is kept
    only when exactly ncol numbers parse and nothing follows the last one."""
    rows = []
    try:
        with open(path, "r", newline="\n") as fh:
            lines = fh.read().split("\n")
    except OSError:
        return rows
    row_re = re.compile(r"^(?:\s*(" + _FLOAT_TOKEN + r")){%d}$" % ncol)
    for data in lines:
        data = data.lstrip(" \t")
        if not row_re.match(data):
            continue
        vals = [np.float32(float(t)) for t in data.split()]
        if len(vals) == ncol and all(np.isfinite(vals)):
            rows.append([float(v) for v in vals])
    return rows


@dataclass
class Config:
    """Mirror of the reference's Config (lib/config.h:86-108)."""
    path: str
    f: dict = field(default_factory=dict)
    i: dict = field(default_factory=dict)
    src: list = field(default_factory=list)
    rec: list = field(default_factory=list)

    @classmethod
    def load(cls, cfgdir: str, overrides: dict | None = None, cwd: str | None = None):
        cfg = dict(overrides or {})
        cfg["config"] = cfgdir
        _load_config_file(os.path.join(cfgdir, "config.ini"), cfg)
        if cfg.get("inherit"):
            inh = cfg["inherit"]
            if cwd and not os.path.isabs(inh):
                inh = os.path.join(cwd, inh)
            _load_config_file(inh, cfg)
        c = cls(path=cfgdir)
        for k, v in cfg.items():
            if k in ("config", "inherit"):
                continue
            fv = _parse_float_token(v)
            if fv is not None:
                c.f[k] = fv
                c.i[k] = int(math.floor(abs(fv) + 0.5)) * (1 if fv >= 0 else -1)
        c.src = _load_rows(os.path.join(cfgdir, "sources.dat"), 7)
        c.rec = _load_rows(os.path.join(cfgdir, "stations.dat"), 2)
        return c

    def fv(self, k):
        return self.f.get(k, 0.0)

    def iv(self, k):
        return self.i.get(k, 0)


# ----------------------------------------------------------------------------
# Model files and grid inference
# ----------------------------------------------------------------------------
def read_bin(path: str) -> np.ndarray:
    """int32 npt followed by float32[npt] (solver/solver.h:109-120,225-252)."""
    raw = np.fromfile(path, dtype=np.uint8)
    npt = int(np.frombuffer(raw[:4].tobytes(), dtype=np.int32)[0])
    return np.frombuffer(raw[4:4 + 4 * npt].tobytes(), dtype=np.float32).copy()


def write_bin(path: str, data) -> None:
    data = np.ascontiguousarray(data, dtype=np.float32).ravel()
    with open(path, "wb") as fh:
        fh.write(np.int32(data.size).tobytes())
        fh.write(data.tobytes())


def infer_grid(xs: np.ndarray, zs: np.ndarray):
    """FdmSolver::init grid inference (solver/fdm.h:354-391), float arithmetic."""
    f32 = np.float32
    npt = xs.size
    xmax = f32(0)
    for v in (xs.max(initial=0),):
        xmax = f32(max(f32(0), f32(v)))
    zmax = f32(max(f32(0), f32(zs.max(initial=0))))
    a = f32(zmax / xmax)
    b = f32(a + f32(1))
    c = f32(1 - npt)
    root = f32(np.sqrt(f32(b * b - f32(f32(4) * a) * c)))
    nx = _round(f32(f32(-b + root) / f32(f32(2) * a))) + 1
    nz = int(npt // nx)
    dx = f32(xmax / f32(nx - 1))
    dz = f32(zmax / f32(nz - 1))
    return nx, nz, float(dx), float(dz), float(xmax), float(zmax)


def calc_idx(coords, L: float, n: int) -> np.ndarray:
    coords = np.ascontiguousarray(coords, dtype=np.float32)
    out = np.zeros(coords.size, dtype=np.int32)
    lib().orc_calc_idx(ctypes.c_int(coords.size), _p(coords), ctypes.c_float(L), ctypes.c_float(n), _p(out))
    return out


def absbound(nx, nz, width, alpha, left, right, bottom, top) -> np.ndarray:
    ab = np.zeros(nx * nz, dtype=np.float32)
    lib().orc_absbound(nx, nz, int(width), ctypes.c_float(alpha), int(left), int(right), int(bottom),
                       int(top), _p(ab))
    return ab


def ricker(nt, dt, f0, t0, angle, amp):
    sx = np.zeros(nt, np.float32)
    sy = np.zeros(nt, np.float32)
    sz = np.zeros(nt, np.float32)
    lib().orc_ricker(nt, ctypes.c_float(dt), ctypes.c_float(f0), ctypes.c_float(t0), ctypes.c_float(angle),
                     ctypes.c_float(amp), _p(sx), _p(sy), _p(sz))
    return sx, sy, sz


def taper(nt, dt) -> np.ndarray:
    tw = np.zeros(nt, np.float32)
    lib().orc_taper(nt, ctypes.c_float(dt), _p(tw))
    return tw


def mesh2grid(nx, nz, dx, dz, px, pz, pvp, pvs, prho, xmax, zmax):
    f32 = np.float32
    lam = np.zeros(nx * nz, f32)
    mu = np.zeros(nx * nz, f32)
    rho = np.zeros(nx * nz, f32)
    arrs = [np.ascontiguousarray(a, dtype=f32) for a in (px, pz, pvp, pvs, prho)]
    dmax = f32(f32(xmax) * f32(xmax) + f32(zmax) * f32(zmax))
    lib().orc_mesh2grid(nx, nz, ctypes.c_float(dx), ctypes.c_float(dz), arrs[0].size, *[_p(a) for a in arrs],
                        ctypes.c_float(dmax), _p(lam), _p(mu), _p(rho))
    return lam, mu, rho


def vps2lm(lam, mu, rho):
    lam = np.ascontiguousarray(lam, np.float32).copy()
    mu = np.ascontiguousarray(mu, np.float32).copy()
    rho = np.ascontiguousarray(rho, np.float32)
    lib().orc_vps2lm(ctypes.c_size_t(lam.size), _p(lam), _p(mu), _p(rho))
    return lam, mu


def gaussian_filter(nx, nz, sigma, data) -> np.ndarray:
    d = np.ascontiguousarray(data, np.float32).copy()
    lib().orc_gaussian(nx, nz, int(sigma), _p(d))
    return d


def gauss_weight(i, n, sigma) -> float:
    f = lib().orc_gauss_weight
    f.restype = ctypes.c_float
    return f(ctypes.c_longlong(i), ctypes.c_longlong(n), ctypes.c_int(sigma))


# ----------------------------------------------------------------------------
# Solver
# ----------------------------------------------------------------------------
@dataclass
class Problem:
    """Everything one solve needs, in the reference layout (k = i*nz + j)."""
    nx: int
    nz: int
    nt: int
    dx: float
    dz: float
    dt: float
    sh: bool
    psv: bool
    sfe: int
    lam: np.ndarray
    mu: np.ndarray
    rho: np.ndarray
    ab: np.ndarray
    stf: tuple          # (stf_x, stf_y, stf_z) each float32[nsrc*nt]
    src_id: tuple       # (x ids, z ids) int32[nsrc]
    rec_id: tuple       # (x ids, z ids) int32[nrec]
    inv_lambda: bool = True
    inv_mu: bool = True
    inv_rho: bool = True

    @property
    def nsrc(self):
        return int(self.src_id[0].size)

    @property
    def nrec(self):
        return int(self.rec_id[0].size)

    def params(self, adj: bool, record_u: bool) -> OrcParams:
        return OrcParams(self.nx, self.nz, self.nt, self.sfe, int(self.sh), int(self.psv), self.nsrc,
                         self.nrec, float(self.dx), float(self.dz), float(self.dt), int(record_u), int(adj),
                         int(self.inv_lambda), int(self.inv_mu), int(self.inv_rho))

    def nckpt(self):
        return (2 if self.sh else 0) + (4 if self.psv else 0)


def _cast(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def forward(pb: Problem, isrc: int, adj: bool = True, record_u: bool | None = None, precision="f32"):
    """FdmSolver::runForward. Returns (out_x, out_y, out_z, ckpt); traces are
    [nrec, nt]; ckpt is [nsfe, nf, nx*nz] (u fields then v fields) or None."""
    dt = np.float32 if precision == "f32" else np.float64
    if record_u is None:
        record_u = adj
    n = pb.nx * pb.nz
    outs = [np.zeros(pb.nrec * pb.nt, dt) for _ in range(3)]
    nsfe = pb.nt // pb.sfe if (adj and pb.sfe) else 0
    ckpt = np.zeros(nsfe * pb.nckpt() * n, dt) if nsfe else None
    mats = [_cast(a, dt) for a in (pb.lam, pb.mu, pb.rho, pb.ab)]
    stf = [_cast(a, dt) for a in pb.stf]
    ids = [_cast(a, np.int32) for a in (*pb.src_id, *pb.rec_id)]
    prm = pb.params(adj, record_u)
    fn = lib().orc_forward_f32 if precision == "f32" else lib().orc_forward_f64
    fn(ctypes.byref(prm), *[_p(a) for a in mats], *[_p(a) for a in stf], *[_p(a) for a in ids],
       ctypes.c_int(isrc), *[_p(a) for a in outs], _p(ckpt))
    outs = [o.reshape(pb.nrec, pb.nt) for o in outs]
    if ckpt is not None:
        ckpt = ckpt.reshape(nsfe, pb.nckpt(), n)
    return outs[0], outs[1], outs[2], ckpt


def adjoint(pb: Problem, adstf, ckpt, kernels=None, precision="f32"):
    """FdmSolver::runAdjoint. adstf = (x, y, z) [nrec, nt]; kernels (k_lambda,
    k_mu, k_rho) are updated in place and returned."""
    dt = np.float32 if precision == "f32" else np.float64
    n = pb.nx * pb.nz
    if kernels is None:
        kernels = [np.zeros(n, dt) for _ in range(3)]
    kernels = [k if (k.dtype == dt and k.flags.c_contiguous) else _cast(k, dt) for k in kernels]
    mats = [_cast(a, dt) for a in (pb.lam, pb.mu, pb.rho, pb.ab)]
    ad = [_cast(a, dt).ravel() for a in adstf]
    ids = [_cast(a, np.int32) for a in pb.rec_id]
    ck = _cast(ckpt, dt).ravel()
    prm = pb.params(True, True)
    fn = lib().orc_adjoint_f32 if precision == "f32" else lib().orc_adjoint_f64
    fn(ctypes.byref(prm), *[_p(a) for a in mats], *[_p(a) for a in ad], *[_p(a) for a in ids], _p(ck),
       *[_p(k) for k in kernels])
    return kernels


# ----------------------------------------------------------------------------
# Misfits (FP64 sums; the reference sums FP32 cuBLAS norms)
# ----------------------------------------------------------------------------
def waveform_misfit(syn, obs, tw, dt):
    """WaveformMisfit::run per trace (misfit/waveform.h:4-8,35-40).
    syn/obs [ntr, nt]. Returns (sum of per-trace values, adstf [ntr, nt])."""
    syn = np.asarray(syn, np.float32)
    obs = np.asarray(obs, np.float32)
    r = (syn - obs) * tw
    ad = (r * tw * np.float32(2))[:, ::-1].astype(np.float32)
    val = np.sqrt((r.astype(np.float64) ** 2).sum(axis=1)) * math.sqrt(np.float32(dt))
    return float(val.sum()), np.ascontiguousarray(ad)


def hilbert_analytic(x):
    """hilbert() (misfit/envelope.h:83-90) with the _hilbert mask
    (envelope.h:4-28): returns the unnormalised inverse transform (n times
    the analytic signal), rows = traces. For even n, bins 1..n/2 are doubled
    (Nyquist included), bin n/2+1 is left as is, higher bins are zeroed; for
    odd n, bins 1..(n-1)/2 are doubled and the rest zeroed."""
    x = np.asarray(x, np.float64)
    n = x.shape[-1]
    h = np.fft.fft(x, axis=-1)
    i = np.arange(n)
    mask = np.ones(n)
    if n % 2 == 0:
        mask[(i > 0) & (i < n // 2 + 1)] = 2
        mask[i > n // 2 + 1] = 0
    else:
        mask[(i > 0) & (i < (n + 1) // 2)] = 2
        mask[(i > 0) & (i >= (n + 1) // 2)] = 0
    return np.fft.ifft(h * mask, axis=-1) * n


def envelope_misfit(syn, obs, dt):
    """EnvelopeMisfit::run per trace (misfit/envelope.h:62-82)."""
    syn = np.asarray(syn, np.float64)
    obs = np.asarray(obs, np.float64)
    n = syn.shape[-1]
    csyn = hilbert_analytic(syn)
    cobs = hilbert_analytic(obs)
    esyn = np.abs(csyn) / n
    eobs = np.abs(cobs) / n
    mx = np.maximum(esyn.max(axis=-1, keepdims=True) * 0.05, 0.05)
    etmp = (esyn - eobs) / (esyn + mx)
    ersd = csyn.imag / n * etmp
    ersd = hilbert_analytic(ersd).imag / n
    ad = (etmp * syn - ersd)[:, ::-1]
    val = np.sqrt(((esyn - eobs) ** 2).sum(axis=-1)) * math.sqrt(np.float32(dt))
    return float(val.sum()), np.ascontiguousarray(ad.astype(np.float32))


def v2u(traces, dt):
    """Velocity -> displacement running sum (misfit/misfit.h:110-120), float."""
    t = np.array(traces, dtype=np.float32, copy=True)
    dt = np.float32(dt)
    t[..., 0] *= dt
    for it in range(1, t.shape[-1]):
        t[..., it] = t[..., it - 1] + t[..., it] * dt
    return t


# ----------------------------------------------------------------------------
# SU traces (solver/solver.h:38-108, misfit/misfit.h:52-90)
# ----------------------------------------------------------------------------
def read_su(path, nrec=None):
    raw = np.fromfile(path, dtype=np.uint8)
    nt = int(np.frombuffer(raw[114:116].tobytes(), dtype=np.int16)[0])
    rec = 240 + 4 * nt
    ntr = raw.size // rec if nrec is None else nrec
    out = np.zeros((ntr, nt), np.float32)
    heads = []
    for ir in range(ntr):
        b = raw[ir * rec:(ir + 1) * rec]
        heads.append(b[:240].copy())
        out[ir] = np.frombuffer(b[240:].tobytes(), dtype=np.float32)
    return out, heads


def _round(v) -> int:
    """std::round: halves away from zero."""
    v = float(v)
    return int(math.floor(abs(v) + 0.5)) * (1 if v >= 0 else -1)


def su_headers(nrec, nt, dt, xs, zs, rec_x, rec_z):
    """The 240-byte headers the reference writes for one shot."""
    f32 = np.float32
    dt_int2 = 0 if float(np.float32(dt)) * 1e6 > 2 ** 15 else int(float(np.float32(dt)) * 1e6)
    heads = []
    for ir in range(nrec):
        h1 = np.zeros(28, np.int32)
        h1[0] = ir + 1
        h1[9] = _round(f32(f32(rec_x[ir]) - f32(xs)))
        h1[18] = _round(f32(xs))
        h1[19] = _round(f32(zs))
        h1[20] = _round(f32(rec_x[ir]))
        h1[21] = _round(f32(rec_z[ir]))
        h2 = np.array([0, nt], np.int16)
        h3 = np.array([dt_int2, 0], np.int16)
        h4 = np.zeros(30, np.float32)
        if nrec > 1:
            h4[1] = f32(f32(rec_x[1]) - f32(rec_x[0]))
        heads.append(h1.tobytes() + h2.tobytes() + h3.tobytes() + h4.tobytes())
    return heads


# ----------------------------------------------------------------------------
# Problem builder from a reference example directory
# ----------------------------------------------------------------------------
def problem_from_config(cfg: Config, model: str = "model_true") -> Problem:
    """Solver::init + FdmSolver::init + importModel, restated on the host."""
    base = cfg.path
    xs = read_bin(os.path.join(base, "model_true", "proc000000_x.bin"))
    zs = read_bin(os.path.join(base, "model_true", "proc000000_z.bin"))
    nx, nz, dx, dz, xmax, zmax = infer_grid(xs, zs)
    nt = cfg.iv("nt")
    dt = cfg.fv("dt")
    px = read_bin(os.path.join(base, model, "proc000000_x.bin"))
    pz = read_bin(os.path.join(base, model, "proc000000_z.bin"))
    mtype = cfg.iv("model_type")
    a = read_bin(os.path.join(base, model, "proc000000_%s.bin" % ("lambda" if mtype else "vp")))
    b = read_bin(os.path.join(base, model, "proc000000_%s.bin" % ("mu" if mtype else "vs")))
    r = read_bin(os.path.join(base, model, "proc000000_rho.bin"))
    lam, mu, rho = mesh2grid(nx, nz, dx, dz, px, pz, a, b, r, xmax, zmax)
    if mtype == 0:
        lam, mu = vps2lm(lam, mu, rho)
    src = np.array(cfg.src, np.float32).reshape(-1, 7)
    rec = np.array(cfg.rec, np.float32).reshape(-1, 2)
    stfs = [np.zeros(len(src) * nt, np.float32) for _ in range(3)]
    for s in range(len(src)):
        sx, sy, sz = ricker(nt, dt, src[s, 3], src[s, 4], src[s, 5], src[s, 6])
        stfs[0][s * nt:(s + 1) * nt] = sx
        stfs[1][s * nt:(s + 1) * nt] = sy
        stfs[2][s * nt:(s + 1) * nt] = sz
    ab = absbound(nx, nz, cfg.iv("abs_width"), cfg.fv("abs_alpha"), cfg.iv("abs_left"), cfg.iv("abs_right"),
                  cfg.iv("abs_bottom"), cfg.iv("abs_top"))
    return Problem(nx=nx, nz=nz, nt=nt, dx=dx, dz=dz, dt=dt, sh=bool(cfg.iv("sh")), psv=bool(cfg.iv("psv")),
                   sfe=cfg.iv("sfe"), lam=lam, mu=mu, rho=rho, ab=ab, stf=tuple(stfs),
                   src_id=(calc_idx(src[:, 0], xmax, nx), calc_idx(src[:, 1], zmax, nz)),
                   rec_id=(calc_idx(rec[:, 0], xmax, nx), calc_idx(rec[:, 1], zmax, nz)),
                   inv_lambda=bool(cfg.iv("inv_lambda")), inv_mu=bool(cfg.iv("inv_mu")),
                   inv_rho=bool(cfg.iv("inv_rho")))


# ----------------------------------------------------------------------------
# The reference's own kernels (ref_harness.cu; needs a GPU and _ref/inv_ref.cubin)
# ----------------------------------------------------------------------------
def ref_available() -> bool:
    return os.path.exists(REF_CUBIN) and os.path.exists(os.path.join(_HERE, "_build", "libref_harness.so"))


def ref_lib():
    """The harness, with the reference's cubin loaded (raises when absent)."""
    global _REF
    if _REF is None:
        lib_ = ctypes.CDLL(os.path.join(_HERE, "_build", "libref_harness.so"))
        lib_.ref_last_error.restype = ctypes.c_char_p
        if lib_.ref_open(REF_CUBIN.encode()) != 0:
            raise RuntimeError("reference kernels: " + lib_.ref_last_error().decode())
        _REF = lib_
    return _REF


def _ref_check(rc, what):
    if rc != 0:
        raise RuntimeError("%s: %s" % (what, ref_lib().ref_last_error().decode()))


def ref_absbound(nx, nz, width, alpha, left, right, bottom, top) -> np.ndarray:
    """initAbsbound (solver/fdm.h:48-74) run by the reference's kernel."""
    out = np.zeros(nx * nz, np.float32)
    _ref_check(ref_lib().ref_absbound(nx, nz, int(width), ctypes.c_float(alpha), int(left), int(right),
                                      int(bottom), int(top), _p(out)), "ref_absbound")
    return out


def ref_forward(pb: Problem, isrc: int, adj: bool = True, record_u: bool | None = None, ab=None):
    """FdmSolver::runForward with the reference's kernels; as forward() (one
    wave system). ab: absorbing profile (default pb.ab)."""
    if record_u is None:
        record_u = adj
    n = pb.nx * pb.nz
    outs = [np.zeros(pb.nrec * pb.nt, np.float32) for _ in range(3)]
    nsfe = pb.nt // pb.sfe if (adj and pb.sfe) else 0
    ckpt = np.zeros(nsfe * pb.nckpt() * n, np.float32) if nsfe else None
    mats = [_cast(a, np.float32) for a in (pb.lam, pb.mu, pb.rho, pb.ab if ab is None else ab)]
    stf = [_cast(a, np.float32) for a in pb.stf]
    ids = [_cast(a, np.int32) for a in (*pb.src_id, *pb.rec_id)]
    prm = pb.params(adj, record_u)
    _ref_check(ref_lib().ref_forward(ctypes.byref(prm), *[_p(a) for a in mats], *[_p(a) for a in stf],
                                     *[_p(a) for a in ids], ctypes.c_int(isrc), *[_p(o) for o in outs], _p(ckpt)),
               "ref_forward")
    outs = [o.reshape(pb.nrec, pb.nt) for o in outs]
    if ckpt is not None:
        ckpt = ckpt.reshape(nsfe, pb.nckpt(), n)
    return outs[0], outs[1], outs[2], ckpt


def ref_adjoint(pb: Problem, adstf, ckpt, kernels=None, ab=None):
    """FdmSolver::runAdjoint with the reference's kernels; as adjoint()."""
    n = pb.nx * pb.nz
    if kernels is None:
        kernels = [np.zeros(n, np.float32) for _ in range(3)]
    kernels = [_cast(k, np.float32).copy() for k in kernels]
    mats = [_cast(a, np.float32) for a in (pb.lam, pb.mu, pb.rho, pb.ab if ab is None else ab)]
    ad = [_cast(a, np.float32).ravel() for a in adstf]
    ids = [_cast(a, np.int32) for a in pb.rec_id]
    ck = _cast(ckpt, np.float32).ravel()
    prm = pb.params(True, True)
    _ref_check(ref_lib().ref_adjoint(ctypes.byref(prm), *[_p(a) for a in mats], *[_p(a) for a in ad],
                                     *[_p(a) for a in ids], _p(ck), *[_p(k) for k in kernels]), "ref_adjoint")
    return kernels


def ref_gaussian(nx, nz, sigma, data) -> np.ndarray:
    """GaussianFilter::init + apply (filter/gaussian.h:37-61) with the reference's kernels."""
    d = np.ascontiguousarray(data, np.float32).copy()
    _ref_check(ref_lib().ref_gaussian(nx, nz, int(sigma), _p(d)), "ref_gaussian")
    return d


def ref_misfit(kind: int, syn, obs, dt: float):
    """The reference's per-trace misfit (misfit/waveform.h, misfit/envelope.h)
    with its kernels, cuFFT and cuBLAS: syn/obs [ntr, nt] -> (values [ntr],
    adstf [ntr, nt])."""
    syn = _cast(syn, np.float32)
    obs = _cast(obs, np.float32)
    ntr, nt = syn.shape
    ad = np.zeros((ntr, nt), np.float32)
    val = np.zeros(ntr, np.float32)
    _ref_check(ref_lib().ref_misfit(int(kind), int(ntr), int(nt), ctypes.c_double(dt), _p(syn), _p(obs), _p(ad),
                                    _p(val)), "ref_misfit")
    return val, ad


def ref_calc(c, ka, a, kb=None, b=None, nx=None, nz=None):
    """device::calc (lib/device.h:157-176) with the reference's kernel, in
    place into c (a float32 grid of nx*nz cells): c = ka*a + kb*b, or ka*a."""
    ca = _cast(a, np.float32)
    cb = None if b is None else _cast(b, np.float32)
    out = np.empty(ca.size, np.float32)
    _ref_check(ref_lib().ref_calc(_p(out), ctypes.c_float(ka), _p(ca), ctypes.c_float(0 if kb is None else kb),
                                  _p(cb), int(nx), int(nz)), "ref_calc")
    c[...] = out.reshape(c.shape)


def ref_dot(a, b) -> np.float32:
    """device::dot (lib/device.h:188-192): cublasSdot."""
    a = _cast(a, np.float32)
    b = _cast(b, np.float32)
    out = ctypes.c_float()
    _ref_check(ref_lib().ref_dot(_p(a), _p(b), int(a.size), ctypes.byref(out)), "ref_dot")
    return np.float32(out.value)


def ref_amax(a) -> np.float32:
    """device::amax (lib/device.h:178-182): cublasIsamax, then |a[i]|."""
    a = _cast(a, np.float32)
    out = ctypes.c_float()
    _ref_check(ref_lib().ref_amax(_p(a), int(a.size), ctypes.byref(out)), "ref_amax")
    return np.float32(out.value)


def ref_polyfit(x, y):
    """Optimizer::polyfit + solveQR (optimizer/optimizer.h:108-172) with
    cuSOLVER, the reference's reduceSystem kernel and cuBLAS: the least-squares
    quadratic through (x, y) as float64 (p0, p1, p2), and the status of the
    reference's cusolverDnDormqr call (0: success)."""
    x = _cast(x, np.float64)
    y = _cast(y, np.float64)
    p = np.zeros(3, np.float64)
    st = ctypes.c_int(-1)
    _ref_check(ref_lib().ref_polyfit(_p(x), _p(y), int(x.size), _p(p), ctypes.byref(st)), "ref_polyfit")
    return p, st.value
