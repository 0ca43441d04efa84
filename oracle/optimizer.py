"""Optimizer oracle — TEST INFRASTRUCTURE ONLY (only tests/ import it).

Restates the reference's inversion loop in float32 scalars, as it computes
them:
  Optimizer::run ............... optimizer/optimizer.h:428-467
  Optimizer::lineSearch ........ optimizer/optimizer.h:360-419
  bracket / backtrack .......... optimizer/optimizer.h:257-357
  getHistory, argmin,
  checkBracket, goodEnough ..... optimizer/optimizer.h:184-256
  polyfit / solveQR ............ optimizer/optimizer.h:109-182
  p_amax/p_dot/p_calc/p_angle .. optimizer/optimizer.h:49-107
  NLCGOptimizer ................ optimizer/nlcg.h:8-52
  LBFGSOptimizer ............... optimizer/lbfgs.h:18-91, including its
      history rotation: `float** &s0 = lbfgs_S[lbfgs_mem - 1]` binds a
      reference to the last slot, which the shift loop then overwrites, so
      after the rotation slot 0 and slot lbfgs_mem-1 share one buffer (the
      newest pair) and the oldest pair's buffer drops out.

The vector primitives are pluggable: ``NumpyOps`` (CPU, float32) or
``RefOps`` (the reference's device::calc kernels, cublasSdot/Isamax and its
cuSOLVER polyfit, through ref_harness.cu on a GPU). The model and kernel
arrays are the caller's, updated in place, as the reference aliases m_new
and g_new to the solver's lambda/mu/rho and k_* (optimizer.h:498-503).

Where the reference is undefined the oracle does what the GB300 optimizer
does and counts the event in ``undefined_steps``. goodEnough leaves
bracket's alpha uninitialised when the fit, converted to float
(optimizer.h:174-177), has no positive curvature: where only the conversion
lost it (p[0] underflows once steps reach ~1e20) the double fit's minimum is
taken, otherwise the search ends at the best point evaluated. A search that
has used the reference's inv_iteration * ls_step entries (optimizer.h:485-487,
written past after that) fails as one past ls_step does.
"""
from __future__ import annotations

import numpy as np

F = np.float32
PI = F(3.1415927)  # host::pi (lib/device.h:68)


class NumpyOps:
    """float32 primitives on the CPU."""

    def calc(self, c, ka, a, kb=None, b=None):
        if b is None:
            c[...] = F(ka) * a
        else:
            c[...] = F(ka) * a + F(kb) * b

    def dot(self, a, b):
        return F(np.dot(a.astype(np.float64), b.astype(np.float64)))

    def amax(self, a):
        return F(np.abs(a).max())

    def polyfit(self, x, y):
        """Householder QR and a triangular solve, as solveQR (no rank cut-off:
        the columns x^2, x, 1 span many decades when steps are ~1e20)."""
        x = np.asarray(x, np.float64)
        y = np.asarray(y, np.float64)
        A = np.stack([x * x, x, np.ones_like(x)], 1)
        q, r = np.linalg.qr(A)
        return np.linalg.solve(r, q.T @ y)


class RefOps:
    """The reference's own device primitives (needs the harness and a GPU)."""

    def __init__(self, orc, nx, nz):
        self.orc, self.nx, self.nz = orc, nx, nz
        self.ormqr_failures = 0

    def calc(self, c, ka, a, kb=None, b=None):
        self.orc.ref_calc(c, ka, a, kb, b, nx=self.nx, nz=self.nz)

    def dot(self, a, b):
        return self.orc.ref_dot(a, b)

    def amax(self, a):
        return self.orc.ref_amax(a)

    def polyfit(self, x, y):
        p, st = self.orc.ref_polyfit(x, y)
        self.ormqr_failures += st != 0
        return p


class Optimizer:
    """NLCG (values["optimizer"] = 0) or L-BFGS (1) over the parameters
    flagged in inv (lambda, mu, rho). m, g: three float32 arrays each (the
    model and the kernels), updated in place. misfit_run(kernel) returns the
    misfit (float32) and, with kernel, writes the new kernels into g."""

    def __init__(self, values, inv, m, g, misfit_run, ops):
        self.type = int(values["optimizer"])
        self.inv = [bool(v) for v in inv]
        self.inv_iteration = int(values["inv_iteration"])
        self.inv_cycle = int(values["inv_cycle"])
        self.ls_step = int(values["ls_step"])
        self.ls_step_max = F(values["ls_step_max"])
        self.ls_step_init = F(values["ls_step_init"])
        self.ls_thresh = F(values["ls_thresh"])
        self.nlcg_type = int(values.get("nlcg_type", 1))
        self.nlcg_thresh = F(values.get("nlcg_thresh", 0))
        self.lbfgs_mem = int(values.get("lbfgs_mem", 5))
        self.lbfgs_thresh = F(values.get("lbfgs_thresh", 0))
        self.lbfgs_used = 0
        self.m_new, self.g_new = m, g
        n = next(m[ip].size for ip in range(3) if self.inv[ip])
        z = lambda: [np.zeros(n, F) for _ in range(3)]
        self.m_old, self.g_old, self.p_new, self.p_old = z(), z(), z(), z()
        self.lbfgs_S = [z() for _ in range(self.lbfgs_mem)]
        self.lbfgs_Y = [z() for _ in range(self.lbfgs_mem)]
        self.misfit_run = misfit_run
        self.ops = ops
        self.ls_lens, self.ls_vals, self.ls_gtg, self.ls_gtp = {}, {}, {}, {}
        self.eval_count = self.inv_count = self.ls_count = 0
        self.ref = F(1)
        self.log = []  # (kind, alpha, value): 1 gradient, 0 line-search step, 2 final
        self.events = []  # restarts and line-search outcomes, as printed
        self.undefined_steps = 0

    # ---- primitives over the inverted parameters (optimizer.h:49-107)
    def p_amax(self, a):
        r = F(0)
        for ip in range(3):
            if self.inv[ip]:
                r = max(r, self.ops.amax(a[ip]))
        return r

    def p_dot(self, a, b):
        r = F(0)
        for ip in range(3):
            if self.inv[ip]:
                r = F(r + self.ops.dot(a[ip], b[ip]))
        return r

    def p_calc(self, c, ka, a, kb=None, b=None):
        for ip in range(3):
            if self.inv[ip]:
                self.ops.calc(c[ip], F(ka), a[ip], None if b is None else F(kb), None if b is None else b[ip])

    def p_copy(self, d, s):
        for ip in range(3):
            if self.inv[ip]:
                d[ip][...] = s[ip]

    def p_angle(self, p, g, k=1):
        xx = self.p_dot(p, p)
        yy = self.p_dot(g, g)
        xy = F(F(k) * self.p_dot(p, g))
        return F(np.arccos(F(xy / F(np.sqrt(F(xx * yy))))))

    # ---- line search (optimizer.h:184-357)
    def history(self, step_count):
        x = [self.ls_lens[self.ls_count - 1 - step_count + i] for i in range(step_count + 1)]
        f = [self.ls_vals[self.ls_count - 1 - step_count + i] for i in range(step_count + 1)]
        for i in range(step_count + 1):
            for j in range(i + 1, step_count + 1):
                if x[j] < x[i]:
                    x[i], x[j] = x[j], x[i]
                    f[i], f[j] = f[j], f[i]
        update_count = sum(1 for i in range(self.ls_count) if abs(float(self.ls_lens[i])) < 1e-6)
        if update_count > 0:
            update_count -= 1
        return x, f, update_count

    @staticmethod
    def argmin(f, n):
        m, idx = f[0], 0
        for i in range(1, n):
            if f[i] < m:
                m, idx = f[i], i
        return idx

    def check_bracket(self, f, n):
        imin = self.argmin(f, n)
        fmin = f[imin]
        if fmin < f[0]:
            for i in range(imin, n):
                if f[i] > fmin:
                    return True
        return False

    def good_enough(self, x, f, n):
        """(bool, x0); x0 is None where the reference leaves it unset."""
        thresh = F(np.log10(self.ls_thresh))
        if not self.check_bracket(f, n):
            return False, None
        idx = self.argmin(f, n) - 1
        fitlen = min(4, n - idx)
        pd = self.ops.polyfit(np.array(x[idx:idx + fitlen], np.float64), np.array(f[idx:idx + fitlen], np.float64))
        p = [F(v) for v in pd]
        if p[0] > 0:
            x0 = F(-p[1] / F(F(2) * p[0]))
        elif pd[0] > 0:  # the float coefficient underflowed: the double fit's minimum
            self.undefined_steps += 1
            x0 = F(-pd[1] / (2 * pd[0]))
        else:
            self.events.append("line search error")
            self.undefined_steps += 1
            return True, None
        for i in range(1, n):
            if abs(F(np.log10(F(x[i] / x0)))) < thresh:
                return True, x0
        return False, x0

    @staticmethod
    def backtrack2(f0, g0, x1, f1, b1, b2):
        b1, b2 = F(b1), F(b2)
        # the slope is gtp/gtg, not gtp: with steps of ~1e20 the float
        # numerator overflows to inf as the reference's does, and the clamp
        # below then takes b2 * x1
        with np.errstate(over="ignore", invalid="ignore"):
            x2 = F(F(F(-g0 * x1) * x1) / F(F(2) * F(F(f1 - f0) - F(g0 * x1))))
        if x2 > F(b2 * x1):
            x2 = F(b2 * x1)
        elif x2 < F(b1 * x1):
            x2 = F(b1 * x1)
        return x2

    def bracket(self, step_count, step_max):
        x, f, update_count = self.history(step_count)
        alpha, status = None, 0
        if step_count == 0:
            if update_count == 0:
                alpha = F(F(1) / self.ls_gtg[self.inv_count - 1])
            else:
                vals = [self.ls_vals[i] for i in range(self.ls_count - 1)]
                idx = self.argmin(vals, self.ls_count - 1)
                alpha = F(F(self.ls_lens[idx] * self.ls_gtp[self.inv_count - 2]) / self.ls_gtp[self.inv_count - 1])
        elif self.check_bracket(f, step_count + 1):
            ok, x0 = self.good_enough(x, f, step_count + 1)
            if ok:
                alpha = x[self.argmin(f, step_count + 1)]
                status = 1
            else:
                alpha = x0
        elif step_count <= self.ls_step:
            i = 1
            while i < step_count + 1 and not f[i] > f[0]:
                i += 1
            if i == step_count + 1:
                alpha = F(1.618034 * float(x[step_count]))
            else:
                slope = F(self.ls_gtp[self.inv_count - 1] / self.ls_gtg[self.inv_count - 1])
                alpha = self.backtrack2(f[0], slope, x[1], f[1], 0.1, 0.5)
        else:
            alpha, status = F(0), -1
        if alpha > step_max:
            if step_count == 0:
                alpha, status = F(0.618034 * float(step_max)), 0
            else:
                alpha, status = step_max, 1
        return alpha, status

    def backtrack(self, step_count, step_max):
        x, f, update_count = self.history(step_count)
        idx = self.argmin(f, step_count + 1)
        if update_count == 0:
            return self.bracket(step_count, step_max)
        if step_count == 0:
            return min(F(1), step_max), 0
        if f[idx] < f[0]:
            return x[idx], 1
        if step_count <= self.ls_step:
            slope = F(self.ls_gtp[self.inv_count - 1] / self.ls_gtg[self.inv_count - 1])
            return self.backtrack2(f[0], slope, x[1], f[1], 0.1, 0.5), 0
        return F(0), -1

    def calc_step(self, step_count, step_max):
        if self.type == 0:
            return self.bracket(step_count, step_max)
        return self.backtrack(step_count, step_max)

    def evaluate(self, kernel, kind, alpha):
        v = F(self.misfit_run(kernel))
        self.log.append((kind, float(alpha), float(v)))
        return v

    def line_search(self, f):
        status, alpha = 0, F(0)
        norm_m = self.p_amax(self.m_new)
        norm_p = self.p_amax(self.p_new)
        gtg = self.p_dot(self.g_new, self.g_new)
        gtp = self.p_dot(self.g_new, self.p_new)
        step_max = F(F(self.ls_step_max * norm_m) / norm_p)
        step_count = 0
        self.ls_lens[self.ls_count] = F(0)
        self.ls_vals[self.ls_count] = f
        self.ls_gtg[self.inv_count - 1] = gtg
        self.ls_gtp[self.inv_count - 1] = gtp
        self.ls_count += 1
        alpha_current = F(0)
        if self.ls_step_init and self.ls_count <= 1:
            alpha = F(F(self.ls_step_init * norm_m) / norm_p)
        else:
            alpha, status = self.calc_step(step_count, step_max)
        while True:
            if self.ls_count >= max(1, self.inv_iteration * self.ls_step):
                self.undefined_steps += 1
                status = -1
            if status >= 0:
                self.p_calc(self.m_new, 1, self.m_new, F(alpha - alpha_current), self.p_new)
                alpha_current = alpha
                self.ls_lens[self.ls_count] = alpha
                self.ls_vals[self.ls_count] = self.evaluate(False, 0, alpha)
                self.ls_count += 1
                self.eval_count += 1
                step_count += 1
                alpha, status = self.calc_step(step_count, step_max)
            if status > 0:
                self.events.append("alpha")
                self.p_calc(self.m_new, 1, self.m_new, F(alpha - alpha_current), self.p_new)
                return status
            if status < 0:
                self.p_calc(self.m_new, 1, self.m_new, F(-alpha_current), self.p_new)
                if self.p_angle(self.p_new, self.g_new, -1) < 1e-3:
                    self.events.append("line search failed")
                    return status
                self.events.append("restarting line search")
                self.restart_search()
                return self.line_search(f)

    def restart_search(self):
        self.p_calc(self.p_new, -1, self.g_new)
        self.ls_count = 0
        self.inv_count = 1
        if self.type == 1:
            self.lbfgs_used = 0

    # ---- search directions
    def direction_nlcg(self):
        self.inv_count += 1
        if self.inv_count == 1:
            self.p_calc(self.p_new, -1, self.g_new)
            return 0
        if self.inv_cycle and self.inv_cycle < self.inv_count:
            self.events.append("restart: periodic")
            return -1
        if self.nlcg_type == 0:
            beta = F(self.p_dot(self.g_new, self.g_new) / self.p_dot(self.g_old, self.g_old))
        elif self.nlcg_type == 1:
            self.p_calc(self.p_new, 1, self.g_new, -1, self.g_old)
            beta = F(self.p_dot(self.g_new, self.p_new) / self.p_dot(self.g_old, self.g_old))
        else:
            beta = F(0)
        self.p_calc(self.p_new, -1, self.g_new, beta, self.p_old)
        if self.p_angle(self.g_new, self.g_old) < self.nlcg_thresh:
            self.events.append("restart: loss of conjugacy")
            return -1
        if self.p_dot(self.p_new, self.g_new) > 0:
            self.events.append("restart: not a descent direction")
            return -1
        return 1

    def direction_lbfgs(self):
        self.inv_count += 1
        if self.inv_count == 1:
            self.p_calc(self.p_new, -1, self.g_new)
            return 0
        if self.inv_cycle and self.inv_cycle < self.inv_count:
            self.events.append("restart: periodic")
            return -1
        S, Y, mem = self.lbfgs_S, self.lbfgs_Y, self.lbfgs_mem
        for i in range(mem - 1, 0, -1):
            S[i] = S[i - 1]
            Y[i] = Y[i - 1]
        S[0] = S[mem - 1]  # s0 is a reference to the last slot, read after the shift
        Y[0] = Y[mem - 1]
        s, y = self.m_old, self.p_old
        self.p_calc(s, 1, self.m_new, -1, self.m_old)
        self.p_copy(S[0], s)
        self.p_calc(y, 1, self.g_new, -1, self.g_old)
        self.p_copy(Y[0], y)
        if self.lbfgs_used < mem:
            self.lbfgs_used += 1
        rh, al = [F(0)] * self.lbfgs_used, [F(0)] * self.lbfgs_used
        self.p_copy(self.p_new, self.g_new)
        sty = yty = F(0)
        for i in range(self.lbfgs_used):
            self.p_copy(s, S[i])
            self.p_copy(y, Y[i])
            rh[i] = F(F(1) / self.p_dot(y, s))
            al[i] = F(rh[i] * self.p_dot(s, self.p_new))
            self.p_calc(self.p_new, 1, self.p_new, F(-al[i]), y)
            if i == 0:
                sty = F(F(1) / rh[i])
                yty = self.p_dot(y, y)
        self.p_calc(self.p_new, F(sty / yty), self.p_new)
        for i in range(self.lbfgs_used - 1, -1, -1):
            self.p_copy(s, S[i])
            self.p_copy(y, Y[i])
            be = F(rh[i] * self.p_dot(y, self.p_new))
            self.p_calc(self.p_new, 1, self.p_new, F(al[i] - be), s)
        angle = self.p_angle(self.g_new, self.p_new)
        if angle >= F(PI / F(2)):
            self.events.append("restart: not a descent direction")
            return -1
        if angle > F(F(PI / F(2)) - self.lbfgs_thresh):
            self.events.append("restart: practical safeguard")
            return -1
        self.p_calc(self.p_new, -1, self.p_new)
        return 1

    def run(self):
        for it in range(self.inv_iteration):
            f = self.evaluate(True, 1, 0.0)
            if it == 0:
                self.ref = f
            self.eval_count += 2
            d = self.direction_nlcg() if self.type == 0 else self.direction_lbfgs()
            if d < 0:
                self.restart_search()
            self.p_copy(self.m_old, self.m_new)
            self.p_copy(self.p_old, self.p_new)
            self.p_copy(self.g_old, self.g_new)
            if self.line_search(f) < 0:
                break
        return self.evaluate(False, 2, 0.0)
