"""The optimizer's line-search step rule (gb_linesearch_step: the host code
of gb_optimizer_run, no device work) against the optimizer oracle's float
restatement of bracket and backtrack (optimizer/optimizer.h:184-357).

Seeded searches over quadratic misfit profiles with noise, three iterations
sharing one history (so that the rules that scale the previous iteration's
step run too), driven by the oracle: at every step both rules see the same
history and must return the same status and the same step."""
import numpy as np
import pytest

from oracle import optimizer as ropt

F = np.float32


def oracle_rule(opt, lens, vals, gtg, gtp, step_count, ls_step, ls_thresh, step_max):
    z = [np.zeros(1, F)] * 3
    values = {"optimizer": opt, "inv_iteration": 1, "inv_cycle": 0, "ls_step": ls_step, "ls_step_max": 0.5,
              "ls_step_init": 0, "ls_thresh": ls_thresh}
    o = ropt.Optimizer(values, (0, 1, 0), z, z, None, ropt.NumpyOps())
    o.ls_lens = {i: F(v) for i, v in enumerate(lens)}
    o.ls_vals = {i: F(v) for i, v in enumerate(vals)}
    o.ls_count = len(lens)
    o.ls_gtg = {i: F(v) for i, v in enumerate(gtg)}
    o.ls_gtp = {i: F(v) for i, v in enumerate(gtp)}
    o.inv_count = len(gtg)
    a, s = o.calc_step(step_count, F(step_max))
    return float(a), s, o.undefined_steps


def simulate(pkg, seed, scale, noise, ls_step):
    """One seeded run; returns (steps compared, statuses seen, undefined)."""
    rng = np.random.default_rng(seed)
    opt = seed % 2
    ls_thresh = float(F(rng.uniform(1.1, 2.0)))
    lens, vals, gtg, gtp = [], [], [], []
    fcur = float(F(rng.uniform(0.5, 2.0)))
    n, seen, undefined = 0, set(), 0
    for it in range(3):
        g2 = float(F(10 ** rng.uniform(-1, 1) / scale))
        gp = float(F(-g2 * rng.uniform(0.2, 1.0)))
        gtg.append(g2)
        gtp.append(gp)
        astar = 10 ** rng.uniform(-1.5, 1.5) / g2
        curv = -gp / astar
        f0 = fcur

        def f(a):
            return float(F(f0 + gp * a + 0.5 * curv * a * a + noise * abs(f0) * rng.standard_normal()))

        step_max = float(F(astar * 10 ** rng.uniform(-0.5, 2)))
        lens.append(0.0)
        vals.append(f0)
        step_count = 0
        while True:
            ap, sp = pkg.linesearch_step(opt, lens, vals, gtg, gtp, step_count, ls_step, ls_thresh, step_max)
            ao, so, un = oracle_rule(opt, lens, vals, gtg, gtp, step_count, ls_step, ls_thresh, step_max)
            undefined += un
            assert sp == so, (seed, it, step_count, ap, ao)
            assert ap == ao or abs(ap - ao) <= 1e-6 * abs(ao), (seed, it, step_count, ap, ao)
            n += 1
            seen.add(so)
            if so != 0:
                break
            lens.append(float(F(ao)))
            vals.append(f(ao))
            step_count += 1
        if so < 0:
            break
        fcur = f(ao)
    return n, seen, undefined


@pytest.mark.parametrize("scale,noise,ls_step", [(1.0, 1e-7, 10), (1.0, 1e-3, 3), (1e23, 1e-7, 10)])
def test_step_rule_matches_oracle(pkg, scale, noise, ls_step):
    """scale 1e23: steps near 1e23, where the float fit's leading coefficient
    underflows and both take the double fit's minimum; noise 1e-3 with
    ls_step 3: fits without curvature and searches that fail."""
    total, statuses, undefined = 0, set(), 0
    for seed in range(150):
        n, seen, un = simulate(pkg, seed, scale, noise, ls_step)
        total += n
        statuses |= seen
        undefined += un
    assert total > 1000
    assert statuses >= {0, 1}
    if noise > 1e-6:
        assert -1 in statuses
    if scale > 1:
        assert undefined > 0  # the underflowed fits were reached


def test_step_rule_rejects_bad_history(pkg):
    with pytest.raises(pkg.GbError):
        pkg.linesearch_step(0, [0.0], [1.0], [1.0], [-1.0], 1, 10, 1.2, 1.0)  # step_count past the history
    with pytest.raises(pkg.GbError):
        # two iterations in the history need two slopes
        pkg.linesearch_step(0, [0.0, 0.5, 0.0], [1.0, 0.5, 0.5], [1.0], [-1.0], 0, 10, 1.2, 1.0)
