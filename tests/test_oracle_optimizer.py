"""The optimizer oracle (oracle/optimizer.py) on the CPU: NLCG and L-BFGS on
a separable quadratic misfit, the line search's decisions, and the
reference's L-BFGS history rotation (optimizer/lbfgs.h:29-36)."""
import numpy as np
import pytest

from oracle import optimizer as ropt

F = np.float32


def quadratic(n=64, seed=0):
    rng = np.random.default_rng(seed)
    w = (0.5 + rng.random(n)).astype(F)
    target = rng.standard_normal(n).astype(F)
    m = [np.zeros(n, F), (target + rng.standard_normal(n).astype(F)).astype(F), np.zeros(n, F)]
    g = [np.zeros(n, F) for _ in range(3)]

    def run(kernel):
        r = (m[1] - target).astype(F)
        if kernel:
            g[1][...] = w * r
        return F(0.5 * np.sum(w.astype(np.float64) * r.astype(np.float64) ** 2))

    return m, g, run


VALUES = {"inv_iteration": 6, "inv_cycle": 0, "ls_step": 10, "ls_step_max": 0.5, "ls_step_init": 0.05,
          "ls_thresh": 1.2, "nlcg_type": 1, "nlcg_thresh": 0.0, "lbfgs_mem": 5, "lbfgs_thresh": 0.0}


@pytest.mark.parametrize("opt,extra", [(0, {}), (0, {"nlcg_type": 0}), (1, {}), (1, {"lbfgs_mem": 2})])
def test_quadratic_misfit_decreases(opt, extra):
    m, g, run = quadratic()
    v = dict(VALUES, optimizer=opt, **extra)
    o = ropt.Optimizer(v, (False, True, False), m, g, run, ropt.NumpyOps())
    final = o.run()
    grads = [e[2] for e in o.log if e[0] == 1]
    assert len(grads) == v["inv_iteration"]
    # not monotone: bracket accepts step_max unevaluated once its
    # extrapolation passes it (optimizer.h:311-319)
    assert final < 0.05 * grads[0], grads
    assert o.undefined_steps == 0
    # the first line search starts at ls_step_init * max|m| / max|p| (optimizer.h:379-381)
    first_step = [e for e in o.log if e[0] == 0][0]
    assert first_step[1] > 0


def test_lbfgs_rotation_aliases_the_last_slot():
    """Three iterations rotate the history twice (A0..A3 the initial slot
    buffers): [A2, A0, A1, A2], then [A1, A2, A0, A1] — slot 0 and slot
    mem-1 always share the newest pair's buffer."""
    m, g, run = quadratic()
    v = dict(VALUES, optimizer=1, lbfgs_mem=4, inv_iteration=3)
    o = ropt.Optimizer(v, (False, True, False), m, g, run, ropt.NumpyOps())
    a = list(o.lbfgs_S)
    o.run()
    assert [s is t for s, t in zip(o.lbfgs_S, (a[1], a[2], a[0], a[1]))] == [True] * 4
    # slot 0 holds the newest pair: the model step of the second line search
    assert np.abs(o.lbfgs_S[0][1]).max() > 0


def test_backtrack2_and_polyfit():
    # the safeguarded quadratic step (optimizer.h:257-266)
    # x2 = -g0 x1^2 / (2 (f1 - f0 - g0 x1)), clamped to [0.1 x1, 0.5 x1]
    assert ropt.Optimizer.backtrack2(F(1), F(-1), F(1), F(2), 0.1, 0.5) == F(0.25)
    assert ropt.Optimizer.backtrack2(F(1), F(-1), F(1), F(10), 0.1, 0.5) == F(0.1)
    assert ropt.Optimizer.backtrack2(F(1), F(-1), F(1), F(0.5), 0.1, 0.5) == F(0.5)
    p = ropt.NumpyOps().polyfit([0.0, 1.0, 2.0, 3.0], [2.0, 1.0, 2.0, 5.0])
    np.testing.assert_allclose(p, [1.0, -2.0, 2.0], atol=1e-12)
