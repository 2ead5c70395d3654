"""Symbolic differentiation used by the adjoint generator, checked numerically
on the CPU (no GPU): derivative expressions vs central differences."""
import random

from xgrid_gb300 import adjoint as A


def evaluate(node, env):
    k = node[0]
    if k == "c":
        return node[1]
    if k in ("p", "l"):
        return env[node[1]]
    if k == "neg":
        return -evaluate(node[1], env)
    a, b = evaluate(node[1], env), evaluate(node[2], env)
    return {"+": a + b, "-": a - b, "*": a * b, "/": a / b}[k]


def test_partials_match_central_differences():
    rng = random.Random(0)
    L = [("l", (0, 1, (0, 0, o))) for o in (-1, 0, 1)]
    K = [("l", (1, 0, (0, 0, o))) for o in (-1, 0, 1)]
    dt = ("p", "dt")
    # u' = u + dt * ((k0 + k1)(u1 - u0) + (k0 + km)(um - u0)) / (1 + k0 * k0)
    flux = A.s_add(A.s_mul(A.s_add(K[1], K[2]), A.s_sub(L[2], L[1])),
                   A.s_mul(A.s_add(K[1], K[0]), A.s_sub(L[0], L[1])))
    expr = A.s_add(L[1], A.s_div(A.s_mul(dt, flux), A.s_add(("c", 1.0), A.s_mul(K[1], K[1]))))
    env = {"dt": 0.3}
    for n in L + K:
        env[n[1]] = rng.uniform(0.1, 1.0)
    for n in L + K:
        d = A.diff(expr, n[1])
        h = 1e-6
        e1, e2 = dict(env), dict(env)
        e1[n[1]] += h
        e2[n[1]] -= h
        fd = (evaluate(expr, e1) - evaluate(expr, e2)) / (2 * h)
        assert abs(evaluate(d, env) - fd) < 1e-7


def test_shift_moves_every_load():
    node = A.s_mul(("l", (0, 1, (0, 0, 1))), ("l", (1, 0, (0, -1, 0))))
    s = A.shift(node, (0, 0, 1))
    assert A.loads_of(s) == [(0, 1, (0, 0, 0)), (1, 0, (0, -1, -1))]


def test_rollout_keeps_every_state_within_the_budget():
    """The rollout's choice between a state pool and checkpoints (host logic, no
    GPU): an explicit interval wins; otherwise every state is kept when ``steps``
    states fit in the budget, else a checkpoint every 20 steps."""
    import xgrid
    import workloads
    from xgrid_gb300.operator import Operator
    xgrid.init(precision="float", cacheroot="/tmp/xgadj", opt_level=3, overstep="wrap")
    k = Operator(workloads.diffuse3d.func, "kernel", "diffuse3d")
    state = 64 ** 3 * 4
    assert A.Rollout(k, 200, 7).checkpoint_interval(state) == 7
    assert A.Rollout(k, 200, 1).checkpoint_interval(state) == 1
    assert A.Rollout(k, 200, state_budget=200 * state).checkpoint_interval(state) == 1
    assert A.Rollout(k, 200, state_budget=200 * state - 1).checkpoint_interval(state) == 20
    import pytest
    with pytest.raises(Exception):
        A.Rollout(k, 0)
