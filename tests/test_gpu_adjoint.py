"""Adjoint kernels generated from the DSL body, behind torch.autograd with
checkpointing: gradients w.r.t. the initial field and the diffusivity field,
checked against PyTorch autograd through a plain tensor stencil (FP32) and
against central finite differences (FP64)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import xgrid
import workloads
from xgrid_gb300 import adjoint
from xgrid_gb300.operator import Operator

pytestmark = pytest.mark.gpu


def torch_step(u, k, dt):
    """The diffuse3d body on tensors: offset +1 along an axis reads index i+1."""
    acc = None
    for d in range(3):
        for s in (-1, 1):  # offset +1 -> roll by -1
            un, kn = torch.roll(u, -s, d), torch.roll(k, -s, d)
            term = (k + kn) * (un - u)
            acc = term if acc is None else acc + term
    return u + dt * acc


def _order_like_kernel(u, k, dt):
    # the kernel sums faces in the order +x0, -x0, +x1, -x1, +x2, -x2
    return torch_step(u, k, dt)


def _inputs(n, dtype, seed=4):
    u0, kap, tgt, dt = workloads.adjoint_setup(n, seed)
    to = lambda a: torch.tensor(a.astype(dtype), device="cuda")
    return to(u0), to(kap), to(tgt), dt


@pytest.mark.parametrize("steps,every", [(13, 5), (8, 20), (13, 1), (6, None)])
def test_adjoint_matches_torch_autograd(cacheroot, steps, every):
    """Checkpointed rollouts (every 5 steps, or one segment) and rollouts that keep
    every state (explicitly, or by the default budget rule at this size)."""
    xgrid.init(precision="float", cacheroot=cacheroot, opt_level=3, overstep="wrap")
    k = Operator(workloads.diffuse3d.func, "kernel", "diffuse3d")
    u0, kap, tgt, dt = _inputs(20, np.float32)
    ro = adjoint.Rollout(k, steps, every)
    a = u0.clone().requires_grad_(True)
    b = kap.clone().requires_grad_(True)
    uT = ro(a, {"k": b}, (dt,))
    loss = ((uT - tgt) ** 2).mean()
    loss.backward()
    ar = u0.clone().requires_grad_(True)
    br = kap.clone().requires_grad_(True)
    u = ar
    for _ in range(steps):
        u = torch_step(u, br, torch.tensor(dt, dtype=torch.float32, device="cuda"))
    lr = ((u - tgt) ** 2).mean()
    lr.backward()
    assert torch.allclose(uT, u, rtol=1e-5, atol=1e-6)
    for g, gr in ((a.grad, ar.grad), (b.grad, br.grad)):
        rel = (g - gr).abs().max() / gr.abs().max()
        assert rel < 1e-4, float(rel)


def test_adjoint_matches_finite_differences_fp64(cacheroot):
    xgrid.init(precision="double", cacheroot=cacheroot, opt_level=3, overstep="wrap")
    k = Operator(workloads.diffuse3d.func, "kernel", "diffuse3d")
    u0, kap, tgt, dt = _inputs(12, np.float64, seed=6)
    steps = 9
    ro = adjoint.Rollout(k, steps, 4)
    a = u0.clone().requires_grad_(True)
    b = kap.clone().requires_grad_(True)
    loss = ((ro(a, {"k": b}, (dt,)) - tgt) ** 2).mean()
    loss.backward()
    gen = torch.Generator(device="cuda").manual_seed(0)
    v = torch.randn(u0.shape, dtype=torch.float64, device="cuda", generator=gen)
    w = torch.randn(u0.shape, dtype=torch.float64, device="cuda", generator=gen) * kap * 0.1

    def L(du, dk):
        with torch.no_grad():
            return float(((ro(u0 + du, {"k": kap + dk}, (dt,)) - tgt) ** 2).mean())

    for eps in (1e-5,):
        fd_u = (L(eps * v, 0 * w) - L(-eps * v, 0 * w)) / (2 * eps)
        fd_k = (L(0 * v, eps * w) - L(0 * v, -eps * w)) / (2 * eps)
        an_u = float((a.grad * v).sum())
        an_k = float((b.grad * w).sum())
        assert abs(fd_u - an_u) <= 1e-7 * max(1.0, abs(an_u)) + 1e-9, (fd_u, an_u)
        assert abs(fd_k - an_k) <= 1e-7 * max(1.0, abs(an_k)) + 1e-9, (fd_k, an_k)


def test_rollout_waits_for_inputs_made_on_the_callers_stream(cacheroot):
    """The rollout runs on the backend's own stream; inputs still being computed
    on the caller's stream (a queue of kernels ahead of them) must be finished
    before the rollout reads them, and its result must be ready for the caller."""
    xgrid.init(precision="double", cacheroot=cacheroot, opt_level=3, overstep="wrap")
    k = Operator(workloads.diffuse3d.func, "kernel", "diffuse3d")
    n = 40
    u0, kap, tgt, dt = workloads.adjoint_setup(n, 6)
    u0, kap = u0.astype(np.float64), kap.astype(np.float64)
    ro = adjoint.Rollout(k, 9, 4)
    base = torch.tensor(u0, device="cuda")
    big = torch.ones((4096, 4096), dtype=torch.float64, device="cuda")
    outs = []
    for scale in (1.0, 1.5):
        for _ in range(3):  # keep the caller's stream busy
            big = big @ big * (1.0 / 4096)
        u_in = base * scale + big[0, 0] * 0.0
        with torch.no_grad():
            outs.append(ro(u_in, {"k": torch.tensor(kap, device="cuda")}, (dt,)).cpu().numpy())
    for scale, got in zip((1.0, 1.5), outs):
        ref = u0 * scale
        for _ in range(9):
            acc = None
            for d in range(3):
                for s in (-1, 1):
                    t = (kap + np.roll(kap, -s, d)) * (np.roll(ref, -s, d) - ref)
                    acc = t if acc is None else acc + t
            ref = ref + dt * acc
        assert np.abs(got - ref).max() < 1e-12


@pytest.mark.parametrize("precision,dtype,tol", [("float", np.float32, 1e-5), ("double", np.float64, 1e-13)])
@pytest.mark.parametrize("shape", [(37, 29, 70), (37, 29, 136)])
def test_staged_and_register_adjoint_agree(cacheroot, precision, dtype, tol, shape):
    """Forward and adjoint steps through the staged z-walks (planes in shared
    memory, the default) and through the register z-walks give the same
    gradients, on extents that are not multiples of the staged column block."""
    xgrid.init(precision=precision, cacheroot=cacheroot, opt_level=3, overstep="wrap")
    rng = np.random.default_rng(9)
    u0 = torch.tensor(rng.random(shape).astype(dtype), device="cuda")
    kap = torch.tensor(rng.uniform(0.01, 0.1, shape).astype(dtype), device="cuda")
    tgt = torch.tensor(rng.random(shape).astype(dtype), device="cuda")
    grads = []
    for staged in (True, False):
        k = Operator(workloads.diffuse3d.func, "kernel", "diffuse3d")
        ro = adjoint.Rollout(k, 7, 3)
        ro.set_zstage(staged)
        a = u0.clone().requires_grad_(True)
        b = kap.clone().requires_grad_(True)
        loss = ((ro(a, {"k": b}, (0.5,)) - tgt) ** 2).mean()
        loss.backward()
        grads.append((a.grad.clone(), b.grad.clone()))
    for g, r in zip(grads[0], grads[1]):
        assert float((g - r).abs().max() / r.abs().max()) < tol


def test_state_budget_chooses_the_mode(cacheroot):
    """Without an explicit interval the rollout keeps every state when the states
    fit in the budget, else checkpoints every 20 steps; both give the same
    gradients."""
    xgrid.init(precision="float", cacheroot=cacheroot, opt_level=3, overstep="wrap")
    u0, kap, tgt, dt = _inputs(16, np.float32)
    state = u0.numel() * 4
    out = []
    for budget, every in ((30 * state, 1), (29 * state, 20)):
        ro = adjoint.Rollout(Operator(workloads.diffuse3d.func, "kernel", "diffuse3d"), 30, state_budget=budget)
        assert ro.checkpoint_interval(state) == every
        a = u0.clone().requires_grad_(True)
        b = kap.clone().requires_grad_(True)
        ((ro(a, {"k": b}, (dt,)) - tgt) ** 2).mean().backward()
        out.append((a.grad, b.grad))
    for g, r in zip(out[0], out[1]):
        assert float((g - r).abs().max() / r.abs().max()) < 1e-6
