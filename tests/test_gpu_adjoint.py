"""The differentiation form: bmxg_forward / bmxg_backward (hand-written adjoint
with checkpointed recomputation) against central finite differences on the
FP64 path, against a forward difference of the oracle's reference-law
trajectory, and through a torch.autograd.Function wrapper.

Spheres start above the growth surface (dz > 0), where the wall law is
continuously differentiable, so finite differences see a smooth trajectory."""
import math

import numpy as np
import pytest

from boltzmannmfx_gb300 import Context, configs
from boltzmannmfx_gb300.abi import BMXG_FP64, Particles

pytestmark = pytest.mark.gpu

DT, T, H = 0.25, 20, 1e-6


def setup(n=600, seed=11):
    rng = np.random.default_rng(seed)
    P = configs.sphere_colony(n, 0.064, 0.064, rng, z_band=(0.0485, 0.0530))
    P["x"] = rng.uniform(0.004, 0.060, n)   # away from the periodic faces: the loss needs no image
    P["y"] = rng.uniform(0.004, 0.060, n)
    prm = configs.deck_params()
    g = configs.box_geometry(0.064, 0.064)
    target = np.stack([P["x"], P["y"], P["z"]]) + rng.normal(0.0, 1e-4, (3, n))
    adh = rng.uniform(0.0, 1e-3, n)
    return prm, g, P, target, adh


def run(ctx, prm, P, k, gamma, mu, adh, x0=None, ckpt=5):
    p = Particles.copy(P)
    if x0 is not None:
        p["x"], p["y"], p["z"] = x0
    prm.stiffness = k
    ctx.set_params(prm)
    ctx.set_state(p)
    ctx.set_ext(gamma, mu, adh)
    ctx.forward(DT, T, ckpt)
    q = p.copy()
    ctx.get_state(q, ("x", "y", "z"))
    return np.stack([q["x"], q["y"], q["z"]])


def loss(xT, target):
    return float(np.mean(np.sum((xT - target) ** 2, axis=0)))


def test_forward_equals_plain_step_at_zero_extensions(gpu_lib):
    prm, g, P, _, _ = setup()
    a = Context(prm, g)
    xa = run(a, prm, P, prm.stiffness, 0.0, 0.0, None)
    b = Context(prm, g)
    b.set_state(P)
    b.step(DT, T, BMXG_FP64)
    q = P.copy()
    b.get_state(q, ("x", "y", "z"))
    assert np.array_equal(xa, np.stack([q["x"], q["y"], q["z"]]))


@pytest.mark.parametrize("ext", [(0.0, 0.0, False), (5e-5, 1e-2, True)])
def test_gradients_match_central_differences(gpu_lib, ext):
    gamma, mu, use_adh = ext
    prm, g, P, target, adh0 = setup()
    adh = adh0 if use_adh else None
    k0 = prm.stiffness
    ctx = Context(prm, g)
    xT = run(ctx, prm, P, k0, gamma, mu, adh)
    gx0, gp, ga = ctx.backward(2.0 * (xT - target) / P.n)
    x0 = np.stack([P["x"], P["y"], P["z"]])
    rng = np.random.default_rng(5)

    def L(**kw):
        return loss(run(ctx, prm, P, kw.get("k", k0), kw.get("gamma", gamma), kw.get("mu", mu),
                        kw.get("adh", adh), x0=kw.get("x0")), target)

    # positions, along a random direction
    d = rng.normal(size=x0.shape)
    fd = (L(x0=x0 + H * d) - L(x0=x0 - H * d)) / (2 * H)
    assert abs(fd - np.sum(gx0 * d)) <= 1e-4 * abs(fd)
    # stiffness
    hk = H * k0
    fd = (L(k=k0 + hk) - L(k=k0 - hk)) / (2 * hk)
    assert abs(fd - gp[0]) <= 1e-4 * abs(fd)
    if gamma > 0.0:
        hg = H * gamma
        fd = (L(gamma=gamma + hg) - L(gamma=gamma - hg)) / (2 * hg)
        assert abs(fd - gp[1]) <= 1e-4 * abs(fd)
    if mu > 0.0:
        hm = H * mu
        fd = (L(mu=mu + hm) - L(mu=mu - hm)) / (2 * hm)
        assert abs(fd - gp[2]) <= 1e-4 * abs(fd)
    if use_adh:
        da = rng.uniform(0.0, 1e-3, P.n)
        fd = (L(adh=adh + H * da) - L(adh=adh - H * da)) / (2 * H)
        assert abs(fd - np.dot(ga, da)) <= 1e-4 * abs(fd)


def test_checkpoint_interval_does_not_change_gradients(gpu_lib):
    prm, g, P, target, adh = setup(n=300)
    out = []
    for ck in (1, 3, 20):
        ctx = Context(prm, g)
        xT = run(ctx, prm, P, prm.stiffness, 5e-5, 1e-2, adh, ckpt=ck)
        out.append(ctx.backward(2.0 * (xT - target) / P.n))
    for o in out[1:]:
        for a, b in zip(o, out[0]):
            assert np.array_equal(a, b)


def test_stiffness_gradient_vs_reference_forward_difference(gpu_lib, oracle_lib):
    """dL/dk of the adjoint at zero extensions against an FP64 forward
    difference of the oracle's trajectory (the reference law)."""
    prm, g, P, target, _ = setup(n=400)
    k0 = prm.stiffness
    ctx = Context(prm, g)
    xT = run(ctx, prm, P, k0, 0.0, 0.0, None)
    _, gp, _ = ctx.backward(2.0 * (xT - target) / P.n)

    def oracle_L(k):
        q = P.copy()
        prm.stiffness = k
        oracle_lib.evolve(prm, [g], [0, P.n], q, DT, T)
        return loss(np.stack([q["x"], q["y"], q["z"]]), target)

    hk = 1e-6 * k0
    fd = (oracle_L(k0 + hk) - oracle_L(k0)) / hk
    prm.stiffness = k0
    assert abs(fd - gp[0]) <= 1e-4 * abs(fd)


def test_torch_autograd_wrapper(gpu_lib):
    torch = pytest.importorskip("torch")
    prm, g, P, target, adh0 = setup(n=300)
    ctx = Context(prm, g)

    class Trajectory(torch.autograd.Function):
        @staticmethod
        def forward(fctx, x0, k, gamma, mu, adh):
            xT = run(ctx, prm, P, float(k), float(gamma), float(mu), adh.detach().numpy(),
                     x0=x0.detach().numpy())
            return torch.from_numpy(xT)

        @staticmethod
        def backward(fctx, gout):
            gx0, gp, ga = ctx.backward(gout.detach().numpy())
            return (torch.from_numpy(gx0), torch.tensor(gp[0], dtype=torch.float64),
                    torch.tensor(gp[1], dtype=torch.float64), torch.tensor(gp[2], dtype=torch.float64),
                    torch.from_numpy(ga))

    x0 = torch.tensor(np.stack([P["x"], P["y"], P["z"]]), requires_grad=True)
    k = torch.tensor(prm.stiffness, dtype=torch.float64, requires_grad=True)
    gamma = torch.tensor(5e-5, dtype=torch.float64, requires_grad=True)
    mu = torch.tensor(1e-2, dtype=torch.float64, requires_grad=True)
    adh = torch.tensor(adh0, requires_grad=True)
    tgt = torch.from_numpy(target)
    L = ((Trajectory.apply(x0, k, gamma, mu, adh) - tgt) ** 2).sum(0).mean()
    L.backward()
    hk = 1e-6 * float(k)
    with torch.no_grad():
        Lp = ((Trajectory.apply(x0, k + hk, gamma, mu, adh) - tgt) ** 2).sum(0).mean()
        Lm = ((Trajectory.apply(x0, k - hk, gamma, mu, adh) - tgt) ** 2).sum(0).mean()
    fd = float(Lp - Lm) / (2 * hk)
    assert abs(fd - float(k.grad)) <= 1e-4 * abs(fd)
    assert x0.grad.shape == x0.shape and torch.isfinite(x0.grad).all()
    assert adh.grad is not None and math.isfinite(float(adh.grad.abs().sum()))
