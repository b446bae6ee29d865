"""The benchmark configurations at their full sizes, through the C ABI.

* 200 000 spheres, 500 FP32F steps through the neighbour-list path
  (k_list_step): at every step the list step's force is compared with the
  FP64 step's from the same positions (the FP64 GPU step is bit-exact to the
  oracle; that is checked at sampled steps of the trajectory here too).
* 50 000 rod segments in 500 branching trees, 200 steps: the first FP64 step
  against the oracle, and FP64 and FP32F trajectories side by side, with the
  FP32F force error measured on the FP32F trajectory's own states every 20
  steps.
* The differentiation form on 20 000 spheres over 200 steps with a
  checkpoint every 20: central differences (h = 1e-6) for the positions, the
  stiffness, the damping, the drag and the per-particle adhesion.

Bars: FP32F force error <= 1e-5 norm-wise relative against FP64; FP64 rod step
within 1e-10 plus 8x the reference's own sensitivity to a last-bit change of
the segment angles; FP64 sphere steps bit-exact; gradients within 1e-4 of the
central differences."""
import numpy as np
import pytest

from boltzmannmfx_gb300 import Context, configs
from boltzmannmfx_gb300.abi import BMXG_FP32F, BMXG_FP64, Particles
from common import relerr, trig_floor, within

pytestmark = pytest.mark.gpu

TOL32 = 1e-5
TOL64 = 1e-10

VEL = ("velx", "vely", "velz")
ROT = ("wx", "wy", "wz")


def fields(Q, names):
    return np.stack([Q[k] for k in names])


def test_sphere_fp32_200k_500_list_steps(gpu_lib, oracle_lib):
    w = configs.sphere_fp32()
    assert w.n == 200_000 and w.steps == 500
    g = w.geoms[0]
    A = Context(w.params, w.geoms)     # the FP32F trajectory (list steps)
    B = Context(w.params, w.geoms)     # FP64 steps from A's positions
    A.set_state(w.particles)
    P = w.particles.copy()
    errs = []
    checked = 0
    # (a one-step call right after a load takes the per-step path; every later
    # call steps over the list)
    for s in range(w.steps):
        B.set_state(P)
        B.step(w.dt, 1, BMXG_FP64)
        V64 = P.copy()
        B.get_state(V64, VEL + ("x", "y", "z"))
        if s in (0, 1, 250, w.steps - 1):  # the FP64 reference along the trajectory, against the oracle
            Pr = P.copy()
            oracle_lib.step(w.params, g, Pr, w.dt, nthreads=8)
            for k in VEL + ("x", "y", "z"):
                assert np.array_equal(V64[k], Pr[k]), (s, k)
            checked += 1
        A.step(w.dt, 1, BMXG_FP32F)
        Q = P.copy()
        A.get_state(Q, VEL + ("x", "y", "z"))
        errs.append(relerr(fields(Q, VEL), fields(V64, VEL)))
        P = Q
    st = A.stats()
    assert st["n_rebins"] < w.steps // 4, "the list path ran"
    errs = np.array(errs)
    print(f"FP32F list step force error vs FP64 over {w.steps} steps: max {errs.max():.3e}, "
          f"median {np.median(errs):.3e}, builds {st['n_rebins']}")
    assert checked == 4
    assert errs.max() <= TOL32, (int(errs.argmax()), float(errs.max()))


def test_rod_trees_50k_200_steps(gpu_lib, oracle_lib):
    w = configs.rod_trees()
    assert w.n == 50_000
    g = w.geoms[0]
    P0 = w.particles
    # first FP64 step against the oracle
    Pr = P0.copy()
    pl = oracle_lib.pairs(w.params, g, Pr)
    fc = oracle_lib.forces(w.params, g, Pr, pl, nthreads=8)
    fv, fw = trig_floor(oracle_lib, w.params, g, P0)
    A = Context(w.params, w.geoms)
    A.set_state(P0)
    A.step(w.dt, 1, BMXG_FP64)
    Q = P0.copy()
    A.get_state(Q)
    assert within(fields(Q, VEL), fc[:3], TOL64, 8 * fv)
    assert within(fields(Q, ROT), fc[3:], TOL64, 8 * fw)
    # FP64 and FP32F trajectories; the FP32F force error on its own states
    A.set_state(P0)
    B = Context(w.params, w.geoms)
    B.set_state(P0)
    C = Context(w.params, w.geoms)
    errs = []
    for s in range(0, 200, 20):
        SB = P0.copy()
        B.get_state(SB)
        C.set_state(SB)
        C.step(w.dt, 1, BMXG_FP64)
        R64 = P0.copy()
        C.get_state(R64)
        C.set_state(SB)
        C.step(w.dt, 1, BMXG_FP32F)
        R32 = P0.copy()
        C.get_state(R32)
        errs.append((relerr(fields(R32, VEL), fields(R64, VEL)), relerr(fields(R32, ROT), fields(R64, ROT))))
        A.step(w.dt, 20, BMXG_FP64)
        B.step(w.dt, 20, BMXG_FP32F)
    QA, QB = P0.copy(), P0.copy()
    A.get_state(QA)
    B.get_state(QB)
    # how far FP64 itself moves after 200 steps from starting positions moved by
    # the size of FP32 rounding (2^-24 of a segment length): contact and bond
    # forces of the tree networks amplify any perturbation, so the FP32F
    # trajectory is held to that spread, not to a fixed bar
    rng = np.random.default_rng(17)
    Pp = P0.copy()
    for k in ("x", "y", "z"):
        Pp[k] = P0[k] + rng.uniform(-1.0, 1.0, w.n) * 2.0 ** -24 * 3.0e-3
    A.set_state(Pp)
    A.step(w.dt, 200, BMXG_FP64)
    QP = P0.copy()
    A.get_state(QP)
    errs = np.array(errs)
    disp = max(relerr(QB[k] - P0[k], QA[k] - P0[k]) for k in ("x", "y", "z"))
    spread = max(relerr(QP[k] - P0[k], QA[k] - P0[k]) for k in ("x", "y", "z"))
    print(f"rods: FP32F force error on its trajectory, max vel {errs[:, 0].max():.3e} rot "
          f"{errs[:, 1].max():.3e}; 200-step displacement FP32F vs FP64 {disp:.3e}, FP64 from positions "
          f"moved by FP32 rounding vs FP64 {spread:.3e}")
    assert errs.max() <= TOL32, errs
    assert disp <= max(10.0 * spread, 1e-6)


@pytest.mark.parametrize("band", ["config", "above"])
def test_adjoint_20k_200_steps_central_differences(gpu_lib, band):
    """Loss: mean over particles of |x_T - target|^2 with the minimum-image
    displacement in the periodic x and y (a particle that wraps stays
    continuous).  The central difference is summed particle by particle from
    the two trajectories, (d+ - d-) . (d+ + d-) / (2 h n): the loss's own
    magnitude would swamp gradients of 1e-13 (adhesion) in the difference of
    two totals.

    The reference's wall law has a kink at dz = 0 (constant below the growth
    surface, cubic above it: bmx_cell_interaction_K.H:1019-1030).  In the
    configuration's band z in [0.040, 0.052] two thirds of the spheres start
    below the surface at 0.048 and rise at about 7e-6 cm a step; those that
    cross it within the 200 steps meet the kink, and a position perturbation
    of h = 1e-6 cm moves roughly a quarter of the crossings to the other side
    of a step boundary -- no derivative exists there for a central difference
    to approach.  So the configuration's own band checks the stiffness and the
    damping (perturbations of 1e-6 of a parameter move a crossing by ~1e-12
    cm); the same size with the band lifted above the surface
    (z in [0.0485, 0.0605], the same width) checks all five."""
    w = configs.adjoint_spheres()
    assert w.n == 20_000
    prm, g = w.params, w.geoms[0]
    P = w.particles.copy()
    if band == "above":
        P["z"] = P["z"] + (0.0485 - 0.040)
    rng = np.random.default_rng(configs.SEED + 1)
    adh0 = rng.uniform(0.0, 1.0e-3, w.n)
    target = np.stack([P["x"], P["y"], P["z"]]) + rng.normal(0.0, 1.0e-4, (3, w.n))
    box = np.array([g.prob_hi[d] - g.prob_lo[d] for d in range(3)])[:, None]
    per = np.array([g.is_periodic[d] for d in range(3)], bool)[:, None]
    k0, gamma0, mu0 = prm.stiffness, 0.05, 1.0e-2
    T, ck, h = 200, 20, 1e-6
    ctx = Context(prm, [g])

    def disp(xT):
        d = xT - target
        return np.where(per, d - box * np.round(d / box), d)

    def run(k=k0, gamma=gamma0, mu=mu0, adh=adh0, x0=None):
        p = Particles.copy(P)
        if x0 is not None:
            p["x"], p["y"], p["z"] = x0
        prm.stiffness = k
        ctx.set_params(prm)
        ctx.set_state(p)
        ctx.set_ext(gamma, mu, adh)
        ctx.forward(w.dt, T, ck)
        q = p.copy()
        ctx.get_state(q, ("x", "y", "z"))
        return disp(np.stack([q["x"], q["y"], q["z"]]))

    def fd(plus, minus, step):
        dp, dm = run(**plus), run(**minus)
        return float(np.sum((dp - dm) * (dp + dm))) / (w.n * 2.0 * step)

    d0 = run()
    gx0, gp, ga = ctx.backward(2.0 * d0 / w.n)
    x0 = np.stack([P["x"], P["y"], P["z"]])
    checks = {}
    d = rng.normal(size=x0.shape)
    checks["positions"] = (fd({"x0": x0 + h * d}, {"x0": x0 - h * d}, h), float(np.sum(gx0 * d)))
    checks["stiffness"] = (fd({"k": k0 * (1 + h)}, {"k": k0 * (1 - h)}, h * k0), gp[0])
    checks["damping"] = (fd({"gamma": gamma0 * (1 + h)}, {"gamma": gamma0 * (1 - h)}, h * gamma0), gp[1])
    checks["drag"] = (fd({"mu": mu0 * (1 + h)}, {"mu": mu0 * (1 - h)}, h * mu0), gp[2])
    da = rng.uniform(0.0, 1.0e-3, w.n)
    checks["adhesion"] = (fd({"adh": adh0 + h * da}, {"adh": adh0 - h * da}, h), float(np.dot(ga, da)))
    prm.stiffness = k0
    for name, (f, an) in checks.items():
        print(f"{band} {name}: central difference {f:.9e}, adjoint {an:.9e}, rel {abs(f - an) / abs(f):.2e}")
    for name, (f, an) in checks.items():
        if band == "above" or name in ("stiffness", "damping"):
            assert abs(f - an) <= 1e-4 * abs(f), (name, f, an)
