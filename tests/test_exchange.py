"""ParticleExchange (bmx_pc_xchng.cpp:13-257 with the exchange kernels of
bmx_chem_K.H:1949-2126) on the reference's 410-segment network: the oracle
port and the GPU kernel against the golden output of the reference's own loop
body, bit for bit, with gentle and with clamping transfer rates."""
import numpy as np
import pytest

from common import geom_of, load, params_of, particles_of

CASES = ("gentle", "clamped")


@pytest.mark.parametrize("case", CASES)
def test_port_matches_golden(oracle_lib, case):
    d, e = load("fungi_network"), load("exchange")
    P = particles_of(d)
    got = oracle_lib.particle_exchange(geom_of(d), P, e["vol"], e["conc"], float(e["dt"]), e["xpar_" + case],
                                       params=params_of(d))
    assert np.array_equal(got, e["out_" + case])
    assert not np.array_equal(got, e["conc"])


def test_port_matches_reference_harness(oracle_lib):
    if not oracle_lib.have_ref():
        pytest.skip("reference harness not built")
    d, e = load("fungi_network"), load("exchange")
    P = particles_of(d)
    rng = np.random.default_rng(4)
    conc = rng.uniform(0.0, 2.0e-3, (3, P.n))
    for xp in ([3e-3, 1e-1, 1.0], [5e3, 1e-4, 2e2]):
        a = oracle_lib.particle_exchange(geom_of(d), P, e["vol"], conc, 0.1, xp, params=params_of(d))
        b = oracle_lib.particle_exchange(geom_of(d), P, e["vol"], conc, 0.1, xp, params=params_of(d), use_ref=True)
        assert np.array_equal(a, b)


def test_spheres_do_not_exchange(oracle_lib):
    from boltzmannmfx_gb300 import configs
    w = configs.sphere_plain()
    P = w.particles
    P.rods = True
    from boltzmannmfx_gb300.abi import Particles
    Q = Particles(P.n, rods=True)
    for k in P.a:
        Q[k] = P[k]
    conc = np.random.default_rng(1).uniform(0, 1e-3, (3, Q.n))
    got = oracle_lib.particle_exchange(w.geoms[0], Q, np.ones(Q.n), conc, 0.25, [1.0, 1.0, 1.0], params=w.params)
    assert np.array_equal(got, conc)


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_gpu_matches_golden(gpu_lib, case):
    from boltzmannmfx_gb300.runtime import Context
    d, e = load("fungi_network"), load("exchange")
    P = particles_of(d)
    ctx = Context(params_of(d), [geom_of(d)])
    ctx.set_state(P)
    got = ctx.particle_exchange(e["vol"], e["conc"], float(e["dt"]), e["xpar_" + case])
    assert np.array_equal(got, e["out_" + case])
