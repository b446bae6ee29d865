"""bmxg_sphere_step_noalloc: the sphere step for callers that may not allocate
device memory (an application that hands out all device memory through its
own arenas, sized up front, where an allocation behind the arena's back can
make the arena's next one fail).  It must give
the same result as the regular entry points -- bit for bit, the bar of every
FP64 sphere test here -- on two calls in a row (the second call reuses the
scratch the first one left behind), and reject sizes beyond its limits.

This file is collected last on purpose, and passes alone in a fresh process
as well as after the other tests."""
import ctypes as C

import numpy as np
import pytest

from boltzmannmfx_gb300 import Context, configs
from boltzmannmfx_gb300.abi import BMXG_ERR_CAPACITY, BMXG_FP64, BMXG_OK, Geometry

pytestmark = pytest.mark.gpu


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def test_noalloc_step_matches_regular_entry_points_twice(gpu_lib):
    torch = pytest.importorskip("torch")
    w = configs.spheres("noalloc", 3000, 0.128, 0.128, 2)
    P, g, prm = w.particles, w.geoms[0], w.params
    # regular path: two FP64 steps through set_state / step / get_state
    ctx = Context(prm, [g])
    ctx.set_state(P)
    ref, ref_ood = [], []
    for _ in range(2):
        ctx.step(w.dt, 1, BMXG_FP64)
        Q = P.copy()
        ctx.get_state(Q)
        ref.append(Q)
        ref_ood.append(ctx.stats()["n_out_of_domain"])
    ctx.close()
    # no-alloc path on device arrays the caller owns
    dev = torch.device("cuda", 0)
    pos = [torch.tensor(P[k], device=dev) for k in ("x", "y", "z")]
    rad = torch.tensor(P["radius"], device=dev)
    stream = torch.cuda.current_stream(dev)
    for call in range(2):
        out = [torch.empty_like(pos[0]) for _ in range(3)]
        vel = [torch.empty_like(pos[0]) for _ in range(3)]
        ood = C.c_int64(-1)
        rc = gpu_lib.bmxg_sphere_step_noalloc(C.byref(prm), C.byref(g), P.n, *map(_ptr, pos), _ptr(rad),
                                              *map(_ptr, out), *map(_ptr, vel), w.dt,
                                              C.c_void_p(stream.cuda_stream), C.byref(ood))
        assert rc == BMXG_OK
        assert ood.value == ref_ood[call], (call, ood.value)
        torch.cuda.synchronize()
        for k, t in zip(("x", "y", "z"), out):
            assert np.array_equal(t.cpu().numpy(), ref[call][k]), (call, k)
        for k, t in zip(("velx", "vely", "velz"), vel):
            assert np.array_equal(t.cpu().numpy(), ref[call][k]), (call, k)
        pos = out


def test_noalloc_rejects_sizes_beyond_its_limits(gpu_lib):
    prm = configs.deck_params()
    g = configs.box_geometry(0.128, 0.128)
    null = C.c_void_p(0)
    args = [null] * 10
    assert gpu_lib.bmxg_sphere_step_noalloc(C.byref(prm), C.byref(g), 32769, *args, 0.25,
                                            null, None) == BMXG_ERR_CAPACITY
    big = Geometry.make((0, 0, 0), (1.0, 1.0, 0.064), (257, 256, 32), (1, 1, 0))
    assert gpu_lib.bmxg_sphere_step_noalloc(C.byref(prm), C.byref(big), 10, *args, 0.25,
                                            null, None) == BMXG_ERR_CAPACITY
