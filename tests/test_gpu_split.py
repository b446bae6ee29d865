"""YEAST division through bmxg_split_cells_aos (host and device records)
against the oracle and the golden vectors of the reference's split loop.

Tolerance: every copied, halved or assigned field is bit-exact.  The fields
that go through acos, sin, cos and pow (positions, radius, area, dadt) take
CUDA's double-precision functions on the device and the C library's on the
host; both are within 2 ulp of the true value, so they agree within
8 x 2^-52 relative (positions: relative to |x| + r)."""
import ctypes as C

import numpy as np
import pytest

from boltzmannmfx_gb300 import runtime
from boltzmannmfx_gb300.abi import (BMXG_DEVICE, BMXG_ERR_ARG, BMXG_ERR_CAPACITY, BMXG_ERR_UNSUPPORTED,
                                    BMXG_HOST, FUNGI, INT_IDX as I, REAL_IDX as R)
from boltzmannmfx_gb300.runtime import BmxgError
from common import load, split_expected_count, split_params, split_records

pytestmark = pytest.mark.gpu

EPS = 2.0 ** -52
TRIG_REALS = (R["radius"], R["area"], R["dadt"])


def assert_same_division(got, ref, n_used):
    """bit-exact outside the transcendental fields, 8 ulp inside them"""
    g, r = got[:n_used], ref[:n_used]
    for f in ("id", "cpu", "idata"):
        assert np.array_equal(g[f], r[f]), f
    exact = [j for j in range(g["rdata"].shape[1]) if j not in TRIG_REALS]
    assert np.array_equal(g["rdata"][:, exact], r["rdata"][:, exact])
    for j in TRIG_REALS:
        a, b = g["rdata"][:, j], r["rdata"][:, j]
        assert np.all(np.abs(a - b) <= 8 * EPS * np.abs(b)), j
    scale = np.abs(r["pos"]) + np.abs(r["rdata"][:, R["radius"]])[:, None]
    assert np.all(np.abs(g["pos"] - r["pos"]) <= 8 * EPS * scale)
    assert got[n_used:].tobytes() == ref[n_used:].tobytes()


def test_golden_host_records(gpu_lib):
    d = load("split_cells")
    a = d["in_rec"].copy()
    k = runtime.split_cells_aos(a, int(d["n"]), split_params(), draws=d["draws"])
    assert k == int(d["num_split"])
    assert_same_division(a, d["out_rec"], int(d["n"]) + k)


@pytest.mark.parametrize("n,seed,frac", [(1, 3, 1.0), (255, 4, 0.3), (257, 5, 0.3), (70_000, 6, 0.1),
                                         (999, 8, 0.0), (700, 9, 1.0)])
def test_host_records_match_oracle(gpu_lib, oracle_lib, n, seed, frac):
    a = split_records(n, 2 * n + 3, seed, frac_divide=frac)
    b = a.copy()
    k = split_expected_count(a, n)
    draws = np.random.default_rng(seed).random(2 * k)
    got = runtime.split_cells_aos(a, n, split_params(), draws=draws, next_id=77, my_proc=2)
    rc, want = oracle_lib.split_cells(b, n, split_params(), draws=draws, next_id=77, my_proc=2)
    assert rc == 0 and got == want == k
    assert_same_division(a, b, n + k)


def test_device_records_and_seeded_draws(gpu_lib, oracle_lib):
    import torch
    n = 50_000
    a = split_records(n, n + n // 2, 13)
    b = a.copy()
    seed = 0x5EED_0000_0000_0042
    dev = torch.from_numpy(a.view(np.uint8)).cuda()
    k = runtime.split_cells_aos(dev.data_ptr(), n, split_params(), seed=seed, next_id=1 << 20, my_proc=1,
                                where=BMXG_DEVICE, cap=len(a))
    torch.cuda.synchronize()
    got = dev.cpu().numpy().view(a.dtype)
    rc, want = oracle_lib.split_cells(b, n, split_params(), seed=seed, next_id=1 << 20, my_proc=1)
    assert rc == 0 and k == want == split_expected_count(a, n)
    assert_same_division(got, b, n + k)


def test_device_draws(gpu_lib, oracle_lib):
    import torch
    n = 20_000
    a = split_records(n, 2 * n, 17)
    b = a.copy()
    k = split_expected_count(a, n)
    draws = np.random.default_rng(18).random(2 * k)
    dev = torch.from_numpy(a.view(np.uint8)).cuda()
    ddr = torch.from_numpy(draws).cuda()
    got_k = runtime.split_cells_aos(dev.data_ptr(), n, split_params(), draws=(ddr.data_ptr(), ddr.numel()),
                                    where=BMXG_DEVICE, cap=len(a))
    torch.cuda.synchronize()
    rc, want = oracle_lib.split_cells(b, n, split_params(), draws=draws)
    assert rc == 0 and got_k == want == k
    assert_same_division(dev.cpu().numpy().view(a.dtype), b, n + k)


def test_full_size_division(gpu_lib, oracle_lib):
    """2.73 M records (the size of the 256-colony workload), device-resident:
    the count, every non-dividing record byte for byte, and the oracle's
    result on every record."""
    import torch
    n = 2_731_333
    a = split_records(n, n + n // 8, 23, frac_divide=0.05)
    b = a.copy()
    dev = torch.from_numpy(a.view(np.uint8)).cuda()
    k = runtime.split_cells_aos(dev.data_ptr(), n, split_params(), seed=99, next_id=n + 1,
                                where=BMXG_DEVICE, cap=len(a))
    got = dev.cpu().numpy().view(a.dtype)
    rc, want = oracle_lib.split_cells(b, n, split_params(), seed=99, next_id=n + 1)
    assert rc == 0 and k == want == split_expected_count(a, n)
    assert_same_division(got, b, n + k)


@pytest.mark.parametrize("where", [BMXG_HOST, BMXG_DEVICE])
def test_errors_write_nothing(gpu_lib, where):
    import torch
    n = 3000
    a = split_records(n, 2 * n, 41)
    k = split_expected_count(a, n)
    draws = np.random.default_rng(42).random(2 * k)

    def call(rec, sp=None, dr=draws, cap=None):
        if where == BMXG_HOST:
            return runtime.split_cells_aos(rec, n, sp or split_params(), draws=dr, cap=cap)
        dev = torch.from_numpy(rec.view(np.uint8)).cuda()
        ddr = torch.from_numpy(np.ascontiguousarray(dr)).cuda()
        try:
            return runtime.split_cells_aos(dev.data_ptr(), n, sp or split_params(), draws=(ddr.data_ptr(), len(dr)),
                                           where=BMXG_DEVICE, cap=len(rec) if cap is None else cap)
        finally:
            torch.cuda.synchronize()
            rec[...] = dev.cpu().numpy().view(rec.dtype)

    before = a.tobytes()
    with pytest.raises(BmxgError) as e:
        call(a, cap=n + k - 1)
    assert e.value.code == BMXG_ERR_CAPACITY and a.tobytes() == before
    with pytest.raises(BmxgError) as e:
        call(a, dr=draws[:-1])
    assert e.value.code == BMXG_ERR_ARG and a.tobytes() == before
    t = a.copy()
    t["idata"][5, I["cell_type"]] = FUNGI
    t["idata"][5, I["position"]] = 1
    tb = t.tobytes()
    with pytest.raises(BmxgError) as e:
        call(t, sp=split_params(brnch_prob=1e-4))
    assert e.value.code == BMXG_ERR_UNSUPPORTED and t.tobytes() == tb
    assert call(t, sp=split_params(brnch_prob=0.0)) == k - int(a["rdata"][5, R["vol"]] > 5.0e-10
                                                                 and a["idata"][5, I["cell_type"]] == 0)


def test_empty_and_bad_layout(gpu_lib):
    L = gpu_lib
    out = C.c_int64(-1)
    sp = split_params()
    assert L.bmxg_split_cells_aos(C.byref(sp), None, 0, 0, 34, 35, None, 0, 0, 1, 0, BMXG_HOST, C.byref(out),
                                  None) == 0 and out.value == 0
    a = split_records(4, 8, 1)
    p = a.ctypes.data_as(C.c_void_p)
    assert L.bmxg_split_cells_aos(C.byref(sp), p, 4, 8, 33, 35, None, 0, 0, 1, 0, BMXG_HOST, C.byref(out),
                                  None) == BMXG_ERR_ARG
    assert L.bmxg_split_cells_aos(C.byref(sp), p, 4, 8, 34, 34, None, 0, 0, 1, 0, BMXG_HOST, C.byref(out),
                                  None) == BMXG_ERR_ARG
    assert L.bmxg_split_cells_aos(C.byref(sp), p, 4, 3, 34, 35, None, 0, 0, 1, 0, BMXG_HOST, C.byref(out),
                                  None) == BMXG_ERR_ARG
