"""Cell division through bmxg_split_cells_aos (host and device records) against
the oracle and the golden vectors of the reference's split loop.

Tolerance: every integer field and every real that the division copies,
halves, adds or takes a square root of is bit-exact.  Reals that go through
acos, sin, cos or pow (positions, the new segments' theta and phi, a YEAST
cell's radius, area and dadt) take CUDA's double-precision functions on the
device and the C library's on the host, each within 2 ulp of the true value;
they agree within 64 x 2^-52 of the field's scale (positions: |x| plus the
largest segment length or radius).  A new segment's angles are the
reference's acos(z) and acos(x / sin theta), whose condition number is
1 / |sin| of the result: a last-bit difference of the argument moves an angle
near 0 or pi by that factor, so angles agree within
128 x 2^-52 x (1 + 1 / |sin angle|)."""
import ctypes as C

import numpy as np
import pytest

from boltzmannmfx_gb300 import runtime
from boltzmannmfx_gb300.abi import BMXG_DEVICE, BMXG_ERR_ARG, BMXG_ERR_CAPACITY, BMXG_HOST, REAL_IDX as R
from boltzmannmfx_gb300.runtime import BmxgError
from common import load, split_expected_count, split_fungi_records, split_params, split_records

pytestmark = pytest.mark.gpu

EPS = 2.0 ** -52
TRIG_REALS = (R["radius"], R["theta"], R["phi"], R["area"], R["vol"], R["dadt"])


def assert_same_division(got, ref, n_used):
    """ints bit-exact; reals bit-exact outside the transcendental fields,
    64 ulp of the field's scale inside them; most of those bit-exact too"""
    g, r = got[:n_used], ref[:n_used]
    for f in ("id", "cpu", "idata"):
        assert np.array_equal(g[f], r[f]), f
    exact = [j for j in range(g["rdata"].shape[1]) if j not in TRIG_REALS]
    assert np.array_equal(g["rdata"][:, exact], r["rdata"][:, exact])
    for j in TRIG_REALS:
        a, b = g["rdata"][:, j], r["rdata"][:, j]
        if j in (R["theta"], R["phi"]):
            tol = 128 * EPS * (1.0 + 1.0 / np.maximum(np.abs(np.sin(b)), 1e-6))
        else:
            tol = 64 * EPS * np.abs(b)
        assert np.all(np.abs(a - b) <= tol), j
    size = max(np.abs(r["rdata"][:, R["c_length"]]).max(), np.abs(r["rdata"][:, R["radius"]]).max())
    assert np.all(np.abs(g["pos"] - r["pos"]) <= 64 * EPS * (np.abs(r["pos"]) + size))
    assert got[n_used:].tobytes() == ref[n_used:].tobytes()
    same = np.mean(g["pos"] == r["pos"])
    assert same > 0.5, same  # a last-bit difference of the trig functions is the exception


@pytest.mark.parametrize("case", ["split_cells", "split_fungi"])
def test_golden_host_records(gpu_lib, case):
    d = load(case)
    a = d["in_rec"].copy()
    kw = {} if case == "split_cells" else dict(brnch_prob=float(d["params"][0]), split_prob=float(d["params"][1]))
    k = runtime.split_cells_aos(a, int(d["n"]), split_params(**kw), draws=d["draws"])
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


@pytest.mark.parametrize("n,seed,bp,sprob", [(400, 1, 0.3, 0.5), (50_000, 2, 0.05, 0.1), (257, 3, 1.0, 0.0)])
def test_fungi_records_match_oracle(gpu_lib, oracle_lib, n, seed, bp, sprob):
    a = split_fungi_records(n, 3 * n, seed)
    b = a.copy()
    sp = split_params(brnch_prob=bp, split_prob=sprob)
    draws = np.random.default_rng(seed + 10).random(8 * n)
    got = runtime.split_cells_aos(a, n, sp, draws=draws, next_id=5, my_proc=1)
    rc, want = oracle_lib.split_cells(b, n, sp, draws=draws, next_id=5, my_proc=1)
    assert rc == 0 and got == want > 0
    assert_same_division(a, b, n + got)


@pytest.mark.parametrize("fungi", [False, True])
def test_device_records_and_seeded_draws(gpu_lib, oracle_lib, fungi):
    import torch
    n = 50_000
    a = split_fungi_records(n, 3 * n, 13) if fungi else split_records(n, n + n // 2, 13)
    b = a.copy()
    seed = 0x5EED_0000_0000_0042
    sp = split_params(brnch_prob=0.2, split_prob=0.5)
    dev = torch.from_numpy(a.view(np.uint8)).cuda()
    k = runtime.split_cells_aos(dev.data_ptr(), n, sp, seed=seed, next_id=1 << 20, my_proc=1,
                                where=BMXG_DEVICE, cap=len(a))
    torch.cuda.synchronize()
    got = dev.cpu().numpy().view(a.dtype)
    rc, want = oracle_lib.split_cells(b, n, sp, seed=seed, next_id=1 << 20, my_proc=1)
    assert rc == 0 and k == want > 0
    assert_same_division(got, b, n + k)


def test_device_draws(gpu_lib, oracle_lib):
    import torch
    n = 20_000
    a = split_fungi_records(n, 3 * n, 17)
    b = a.copy()
    sp = split_params(brnch_prob=0.2, split_prob=0.5)
    draws = np.random.default_rng(18).random(8 * n)
    dev = torch.from_numpy(a.view(np.uint8)).cuda()
    ddr = torch.from_numpy(draws).cuda()
    got_k = runtime.split_cells_aos(dev.data_ptr(), n, sp, draws=(ddr.data_ptr(), ddr.numel()),
                                    where=BMXG_DEVICE, cap=len(a))
    torch.cuda.synchronize()
    rc, want = oracle_lib.split_cells(b, n, sp, draws=draws)
    assert rc == 0 and got_k == want > 0
    assert_same_division(dev.cpu().numpy().view(a.dtype), b, n + got_k)


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
def test_errors_write_nothing(gpu_lib, oracle_lib, where):
    import torch
    n = 3000
    a = split_fungi_records(n, 3 * n, 41)
    sp = split_params(brnch_prob=0.2, split_prob=0.5)
    full = np.random.default_rng(42).random(8 * n)
    rc, k = oracle_lib.split_cells(a.copy(), n, sp, draws=full)
    assert rc == 0 and k > 0

    def used_draws():
        for m in range(0, 8 * n + 1, 64):  # the shortest prefix the oracle accepts
            if oracle_lib.split_cells(a.copy(), n, sp, draws=full[:m])[0] == 0:
                return m
        return None

    m = used_draws()
    while oracle_lib.split_cells(a.copy(), n, sp, draws=full[:m - 1])[0] == 0:
        m -= 1

    def call(rec, dr, cap=None):
        if where == BMXG_HOST:
            return runtime.split_cells_aos(rec, n, sp, draws=dr, cap=cap)
        dev = torch.from_numpy(rec.view(np.uint8)).cuda()
        ddr = torch.from_numpy(np.ascontiguousarray(dr)).cuda()
        try:
            return runtime.split_cells_aos(dev.data_ptr(), n, sp, draws=(ddr.data_ptr(), len(dr)),
                                           where=BMXG_DEVICE, cap=len(rec) if cap is None else cap)
        finally:
            torch.cuda.synchronize()
            rec[...] = dev.cpu().numpy().view(rec.dtype)

    before = a.tobytes()
    with pytest.raises(BmxgError) as e:
        call(a, full, cap=n + k - 1)
    assert e.value.code == BMXG_ERR_CAPACITY and a.tobytes() == before
    with pytest.raises(BmxgError) as e:
        call(a, full[:m - 1])
    assert e.value.code == BMXG_ERR_ARG and a.tobytes() == before
    assert call(a, full[:m]) == k


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


def test_other_layouts_match_oracle(gpu_lib, oracle_lib):
    """records with more reals and ints than BMX's 34 / 35, and a species block
    shorter than the increments the division halves (num_reals 3: the
    daughter's first_data + 6..8 are not copied, and the reference halves what
    the new record held), through the raw C ABI of both"""
    from boltzmannmfx_gb300.abi import aos_dtype
    n, cap, nreal, nint = 3000, 9000, 40, 40
    src = split_fungi_records(n, cap, 61)
    a = np.zeros(cap, aos_dtype(nreal, nint))
    a["pos"] = src["pos"]
    a["rdata"][:, :34] = src["rdata"]
    a["rdata"][:, 34:] = np.random.default_rng(62).normal(size=(cap, 6))
    a["id"], a["cpu"] = src["id"], src["cpu"]
    a["idata"][:, :35] = src["idata"]
    a["idata"][:, 35:] = 11
    a0 = a
    draws = np.random.default_rng(63).random(8 * n)
    for sp in (split_params(brnch_prob=0.3, split_prob=0.5, num_reals=12, num_ints=3),
               split_params(brnch_prob=0.3, split_prob=0.5, num_reals=3)):
        a, b = a0.copy(), a0.copy()
        out_g, out_o = C.c_int64(0), C.c_int64(0)
        rc = gpu_lib.bmxg_split_cells_aos(C.byref(sp), a.ctypes.data_as(C.c_void_p), n, cap, nreal, nint,
                                          draws.ctypes.data_as(C.c_void_p), draws.size, 0, 1, 0, BMXG_HOST,
                                          C.byref(out_g), None)
        ro = oracle_lib.lib().orc_split_cells_aos(C.byref(sp), b.ctypes.data_as(C.c_void_p), n, cap, nreal,
                                                  nint, draws.ctypes.data_as(C.c_void_p), draws.size, 0, 1, 0,
                                                  C.byref(out_o))
        assert rc == ro == 0 and out_g.value == out_o.value > 0
        assert_same_division(a, b, n + out_g.value)


def test_fungi_division_repeats_byte_for_byte(gpu_lib, oracle_lib):
    """The division list is filled in atomic arrival order within each kind of
    division, so its order changes from run to run; the result must not.  Each
    division writes only its mother's and its daughters' records (a side branch
    or a two-way split edits the bond tables of those records alone), so the
    bytes are the same whatever the order.  Checked on the reference's shipped
    410-segment network (tips at the limits, bonded neighbours that several
    divisions share) and on 50 000 seeded segments, device records and draws
    from the sequence, three runs each: byte-identical, and the oracle's
    result within 1e-9 of each field's scale (the bar of the pipeline test on
    the same network)."""
    import torch
    from test_gpu_aos import NINT, NREAL, to_aos
    from boltzmannmfx_gb300.abi import aos_dtype
    from common import particles_of

    d = load("fungi_network")
    P0 = particles_of(d)
    n0 = P0.n
    net = np.zeros(6 * n0, aos_dtype(NREAL, NINT))
    b = to_aos(P0)
    for f in ("pos", "rdata", "idata"):
        net[f][:n0] = b[f]
    net["id"][:n0], net["cpu"][:n0] = P0["id"], P0["cpu"]
    net["rdata"][:n0, R["vol"]] = np.pi * P0["radius"] ** 2 * P0["c_length"]
    cases = [(net, n0, split_params(max_len=0.0030, max_rad=0.00025, brnch_prob=0.5, split_prob=0.5,
                                    split_len=0.0025), 31, True),
             (split_fungi_records(50_000, 150_000, 29), 50_000, split_params(brnch_prob=0.3, split_prob=0.5), 37,
              False)]
    for a, n, sp, seed, network in cases:
        draws = np.random.default_rng(seed).random(8 * n)
        outs = []
        for _ in range(3):
            dev = torch.from_numpy(a.copy().view(np.uint8)).cuda()
            ddr = torch.from_numpy(draws).cuda()
            k = runtime.split_cells_aos(dev.data_ptr(), n, sp, draws=(ddr.data_ptr(), ddr.numel()), next_id=10 ** 6,
                                        where=BMXG_DEVICE, cap=len(a))
            torch.cuda.synchronize()
            outs.append((k, dev.cpu().numpy().tobytes()))
        assert outs[0][0] > 0
        assert all(o == outs[0] for o in outs[1:]), "division result depends on the run"
        ref = a.copy()
        rc, want = oracle_lib.split_cells(ref, n, sp, draws=draws, next_id=10 ** 6)
        assert rc == 0 and want == outs[0][0]
        got = np.frombuffer(outs[0][1], a.dtype)
        # the oracle: within 1e-9 of each field's scale, the pipeline test's bar
        # (the strict per-value bar of this file is held by the tests above; a
        # repeat test needs the other result only as a sanity check)
        from test_gpu_pipeline import assert_close
        assert_close(got, ref, n + want, "network" if network else "seeded segments")
