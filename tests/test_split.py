"""Cell division (split_particles) -- the oracle restatement against the
reference's own split loop bodies and against the committed golden vectors,
branch coverage of the FUNGI cases, and the call's error contract.  CPU only."""
import ctypes as C

import numpy as np
import pytest

from boltzmannmfx_gb300.abi import (BMXG_ERR_ARG, BMXG_ERR_CAPACITY, FUNGI, YEAST, INT_IDX as I,
                                    REAL_IDX as R, aos_dtype)
from common import load, split_expected_count, split_fungi_records, split_params, split_records


def test_aos_dtype_is_amrex_layout():
    dt = aos_dtype()
    assert dt.itemsize == 448
    assert dt.fields["rdata"][1] == 24 and dt.fields["id"][1] == 24 + 34 * 8
    assert dt.fields["idata"][1] == 24 + 34 * 8 + 8


def test_oracle_matches_golden(oracle_lib):
    d = load("split_cells")
    a = d["in_rec"].copy()
    rc, k = oracle_lib.split_cells(a, int(d["n"]), split_params(), draws=d["draws"])
    assert rc == 0 and k == int(d["num_split"])
    assert a.tobytes() == d["out_rec"].tobytes()


@pytest.mark.parametrize("n,seed,frac", [(1, 3, 1.0), (257, 5, 0.3), (4000, 7, 0.05), (999, 8, 0.0),
                                         (700, 9, 1.0)])
def test_oracle_matches_reference(oracle_lib, n, seed, frac):
    oracle_lib.build(ref=None)
    if not oracle_lib.have_ref():
        pytest.skip("reference tree not present")
    a = split_records(n, 2 * n + 4, seed, frac_divide=frac)
    b = a.copy()
    k = split_expected_count(a, n)
    draws = np.random.default_rng(seed).random(2 * k)
    rc1, k1 = oracle_lib.split_cells(a, n, split_params(), draws=draws)
    rc2, k2 = oracle_lib.split_cells(b, n, split_params(), draws=draws, use_ref=True)
    assert (rc1, k1) == (rc2, k2) == (0, k)
    assert a.tobytes() == b.tobytes()


def test_division_properties(oracle_lib):
    n = 3000
    a = split_records(n, 2 * n, 11)
    before = a.copy()
    k = split_expected_count(a, n)
    draws = np.random.default_rng(12).random(2 * k)
    rc, ns = oracle_lib.split_cells(a, n, split_params(), draws=draws, next_id=10_000, my_proc=3)
    assert rc == 0 and ns == k > 0
    div = np.flatnonzero((before["idata"][:n, I["cell_type"]] == 0) & (before["rdata"][:n, R["vol"]] > 5.0e-10))
    kids = np.arange(n, n + k)
    # untouched: every record that does not divide, every daughter slot past n + k
    keep = np.setdiff1d(np.arange(n), div)
    assert a[keep].tobytes() == before[keep].tobytes()
    assert a[n + k:].tobytes() == before[n + k:].tobytes()
    # volume halves exactly; the pair straddles the mother's centre 0.8 r apart
    assert np.array_equal(a["rdata"][div, R["vol"]], before["rdata"][div, R["vol"]] / 2.0)
    assert np.array_equal(a["rdata"][kids, R["vol"]], a["rdata"][div, R["vol"]])
    mid = 0.5 * (a["pos"][div] + a["pos"][kids])
    assert np.abs(mid - before["pos"][div]).max() < 1e-18
    sep = np.linalg.norm(a["pos"][kids] - a["pos"][div], axis=1)
    assert np.allclose(sep, 0.8 * before["rdata"][div, R["radius"]], rtol=1e-12)
    assert np.array_equal(a["id"][kids], 10_000 + np.arange(k))
    assert np.array_equal(a["idata"][kids, I["id"]], a["id"][kids])
    assert np.all(a["cpu"][kids] == 3) and np.all(a["idata"][kids, I["cpu"]] == 3)
    assert np.all(a["idata"][kids, I["fuse_tip"]] == 0) and np.all(a["rdata"][kids, R["bond_scale"]] == 1.0)
    f = R["first_data"]
    assert np.array_equal(a["rdata"][div, f + 6:f + 9], 0.5 * before["rdata"][div, f + 6:f + 9])
    assert np.array_equal(a["rdata"][kids, f + 6:f + 9], a["rdata"][div, f + 6:f + 9])
    # the rest of the copied block comes from the mother as she was
    same = [j for j in range(34) if j not in (R["radius"], R["area"], R["vol"], R["dadt"], R["bond_scale"])
            and not f + 6 <= j < f + 9]
    assert np.array_equal(a["rdata"][kids][:, same], before["rdata"][div][:, same])


def seeded_sequence(O, a, n, sp, seed):
    """The draw sequence that equals the seeded mode: each cell's checkSplit
    draw is draw 0 of its (id, cpu) counter, its division's draws 1, 2, ..."""
    checks = []
    for i in range(n):
        q, r = a["idata"][i], a["rdata"][i]
        if q[I["cell_type"]] == FUNGI and ((q[I["position"]] == 0 and r[R["radius"]] >= sp.max_rad)
                                           or q[I["position"]] in (1, 2)):
            checks.append(O.split_uniform(seed, a["id"][i], a["cpu"][i], 0))
    kinds, _ = decisions(a, n, sp, checks)
    need = {"cell": 2, "tip": 2, "two": 4, "branch": 3, "halve": 0}
    div = [O.split_uniform(seed, a["id"][i], a["cpu"][i], 1 + j) for i, k in kinds for j in range(need[k])]
    return np.array(checks + div)


@pytest.mark.parametrize("fungi", [False, True])
def test_seeded_draws(oracle_lib, fungi):
    n = 500
    a = split_fungi_records(n, 3 * n, 21) if fungi else split_records(n, 2 * n, 21)
    b = a.copy()
    seed = 0xB0A7_5EED_1234_5678
    sp = split_params(brnch_prob=0.3, split_prob=0.5)
    draws = seeded_sequence(oracle_lib, a, n, sp, seed)
    assert np.all((draws >= 0.0) & (draws < 1.0))
    rc1, k1 = oracle_lib.split_cells(a, n, sp, seed=seed)
    rc2, k2 = oracle_lib.split_cells(b, n, sp, draws=draws)
    assert rc1 == rc2 == 0 and k1 == k2 > 0
    assert a.tobytes() == b.tobytes()


def decisions(a, n, sp, draws):
    """checkSplit over the records with a draw sequence (bmx_chem_K.H:23-69),
    restated here: the kind of each division and the draws the call takes."""
    kinds, t = [], 0
    for i in range(n):
        q, r = a["idata"][i], a["rdata"][i]
        if q[I["cell_type"]] == YEAST:
            if r[R["vol"]] > sp.max_vol:
                kinds.append((i, "cell"))
            continue
        pos, nb = q[I["position"]], q[I["n_bnds"]]
        if pos == 0 and r[R["radius"]] >= sp.max_rad:
            x = draws[t]
            t += 1
            if r[R["c_length"]] >= sp.max_len:
                kinds.append((i, "halve" if nb == 0 else ("tip" if x > sp.split_prob else "two")))
        elif pos in (1, 2):
            x = draws[t]
            t += 1
            if x < sp.brnch_prob:
                kinds.append((i, "halve" if nb == 0 else "branch"))
    need = {"cell": 2, "tip": 2, "two": 4, "branch": 3, "halve": 0}
    return kinds, t + sum(need[k] for _, k in kinds)


def test_oracle_matches_golden_fungi(oracle_lib):
    d = load("split_fungi")
    a = d["in_rec"].copy()
    sp = split_params(brnch_prob=float(d["params"][0]), split_prob=float(d["params"][1]))
    rc, k = oracle_lib.split_cells(a, int(d["n"]), sp, draws=d["draws"])
    assert rc == 0 and k == int(d["num_split"])
    assert a.tobytes() == d["out_rec"].tobytes()
    kinds, used = decisions(d["in_rec"], int(d["n"]), sp, d["draws"])
    assert used == len(d["draws"])
    assert {k for _, k in kinds} == {"cell", "tip", "two", "branch", "halve"}


@pytest.mark.parametrize("n,seed,bp,sprob", [(400, 1, 0.3, 0.5), (3000, 2, 0.05, 0.1), (50, 3, 1.0, 0.0),
                                             (1000, 4, 0.0, 1.0)])
def test_oracle_matches_reference_fungi(oracle_lib, n, seed, bp, sprob):
    oracle_lib.build(ref=None)
    if not oracle_lib.have_ref():
        pytest.skip("reference tree not present")
    a = split_fungi_records(n, 4 * n, seed)
    b = a.copy()
    sp = split_params(brnch_prob=bp, split_prob=sprob)
    kinds, need = decisions(a, n, sp, np.random.default_rng(seed + 10).random(8 * n))
    draws = np.random.default_rng(seed + 10).random(8 * n)[:need]
    rc2, k2, used = oracle_lib.split_cells(b, n, sp, draws=draws, use_ref=True, return_used=True)
    rc1, k1 = oracle_lib.split_cells(a, n, sp, draws=draws)
    assert rc1 == rc2 == 0 and k1 == k2 == sum(2 if k == "two" else 1 for _, k in kinds)
    assert used == need
    assert a.tobytes() == b.tobytes()


def test_error_contract(oracle_lib):
    n = 400
    a = split_records(n, 2 * n, 31)
    k = split_expected_count(a, n)
    draws = np.random.default_rng(32).random(2 * k)
    before = a.tobytes()
    # too little room: the count comes back, nothing is written
    rc, ns = oracle_lib.split_cells(a[:n + k - 1], n, split_params(), draws=draws)
    assert (rc, ns) == (BMXG_ERR_CAPACITY, k) and a.tobytes() == before
    # too few draws
    rc, ns = oracle_lib.split_cells(a, n, split_params(), draws=draws[:-1])
    assert rc == BMXG_ERR_ARG and a.tobytes() == before
    f = split_fungi_records(300, 1200, 33)
    fb = f.tobytes()
    sp = split_params(brnch_prob=0.5, split_prob=0.5)
    kinds, need = decisions(f, 300, sp, np.full(2400, 0.25))
    rc, _ = oracle_lib.split_cells(f, 300, sp, draws=np.full(need - 1, 0.25))
    assert rc == BMXG_ERR_ARG and f.tobytes() == fb
    rc, ns = oracle_lib.split_cells(f, 300, sp, draws=np.full(need, 0.25))
    assert rc == 0 and ns == sum(2 if k == "two" else 1 for _, k in kinds)
    # layout limits
    L = oracle_lib.lib()
    out = C.c_int64(0)
    p = a.ctypes.data_as(C.c_void_p)
    assert L.orc_split_cells_aos(C.byref(split_params()), p, n, 2 * n, 33, 35, None, 0, 0, 1, 0,
                                 C.byref(out)) == BMXG_ERR_ARG
    assert L.orc_split_cells_aos(C.byref(split_params(num_reals=10)), p, n, 2 * n, 34, 35, None, 0, 0, 1, 0,
                                 C.byref(out)) == BMXG_ERR_ARG
    assert L.orc_split_cells_aos(C.byref(split_params()), p, 0, 0, 34, 35, None, 0, 0, 1, 0,
                                 C.byref(out)) == 0 and out.value == 0
