"""Fixture I/O of libbmxg (bmxg_read_ascii / bmxg_write_ascii / bmxg_write_vtk /
bmxg_read_checkpoint; host functions, no device): against independent
restatements of the two file formats, on the reference's own fixtures where
the reference tree is present, and by round trip."""
import math
import os

import numpy as np
import pytest

from boltzmannmfx_gb300 import configs
from boltzmannmfx_gb300.abi import BMXG_ERR_ARG, BMXG_ERR_UNSUPPORTED, FUNGI, Particles
from boltzmannmfx_gb300.runtime import BmxgError, read_ascii, read_checkpoint, write_ascii, write_vtk
from common import load

from oracle.oracle import REF_TREE as REF  # noqa: E402  (BMX_REFERENCE, else the oracle recipe's default)
CHK = os.path.join(REF, "exec/fungi/chk357900/particles")
need_ref = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "exec")), reason="reference tree not present")

REAL_OUT = ("x", "y", "z", "radius", "c_length", "theta", "phi", "area", "velx", "vely", "velz", "wx", "wy", "wz")


def ascii_tokens(path):
    """The reference's stream read (bmx_pc_init.cpp:34-78): count, then 27
    values per particle; returns (count, rows of 27)."""
    tok = open(path).read().split()
    n = int(tok[0])
    vals = [float(t) for t in tok[1:1 + 27 * n]]
    return n, np.array(vals).reshape(n, 27)


@need_ref
@pytest.mark.parametrize("rel", ["exec/wall_test/fungi_init_cfg.dat", "exec/fungi/fungi_init_cfg.dat"])
def test_read_reference_ascii_fixtures(rel):
    path = os.path.join(REF, rel)
    n, rows = ascii_tokens(path)
    P = read_ascii(path)
    assert P.n == n
    cols = {"x": 0, "y": 1, "z": 2, "radius": 3, "c_length": 4, "theta": 5, "phi": 6, "area": 7,
            "velx": 9, "vely": 10, "velz": 11, "wx": 12, "wy": 13, "wz": 14}
    for k, c in cols.items():
        assert np.array_equal(P[k], rows[:, c]), k
    assert np.array_equal(P["cell_type"], rows[:, 26].astype(np.int32))
    assert np.array_equal(P["id"], np.arange(1, n + 1)) and (P["cpu"] == 0).all()
    assert (P["bond_scale"] == 1.0).all() and (P["n_bnds"] == 0).all()


def mixed_state(seed=3):
    rng = np.random.default_rng(seed)
    w = configs.rod_trees(seed=seed, ntrees=3, per_tree=20, lx=0.032, ly=0.032)
    S = configs.sphere_colony(40, 0.032, 0.032, rng)
    P = Particles.concat([w.particles, S])
    for k in ("velx", "vely", "velz", "wx", "wy", "wz"):
        P[k] = rng.normal(0.0, 1e-6, P.n)
    return P


def test_ascii_round_trip(tmp_path):
    P = mixed_state()
    path = str(tmp_path / "particles.dat")
    write_ascii(path, P)
    Q = read_ascii(path)
    assert Q.n == P.n
    for k in REAL_OUT + ("cell_type",):
        assert np.array_equal(Q[k], P[k]), k
    n, rows = ascii_tokens(path)
    # vol column: the shape's volume
    r, L = P["radius"], P["c_length"]
    vol = np.where(P["cell_type"] == FUNGI, math.pi * r * r * L, 4.0 / 3.0 * math.pi * r ** 3)
    assert np.allclose(rows[:, 8], vol, rtol=1e-15, atol=0.0)


def test_ascii_errors(tmp_path):
    with pytest.raises(BmxgError) as e:
        read_ascii(str(tmp_path / "missing.dat"))
    assert e.value.code == BMXG_ERR_ARG
    bad = tmp_path / "short.dat"
    bad.write_text("3\n1 2 3\n")
    with pytest.raises(BmxgError) as e:
        read_ascii(str(bad))
    assert e.value.code == BMXG_ERR_ARG


def test_vtk_layout(tmp_path):
    P = mixed_state(5)
    conc = np.linspace(0.0, 1.0, P.n)
    path = str(tmp_path / "p.vtk")
    write_vtk(path, P, conc)
    lines = open(path).read().split("\n")
    assert lines[0].startswith("# vtk DataFile Version 3.0")
    i = lines.index(f"POINTS {2 * P.n} float")
    pts = []
    k = i + 1
    while len(pts) < 2 * P.n:
        if lines[k].strip():
            pts.append([float(v) for v in lines[k].split()])
        k += 1
    pts = np.array(pts)
    n = np.stack([np.sin(P["theta"]) * np.cos(P["phi"]), np.sin(P["theta"]) * np.sin(P["phi"]),
                  np.cos(P["theta"])], axis=1)
    c = np.stack([P["x"], P["y"], P["z"]], axis=1)
    half = 0.5 * P["c_length"][:, None] * n
    assert np.allclose(pts[0::2], c + half, rtol=0, atol=1e-8)   # precision(8) text
    assert np.allclose(pts[1::2], c - half, rtol=0, atol=1e-8)
    assert f"POLYGONS {P.n} {3 * P.n}" in lines
    assert f"CELL_DATA {P.n}" in lines and f"POINT_DATA {2 * P.n}" in lines
    j = lines.index("SCALARS conc_B float")
    vals = np.array([float(v) for l in lines[j + 2:j + 2 + P.n] for v in l.split()])
    assert np.allclose(vals, np.repeat(conc, 2), rtol=1e-6, atol=0)


def read_chk_restated(d, level):
    """Independent restatement of the Version_Two_Dot_One_double particle
    files: Header grid table, then per grid (2 + n_int) int32 and
    (3 + n_real) float64 per particle."""
    tok = open(os.path.join(d, "Header")).read().split()
    assert tok[0] == "Version_Two_Dot_One_double"
    p = 2
    nr = int(tok[p]); p += 1 + nr
    ni = int(tok[p]); p += 1 + ni
    p += 1                      # is_checkpoint
    p += 2                      # count, next id
    finest = int(tok[p]); p += 1
    ng = [int(tok[p + k]) for k in range(finest + 1)]; p += finest + 1
    ints, reals = [], []
    for lev in range(finest + 1):
        for g in range(ng[lev]):
            which, cnt, where = (int(t) for t in tok[p:p + 3]); p += 3
            if cnt == 0 or lev != level:
                continue
            b = open(os.path.join(d, f"Level_{lev}", f"DATA_{which:05d}"), "rb").read()[where:]
            ints.append(np.frombuffer(b[:cnt * (2 + ni) * 4], "<i4").reshape(cnt, 2 + ni))
            reals.append(np.frombuffer(b[cnt * (2 + ni) * 4:cnt * ((2 + ni) * 4 + (3 + nr) * 8)], "<f8")
                         .reshape(cnt, 3 + nr))
    return np.concatenate(ints), np.concatenate(reals)


@need_ref
def test_read_reference_checkpoint():
    P = read_checkpoint(CHK, 2)
    iv, rv = read_chk_restated(CHK, 2)
    assert P.n == 410 == len(iv)
    for k, c in (("x", 0), ("y", 1), ("z", 2), ("radius", 3), ("c_length", 4), ("theta", 5), ("phi", 6),
                 ("area", 7), ("velx", 9), ("wz", 14)):
        assert np.array_equal(P[k], rv[:, c]), k
    # integer components of the 33-int layout (intIdx without fuse_tip, fix_site)
    ic = iv[:, 2:]
    assert np.array_equal(P["cell_type"], ic[:, 5]) and np.array_equal(P["n_bnds"], ic[:, 6])
    assert np.array_equal(P["seg_id1"].reshape(4, -1), ic[:, 7:11].T)
    assert np.array_equal(P["site"].reshape(4, -1), ic[:, 15:19].T)
    assert np.array_equal(P["dltd"].reshape(6, -1), ic[:, 25:31].T)
    assert np.array_equal(P["id"], ic[:, 31]) and np.array_equal(P["cpu"], ic[:, 32])
    assert (P["bond_scale"] == 1.0).all() and (P["fuse_tip"] == 0).all() and (P["fix_site"] == 0).all()
    # the mapping is the right one: ids are unique and the bond tables pair up
    n = P.n
    key = {(int(P["id"][i]), int(P["cpu"][i])): i for i in range(n)}
    assert len(key) == n
    s1, s2 = P["seg_id1"].reshape(4, n), P["seg_id2"].reshape(4, n)
    tot = ok = 0
    for i in range(n):
        for k in range(P["n_bnds"][i]):
            tot += 1
            j = key.get((int(s1[k, i]), int(s2[k, i])))
            if j is not None and any((int(s1[m, j]), int(s2[m, j])) == (int(P["id"][i]), int(P["cpu"][i]))
                                     for m in range(P["n_bnds"][j])):
                ok += 1
    assert tot > 900 and ok >= 0.99 * tot
    assert ((P["position"] >= 0) & (P["position"] <= 3)).all()
    assert (P["cell_type"] == FUNGI).all()


@need_ref
def test_network_golden_matches_checkpoint():
    """The committed network vectors (GPU tests use them) are this reader's."""
    P = read_checkpoint(CHK, 2)
    d = load("fungi_network")
    for k in ("x", "y", "z", "theta", "phi", "c_length", "n_bnds", "seg_id1", "site"):
        assert np.array_equal(P[k], d["in_" + k]), k


def test_checkpoint_errors(tmp_path):
    with pytest.raises(BmxgError) as e:
        read_checkpoint(str(tmp_path))
    assert e.value.code == BMXG_ERR_ARG
    (tmp_path / "Header").write_text("Version_Two_Dot_One_single\n3\n0\n0\n1\n0\n1\n0\n1\n0 0 0\n")
    with pytest.raises(BmxgError) as e:
        read_checkpoint(str(tmp_path))
    assert e.value.code == BMXG_ERR_UNSUPPORTED


def test_checkpoint_round_trip_current_layout(tmp_path):
    """A checkpoint written in the current 34 + 35 layout by this restatement
    reads back field for field."""
    P = mixed_state(7)
    n = P.n
    P["n_bnds"][:] = np.arange(n) % 3
    nr, ni = 34, 35
    rc = np.zeros((n, 3 + nr))
    rc[:, 0], rc[:, 1], rc[:, 2] = P["x"], P["y"], P["z"]
    for k, c in (("radius", 0), ("c_length", 1), ("theta", 2), ("phi", 3), ("area", 4), ("velx", 6),
                 ("vely", 7), ("velz", 8), ("wx", 9), ("wy", 10), ("wz", 11), ("bond_scale", 24)):
        rc[:, 3 + c] = P[k]
    ic = np.zeros((n, 2 + ni), np.int32)
    ic[:, 2 + 5] = P["cell_type"]
    ic[:, 2 + 6] = P["n_bnds"]
    ic[:, 2 + 7:2 + 11] = P["seg_id1"].reshape(4, n).T
    ic[:, 2 + 25] = 1      # fuse_tip
    ic[:, 2 + 32] = 2      # fix_site
    ic[:, 2 + 33] = np.arange(10, 10 + n)
    ic[:, 2 + 34] = 5
    d = tmp_path / "particles"
    (d / "Level_0").mkdir(parents=True)
    head = ["Version_Two_Dot_One_double", "3", str(nr)] + [f"real_comp{k}" for k in range(nr)]
    head += [str(ni)] + [f"int_comp{k}" for k in range(ni)]
    head += ["1", str(n), str(n + 1), "0", "1", f"0 {n} 0"]
    (d / "Header").write_text("\n".join(head) + "\n")
    (d / "Level_0" / "DATA_00000").write_bytes(ic.astype("<i4").tobytes() + rc.astype("<f8").tobytes())
    Q = read_checkpoint(str(d))
    assert Q.n == n
    for k in REAL_OUT + ("bond_scale", "cell_type", "n_bnds", "seg_id1"):
        assert np.array_equal(Q[k], P[k]), k
    assert (Q["fuse_tip"] == 1).all() and (Q["fix_site"] == 2).all()
    assert np.array_equal(Q["id"], np.arange(10, 10 + n)) and (Q["cpu"] == 5).all()
