"""asc-convert (edge list -> graph files) against the oracle's restatement of
the reference converter (converter/converter.cpp). CPU only."""
import os
import subprocess

import numpy as np
import pytest

import ascetic_gb300 as A
import oracle
from ascetic_gb300 import formats as F

EXE = A.CONVERT_PATH


def run(*args):
    return subprocess.run([EXE] + [str(a) for a in args], capture_output=True, text=True)


def write_text(path, lines):
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def check_outputs(stem, src, dst, weights, compat=False):
    V, ptr, order, outdeg = oracle.converter(src, dst, compat=compat)
    g = F.read(stem + ".bcsr", F.FMT_BCSR)
    assert np.array_equal(g["ptr"], ptr)
    assert np.array_equal(g["col"], np.asarray(dst, np.uint32)[order])
    g = F.read(stem + ".bwcsr", F.FMT_BWCSR)
    assert np.array_equal(g["ptr"], ptr)
    assert np.array_equal(g["adj"][:, 0], np.asarray(dst, np.uint32)[order])
    assert np.array_equal(g["adj"][:, 1], np.asarray(weights, np.uint32)[order])
    Vc, cptr, corder, _ = oracle.converter(src, dst, by_dst=True, compat=compat)
    g = F.read(stem + ".bcsc", F.FMT_BCSC)
    assert Vc == V and np.array_equal(g["ptr"], cptr)
    assert np.array_equal(g["col"], np.asarray(src, np.uint32)[corder])
    assert np.array_equal(g["outdeg"], outdeg)
    g = F.read(stem + ".bcsr32", F.FMT_BCSR32)
    assert np.array_equal(g["ptr"], ptr)
    return V


def test_text_to_all_formats(tmp_path):
    lines = ["# comment", "% another", "", "0 1", "0 2", "2 2", "  1\t0", "0 1", "4 5", "5 0", "3 7"]
    src = [0, 0, 2, 1, 0, 4, 5, 3]
    dst = [1, 2, 2, 0, 1, 5, 0, 7]
    path = tmp_path / "g.txt"
    write_text(path, lines)
    r = run(path, "--to", "toB,bcsr,bwcsr,bcsc,bcsr32")
    assert r.returncode == 0, r.stderr
    stem = str(tmp_path / "g")
    V = check_outputs(stem, src, dst, oracle.converter_ref_weights(len(src)))
    assert V == 8  # vertex 7 appears only as a destination, 6 not at all
    pairs = np.fromfile(stem + ".toB", np.uint32).reshape(-1, 2)
    assert np.array_equal(pairs[:, 0], src) and np.array_equal(pairs[:, 1], dst)
    # the binary pair file converts to the same graphs
    r = run(stem + ".toB", "--to", "bcsr,bwcsr,bcsc,bcsr32", "--out", tmp_path / "h")
    assert r.returncode == 0, r.stderr
    check_outputs(str(tmp_path / "h"), src, dst, oracle.converter_ref_weights(len(src)))


def test_compat_offsets(tmp_path):
    # the last vertex with edges (2) is followed by vertices without any: the
    # reference's offsets step back one there, moving an edge to vertex V-1
    src, dst = [0, 0, 2, 2], [1, 4, 0, 3]
    path = tmp_path / "c.txt"
    write_text(path, ["%d %d" % e for e in zip(src, dst)])
    assert run(path, "--compat", "--to", "bcsr,bwcsr,bcsc,bcsr32").returncode == 0
    check_outputs(str(tmp_path / "c"), src, dst, oracle.converter_ref_weights(4), compat=True)
    g = F.read(str(tmp_path / "c.bcsr"))
    deg = np.diff(g["ptr"].astype(np.int64))
    assert deg.tolist() == [2, 0, 1, 0, 1]
    assert run(path, "--to", "bcsr", "--out", tmp_path / "x").returncode == 0
    assert np.diff(F.read(str(tmp_path / "x.bcsr"))["ptr"].astype(np.int64)).tolist() == [2, 0, 2, 0, 0]


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_random_edge_lists(tmp_path, seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 400))
    V = int(rng.integers(1, 60))
    src = rng.integers(0, V, n).tolist()
    dst = rng.integers(0, V, n).tolist()
    w = rng.integers(0, 1000, n).tolist()
    path = tmp_path / "r.el"
    write_text(path, ["%d %d %d" % e for e in zip(src, dst, w)])
    assert run(path, "--weights", "column", "--to", "bcsr,bwcsr,bcsc,bcsr32").returncode == 0
    check_outputs(str(tmp_path / "r"), src, dst, w)
    for compat in (False, True):
        assert run(path, "--compat" if compat else "--seed", *([] if compat else ["5"]), "--to",
                   "bcsr,bwcsr,bcsc,bcsr32", "--out", tmp_path / "s").returncode == 0
        check_outputs(str(tmp_path / "s"), src, dst, oracle.converter_ref_weights(n), compat=compat)


def test_symmetrize_transpose_and_uniform_weights(tmp_path):
    src, dst = [0, 1, 1, 3], [1, 2, 3, 0]
    path = tmp_path / "t.txt"
    write_text(path, ["%d %d" % e for e in zip(src, dst)])
    r = run(path, "--symmetrize", "--weights", "uniform:1:63", "--seed", "9", "--to", "bcsr,bwcsr,bcsc,bcsr32")
    assert r.returncode == 0, r.stderr
    g = F.read(str(tmp_path / "t.bwcsr"), F.FMT_BWCSR)
    w = g["adj"][:, 1]
    assert w.min() >= 1 and w.max() <= 63
    # a reversed edge carries its original's weight: read the weights back per edge
    wmap = {}
    ptr = g["ptr"]
    for u in range(len(ptr) - 1):
        for k in range(int(ptr[u]), int(ptr[u + 1])):
            wmap.setdefault((u, int(g["adj"][k, 0])), []).append(int(g["adj"][k, 1]))
    for s, d in zip(src, dst):
        assert wmap[(s, d)] == wmap[(d, s)]
    orig_w = [wmap[(s, d)][0] for s, d in zip(src, dst)]
    check_outputs(str(tmp_path / "t"), src + dst, dst + src, orig_w + orig_w)
    assert run(path, "--transpose", "--to", "bcsr,bwcsr,bcsc,bcsr32", "--out", tmp_path / "u").returncode == 0
    check_outputs(str(tmp_path / "u"), dst, src, oracle.converter_ref_weights(4))


def test_errors(tmp_path):
    r = subprocess.run([EXE], capture_output=True, text=True)
    assert r.returncode == 1 and "usage: asc-convert" in r.stderr
    bad = tmp_path / "bad.txt"
    write_text(bad, ["0 1", "1 x"])
    r = run(bad)
    assert r.returncode == 2 and "line 2" in r.stderr
    write_text(bad, ["0 1", "4294967295 0"])
    assert run(bad).returncode == 2
    write_text(bad, ["0 1", "1 2 3"])
    r = run(bad)
    assert r.returncode == 2 and "columns" in r.stderr
    write_text(bad, ["0 1"])
    assert run(bad, "--weights", "column").returncode == 2
    assert run(bad, "--to", "csv").returncode == 2
    odd = tmp_path / "odd.toB"
    odd.write_bytes(b"\x00" * 12)
    assert run(odd).returncode == 2
    assert run(tmp_path / "missing.txt").returncode == 2
