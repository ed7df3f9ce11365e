"""Host logic of adaptive refinement (athena-gamma_gb300/csrc/athg_amr.cpp) on the CPU:
the gid order of the reference's block tree (pinned by the block lists of the reference's
own adaptive runs, tests/golden/amr_*.npz), MeshBlockTree refinement with the 2:1 level
rule, derefinement of complete octets only, and MeshRefinement::CheckRefinementCondition
(mesh/mesh_refinement.cpp:1003-1062)."""
import itertools
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "athena-gamma_gb300", "csrc")
sys.path.insert(0, HERE)
import amr_golden  # noqa: E402


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    out = str(tmp_path_factory.mktemp("amr") / "amr_check")
    subprocess.run([gxx, "-std=c++17", "-O1", "-I", CSRC, os.path.join(HERE, "amr_check.cpp"),
                    os.path.join(CSRC, "athg_amr.cpp"), "-o", out], check=True)
    return out


def tree(exe, nrb, leaves, flags=None):
    flags = flags or [0] * len(leaves)
    txt = "tree %d %d %d %d\n" % (nrb + (len(leaves),))
    txt += "".join("%d %d %d %d %d\n" % (tuple(l) + (f,)) for l, f in zip(leaves, flags))
    r = subprocess.run([exe], input=txt, capture_output=True, text=True, check=True)
    lines = r.stdout.splitlines()
    order = [int(x) for x in lines[0].split()[1:]]
    changed = lines[1] == "changed 1"
    out = [tuple(int(x) for x in ln.split()) for ln in lines[2:]]
    return order, changed, out


def flag(exe, maxeps, thr, level, max_level, dthr, dcount, nbl=None):
    nbl = nbl if nbl is not None else [level] * 27
    txt = "flag %r %r 0.25 %d %d %d %d %s\n" % (maxeps, thr, level, max_level, dthr, dcount,
                                               " ".join(str(x) for x in nbl))
    r = subprocess.run([exe], input=txt, capture_output=True, text=True, check=True)
    f, c = r.stdout.split()
    return int(f), int(c)


def sort_key(b):
    return (b[0], b[3], b[2], b[1])


def box(b):
    s = 2.0 ** -b[0]
    return np.array(b[1:]) * s, (np.array(b[1:]) + 1) * s


def balanced(leaves):
    """Every two leaves that touch (faces, edges or corners) differ by at most one level."""
    for a, b in itertools.combinations(leaves, 2):
        if abs(a[0] - b[0]) <= 1:
            continue
        (alo, ahi), (blo, bhi) = box(a), box(b)
        if np.all(alo <= bhi) and np.all(blo <= ahi):
            return False
    return True


def volume(leaves):
    return sum(8.0 ** -b[0] for b in leaves)


@pytest.mark.parametrize("name", list(amr_golden.CASES))
def test_tree_order_matches_reference_dumps(exe, name):
    ref = amr_golden.load(name)
    nrb = (amr_golden.CASES[name][8] // amr_golden.CASES[name][9],) * 3
    off = 0
    for nb in ref["dump_nblocks"]:
        dump = [tuple(int(x) for x in b) for b in ref["dump_blocks"][off:off + nb]]
        off += nb
        leaves = sorted(dump, key=sort_key)
        order, changed, out = tree(exe, nrb, leaves)
        assert not changed and out == leaves
        assert [leaves[g] for g in order] == dump


def uniform(n):
    return sorted([(0, i, j, k) for i in range(n) for j in range(n) for k in range(n)],
                  key=sort_key)


def test_refine_keeps_levels_within_one(exe):
    leaves = uniform(4)
    _, changed, l1 = tree(exe, (4, 4, 4), leaves, [int(b == (0, 1, 1, 1)) for b in leaves])
    assert changed and len(l1) == 63 + 8 and volume(l1) == 64
    # refining the child at the octant's low corner pulls the level-0 neighbours touching it
    # up to level 1
    _, changed, l2 = tree(exe, (4, 4, 4), l1, [int(b == (1, 2, 2, 2)) for b in l1])
    assert changed and volume(l2) == 64
    assert sum(1 for b in l2 if b[0] == 2) == 8
    assert balanced(l2)
    assert all(b[0] <= 2 for b in l2)
    # a root block touching the level-2 octant was refined
    assert (0, 0, 0, 0) not in l2 and (1, 1, 1, 1) in l2
    # derefining every level-1 block where allowed keeps the tree balanced
    _, _, l3 = tree(exe, (4, 4, 4), l2, [-1 if b[0] == 1 else 0 for b in l2])
    assert balanced(l3) and volume(l3) == 64
    assert sum(1 for b in l3 if b[0] == 2) == 8


def test_derefine_needs_eight_children(exe):
    leaves = uniform(4)
    _, _, l1 = tree(exe, (4, 4, 4), leaves, [int(b == (0, 1, 1, 1)) for b in leaves])
    kids = [b for b in l1 if b[0] == 1]
    # seven of eight: unchanged
    fl = [-1 if b in kids[:7] else 0 for b in l1]
    _, changed, same = tree(exe, (4, 4, 4), l1, fl)
    assert not changed and same == l1
    # all eight: the parent comes back
    _, changed, back = tree(exe, (4, 4, 4), l1, [-1 if b in kids else 0 for b in l1])
    assert changed and back == leaves


def test_refinement_flags(exe):
    # above the threshold: refine below the top level, keep at it; counter reset
    assert flag(exe, 1.0, 0.5, 0, 1, 3, 2) == (1, 0)
    assert flag(exe, 1.0, 0.5, 1, 1, 3, 2) == (0, 0)
    # between deref_fraction * threshold and threshold: keep, counter reset
    assert flag(exe, 0.2, 0.5, 1, 1, 3, 2) == (0, 0)
    # below: root blocks stay; finer blocks count up and derefine at the count
    assert flag(exe, 0.01, 0.5, 0, 1, 3, 2) == (0, 0)
    assert flag(exe, 0.01, 0.5, 1, 1, 3, 1) == (0, 2)
    assert flag(exe, 0.01, 0.5, 1, 1, 3, 2) == (-1, 3)
    # a finer neighbour blocks derefinement (the counter still counts)
    nbl = [1] * 27
    nbl[5] = 2
    assert flag(exe, 0.01, 0.5, 1, 2, 3, 2, nbl) == (0, 3)
