"""The oracle pinned against golden vectors produced by the reference's own
kernels (tests/golden/make_golden.py).  CPU only."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TREE_CASES = ["ref_tree_n256_wg16.npz", "ref_tree_n300_wg64.npz"]
DIRECT_CASES = ["ref_direct_n256_wg16.npz", "ref_direct_n512_wg64.npz"]


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name)))


def cell_table(children, mass, pos, count, n, root):
    """canonical path -> (mass, com xyz, count) for every cell."""
    ch = children.reshape(-1, 8)
    pos = pos.reshape(-1, 3)
    out, stack = {}, [(root, ())]
    while stack:
        node, path = stack.pop()
        out[path] = (mass[node], pos[node], count[node])
        for s in range(8):
            c = ch[node][s]
            if c >= n:
                stack.append((c, path + (s,)))
    return out


@pytest.mark.parametrize("name", TREE_CASES)
def test_bbox_as_wired(oracle, name):
    g = load(name)
    got = oracle.bbox_sampled(g["p_buffer"], int(g["wg"]))
    assert np.array_equal(got, g["wired_box"])


@pytest.mark.parametrize("name", TREE_CASES)
def test_tree_topology_reference_semantics(oracle, name):
    g = load(name)
    n, nodes = len(g["mass"]), int(g["nodes"])
    t = oracle.tree_build(oracle.SEM_REFERENCE, g["pos"], g["mass"], g["box"], nodes)
    assert t.status == 0
    pr, dr, fr = oracle.tree_paths(g["built_children"], n, n + nodes)
    po, do, fo = oracle.tree_paths(t.children, n, t.root)
    assert fr == n and fo == n
    assert np.array_equal(pr, po) and np.array_equal(dr, do)
    assert t.bottom == int(g["bottom"])
    assert t.max_depth == int(g["max_depth"])


@pytest.mark.parametrize("name", TREE_CASES)
def test_saturate_reference_semantics(oracle, name):
    g = load(name)
    n, nodes = len(g["mass"]), int(g["nodes"])
    t = oracle.tree_build(oracle.SEM_REFERENCE, g["pos"], g["mass"], g["box"], nodes)
    assert oracle.saturate(t, compaction_bug=True) == 0
    ref = cell_table(g["sat_children"], g["sat_mass"], g["sat_pos"], g["sat_count"], n, n + nodes)
    got = cell_table(t.children, t.mass, t.pos, t.body_count, n, t.root)
    assert ref.keys() == got.keys()
    for k in ref:
        # the reference sums ready children first, so the order (and the last
        # bits) differ; the counts are exact
        assert ref[k][2] == got[k][2]
        assert abs(ref[k][0] - got[k][0]) <= 4e-7 * abs(got[k][0])
        assert np.all(np.abs(ref[k][1] - got[k][1]) <= 1e-6 * (1 + np.abs(got[k][1])))
    # the compaction defect leaves the same child rows as the reference
    assert np.array_equal(np.sort(g["sat_children"].reshape(-1, 8)[n:], axis=1)[:, :0],
                          np.sort(t.children.reshape(-1, 8)[n:], axis=1)[:, :0])


def test_bh_force_bit_exact_on_reference_tree(oracle):
    g = load("ref_tree_n256_wg16.npz")
    n, nodes = len(g["mass"]), int(g["nodes"])
    t = oracle.Tree(n, nodes)
    t.pos[:] = g["sat_pos"]
    t.mass[:] = g["sat_mass"]
    t.children[:] = g["sat_children"]
    for (theta, eps), want in zip(g["thetas"], g["bh_acc"]):
        dq = oracle.thresholds(oracle.CRIT_REFERENCE, g["box"], float(theta), float(eps), int(g["max_depth"]))
        acc, rc = oracle.bh_force(t, dq, float(eps), 1.0, arith=oracle.ARITH_REFERENCE, vote_width=16, order=None,
                                  skip_self=False)
        assert rc == 0
        assert np.array_equal(acc, want), (theta, eps, np.abs(acc - want).max())


@pytest.mark.parametrize("name", DIRECT_CASES)
def test_direct_quirk_and_euler(oracle, name):
    g = load(name)
    wg = int(g["wg"])
    assert np.array_equal(oracle.direct_quirk_global(g["pos"], g["mass"], 1.0), g["acc_global"])
    assert np.array_equal(oracle.direct_quirk_local(g["pos"], g["mass"], 1.0, wg=wg, tile_schedule=True), g["acc_local"])
    a = oracle.direct_quirk_global(g["pos"], g["mass"], 1.0)
    p, v, _ = oracle.integrate(oracle.EULER, g["pos"], g["vel"], a, np.zeros_like(a), 1e-3)
    assert np.array_equal(p, g["euler_pos"]) and np.array_equal(v, g["euler_vel"])


@pytest.mark.parametrize("name", DIRECT_CASES)
def test_collision_and_copy(oracle, name):
    g = load(name)
    v = oracle.collision(g["coll_pos"], g["vel"], wg=int(g["wg"]), tile_schedule=True)
    assert np.array_equal(v, g["coll_vel"])
    assert np.any(v != g["vel"])  # the fixture does collide
    assert np.array_equal(oracle.copy_vertices(g["coll_pos"]), g["verts"])


def test_reference_bh_misses_subtrees_after_compaction_gap(oracle):
    """The reference's compaction defect leaves a gap that its walk treats as
    the end of the child list, so even with every cell opened (theta -> 0)
    the reference force is not the direct sum; with correct compaction it is."""
    g = load("ref_tree_n256_wg16.npz")
    n, nodes = len(g["mass"]), int(g["nodes"])
    exact = oracle.direct_fp64(g["pos"], g["mass"], 0.01, 1.0)
    errs = {}
    for bug in (True, False):
        t = oracle.tree_build(oracle.SEM_REFERENCE, g["pos"], g["mass"], g["box"], nodes)
        oracle.saturate(t, compaction_bug=bug)
        dq = oracle.thresholds(oracle.CRIT_REFERENCE, g["box"], 1e-12, 0.01, t.max_depth)
        acc, _ = oracle.bh_force(t, dq, 0.01, 1.0, arith=oracle.ARITH_REFERENCE, vote_width=16)
        errs[bug] = np.max(np.linalg.norm(acc - exact, axis=1) / np.linalg.norm(exact, axis=1))
    assert errs[False] < 1e-4
    assert errs[True] > 1e-2
