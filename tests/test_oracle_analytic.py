"""Known answers the oracle reproduces, independent of the reference: the
forces of two bodies and of a symmetric nine-body set in closed form, and
the trees of hand-built point sets, whose octant paths follow from the
binary expansion of the coordinates.  (The reference ships no golden vectors;
these and the reference's own kernels, run through the emulator, are the
oracle's pins.)"""
import numpy as np
import pytest


def two_bodies():
    pos = np.array([[0.25, -0.5, 1.0], [-0.75, 0.5, 0.0]], np.float32)
    mass = np.array([0.3, 2.0], np.float32)
    return pos, mass


def nine_bodies():
    corners = [[x, y, z] for y in (1.0, -1.0) for x in (1.0, -1.0) for z in (1.0, -1.0)]
    return np.array(corners + [[0.0, 0.0, 0.0]], np.float32), np.ones(9, np.float32)


def analytic_two_body(pos, mass, eps, G):
    d = pos[1].astype(np.float64) - pos[0].astype(np.float64)
    s = (np.dot(d, d) + eps * eps) ** 1.5
    return np.stack([G * float(mass[1]) * d / s, -G * float(mass[0]) * d / s])


@pytest.mark.parametrize("eps", [0.0, 0.05])
def test_two_body_forces(oracle, eps):
    pos, mass = two_bodies()
    want = analytic_two_body(pos, mass, eps, 1.5)
    np.testing.assert_allclose(oracle.direct_fp64(pos, mass, eps, 1.5), want, rtol=1e-12, atol=0)
    # FP32 paths: eps enters as float32(eps)
    want = analytic_two_body(pos, mass, float(np.float32(eps)), 1.5)
    np.testing.assert_allclose(oracle.direct_fp32(pos, mass, eps, 1.5), want, rtol=2e-6, atol=0)
    acc, _, _ = oracle.bh_step_forces(pos, mass, 0.5, eps, 1.5, nodes=64)
    np.testing.assert_allclose(acc, want, rtol=2e-6, atol=0)


def test_nine_body_symmetry(oracle):
    """Eight equal masses on the corners of a cube pull the ninth, at the
    centre, equally in opposite directions: its acceleration is zero to the
    rounding of a sum of eight terms +-c; total momentum is conserved to
    rounding; every corner is pulled inwards along each axis."""
    pos, mass = nine_bodies()
    for acc, ulp in ((oracle.direct_fp64(pos, mass, 0.01, 1.0), 2.0 ** -52),
                     (oracle.direct_fp32(pos, mass, 0.01, 1.0), 2.0 ** -23),
                     (oracle.bh_step_forces(pos, mass, 0.0, 0.01, 1.0, nodes=64)[0], 2.0 ** -23)):
        c = 1.0 / 3.0 ** 1.5  # one corner's pull on the centre, per axis (eps aside)
        assert np.max(np.abs(acc[8])) <= 8 * c * 4 * ulp
        # corners: |a| = G m sum over the other bodies, all pointing inwards
        assert np.all(np.sign(acc[:8]) == -np.sign(pos[:8]))
        p = np.sum(mass[:, None].astype(np.float64) * acc, axis=0)
        assert np.max(np.abs(p)) <= 1e-6 * np.max(np.abs(acc))


def one_per_octant():
    pos = np.array([[x, y, z] for y in (0.5, -0.5) for x in (0.5, -0.5) for z in (0.5, -0.5)], np.float32)
    return pos, np.ones(8, np.float32)


def slot_of(p, c=(0.0, 0.0, 0.0)):
    return 4 * (p[1] < c[1]) + 2 * (p[0] < c[0]) + (p[2] < c[2])


def test_one_body_per_octant(oracle):
    """Each body is alone in its octant of the root: no cell is made and the
    root's slot 4(y<c) + 2(x<c) + (z<c) holds that body."""
    pos, mass = one_per_octant()
    t = oracle.tree_build(oracle.SEM_GEOMETRIC, pos, mass, oracle.bbox_exact(pos), 64)
    assert t.status == 0 and t.root - t.bottom == 0
    row = t.children.reshape(-1, 8)[t.root]
    assert [slot_of(pos[b]) for b in row] == list(range(8))


def chain_bodies():
    """Anchors at two corners fix the box to [-1, 1]^3; A = (x, x, x) with
    x = float32(0.1) and B = A + 2^-10 along x share every octant until a
    cut plane falls between them, which first happens at depth 10."""
    x = np.float32(0.1)
    b = np.float32(x + np.float32(2.0 ** -10))
    pos = np.array([[-1, -1, -1], [1, 1, 1], [x, x, x], [b, x, x]], np.float32)
    return pos, np.ones(4, np.float32)


def chain_expected():
    """Octant paths from the binary digits: below the root (slot 0, all
    coordinates >= 0) the cell at depth d is cut at x's digit d: digit 0 ->
    slot 7 (all three coordinates below the centre), 1 -> slot 0.  A and B
    first differ in digit 10 (B's x is above that cut: slot 5)."""
    x = float(np.float32(0.1))
    digits = [int(x * 2 ** k) & 1 for k in range(1, 11)]
    a = [0] + [0 if d else 7 for d in digits]
    bpath = a[:-1] + [5]
    return a, bpath


def test_chain_separates_at_depth_10(oracle):
    pos, mass = chain_bodies()
    t = oracle.tree_build(oracle.SEM_GEOMETRIC, pos, mass, oracle.bbox_exact(pos), 64)
    assert t.status == 0
    assert t.root - t.bottom == 10 and t.max_depth == 10
    paths, depth, found = oracle.tree_paths(t.children, 4, t.root)
    assert found == 4
    a, b = chain_expected()
    assert list(paths[2, :depth[2]]) == a and list(paths[3, :depth[3]]) == b
    assert list(paths[0, :depth[0]]) == [7] and list(paths[1, :depth[1]]) == [0, 0]


def _cell_table(children, mass, pos, count, n, root):
    """(mass, centre, body count) of every cell, keyed by its octant path."""
    ch = children.reshape(-1, 8)
    pos = pos.reshape(-1, 3)
    out, stack = {}, [(root, ())]
    while stack:
        node, path = stack.pop()
        out[path] = (float(mass[node]), tuple(float(v) for v in pos[node]), int(count[node]))
        for s in range(8):
            c = ch[node][s]
            if c >= n:
                stack.append((c, path + (s,)))
    return out


@pytest.mark.parametrize("semantics", ["geometric", "reference"])
def test_tree_does_not_depend_on_insertion_order(oracle, semantics):
    """For distinct points the octree is a function of the point set: built
    from the bodies in a shuffled order it has the same octant path for every
    body, the same cells with the same summaries (children are summed in slot
    order) and the same in-order listing of the bodies.  This is what lets a
    sequential CPU build check the concurrent GPU build."""
    O = oracle
    sem = O.SEM_GEOMETRIC if semantics == "geometric" else O.SEM_REFERENCE
    n = 3000
    rng = np.random.default_rng(17)
    pos = (rng.normal(size=(n, 3)) * np.array([1.0, 1.0, 0.3])).astype(np.float32)
    mass = (0.5 + rng.random(n)).astype(np.float32)
    perm = rng.permutation(n)
    box = O.bbox_exact(pos)
    built = []
    for p, m in ((pos, mass), (pos[perm], mass[perm])):
        t = O.tree_build(sem, p, m, box)
        assert t.status == 0
        octant = t.children.copy()
        assert O.saturate(t) == 0
        paths, depth, found = O.tree_paths(octant, n, t.root)
        assert found == n
        srt, k = O.sort_bodies(t.children, n, t.root)
        assert k == n
        table = _cell_table(octant, t.mass, t.pos, t.body_count, n, t.root)
        built.append((paths, depth, srt, table, t.root - t.bottom, t.max_depth))
    (pa, da, sa, ta, ca, ma), (pb, db, sb, tb, cb, mb) = built
    assert ca == cb and ma == mb
    assert np.array_equal(pb, pa[perm]) and np.array_equal(db, da[perm])
    assert np.array_equal(perm[sb], sa)
    assert ta == tb


def test_sort_lists_every_cell_contiguously(oracle):
    """The in-order sort puts the bodies of every cell in one contiguous run
    of the sorted order, as long as the cell's body count (so a warp group of
    32 consecutive sorted bodies spans few cells: the walk's vote groups)."""
    O = oracle
    n = 4000
    rng = np.random.default_rng(23)
    pos = rng.normal(size=(n, 3)).astype(np.float32)
    mass = np.full(n, 1.0 / n, np.float32)
    t = O.tree_build(O.SEM_GEOMETRIC, pos, mass, O.bbox_exact(pos))
    assert t.status == 0 and O.saturate(t) == 0
    srt, k = O.sort_bodies(t.children, n, t.root)
    assert k == n and np.array_equal(np.sort(srt), np.arange(n))
    where = np.empty(n, np.int64)
    where[srt] = np.arange(n)
    ch = t.children.reshape(-1, 8)

    def span(node):  # (first, last, bodies) of the node's subtree in the sorted order
        if node < n:
            return where[node], where[node], 1
        lo, hi, cnt = n, -1, 0
        for c in ch[node]:
            if c >= 0:
                a, b, m = span(c)
                lo, hi, cnt = min(lo, a), max(hi, b), cnt + m
        assert hi - lo + 1 == cnt == t.body_count[node]
        return lo, hi, cnt

    assert span(t.root) == (0, n - 1, n)
