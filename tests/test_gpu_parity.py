"""Parity of the CUDA path (through the C ABI) against the CPU oracle.

Bit-exact: bounding box, tree topology in canonical octant-path form, cell
masses / centres of mass / body counts, the sort permutation, the opening
thresholds, the collision update and copy_vertices.  Within tolerance (the
GPU uses the MUFU rsqrt and a different summation order): accelerations and
positions after k steps.  Tolerances are stated per test.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def ball(n, seed, r=1.0):
    rng = np.random.default_rng(seed)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    p = d * (r * rng.random(n) ** (1 / 3))[:, None]
    return p.astype(np.float32)


def normal(n, seed, sigma=(1.0, 1.0, 1.0)):
    rng = np.random.default_rng(seed)
    return (rng.normal(size=(n, 3)) * np.asarray(sigma)).astype(np.float32)


def masses(n, seed, kind="equal"):
    if kind == "equal":
        return np.full(n, 1.0 / n, np.float32)
    rng = np.random.default_rng(seed + 1)
    m = np.exp(0.5 * rng.normal(size=n))
    return (m / m.sum()).astype(np.float32)


def bh_sim(nb, pos, mass, theta, eps, G=1.0, tree=0, crit=0, method=2, precision=0, vel=None, cap=0, quad=0):
    sim = nb.Simulation(num_of_bodies=len(mass), algo_config=nb.BARNES_HUT, theta=theta, epsilon=eps,
                        gravitational_constant=G, tree_semantics=tree, theta_semantics=crit,
                        numerical_method=method, precision=precision, cell_capacity=cap, multipole=quad)
    sim.set_state(pos, mass, vel)
    return sim


def cell_table(children, mass, pos, count, n, root):
    ch = children.reshape(-1, 8)
    pos = pos.reshape(-1, 3)
    out, stack = {}, [(root, ())]
    while stack:
        node, path = stack.pop()
        out[path] = (mass[node], tuple(pos[node]), count[node])
        for s in range(8):
            c = ch[node][s]
            if c >= n:
                stack.append((c, path + (s,)))
    return out


def rel_to_typical(a, b):
    """max |a_i - b_i| / rms |b|: error relative to the typical acceleration."""
    scale = np.sqrt(np.mean(np.sum(b.astype(np.float64) ** 2, axis=1)))
    return float(np.max(np.linalg.norm(a.astype(np.float64) - b, axis=1)) / scale)


CASES = [
    ("ball", 262144, 0.5, 0.01, 0, 0),  # the plain Barnes-Hut configuration's size
    ("ball", 20000, 0.5, 0.01, 0, 0),
    ("normal", 30000, 0.5, 0.005, 0, 0),
    ("normal", 12345, 0.3, 0.005, 0, 0),
    ("ball", 16384, 0.5, 0.01, 1, 1),   # the reference's tree and thresholds
    ("normal", 9000, 1.5, 0.01, 1, 1),  # the reference's default theta
]


@pytest.mark.parametrize("kind,n,theta,eps,tree,crit", CASES)
def test_bh_stages_against_oracle(gpu, oracle, kind, n, theta, eps, tree, crit):
    nb = gpu
    pos = ball(n, n) if kind == "ball" else normal(n, n, (1.0, 1.0, 0.2))
    mass = masses(n, n, "equal" if kind == "ball" else "lognormal")
    sim = bh_sim(nb, pos, mass, theta, eps, tree=tree, crit=crit)
    sim.step(0.0, 1)  # dt = 0: forces only, positions unchanged
    # 1. bounding box, bit-exact
    box = sim.stage_debug(nb.DEBUG_BBOX)
    assert np.array_equal(box, oracle.bbox_exact(pos))
    info = sim.stage_debug(nb.DEBUG_TREE_INFO)
    cap = int(info[1])
    # 2. topology, bit-exact in canonical path form
    sem = oracle.SEM_REFERENCE if tree else oracle.SEM_GEOMETRIC
    t = oracle.tree_build(sem, pos, mass, box, cap)
    assert t.status == 0
    children = sim.stage_debug(nb.DEBUG_CHILDREN)
    pg, dg, fg = oracle.tree_paths(children, n, n + cap)
    po, do, fo = oracle.tree_paths(t.children, n, t.root)
    assert fg == n and fo == n
    assert np.array_equal(dg, do) and np.array_equal(pg, po)
    assert int(info[3]) == t.max_depth
    assert int(info[2]) == t.bottom  # the same number of cells
    # 3. summarisation, bit-exact (children summed in slot order); cells are
    #    keyed by their octant path, taken before the oracle compacts slots
    octant_children = t.children.copy()
    assert oracle.saturate(t) == 0
    mg = sim.stage_debug(nb.DEBUG_NODE_MASS)
    xg = sim.stage_debug(nb.DEBUG_NODE_POS)
    cg = sim.stage_debug(nb.DEBUG_BODY_COUNT)
    tg = cell_table(children, mg, xg, cg, n, n + cap)
    to = cell_table(octant_children, t.mass, t.pos, t.body_count, n, t.root)
    assert tg.keys() == to.keys()
    bad = [k for k in to if tg[k] != to[k]]
    assert not bad, (len(bad), bad[:3])
    assert cg[n + cap] == n
    # 4. sort permutation, bit-exact
    srt_o, k = oracle.sort_bodies(t.children, n, t.root)
    srt_g = sim.stage_debug(nb.DEBUG_SORTED)
    assert k == n
    assert np.array_equal(srt_g, srt_o)
    # 5. thresholds, bit-exact
    crit_o = oracle.CRIT_REFERENCE if crit else oracle.CRIT_STANDARD
    dq = oracle.thresholds(crit_o, box, theta, eps, t.max_depth)
    assert np.array_equal(sim.stage_debug(nb.DEBUG_DQ), dq)
    # 6. accelerations: same votes (warps of 32 in sort order), same d^2 arithmetic;
    #    the GPU's rsqrt and summation order stay within 2e-5 of the typical |a|
    acc_o, rc = oracle.bh_force(t, dq, eps, 1.0, arith=oracle.ARITH_FMA, vote_width=32, order=srt_o)
    assert rc == 0
    _, _, acc_g, _ = sim.get_state()
    err = rel_to_typical(acc_g, acc_o)
    assert err < 2e-5, err


@pytest.mark.parametrize("kind,n,theta,eps,comp", [("ball", 20000, 0.5, 0.01, 0), ("normal", 30000, 0.5, 0.005, 1),
                                                   ("normal", 7777, 0.8, 0.005, 0)])
def test_bh_quadrupole_against_oracle(gpu, oracle, kind, n, theta, eps, comp):
    """Cell quadrupoles bit-exact (same slot order and roundings); forces with
    the quadrupole term within 2e-5 of the typical |a|."""
    nb = gpu
    pos = ball(n, n) if kind == "ball" else normal(n, n, (1.0, 1.0, 0.2))
    mass = masses(n, n, "equal" if kind == "ball" else "lognormal")
    sim = bh_sim(nb, pos, mass, theta, eps, quad=1, precision=comp)
    sim.step(0.0, 1)
    info = sim.stage_debug(nb.DEBUG_TREE_INFO)
    cap = int(info[1])
    acc_o, t, srt = oracle.bh_step_forces(pos, mass, theta, eps, 1.0, nodes=cap, quadrupole=True,
                                          compensated=bool(comp))
    children = sim.stage_debug(nb.DEBUG_CHILDREN)
    qg = sim.stage_debug(nb.DEBUG_NODE_QUAD).reshape(-1, 6)
    qo = oracle.quadrupoles(t).reshape(-1, 6)
    # same cells by octant path: compare the quadrupole of every cell
    tg = cell_table(children, np.zeros(len(qg)), qg[:, :3].ravel(), np.arange(len(qg)), n, n + cap)
    octant = oracle.tree_build(oracle.SEM_GEOMETRIC, pos, mass, sim.stage_debug(nb.DEBUG_BBOX), cap).children
    to = cell_table(octant, np.zeros(len(qo)), qo[:, :3].ravel(), np.arange(len(qo)), n, t.root)
    assert tg.keys() == to.keys()
    for k in to:
        assert np.array_equal(qg[tg[k][2]], qo[to[k][2]]), k
    _, _, acc_g, _ = sim.get_state()
    err = rel_to_typical(acc_g, acc_o)
    assert err < 2e-5, err


def test_bh_accuracy_vs_fp64(gpu, oracle):
    """theta=0.5 standard criterion with quadrupoles: RMS relative force error
    vs FP64 <= 1e-3 (monopole alone is about 4e-3 here); the GPU FP64 probe
    agrees with the CPU FP64 oracle."""
    nb = gpu
    n = 65536
    pos = normal(n, 5, (1.0, 1.0, 0.2))
    mass = masses(n, 5, "lognormal")
    sample = np.random.default_rng(0).choice(n, 2048, replace=False).astype(np.int32)
    mono = bh_sim(nb, pos, mass, 0.5, 0.005)
    mono.step(0.0, 1)
    _, rms_mono, _ = mono.force_error(sample)
    sim = bh_sim(nb, pos, mass, 0.5, 0.005, quad=1)
    sim.step(0.0, 1)
    mx, rms, per = sim.force_error(sample)
    assert rms <= 1e-3, rms
    assert rms < rms_mono / 3, (rms, rms_mono)
    a64 = oracle.direct_fp64(pos, mass, 0.005, 1.0, targets=sample[:256])
    _, _, acc_g, _ = sim.get_state()
    e_cpu = np.linalg.norm(acc_g[sample[:256]] - a64, axis=1) / np.linalg.norm(a64, axis=1)
    # both are FP64 sums in different orders; cancellation in a64 amplifies
    # their last-bit differences, so the errors agree to 1e-4 of themselves
    assert np.allclose(e_cpu, per[:256], rtol=1e-4, atol=1e-12)


@pytest.mark.parametrize("algo,quirk,n", [(1, 0, 4096), (2, 0, 4096), (2, 0, 5000), (2, 0, 70000), (1, 1, 3000),
                                          (2, 1, 3000), (1, 0, 1000)])
def test_direct_against_oracle(gpu, oracle, algo, quirk, n):
    nb = gpu
    pos = normal(n, 100 + n)
    mass = masses(n, n, "lognormal")
    sim = nb.Simulation(num_of_bodies=n, algo_config=algo, force_law=quirk, epsilon=0.05,
                        gravitational_constant=1.0)
    sim.set_state(pos, mass)
    sim.step(0.0, 1)
    _, _, acc_g, _ = sim.get_state()
    if quirk:
        # the reference's arithmetic; the GPU visits every j once (no tile-0 reload)
        acc_o = oracle.direct_quirk_global(pos, mass, 1.0) if algo == 1 else \
            oracle.direct_quirk_local(pos, mass, 1.0, tile_schedule=False)
    else:
        acc_o = oracle.direct_fp32(pos, mass, 0.05, 1.0)
    err = rel_to_typical(acc_g, acc_o)
    assert err < 2e-5, err


def test_direct_trajectory_config1(gpu, oracle):
    """N=4096 normal(0,1), m=1/N, G=1, eps=0.05, dt=1e-3, 20 Euler steps of the
    global direct sum: positions within 1e-5 (relative to their spread)."""
    nb = gpu
    n, steps, dt = 4096, 20, 1e-3
    pos = normal(n, 0)
    mass = masses(n, 0)
    sim = nb.Simulation(num_of_bodies=n, algo_config=nb.BRUTE_FORCE_GLOBAL, epsilon=0.05, gravitational_constant=1.0)
    sim.set_state(pos, mass)
    sim.step(dt, steps)
    pg, vg, _, _ = sim.get_state()
    p, v, a = pos.copy(), np.zeros_like(pos), np.zeros_like(pos)
    for _ in range(steps):
        acc = oracle.direct_fp32(p, mass, 0.05, 1.0)
        p, v, a = oracle.integrate(oracle.EULER, p, v, acc, a, dt)
    assert np.max(np.abs(pg - p)) < 1e-5 * np.std(p)
    assert np.max(np.abs(vg - v)) < 1e-4 * np.std(v)


def test_bh_trajectory(gpu, oracle):
    """BH (standard semantics), 5 Euler steps at N=16384: positions within 1e-5."""
    nb = gpu
    n, steps, dt, theta, eps = 16384, 5, 1e-3, 0.5, 0.01
    pos = ball(n, 3)
    mass = masses(n, 3)
    sim = bh_sim(nb, pos, mass, theta, eps)
    sim.step(dt, steps)
    pg, _, _, _ = sim.get_state()
    p, v, a = pos.copy(), np.zeros_like(pos), np.zeros_like(pos)
    for _ in range(steps):
        acc, _, _ = oracle.bh_step_forces(p, mass, theta, eps, 1.0)
        p, v, a = oracle.integrate(oracle.EULER, p, v, acc, a, dt)
    assert np.max(np.abs(pg - p)) < 1e-5 * np.std(p)


@pytest.mark.parametrize("method", [1, 2, 3])
def test_integrators(gpu, oracle, method):
    nb = gpu
    n, dt = 2048, 2e-3
    pos = normal(n, 9)
    mass = masses(n, 9)
    vel = (np.random.default_rng(1).normal(size=(n, 3)) * 0.1).astype(np.float32)
    sim = nb.Simulation(num_of_bodies=n, algo_config=nb.BRUTE_FORCE_LOCAL, epsilon=0.05, gravitational_constant=1.0,
                        numerical_method=method)
    sim.set_state(pos, mass, vel)
    sim.step(dt, 2)
    pg, vg, _, _ = sim.get_state()
    p, v, a = pos.copy(), vel.copy(), np.zeros_like(pos)
    for k in range(2):
        acc = oracle.direct_fp32(p, mass, 0.05, 1.0)
        p, v, a = oracle.integrate(method, p, v, acc, a, dt, primed=k > 0)
    assert np.max(np.abs(pg - p)) < 1e-6 * np.std(p)
    assert np.max(np.abs(vg - v)) < 1e-5 * np.std(v)


@pytest.mark.parametrize("n,sigma", [(3000, 0.05), (700, 0.02), (40000, 0.12), (65537, 0.15)])
def test_collision_bit_exact(gpu, oracle, n, sigma):
    """The collision update alone (no gravity, dt = 0) equals the oracle's
    ordered reflections bit for bit: small systems take the warp form (one
    target per warp), large ones the block form (one target per thread)."""
    nb = gpu
    pos = normal(n, 77, (sigma, sigma, sigma))
    mass = masses(n, 77)
    vel = (np.random.default_rng(2).normal(size=(n, 3)) * 0.1).astype(np.float32)
    sim = nb.Simulation(num_of_bodies=n, algo_config=nb.BRUTE_FORCE_GLOBAL, collision=1, gravitational_constant=0.0)
    sim.set_state(pos, mass, vel)
    sim.step(0.0, 1)  # no gravity, no drift: the collision update alone
    pg, vg, _, _ = sim.get_state()
    assert np.array_equal(pg, pos)
    vo = oracle.collision(pos, vel)
    assert np.any(vo != vel)
    assert np.array_equal(vg, vo)


def test_copy_vertices(gpu, oracle):
    nb = gpu
    n = 1000
    pos = normal(n, 4)
    sim = nb.Simulation(num_of_bodies=n)
    sim.set_state(pos, masses(n, 4))
    assert np.array_equal(sim.copy_vertices(), oracle.copy_vertices(pos))


@pytest.mark.parametrize("n,offset", [(1000, 0), (70000, 0), (70000, 4), (256 * 40, 8)])
def test_page_locked_host_arrays(gpu, oracle, n, offset):
    """Page-locked host arrays are packed and unpacked by the device in
    place (float4 tiles when 16-byte aligned, single floats otherwise); the
    state and the vertices equal those of ordinary host arrays bit for bit."""
    import ctypes
    nb = gpu
    L = nb.load()
    pos, mass = normal(n, 21), masses(n, 21, "lognormal")
    vel = (0.1 * normal(n, 22)).astype(np.float32)
    plain = bh_sim(nb, pos, mass, 0.5, 0.01, vel=vel)
    plain.step(1e-3, 2)
    want = plain.get_state()
    want_v = plain.copy_vertices()
    plain.close()

    sizes = (12 * n, 12 * n, 4 * n, 12 * n, 12 * n, 16 * n)
    bufs = [L.nb_host_alloc(b + offset) for b in sizes]
    assert all(bufs)
    try:
        arr = [np.ctypeslib.as_array((ctypes.c_float * (b // 4)).from_address(p + offset)) for p, b in zip(bufs, sizes)]
        arr[0][:] = pos.ravel()
        arr[1][:] = vel.ravel()
        arr[2][:] = mass
        # another state first, so that the page-locked one must replace it
        sim = bh_sim(nb, normal(n, 99), masses(n, 99), 0.5, 0.01)
        addr = [p + offset for p in bufs]
        assert L.nb_set_state(sim.h, addr[0], addr[1], addr[2], n) == 0
        sim.step(1e-3, 2)
        assert L.nb_get_state(sim.h, addr[3], addr[4], None, None) == 0
        np.testing.assert_array_equal(arr[3].reshape(n, 3), want[0])
        np.testing.assert_array_equal(arr[4].reshape(n, 3), want[1])
        assert L.nb_copy_vertices(sim.h, addr[5], 0) == 0
        np.testing.assert_array_equal(arr[5].reshape(n, 4), want_v)
        sim.close()
    finally:
        for p in bufs:
            L.nb_host_free(p)


def test_reused_output_arrays(gpu):
    """get_state / positions / a batch's get_state write into the caller's
    arrays when given them, with the same values as fresh arrays."""
    nb = gpu
    n = 5000
    pos, mass = normal(n, 31), masses(n, 31, "lognormal")
    vel = (0.1 * normal(n, 32)).astype(np.float32)
    with bh_sim(nb, pos, mass, 0.5, 0.01, vel=vel) as sim:
        sim.step(1e-3, 2)
        want = sim.get_state()
        out = tuple(np.full_like(a, np.nan) for a in want)
        got = sim.get_state(out=out)
        assert all(g is o for g, o in zip(got, out))
        for g, w in zip(got, want):
            np.testing.assert_array_equal(g, w)
        p = np.empty((n, 3), np.float32)
        assert sim.positions(out=p) is p
        np.testing.assert_array_equal(p, want[0])
        v = np.empty((n, 3), np.float32)
        pp, vv = sim.positions(with_velocities=True, out=(p, v))
        assert pp is p and vv is v
        np.testing.assert_array_equal(v, want[1])
        with pytest.raises(ValueError):
            sim.positions(out=np.empty((n, 4), np.float32))
    cfg = nb.default_config(num_of_bodies=n, algo_config=nb.BARNES_HUT, theta=0.5, epsilon=0.01,
                            gravitational_constant=1.0)
    with nb.Batch([cfg]) as b:
        b.set_state(0, pos, mass, vel)
        b.step(1e-3, 2)
        out = tuple(np.full_like(a, np.nan) for a in want)
        got = b.get_state(0, out=out)
        assert all(g is o for g, o in zip(got, out))
        np.testing.assert_array_equal(got[0], want[0])
        np.testing.assert_array_equal(got[1], want[1])


def test_known_answer_sets(gpu, oracle):
    """The hand-built sets of the oracle's known-answer tests
    (test_oracle_analytic.py) through the C ABI: two-body forces against the
    closed form, the nine-body centre at rest to rounding, the root of one
    body per octant and the tree of two bodies that separate at depth 10."""
    import test_oracle_analytic as K
    nb = gpu

    def accel(pos, mass, algo, eps, G, theta=0.5):
        with nb.Simulation(num_of_bodies=len(mass), algo_config=algo, theta=theta, epsilon=eps,
                           gravitational_constant=G) as sim:
            sim.set_state(pos, mass)
            sim.step(0.0, 1)
            return sim.get_state()[2]

    pos, mass = K.two_bodies()
    want = K.analytic_two_body(pos, mass, float(np.float32(0.05)), 1.5)
    for algo in (nb.BRUTE_FORCE_GLOBAL, nb.BRUTE_FORCE_LOCAL, nb.BARNES_HUT):
        np.testing.assert_allclose(accel(pos, mass, algo, 0.05, 1.5), want, rtol=2e-6, atol=0, err_msg=str(algo))

    pos, mass = K.nine_bodies()
    for algo in (nb.BRUTE_FORCE_GLOBAL, nb.BRUTE_FORCE_LOCAL, nb.BARNES_HUT):
        acc = accel(pos, mass, algo, 0.01, 1.0, theta=0.0)
        assert np.max(np.abs(acc[8])) <= 8 * 3.0 ** -1.5 * 4 * 2.0 ** -23, (algo, acc[8])
        assert np.all(np.sign(acc[:8]) == -np.sign(pos[:8])), algo

    pos, mass = K.one_per_octant()
    with bh_sim(nb, pos, mass, 0.5, 0.01) as sim:
        sim.step(0.0, 1)
        info = sim.stage_debug(nb.DEBUG_TREE_INFO)
        cap = int(info[1])
        root_row = sim.stage_debug(nb.DEBUG_CHILDREN).reshape(-1, 8)[8 + cap]
        assert int(info[2]) == 8 + cap  # no cell
        assert [K.slot_of(pos[b]) for b in root_row] == list(range(8))

    pos, mass = K.chain_bodies()
    with bh_sim(nb, pos, mass, 0.5, 0.01) as sim:
        sim.step(0.0, 1)
        info = sim.stage_debug(nb.DEBUG_TREE_INFO)
        cap = int(info[1])
        assert 4 + cap - int(info[2]) == 10 and int(info[3]) == 10
        paths, depth, found = oracle.tree_paths(sim.stage_debug(nb.DEBUG_CHILDREN), 4, 4 + cap)
        a, b = K.chain_expected()
        assert found == 4 and list(paths[2, :depth[2]]) == a and list(paths[3, :depth[3]]) == b


def test_compensated_accumulation(gpu, oracle):
    nb = gpu
    n = 20000
    pos = normal(n, 6, (1.0, 1.0, 0.2))
    mass = masses(n, 6, "lognormal")
    sim = bh_sim(nb, pos, mass, 0.5, 0.005, precision=nb.PRECISION_COMPENSATED)
    sim.step(0.0, 1)
    acc_o, t, srt = oracle.bh_step_forces(pos, mass, 0.5, 0.005, 1.0, compensated=True)
    _, _, acc_g, _ = sim.get_state()
    assert rel_to_typical(acc_g, acc_o) < 2e-5


def test_update_clamps_frame_time(gpu):
    nb = gpu
    n = 512
    pos = normal(n, 8)
    mass = masses(n, 8)
    a = nb.Simulation(num_of_bodies=n, gravitational_constant=1.0, simulation_speed_mul=2.0)
    b = nb.Simulation(num_of_bodies=n, gravitational_constant=1.0, simulation_speed_mul=2.0)
    a.set_state(pos, mass)
    b.set_state(pos, mass)
    a.update(1.0)          # clamped to 5e-3, times speed 2
    b.step(0.01, 1)
    assert np.array_equal(a.get_state()[0], b.get_state()[0])


def test_cell_overflow_reports_and_keeps_state(gpu):
    nb = gpu
    n = 5000
    pos = ball(n, 1)
    mass = masses(n, 1)
    sim = bh_sim(nb, pos, mass, 0.5, 0.01, cap=64)
    st = sim.step(1e-3, 3, check=False)
    assert st == nb.ERR_CELL_OVERFLOW
    p, _, _, _ = sim.get_state()
    assert np.array_equal(p, pos)


def test_nonfinite_input_reported(gpu):
    nb = gpu
    n = 1000
    pos = ball(n, 2)
    pos[17, 1] = np.nan
    sim = bh_sim(nb, pos, masses(n, 2), 0.5, 0.01)
    assert sim.step(1e-3, 1, check=False) == nb.ERR_NONFINITE


def test_coincident_bodies_do_not_hang(gpu):
    nb = gpu
    n = 1000
    pos = ball(n, 3)
    pos[5] = pos[6]
    sim = bh_sim(nb, pos, masses(n, 3), 0.5, 0.01)
    st = sim.step(1e-3, 1, check=False)
    assert st in (nb.ERR_DEPTH, nb.ERR_CELL_OVERFLOW)


def test_tree_after_steps_equals_the_oracle(gpu, oracle):
    """After steps (integrated positions, buffers flipped, the previous tree
    overwritten) the tree (octant paths), the summaries and the sort equal
    the oracle's build on the same positions, bit for bit."""
    nb = gpu
    n = 30000
    pos = normal(n, 77, (1.0, 1.0, 0.2))
    mass = masses(n, 77, "lognormal")
    sim = bh_sim(nb, pos, mass, 0.5, 0.005)
    sim.step(1e-3, 2)
    cur = sim.get_state()[0]
    sim.step(0.0, 1)  # positions unchanged: the tree of `cur`
    box = sim.stage_debug(nb.DEBUG_BBOX)
    info = sim.stage_debug(nb.DEBUG_TREE_INFO)
    cap = int(info[1])
    t = oracle.tree_build(oracle.SEM_GEOMETRIC, cur, mass, box, cap)
    children = sim.stage_debug(nb.DEBUG_CHILDREN)
    pg, dg, fg = oracle.tree_paths(children, n, n + cap)
    po, do, fo = oracle.tree_paths(t.children, n, t.root)
    assert fg == n and np.array_equal(pg, po) and np.array_equal(dg, do)
    octant_children = t.children.copy()
    assert oracle.saturate(t) == 0
    tg = cell_table(children, sim.stage_debug(nb.DEBUG_NODE_MASS), sim.stage_debug(nb.DEBUG_NODE_POS),
                    sim.stage_debug(nb.DEBUG_BODY_COUNT), n, n + cap)
    to = cell_table(octant_children, t.mass, t.pos, t.body_count, n, t.root)
    assert tg == to
    srt_o, _ = oracle.sort_bodies(t.children, n, t.root)
    assert np.array_equal(sim.stage_debug(nb.DEBUG_SORTED), srt_o)
    sim.close()


@pytest.mark.parametrize("kind", ["ball", "normal"])
def test_five_top_levels_equal_the_oracle(gpu, oracle, kind):
    """At N = 2^20 the build first creates the cells of five top levels from
    region counts (levels 1-4 in one block, level 5 over a grid) and starts
    every insertion below them.  The tree in octant-path form, its cell
    count and depth, the cell summaries and the sort still equal the
    oracle's build bit for bit."""
    nb = gpu
    n = 1 << 20
    pos = ball(n, 11) if kind == "ball" else normal(n, 11, (1.0, 1.0, 0.2))
    mass = masses(n, 11, "equal" if kind == "ball" else "lognormal")
    sim = bh_sim(nb, pos, mass, 0.5, 0.01)
    sim.step(0.0, 1)
    box = sim.stage_debug(nb.DEBUG_BBOX)
    info = sim.stage_debug(nb.DEBUG_TREE_INFO)
    cap = int(info[1])
    t = oracle.tree_build(oracle.SEM_GEOMETRIC, pos, mass, box, cap)
    assert t.status == 0
    children = sim.stage_debug(nb.DEBUG_CHILDREN)
    pg, dg, fg = oracle.tree_paths(children, n, n + cap)
    po, do, fo = oracle.tree_paths(t.children, n, t.root)
    assert fg == n and np.array_equal(pg, po) and np.array_equal(dg, do)
    assert int(info[2]) == t.bottom and int(info[3]) == t.max_depth
    octant_children = t.children.copy()
    assert oracle.saturate(t) == 0
    tg = cell_table(children, sim.stage_debug(nb.DEBUG_NODE_MASS), sim.stage_debug(nb.DEBUG_NODE_POS),
                    sim.stage_debug(nb.DEBUG_BODY_COUNT), n, n + cap)
    to = cell_table(octant_children, t.mass, t.pos, t.body_count, n, t.root)
    assert tg == to
    srt_o, _ = oracle.sort_bodies(t.children, n, t.root)
    assert np.array_equal(sim.stage_debug(nb.DEBUG_SORTED), srt_o)
    sim.close()


def test_bounded_wait_gives_up_and_the_handle_recovers(gpu):
    """The timeout path, exercised without a hang: with the tree stages' wait
    cap at one iteration the sort's waits for parents give up, the step
    returns NB_ERR_SPIN_TIMEOUT and keeps the step-start state; with the
    default cap restored the same handle steps exactly as a fresh one."""
    nb = gpu
    n = 200000
    pos = normal(n, 5, (1.0, 1.0, 0.2))
    mass = masses(n, 5, "lognormal")
    sim = bh_sim(nb, pos, mass, 0.5, 0.005)
    sim.set_spin_cap(1)
    seen_timeout = False
    for _ in range(3):
        before = sim.get_state()[0]
        st = sim.step(1e-3, 1, check=False)
        assert st in (0, nb.ERR_SPIN_TIMEOUT)
        if st:
            seen_timeout = True
            np.testing.assert_array_equal(sim.get_state()[0], before)
    assert seen_timeout
    sim.set_spin_cap(0)
    sim.set_state(pos, mass)
    assert sim.step(1e-3, 2, check=False) == 0
    fresh = bh_sim(nb, pos, mass, 0.5, 0.005)
    fresh.step(1e-3, 2)
    np.testing.assert_array_equal(sim.get_state()[0], fresh.get_state()[0])
    sim.close()
    fresh.close()


@pytest.mark.parametrize("quad,precision", [(0, 0), (1, 1)])
def test_repeated_runs_are_bit_identical(gpu, quad, precision):
    """The tree build, the sort and the walk run on many threads in a
    schedule-dependent order, but slots are summed in slot order and every
    group walks in its own fixed order: two runs of the same steps give the
    same bits (positions, velocities, accelerations)."""
    nb = gpu
    n = 100000
    pos = normal(n, 8, (1.0, 1.0, 0.2))
    mass = masses(n, 8, "lognormal")
    out = []
    for _ in range(2):
        sim = bh_sim(nb, pos, mass, 0.5, 0.005, quad=quad, precision=precision)
        sim.step(1e-3, 4)
        out.append(sim.get_state()[:3])
        sim.close()
    for a, b in zip(*out):
        np.testing.assert_array_equal(a, b)


def test_largest_tree_and_the_size_limit(gpu):
    """The walk packs (level << 26) | node, so N + cells + 1 < 2^26: N = 2^24
    steps normally (with the default 2N cells), and a size past the limit is
    refused at creation with NB_ERR_UNSUPPORTED."""
    nb = gpu
    n = 1 << 24
    rng = np.random.default_rng(1)
    pos = rng.normal(size=(n, 3)).astype(np.float32)
    mass = np.full(n, 1.0 / n, np.float32)
    sim = bh_sim(nb, pos, mass, 0.7, 0.01)
    sim.step(1e-3, 1)
    p = sim.get_state()[0]
    assert np.all(np.isfinite(p))
    info = sim.stage_debug(nb.DEBUG_TREE_INFO)
    assert int(info[1]) == 2 * n  # cell capacity
    sim.close()
    with pytest.raises(nb.NbError) as e:
        nb.Simulation(num_of_bodies=23_000_000, algo_config=nb.BARNES_HUT)
    assert e.value.status == nb.ERR_UNSUPPORTED


@pytest.mark.parametrize("n", [1, 3, 31, 32, 33, 65])
def test_ragged_small_systems(gpu, oracle, n):
    """Sizes around one warp group of 32 bodies, and a single body, through
    every algorithm with and without softening: a lone body feels no force
    and drifts with its velocity; the direct sums equal the FP64 sum within
    1e-5 of the typical acceleration (MUFU rsqrt, FP32 sums); the tree walk
    (monopole and quadrupole, plain and compensated) equals the oracle's
    walk with the same votes within 2e-5 of the typical acceleration."""
    nb = gpu
    pos = normal(n, 500 + n)
    mass = masses(n, 500 + n, "lognormal")
    for eps in (0.01, 0.0):
        ref = oracle.direct_fp64(pos, mass, eps, 1.0)
        for algo in (nb.BRUTE_FORCE_GLOBAL, nb.BRUTE_FORCE_LOCAL):
            with nb.Simulation(num_of_bodies=n, algo_config=algo, epsilon=eps, gravitational_constant=1.0) as sim:
                sim.set_state(pos, mass)
                sim.step(0.0, 1)
                acc = sim.get_state()[2]
            if n == 1:
                assert np.array_equal(acc, np.zeros((1, 3), np.float32)), (algo, eps, acc)
            else:
                assert rel_to_typical(acc, ref) < 1e-5, (algo, eps)
        for quad in (0, 1):
            for comp in (0, 1):
                want, _, _ = oracle.bh_step_forces(pos, mass, 0.5, eps, 1.0, quadrupole=bool(quad),
                                                   compensated=bool(comp))
                with bh_sim(nb, pos, mass, 0.5, eps, quad=quad, precision=comp) as sim:
                    sim.step(0.0, 1)
                    acc = sim.get_state()[2]
                if n == 1:
                    assert np.array_equal(acc, np.zeros((1, 3), np.float32)), (quad, comp, eps, acc)
                else:
                    assert rel_to_typical(acc, want) < 2e-5, (quad, comp, eps)
    if n == 1:
        vel = np.array([[0.5, -0.25, 2.0]], np.float32)
        with bh_sim(nb, pos, mass, 0.5, 0.01, vel=vel) as sim:
            sim.step(np.float32(0.125), 4)
            p = sim.get_state()[0]
        want = pos.copy()
        for _ in range(4):
            want = (want + vel * np.float32(0.125)).astype(np.float32)
        assert np.array_equal(p, want)


@pytest.mark.parametrize("eps", [0.01, 0.0])
def test_theta_zero_opens_every_cell(gpu, oracle, eps):
    """theta = 0 accepts no cell, so the walk reaches every body: the
    accelerations equal the FP64 direct sum to FP32 rounding (with eps = 0
    the self pair is skipped)."""
    nb = gpu
    n = 4000
    pos = ball(n, 21)
    mass = masses(n, 21, "lognormal")
    sim = bh_sim(nb, pos, mass, 0.0, eps)
    sim.step(0.0, 1)
    acc = sim.get_state()[2]
    sim.close()
    ref = oracle.direct_fp64(pos, mass, eps, 1.0)
    rel = np.linalg.norm(acc - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert np.sqrt(np.mean(rel ** 2)) < 2e-5 and np.max(rel) < 2e-3
