"""Batched systems (nb_batch_*) against standalone handles and the oracle.

A batched Barnes-Hut system runs the same per-item device code as a
standalone handle on the same bounding box, so its trajectory must be
bit-identical to nb_step's.  A batched direct-sum system uses another tile
order than the standalone tiled kernel, so it is compared within FP32
summation-order tolerance, and against the oracle's FP32 direct sum.
"""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def normal(n, seed, sigma=(1.0, 1.0, 0.2)):
    rng = np.random.default_rng(seed)
    return (rng.normal(size=(n, 3)) * np.asarray(sigma)).astype(np.float32)


def lognormal_mass(n, seed):
    rng = np.random.default_rng(seed + 7)
    m = np.exp(0.5 * rng.normal(size=n))
    return (m / m.sum()).astype(np.float32)


def small_vel(n, seed):
    rng = np.random.default_rng(seed + 13)
    return (0.05 * rng.normal(size=(n, 3))).astype(np.float32)


def cfg(nb, n, bh, method=2, precision=0, quad=0, theta=0.5, eps=0.01, cap=0):
    return nb.default_config(num_of_bodies=n, algo_config=nb.BARNES_HUT if bh else nb.BRUTE_FORCE_LOCAL,
                             theta=theta, epsilon=eps, direct_epsilon=eps, gravitational_constant=1.0,
                             numerical_method=method, precision=precision, multipole=quad, cell_capacity=cap)


def standalone(nb, c, pos, mass, vel, dt, steps):
    with nb.Simulation(c) as s:
        s.set_state(pos, mass, vel)
        s.step(dt, steps)
        return s.get_state()


SIZES = [(3000, True), (777, False), (20000, True), (100, False), (4096, False), (1, True), (9001, True),
         (31, False)]


@pytest.mark.parametrize("method,precision,quad", [(2, 0, 0), (3, 1, 1), (1, 0, 1)])
def test_mixed_batch_matches_standalone(gpu, method, precision, quad):
    nb = gpu
    cfgs = [cfg(nb, n, bh, method, precision, quad) for n, bh in SIZES]
    states = [(normal(n, 100 + k), lognormal_mass(n, 100 + k), small_vel(n, 100 + k))
              for k, (n, _) in enumerate(SIZES)]
    dt, steps = 1e-3, 3
    with nb.Batch(cfgs) as b:
        for k, (p, m, v) in enumerate(states):
            b.set_state(k, p, m, v)
        b.step(dt, 2)
        b.step(dt, 1)  # a second call replays the same graph
        info = b.info()
        assert info["systems"] == len(SIZES)
        assert info["tree_systems"] == sum(1 for _, bh in SIZES if bh)
        # reset bbox top-count top-cells build used summarize sort force direct flip
        assert info["launches_per_step"] == 11
        for k, ((n, bh), (p, m, v)) in enumerate(zip(SIZES, states)):
            got = b.get_state(k)
            ref = standalone(nb, cfgs[k], p, m, v, dt, steps)
            np.testing.assert_array_equal(got[3], m)
            if bh:
                for a, r, what in zip(got[:3], ref[:3], ("pos", "vel", "acc")):
                    np.testing.assert_array_equal(a, r, err_msg=f"system {k} (BH n={n}) {what}")
            else:
                # FP32 sums of n terms in another order: |delta a| <= ~n ulp of
                # the largest terms; positions move by dt^2 * that
                scale = np.sqrt(np.mean(np.sum(ref[2].astype(np.float64) ** 2, axis=1))) + 1e-30
                assert np.max(np.abs(got[2] - ref[2])) / scale < 1e-4, f"system {k} acc"
                np.testing.assert_allclose(got[0], ref[0], rtol=0, atol=1e-6)
                np.testing.assert_allclose(got[1], ref[1], rtol=0, atol=1e-5)


def test_large_trees_match_standalone(gpu):
    """Systems large enough for top levels: a batched tree builds at most 4
    of them, a standalone 2^20-body tree 5; the cell numbering differs, the
    trees and every result bit do not."""
    nb = gpu
    sizes = [1 << 20, 200000, 70000]
    cfgs = [cfg(nb, n, True, quad=1) for n in sizes]
    states = [(normal(n, 300 + k), lognormal_mass(n, 300 + k), small_vel(n, 300 + k)) for k, n in enumerate(sizes)]
    dt, steps = 1e-3, 2
    with nb.Batch(cfgs) as b:
        for k, (p, m, v) in enumerate(states):
            b.set_state(k, p, m, v)
        b.step(dt, steps)
        for k, (p, m, v) in enumerate(states):
            got = b.get_state(k)
            ref = standalone(nb, cfgs[k], p, m, v, dt, steps)
            for a, r, what in zip(got[:3], ref[:3], ("pos", "vel", "acc")):
                np.testing.assert_array_equal(a, r, err_msg=f"system {k} (n={sizes[k]}) {what}")


def test_reference_tree_semantics_match_standalone(gpu):
    """Batched trees with the reference's tree and opening semantics (the
    insertions start at the root; no top levels) against standalone handles
    with the same settings, bit for bit, beside a default-semantics tree."""
    nb = gpu
    sizes = [(30000, 1), (50000, 0), (9001, 1)]
    cfgs = []
    for n, ref in sizes:
        c = cfg(nb, n, True)
        c.tree_semantics = ref
        c.theta_semantics = ref
        cfgs.append(c)
    states = [(normal(n, 500 + k), lognormal_mass(n, 500 + k), small_vel(n, 500 + k))
              for k, (n, _) in enumerate(sizes)]
    dt, steps = 1e-3, 3
    with nb.Batch(cfgs) as b:
        for k, (p, m, v) in enumerate(states):
            b.set_state(k, p, m, v)
        b.step(dt, steps)
        for k, (p, m, v) in enumerate(states):
            got = b.get_state(k)
            ref = standalone(nb, cfgs[k], p, m, v, dt, steps)
            for a, r, what in zip(got[:3], ref[:3], ("pos", "vel", "acc")):
                np.testing.assert_array_equal(a, r, err_msg=f"system {k} {what}")


def test_collision_in_a_batch_matches_standalone(gpu, oracle):
    """Systems with collision = 1 in a batch run the same collision update as
    a standalone handle after their integration: tree systems (gravity on)
    and direct systems (gravity off, so both paths integrate the same
    positions) equal nb_step on standalone handles bit for bit, next to a
    system without collisions; the direct system also equals the oracle's
    integrate-then-collide."""
    nb = gpu
    specs = [(20000, True, 1.0, 0.08), (3000, False, 0.0, 0.03), (9001, True, 1.0, 0.05), (40000, False, 0.0, 0.1),
             (5000, True, 1.0, 0.05)]
    cfgs, states = [], []
    for k, (n, bh, G, sigma) in enumerate(specs):
        c = cfg(nb, n, bh)
        c.gravitational_constant = G
        c.collision = 0 if k == 4 else 1
        cfgs.append(c)
        states.append((normal(n, 900 + k, (sigma, sigma, sigma)), lognormal_mass(n, 900 + k),
                       (10 * small_vel(n, 900 + k)).astype(np.float32)))
    dt, steps = 1e-3, 3
    with nb.Batch(cfgs) as b:
        for k, (p, m, v) in enumerate(states):
            b.set_state(k, p, m, v)
        b.step(dt, steps)
        got = [b.get_state(k) for k in range(len(cfgs))]
    for k, (p, m, v) in enumerate(states):
        ref = standalone(nb, cfgs[k], p, m, v, dt, steps)
        for a, r, what in zip(got[k][:2], ref[:2], ("pos", "vel")):
            np.testing.assert_array_equal(a, r, err_msg=f"system {k} {what}")
    # the direct system without gravity against the oracle, step by step
    p, m, v = states[1]
    x, u, a = p.copy(), v.copy(), np.zeros_like(p)
    moved = False
    for _ in range(steps):
        x, u, a = oracle.integrate(oracle.EULER, x, u, np.zeros_like(x), a, dt)
        u2 = oracle.collision(x, u)
        moved |= bool(np.any(u2 != u))
        u = u2
    assert moved  # contacts happened
    np.testing.assert_array_equal(got[1][0], x)
    np.testing.assert_array_equal(got[1][1], u)


def test_direct_systems_against_oracle(gpu, oracle):
    nb = gpu
    sizes = [257, 1000, 2048, 5]
    eps = 0.02
    cfgs = [cfg(nb, n, False, 2, eps=eps) for n in sizes]
    states = [(normal(n, 7 * n, (1, 1, 1)), lognormal_mass(n, n)) for n in sizes]
    with nb.Batch(cfgs) as b:
        for k, (p, m) in enumerate(states):
            b.set_state(k, p, m)
        b.step(0.0, 1)  # dt = 0: accelerations only
        for k, (p, m) in enumerate(states):
            acc = b.get_state(k)[2]
            ref = oracle.direct_fp64(p, m, eps, 1.0)
            scale = np.sqrt(np.mean(np.sum(ref ** 2, axis=1)))
            err = np.max(np.linalg.norm(acc - ref, axis=1)) / scale
            assert err < 2e-5, f"system {k}: {err}"
            np.testing.assert_array_equal(b.get_state(k)[0], p)  # dt = 0 leaves positions


def test_failed_system_is_isolated(gpu):
    """A system whose tree overflows its cells reports the status and keeps its
    state; the systems beside it advance exactly as alone."""
    nb = gpu
    sizes = [5000, 5000, 3000]
    cfgs = [cfg(nb, 5000, True), cfg(nb, 5000, True, cap=64), cfg(nb, 3000, False)]
    states = [(normal(n, 50 + k), lognormal_mass(n, 50 + k), small_vel(n, 50 + k)) for k, n in enumerate(sizes)]
    with nb.Batch(cfgs) as b:
        for k, (p, m, v) in enumerate(states):
            b.set_state(k, p, m, v)
        st = b.step(1e-3, 2, check=False)
        assert st == 4  # NB_ERR_CELL_OVERFLOW
        assert b.system_status(1) == 4
        assert b.system_status(0) == 0 and b.system_status(2) == 0
        p1, v1, _, _ = b.get_state(1)
        np.testing.assert_array_equal(p1, states[1][0])
        np.testing.assert_array_equal(v1, states[1][2])
        ref0 = standalone(nb, cfgs[0], *states[0], 1e-3, 2)
        np.testing.assert_array_equal(b.get_state(0)[0], ref0[0])


def test_autotune_cache_and_unchanged_state(gpu, tmp_path):
    nb = gpu
    sizes = [512, 1500, 4000, 64, 9000]
    cfgs = [cfg(nb, n, False, 3) for n in sizes]
    states = [(normal(n, n), lognormal_mass(n, n), small_vel(n, n)) for n in sizes]
    cache = tmp_path / "tune.json"

    def run(tune):
        with nb.Batch(cfgs) as b:
            for k, (p, m, v) in enumerate(states):
                b.set_state(k, p, m, v)
            b.step(1e-3, 1)
            chosen = b.autotune(str(cache)) if tune else None
            b.step(1e-3, 2)
            return chosen, b.info()["direct_variant"], [b.get_state(k) for k in range(len(sizes))]

    chosen, variant, tuned = run(True)
    assert 0 <= chosen < 11 and variant == chosen
    table = json.loads(cache.read_text())
    assert list(table.values()) == [chosen]
    chosen2, _, again = run(True)  # read back from the cache
    assert chosen2 == chosen
    for a, r in zip(tuned, again):
        for x, y in zip(a, r):
            np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("method,precision,quad", [(3, 0, 0), (2, 1, 1)])
def test_autotune_tree_shapes(gpu, tmp_path, method, precision, quad):
    """The tree stages' launch shapes (force warps per block, force grid,
    build chunk, top-level cap) are timed on the batch with dt = 0: the
    state is bit for bit the same after tuning, the choice is one of the
    candidates and is read back from the cache, and a tuned batch steps its
    tree systems exactly as an untuned batch and as standalone handles (no
    shape changes a result)."""
    nb = gpu
    specs = [(20000, True), (3000, False), (70000, True), (9001, True), (140000, True)]
    cfgs = [cfg(nb, n, bh, method, precision, quad) for n, bh in specs]
    states = [(normal(n, 300 + k), lognormal_mass(n, 300 + k), small_vel(n, 300 + k))
              for k, (n, _) in enumerate(specs)]
    cache = tmp_path / "tune.json"
    dt = 1e-3

    def run(tune):
        with nb.Batch(cfgs) as b:
            for k, (p, m, v) in enumerate(states):
                b.set_state(k, p, m, v)
            b.step(dt, 1)
            before = [b.get_state(k) for k in range(len(specs))]
            shape = None
            if tune:
                b.autotune(str(cache))
                shape = b.tree_shape()
                after = [b.get_state(k) for k in range(len(specs))]
                for k, (x, y) in enumerate(zip(before, after)):
                    for u, w, what in zip(x, y, ("pos", "vel", "acc", "mass")):
                        np.testing.assert_array_equal(u, w, err_msg=f"tuning changed system {k} {what}")
            b.step(dt, 2)
            return shape, [b.get_state(k) for k in range(len(specs))]

    shape, tuned = run(True)
    assert shape["force_warps"] in (2, 4, 8) and shape["force_grid_pct"] in (100, 75, 50)
    assert shape["build_chunk"] in (0, 1024, 2048, 4096) and shape["top_levels"] in (0, 2, 3, 4)
    table = json.loads(cache.read_text())
    assert any(k.startswith("batch_tree/") for k in table) and any(k.startswith("batch_direct/") for k in table)
    shape2, again = run(True)  # read back from the cache
    assert shape2 == shape
    _, plain = run(False)
    for k, (n, bh) in enumerate(specs):
        if not bh:
            continue
        ref = standalone(nb, cfgs[k], *states[k], dt, 3)
        for a, b_, r, what in zip(tuned[k][:3], plain[k][:3], ref[:3], ("pos", "vel", "acc")):
            np.testing.assert_array_equal(a, b_, err_msg=f"system {k} {what}: tuned vs untuned batch")
            np.testing.assert_array_equal(a, r, err_msg=f"system {k} {what}: tuned batch vs standalone")
        for x, y in zip(tuned[k], again[k]):
            np.testing.assert_array_equal(x, y)


def test_batch_rejects_mixed_settings(gpu):
    nb = gpu
    with pytest.raises(nb.NbError) as e:
        nb.Batch([cfg(nb, 100, True, 2), cfg(nb, 100, True, 3)])
    assert e.value.status == 10  # NB_ERR_UNSUPPORTED
    with pytest.raises(nb.NbError):
        nb.Batch([cfg(nb, 100, False, eps=0.0)])
    with pytest.raises(nb.NbError):
        nb.Batch([])


def test_many_small_systems(gpu):
    """512 systems of 256..4096 bodies: every BH system bit-identical to its
    standalone run (checked on a sample), energy-like sanity on all."""
    nb = gpu
    rng = np.random.default_rng(3)
    sizes = [int(x) for x in rng.integers(256, 4097, size=512)]
    cfgs = [cfg(nb, n, k % 2 == 0) for k, n in enumerate(sizes)]
    states = [(normal(n, 1000 + k), lognormal_mass(n, 1000 + k), small_vel(n, 1000 + k))
              for k, n in enumerate(sizes)]
    with nb.Batch(cfgs) as b:
        for k, (p, m, v) in enumerate(states):
            b.set_state(k, p, m, v)
        b.step(1e-3, 3)
        for k in (0, 2, 100, 510):
            ref = standalone(nb, cfgs[k], *states[k], 1e-3, 3)
            np.testing.assert_array_equal(b.get_state(k)[0], ref[0])
        for k in range(len(sizes)):
            p = b.get_state(k)[0]
            assert np.all(np.isfinite(p))
            assert np.max(np.abs(p - states[k][0])) < 0.05


def test_more_systems_than_one_scan_block(gpu):
    """1100 tree systems: the used-cell scan runs over more systems than its
    1024 threads (two chunks with a carry); every system equals its
    standalone step (checked on a sample that spans both chunks)."""
    nb = gpu
    rng = np.random.default_rng(11)
    sizes = [int(x) for x in rng.integers(64, 600, size=1100)]
    cfgs = [cfg(nb, n, True) for n in sizes]
    states = [(normal(n, 3000 + k), lognormal_mass(n, 3000 + k), small_vel(n, 3000 + k))
              for k, n in enumerate(sizes)]
    with nb.Batch(cfgs) as b:
        for k, (p, m, v) in enumerate(states):
            b.set_state(k, p, m, v)
        b.step(1e-3, 2)
        for k in (0, 1023, 1024, 1099):
            ref = standalone(nb, cfgs[k], *states[k], 1e-3, 2)
            np.testing.assert_array_equal(b.get_state(k)[0], ref[0])
            np.testing.assert_array_equal(b.get_state(k)[1], ref[1])
