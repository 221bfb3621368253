"""The oracle against the reference's own kernels run live by the emulator
(oracle/_ref, built from the reference sources).  Skips where the sources
are absent."""
import numpy as np
import pytest

from oracle import refemu

pytestmark = pytest.mark.skipif(not refemu.available(), reason="reference sources not present")


def bodies(n, seed, scale=1.0):
    rng = np.random.default_rng(seed)
    pos = (rng.normal(size=(n, 3)) * scale).astype(np.float32)
    mass = (np.abs(rng.normal(0.5, 0.25, n)) + 1e-3).astype(np.float32)
    return pos, mass


@pytest.mark.parametrize("n,seed,wg", [(200, 11, 16), (777, 12, 64), (1500, 13, 256)])
def test_tree_and_bbox_live(oracle, n, seed, wg):
    pos, mass = bodies(n, seed)
    rs = refemu.RefSim(n, wg)
    rs.set_bodies(pos.ravel(), mass)
    if n >= 2 * wg:
        assert np.array_equal(rs.bbox_as_wired(), oracle.bbox_sampled(rs.get(rs.POS, np.float32), wg))
    box = oracle.bbox_exact(pos)
    rs.set_boundary(box)
    rs.init()
    rs.build_tree()
    t = oracle.tree_build(oracle.SEM_REFERENCE, pos, mass, box, rs.nodes)
    pr, dr, _ = oracle.tree_paths(rs.get(rs.CHILDREN, np.int32), n, n + rs.nodes)
    po, do, _ = oracle.tree_paths(t.children, n, t.root)
    assert np.array_equal(pr, po) and np.array_equal(dr, do)
    assert int(rs.get(rs.MAX_DEPTH, np.int32)[0]) == t.max_depth


@pytest.mark.parametrize("theta,eps", [(0.5, 0.01), (0.9, 0.02)])
def test_bh_force_live_bit_exact(oracle, theta, eps):
    n = 320
    pos, mass = bodies(n, 21)
    box = oracle.bbox_exact(pos)
    rs = refemu.RefSim(n, 16)
    rs.set_bodies(pos.ravel(), mass)
    rs.set_boundary(box)
    rs.init()
    rs.build_tree()
    rs.saturate_tree()
    t = oracle.Tree(n, rs.nodes)
    t.pos[:] = rs.get(rs.POS, np.float32)
    t.mass[:] = rs.get(rs.MASS, np.float32)
    t.children[:] = rs.get(rs.CHILDREN, np.int32)
    md = int(rs.get(rs.MAX_DEPTH, np.int32)[0])
    want = rs.accelerations_via_leapfrog(theta, eps, 1.0, "bh")
    dq = oracle.thresholds(oracle.CRIT_REFERENCE, box, theta, eps, md)
    got, _ = oracle.bh_force(t, dq, eps, 1.0, arith=oracle.ARITH_REFERENCE, vote_width=16, skip_self=False)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("n,wg", [(256, 16), (512, 256)])
def test_direct_and_collision_live(oracle, n, wg):
    pos, mass = bodies(n, 31)
    rs = refemu.RefSim(n, wg)
    rs.set_bodies(pos.ravel(), mass)
    assert np.array_equal(rs.accelerations_via_leapfrog(0, 0, 1.0, "global"),
                          oracle.direct_quirk_global(pos, mass, 1.0))
    rs.set_bodies(pos.ravel(), mass)
    assert np.array_equal(rs.accelerations_via_leapfrog(0, 0, 1.0, "local"),
                          oracle.direct_quirk_local(pos, mass, 1.0, wg=wg, tile_schedule=True))
    cpos, _ = bodies(n, 32, scale=0.05)
    vel = (np.random.default_rng(3).normal(size=(n, 3)) * 0.1).astype(np.float32)
    rs.set_bodies(cpos.ravel(), mass, vel.ravel(), None)
    rs.collision()
    assert np.array_equal(rs.get(rs.VEL, np.float32).reshape(n, 3), oracle.collision(cpos, vel, wg=wg, tile_schedule=True))
