"""Generate the golden fixtures of tests/golden/ from the reference's OWN
kernels (kernels/*.cl of Ace-of-Heartz/NBodySimulation), run on the CPU by
the emulator in oracle/_ref (built from the reference sources by
oracle/ref/Makefile).  Needs the reference sources; the fixtures are
committed so the oracle can be checked where the sources are absent.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import oracle as O  # noqa: E402
from oracle import refemu as R  # noqa: E402


def bodies(n, seed, scale=1.0):
    rng = np.random.default_rng(seed)
    pos = (rng.normal(size=(n, 3)) * scale).astype(np.float32)
    mass = (np.abs(rng.normal(0.5, 0.25, n)) + 1e-3).astype(np.float32)
    vel = (rng.normal(size=(n, 3)) * 0.1).astype(np.float32)
    return pos, mass, vel


def tree_case(n, seed, wg, thetas):
    pos, mass, _ = bodies(n, seed)
    rs = R.RefSim(n, wg)
    rs.set_bodies(pos.ravel(), mass)
    wired = rs.bbox_as_wired()
    p_buffer = rs.get(rs.POS, np.float32).copy()
    box = O.bbox_exact(pos)
    rs.set_boundary(box)
    rs.init()
    rs.build_tree()
    built_children = rs.get(rs.CHILDREN, np.int32).copy()
    bottom = int(rs.get(rs.BOTTOM, np.int32)[0])
    max_depth = int(rs.get(rs.MAX_DEPTH, np.int32)[0])
    rs.saturate_tree()
    out = dict(pos=pos, mass=mass, wg=wg, nodes=rs.nodes, wired_box=wired, p_buffer=p_buffer[: 6 * wg],
               box=box, built_children=built_children, bottom=bottom, max_depth=max_depth,
               sat_children=rs.get(rs.CHILDREN, np.int32), sat_pos=rs.get(rs.POS, np.float32),
               sat_mass=rs.get(rs.MASS, np.float32), sat_count=rs.get(rs.BODY_COUNT, np.int32))
    accs = []
    for theta, eps in thetas:
        accs.append(rs.accelerations_via_leapfrog(theta, eps, 1.0, "bh"))
    out["thetas"] = np.array(thetas, np.float32)
    out["bh_acc"] = np.stack(accs) if accs else np.zeros((0, n, 3), np.float32)
    return out


def direct_case(n, seed, wg):
    pos, mass, vel = bodies(n, seed)
    rs = R.RefSim(n, wg)
    rs.set_bodies(pos.ravel(), mass)
    acc_global = rs.accelerations_via_leapfrog(0, 0, 1.0, "global")
    rs.set_bodies(pos.ravel(), mass)
    acc_local = rs.accelerations_via_leapfrog(0, 0, 1.0, "local")
    rs.set_bodies(pos.ravel(), mass, vel.ravel(), np.zeros((n, 3), np.float32))
    rs.update_global(1e-3, 1.0, 2)
    euler_pos = rs.get(rs.POS, np.float32)[: 3 * n].reshape(n, 3).copy()
    euler_vel = rs.get(rs.VEL, np.float32).reshape(n, 3).copy()
    cpos, _, _ = bodies(n, seed + 100, scale=0.05)
    rs.set_bodies(cpos.ravel(), mass, vel.ravel(), None)
    rs.collision()
    coll_vel = rs.get(rs.VEL, np.float32).reshape(n, 3).copy()
    verts = rs.copy_vertices()
    return dict(pos=pos, mass=mass, vel=vel, wg=wg, acc_global=acc_global, acc_local=acc_local,
                euler_pos=euler_pos, euler_vel=euler_vel, coll_pos=cpos, coll_vel=coll_vel, verts=verts)


def main():
    R.build()
    np.savez_compressed(os.path.join(HERE, "ref_tree_n256_wg16.npz"),
                        **tree_case(256, 0, 16, [(0.5, 0.01), (1.5, 0.01), (0.2, 0.05)]))
    np.savez_compressed(os.path.join(HERE, "ref_tree_n300_wg64.npz"), **tree_case(300, 3, 64, []))
    np.savez_compressed(os.path.join(HERE, "ref_direct_n256_wg16.npz"), **direct_case(256, 7, 16))
    np.savez_compressed(os.path.join(HERE, "ref_direct_n512_wg64.npz"), **direct_case(512, 8, 64))
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
