"""Parity at the benchmarked sizes and the FP64 diagnostics.

* The 4,194,304-body precision workload (normal positions sigma = (1, 1,
  0.2), lognormal masses, theta = 0.5, eps = 0.005, quadrupoles, compensated
  sums): bounding box, tree in octant-path form, cell masses / centres /
  body counts and the sort permutation bit-exact against the oracle's build
  (kernels/build_tree.cl:42-161, kernels/saturate_tree.cl:39-145);
  accelerations of 8192 bodies (256 whole warp groups) within 2e-5 of the
  oracle's walk on the same tree (kernels/calculate_forces.cl:84-147), and
  their RMS error against an FP64 direct sum at most 1e-3.
* The plain Barnes-Hut configuration, 262,144 bodies in the unit ball with
  circular velocities about z, 50 Euler steps against the oracle's 50 steps
  (positions within 1e-5 of their spread), and the tiled direct sum on the
  same bodies.
* nb_diagnostics against an FP64 numpy computation on the same state, and
  conservation of momentum over direct-sum steps.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HEADLINE = dict(n=4194304, theta=0.5, eps=0.005, sigma=(1.0, 1.0, 0.2))


def rel_to_typical(a, b):
    scale = np.sqrt(np.mean(np.sum(np.asarray(b, np.float64) ** 2, axis=1)))
    return float(np.max(np.linalg.norm(np.asarray(a, np.float64) - b, axis=1)) / scale)


def bfs_cells(children, n, root):
    """Cells in breadth-first order, children in slot order: the same
    sequence for two trees of one topology in octant-slot form."""
    ch = children.reshape(-1, 8)
    front = np.array([root], np.int64)
    out = [front]
    while len(front):
        c = ch[front].ravel()
        front = c[c >= n].astype(np.int64)
        out.append(front)
    return np.concatenate(out)


def test_headline_4m_against_the_oracle(gpu, oracle):
    nb, O = gpu, oracle
    n, theta, eps = HEADLINE["n"], HEADLINE["theta"], HEADLINE["eps"]
    cfg = nb.default_config(num_of_bodies=n, pos_config=nb.NORMAL_SIGMA_POS, pos_sigma=HEADLINE["sigma"],
                            mass_config=nb.MASS_LOGNORMAL, mass_lognormal_sigma=0.5, vel_config=nb.FUNC_ZERO_VEL,
                            seed=0)
    pos, _, mass = nb.generate_ic(cfg)
    sim = nb.Simulation(num_of_bodies=n, algo_config=nb.BARNES_HUT, theta=theta, epsilon=eps,
                        gravitational_constant=1.0, numerical_method=nb.EULER, precision=nb.PRECISION_COMPENSATED,
                        multipole=nb.MULTIPOLE_QUADRUPOLE)
    sim.set_state(pos, mass)
    sim.step(0.0, 1)
    box = sim.stage_debug(nb.DEBUG_BBOX)
    info = sim.stage_debug(nb.DEBUG_TREE_INFO)
    cap = int(info[1])
    children = sim.stage_debug(nb.DEBUG_CHILDREN)
    mg, xg, cg = (sim.stage_debug(nb.DEBUG_NODE_MASS), sim.stage_debug(nb.DEBUG_NODE_POS),
                  sim.stage_debug(nb.DEBUG_BODY_COUNT))
    srt_g = sim.stage_debug(nb.DEBUG_SORTED)
    acc_g = sim.get_state()[2]
    sim.close()

    # bounding box and tree, bit-exact
    assert np.array_equal(box, O.bbox_exact(pos))
    t = O.tree_build(O.SEM_GEOMETRIC, pos, mass, box, cap)
    assert t.status == 0
    assert int(info[2]) == t.bottom and int(info[3]) == t.max_depth
    pg, dg, fg = O.tree_paths(children, n, n + cap)
    po, do, fo = O.tree_paths(t.children, n, t.root)
    assert fg == fo == n
    assert np.array_equal(dg, do) and np.array_equal(pg, po)
    del pg, po
    # cell summaries, bit-exact, cells matched by their place in the tree
    octant = t.children.copy()
    assert O.saturate(t) == 0
    cells_g, cells_o = bfs_cells(children, n, n + cap), bfs_cells(octant, n, t.root)
    assert len(cells_g) == len(cells_o) == t.root - t.bottom + 1
    assert np.array_equal(mg[cells_g], t.mass[cells_o])
    assert np.array_equal(xg.reshape(-1, 3)[cells_g], t.pos.reshape(-1, 3)[cells_o])
    assert np.array_equal(cg[cells_g], t.body_count[cells_o])
    del octant, children
    # sort permutation, bit-exact
    srt_o, k = O.sort_bodies(t.children, n, t.root)
    assert k == n and np.array_equal(srt_g, srt_o)
    # accelerations of 256 whole warp groups (the GPU's vote groups): the
    # oracle walks the same groups of the same tree
    groups = np.linspace(0, n // 32 - 1, 256).astype(np.int64)
    order = srt_o[(groups[:, None] * 32 + np.arange(32)[None, :]).ravel()]
    dq = O.thresholds(O.CRIT_STANDARD, box, theta, eps, t.max_depth)
    acc_o, rc = O.bh_force(t, dq, eps, 1.0, vote_width=32, order=order, compensated=True, quad=O.quadrupoles(t))
    assert rc == 0
    err = rel_to_typical(acc_g[order], acc_o[order])
    assert err < 2e-5, err
    # accuracy against the FP64 direct sum on those 8192 bodies
    a64 = O.direct_fp64(pos, mass, eps, 1.0, targets=order)
    rel = np.linalg.norm(acc_g[order] - a64, axis=1) / np.linalg.norm(a64, axis=1)
    rms = float(np.sqrt(np.mean(rel ** 2)))
    assert rms <= 1e-3, rms


BALL = dict(n=262144, theta=0.5, eps=0.01, dt=1e-3, steps=50)


def ball_state(nb, n):
    cfg = nb.default_config(num_of_bodies=n, pos_config=nb.BALL_POS, starting_volume_radius=1.0,
                            vel_config=nb.CIRCULAR_Z_VEL, mass_config=nb.MASS_EQUAL, gravitational_constant=1.0,
                            seed=0)
    return nb.generate_ic(cfg)


def test_ball_262k_50_steps_against_the_oracle(gpu, oracle):
    """The plain Barnes-Hut configuration for its 50 steps (monopole, FP32,
    Euler) on the GPU and in the oracle (its parallel whole step, equal to
    the sequential restatement bit for bit): positions within 1e-5 of their
    spread, velocities within 1e-4 of theirs.  The two runs part only by the
    GPU's rsqrt and summation order (about 1e-7 of |a| per step)."""
    nb, O = gpu, oracle
    n = BALL["n"]
    pos, vel, mass = ball_state(nb, n)
    sim = nb.Simulation(num_of_bodies=n, algo_config=nb.BARNES_HUT, theta=BALL["theta"], epsilon=BALL["eps"],
                        gravitational_constant=1.0, numerical_method=nb.EULER)
    sim.set_state(pos, mass, vel)
    sim.step(BALL["dt"], BALL["steps"])
    pg, vg, _, _ = sim.get_state()
    sim.close()
    p, v, a = pos.copy(), vel.copy(), np.zeros_like(pos)
    pipe = O.Pipeline(n)
    for _ in range(BALL["steps"]):
        pipe.step(p, v, a, mass, BALL["theta"], BALL["eps"], 1.0, BALL["dt"], quadrupole=False, compensated=False)
    pipe.close()
    assert np.max(np.abs(pg - p)) < 1e-5 * np.std(p)
    assert np.max(np.abs(vg - v)) < 1e-4 * np.std(v)
    assert np.max(np.abs(p - pos)) > 100 * 1e-5 * np.std(p)  # the bodies did move


def test_ball_262k_tiled_direct_against_the_oracle(gpu, oracle):
    """The tiled direct sum on the same 262,144 bodies, first and last 2048
    targets.  Sums of 262,144 FP32 terms in two orders each sit about 3e-5 of
    the typical |a| from the FP64 sum, so the GPU is held to: within 1e-4 of
    the oracle's FP32 sum, and no further from the FP64 sum than 1.5 times
    the oracle's own FP32 error."""
    nb, O = gpu, oracle
    n = BALL["n"]
    pos, vel, mass = ball_state(nb, n)
    sim = nb.Simulation(num_of_bodies=n, algo_config=nb.BRUTE_FORCE_LOCAL, epsilon=BALL["eps"],
                        direct_epsilon=BALL["eps"], gravitational_constant=1.0)
    sim.set_state(pos, mass, vel)
    sim.step(0.0, 1)
    acc_g = sim.get_state()[2]
    sim.close()
    for i0, i1 in ((0, 2048), (n - 2048, n)):
        acc_o = O.direct_fp32(pos, mass, BALL["eps"], 1.0, i0, i1)[i0:i1]
        a64 = O.direct_fp64(pos, mass, BALL["eps"], 1.0, targets=np.arange(i0, i1, dtype=np.int32))
        err = rel_to_typical(acc_g[i0:i1], acc_o)
        assert err < 1e-4, (i0, err)
        e_gpu, e_orc = rel_to_typical(acc_g[i0:i1], a64), rel_to_typical(acc_o, a64)
        assert e_gpu <= 1.5 * e_orc, (i0, e_gpu, e_orc)


def diagnostics_fp64(pos, vel, mass, eps, G):
    x, v, m = pos.astype(np.float64), vel.astype(np.float64), mass.astype(np.float64)
    out = {"kinetic": 0.5 * np.sum(m * np.sum(v * v, axis=1)), "mass": np.sum(m)}
    p = np.sum(m[:, None] * v, axis=0)
    lmom = np.sum(m[:, None] * np.cross(x, v), axis=0)
    out.update(px=p[0], py=p[1], pz=p[2], lx=lmom[0], ly=lmom[1], lz=lmom[2])
    pe = 0.0
    n = len(m)
    for i0 in range(0, n, 512):
        d = x[i0:i0 + 512, None, :] - x[None, :, :]
        r = np.sqrt(np.sum(d * d, axis=2) + eps * eps)
        pair = m[i0:i0 + 512, None] * m[None, :] / r
        idx = np.arange(i0, min(n, i0 + 512))
        pair[idx - i0, idx] = 0.0
        pe -= 0.5 * G * np.sum(pair)
    out["potential"] = pe
    scales = {"kinetic": out["kinetic"], "mass": out["mass"], "potential": abs(pe),
              "p": np.sum(m * np.linalg.norm(v, axis=1)),
              "l": np.sum(m * np.linalg.norm(np.cross(x, v), axis=1))}
    return out, scales


@pytest.mark.parametrize("algo", ["direct", "tree"])
def test_diagnostics_match_fp64_numpy(gpu, algo):
    nb = gpu
    n, eps, G = 5000, 0.05, 0.7
    rng = np.random.default_rng(31)
    pos = (rng.normal(size=(n, 3)) * (1.0, 1.0, 0.3)).astype(np.float32)
    vel = (0.2 * rng.normal(size=(n, 3))).astype(np.float32)
    m = np.exp(0.5 * rng.normal(size=n))
    mass = (m / m.sum()).astype(np.float32)
    sim = nb.Simulation(num_of_bodies=n, algo_config=nb.BRUTE_FORCE_LOCAL if algo == "direct" else nb.BARNES_HUT,
                        epsilon=eps, direct_epsilon=eps, gravitational_constant=G)
    sim.set_state(pos, mass, vel)
    d = sim.diagnostics(with_potential=True)
    d_nopot = sim.diagnostics(with_potential=False)
    sim.close()
    # the library holds eps and G as float32 (nb_config); the FP64 sums take those values
    want, sc = diagnostics_fp64(pos, vel, mass, float(np.float32(eps)), float(np.float32(G)))
    tol = 1e-12
    for k in ("kinetic", "mass", "potential"):
        assert abs(d[k] - want[k]) <= tol * sc[k], (k, d[k], want[k])
    for k in ("px", "py", "pz"):
        assert abs(d[k] - want[k]) <= tol * sc["p"], (k, d[k], want[k])
    for k in ("lx", "ly", "lz"):
        assert abs(d[k] - want[k]) <= tol * sc["l"], (k, d[k], want[k])
    # FP64 atomics add the blocks' partial sums in arrival order: equal to rounding
    assert d_nopot["potential"] == 0.0 and abs(d_nopot["kinetic"] - d["kinetic"]) <= tol * sc["kinetic"]


def test_direct_sum_conserves_momentum(gpu):
    """Pairwise forces are antisymmetric: over 10 Euler steps of the direct
    sum from rest, linear and angular momentum stay zero to FP32 rounding of
    the accelerations (1e-5 of sum m|v| and of sum m|x cross v|), and the
    energy drifts by less than 1e-4 of itself."""
    nb = gpu
    n, eps, dt = 4096, 0.05, 1e-3
    rng = np.random.default_rng(5)
    pos = rng.normal(size=(n, 3)).astype(np.float32)
    m = np.exp(0.5 * rng.normal(size=n))
    mass = (m / m.sum()).astype(np.float32)
    sim = nb.Simulation(num_of_bodies=n, algo_config=nb.BRUTE_FORCE_LOCAL, epsilon=eps, direct_epsilon=eps,
                        gravitational_constant=1.0, numerical_method=nb.EULER)
    sim.set_state(pos, mass, np.zeros_like(pos))
    e0 = sim.diagnostics(with_potential=True)
    sim.step(dt, 10)
    d = sim.diagnostics(with_potential=True)
    x, v, _, _ = sim.get_state()
    sim.close()
    _, sc = diagnostics_fp64(x, v, mass, float(np.float32(eps)), 1.0)
    assert sc["p"] > 0
    assert np.linalg.norm([d["px"], d["py"], d["pz"]]) <= 1e-5 * sc["p"]
    assert np.linalg.norm([d["lx"], d["ly"], d["lz"]]) <= 1e-5 * sc["l"]
    E0, E1 = e0["kinetic"] + e0["potential"], d["kinetic"] + d["potential"]
    assert abs(E1 - E0) <= 1e-4 * abs(E0), (E0, E1)


def test_diagnostics_under_kdk_use_the_half_step_velocities(gpu):
    """Under the KDK leapfrog the stored velocities are v(t - dt/2) while the
    positions are at t; nb_diagnostics reports the moments of the stored
    velocities (what nb_get_state returns), to FP64 rounding."""
    nb = gpu
    n, eps = 2048, 0.05
    rng = np.random.default_rng(8)
    pos = rng.normal(size=(n, 3)).astype(np.float32)
    vel = (0.1 * rng.normal(size=(n, 3))).astype(np.float32)
    mass = np.full(n, 1.0 / n, np.float32)
    sim = nb.Simulation(num_of_bodies=n, algo_config=nb.BRUTE_FORCE_LOCAL, epsilon=eps, direct_epsilon=eps,
                        gravitational_constant=1.0, numerical_method=nb.KDK_LEAPFROG)
    sim.set_state(pos, mass, vel)
    sim.step(1e-3, 3)
    x, v, _, _ = sim.get_state()
    d = sim.diagnostics()
    sim.close()
    want, sc = diagnostics_fp64(x, v, mass, eps, 1.0)
    assert abs(d["kinetic"] - want["kinetic"]) <= 1e-12 * sc["kinetic"]
    for k in ("px", "py", "pz"):
        assert abs(d[k] - want[k]) <= 1e-12 * sc["p"]
