"""The oracle's parallel whole step (oracle/nbpipeline.c), the timed CPU
baseline, against the sequential restatement: same tree (octant paths), same
sort, bit-identical accelerations and Euler update; and its seeded initial
conditions against the library's generator (same bytes)."""
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("n,seed", [(100_000, 0), (4097, 3)])
def test_generated_ic_matches_the_library(oracle, nbgb_lib, n, seed):
    nb, O = nbgb_lib, oracle
    cfg = nb.default_config(num_of_bodies=n, pos_config=nb.NORMAL_SIGMA_POS, pos_sigma=(1.0, 1.0, 0.2),
                            mass_config=nb.MASS_LOGNORMAL, mass_lognormal_sigma=0.5, vel_config=nb.FUNC_ZERO_VEL,
                            seed=seed)
    p_lib, _, m_lib = nb.generate_ic(cfg)
    p_orc, m_orc = O.generate_ic(n, seed, O.POS_NORMAL_SIGMA, (1.0, 1.0, 0.2), mass_mode=O.MASS_LOGNORMAL,
                                 mass_sigma=0.5)
    assert np.array_equal(p_lib, p_orc) and np.array_equal(m_lib, m_orc)
    cfg = nb.default_config(num_of_bodies=n, pos_config=nb.UNIFORM_POS, starting_volume_radius=1.5,
                            mass_config=nb.MASS_EQUAL, seed=seed)
    p_lib, _, m_lib = nb.generate_ic(cfg)
    p_orc, m_orc = O.generate_ic(n, seed, O.POS_UNIFORM, radius=1.5, mass_mode=O.MASS_EQUAL)
    assert np.array_equal(p_lib, p_orc) and np.array_equal(m_lib, m_orc)


@pytest.mark.parametrize("n", [3000, 60_000])
def test_parallel_step_equals_the_sequential_oracle(oracle, n):
    O = oracle
    pos, mass = O.generate_ic(n, 11, O.POS_NORMAL_SIGMA, (1.0, 1.0, 0.2), mass_mode=O.MASS_LOGNORMAL,
                              mass_sigma=0.5)
    vel = np.zeros_like(pos)
    acc = np.zeros_like(pos)
    pipe = O.Pipeline(n)
    theta, eps, G, dt = 0.5, 0.005, 1.0, 1e-3
    x0, v0 = pos.copy(), vel.copy()
    for step in range(2):  # the second step reuses every buffer of the first
        pipe.step(pos, vel, acc, mass, theta, eps, G, dt, quadrupole=True, compensated=True)
        a_ref, t, srt_ref = O.bh_step_forces(x0, mass, theta, eps, G, compensated=True, quadrupole=True,
                                             nodes=2 * n)
        children, srt, bottom, _ = pipe.export()
        assert np.array_equal(srt, srt_ref), step
        assert np.array_equal(acc, a_ref), step
        assert t.root - t.bottom == n + 2 * n - bottom  # same number of cells
        pg, dg, fg = O.tree_paths(children, n, n + 2 * n)
        po, do, fo = O.tree_paths(t.children, n, t.root)
        assert fg == fo == n and np.array_equal(pg, po) and np.array_equal(dg, do)
        x0, v0, _ = O.integrate(O.EULER, x0, v0, a_ref, np.zeros_like(x0), dt)
        assert np.array_equal(pos, x0) and np.array_equal(vel, v0), step
    pipe.close()


def test_parallel_step_monopole_fp32_equals_the_sequential_oracle(oracle):
    O = oracle
    n = 20_000
    pos, mass = O.generate_ic(n, 5, O.POS_UNIFORM, radius=1.0, mass_mode=O.MASS_EQUAL)
    vel, acc = np.zeros_like(pos), np.zeros_like(pos)
    x0 = pos.copy()
    pipe = O.Pipeline(n)
    pipe.step(pos, vel, acc, mass, 0.7, 0.01, 1.0, 1e-3, quadrupole=False, compensated=False)
    a_ref, _, _ = O.bh_step_forces(x0, mass, 0.7, 0.01, 1.0, nodes=2 * n)
    assert np.array_equal(acc, a_ref)
    assert pipe.stats.sum() > n  # interaction counters filled


def test_parallel_step_reports_coincident_bodies(oracle):
    O = oracle
    n = 5000
    pos, mass = O.generate_ic(n, 1, O.POS_UNIFORM, radius=1.0, mass_mode=O.MASS_EQUAL)
    pos[7] = pos[8]  # two bodies at one point never part: the depth limit ends the build
    pipe = O.Pipeline(n)
    with pytest.raises(RuntimeError):
        pipe.step(pos, np.zeros_like(pos), np.zeros_like(pos), mass, 0.5, 0.01, 1.0, 1e-3)


def test_reference_arm_runs_without_the_gpu_library(oracle):
    """bench.py --impl reference: whole steps on the CPU, the config of the
    GPU arm, and libnbgb.so never mapped into the process."""
    code = (
        "import sys, json; sys.argv = ['bench.py', '--impl', 'reference', '--n', '4096', '--steps', '1', "
        "'--warmup', '3']; sys.path.insert(0, %r); import bench; bench.main(); "
        "maps = open('/proc/self/maps').read(); print('LIBNBGB' if 'libnbgb' in maps else 'CLEAN')" % ROOT)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    assert lines[-1] == "CLEAN"
    import json
    sys.path.insert(0, ROOT)
    import bench
    line = json.loads(lines[-2])
    assert line["impl"] == "reference" and line["steps"] == 1 and line["warmup"] == 3
    assert line["config"] == bench.step_config(4096, 1)
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert abs(line["ms_per_step"] - 1e3 * 4096 / line["value"]) < 1e-6 * line["ms_per_step"]
