"""Job server (nb_server_*): continuous batching on the GPU.

The same job gives the same result alone and in a mix of other jobs that
arrive before, during and after it (bit-identical: every job's work is
independent of its neighbours in the batch), and tree jobs equal a
standalone handle's nb_step bit for bit.  Snapshots every k steps equal the
standalone state after that many steps.  Admission respects the slot count
and the device-memory budget.
"""
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

WAIT_S = 120.0


def normal(n, seed, sigma=(1.0, 1.0, 1.0)):
    rng = np.random.default_rng(seed)
    return (rng.normal(size=(n, 3)) * np.asarray(sigma)).astype(np.float32)


def job_state(n, seed):
    rng = np.random.default_rng(seed + 5)
    m = np.full(n, 1.0 / n, np.float32)
    return normal(n, seed), (0.05 * rng.normal(size=(n, 3))).astype(np.float32), m


def jcfg(nb, n, bh=True, theta=0.5, eps=0.01, cap=0, method=2):
    return nb.default_config(num_of_bodies=n, algo_config=nb.BARNES_HUT if bh else nb.BRUTE_FORCE_LOCAL,
                             theta=theta, epsilon=eps, direct_epsilon=eps, gravitational_constant=1.0,
                             numerical_method=method, cell_capacity=cap)


def run_alone(nb, cfg, steps, dt, state, **server_kw):
    pos, vel, mass = state
    with nb.Server(**server_kw) as srv:
        j = srv.submit(cfg, steps, dt, pos, mass, vel)
        assert srv.wait(j, WAIT_S) == 0
        return srv.result(j, cfg.num_of_bodies)


def standalone(nb, cfg, steps, dt, state):
    pos, vel, mass = state
    with nb.Simulation(cfg) as s:
        s.set_state(pos, mass, vel)
        s.step(dt, steps)
        p, v, _, _ = s.get_state()
        return p, v


def test_same_alone_and_in_mix(gpu):
    nb = gpu
    dt = 1e-3
    target_bh = (jcfg(nb, 20000, True, theta=0.6), 37, job_state(20000, 1))
    target_direct = (jcfg(nb, 3000, False), 23, job_state(3000, 2))
    alone_bh = run_alone(nb, *target_bh[:2], dt, target_bh[2])
    alone_direct = run_alone(nb, *target_direct[:2], dt, target_direct[2])

    others = [(jcfg(nb, n, bh), steps, job_state(n, 100 + k))
              for k, (n, bh, steps) in enumerate([(50000, True, 60), (1500, False, 15), (9000, True, 44),
                                                  (70000, True, 12), (4096, False, 90), (12345, True, 31)])]
    with nb.Server() as srv:
        ids = []
        for c, steps, (p, v, m) in others[:3]:
            ids.append(srv.submit(c, steps, dt, p, m, v))
        time.sleep(0.02)  # the first jobs are running when the targets arrive
        tb = srv.submit(target_bh[0], target_bh[1], dt, target_bh[2][0], target_bh[2][2], target_bh[2][1])
        for c, steps, (p, v, m) in others[3:5]:
            ids.append(srv.submit(c, steps, dt, p, m, v))
        td = srv.submit(target_direct[0], target_direct[1], dt, target_direct[2][0], target_direct[2][2],
                        target_direct[2][1])
        time.sleep(0.01)
        c, steps, (p, v, m) = others[5]
        ids.append(srv.submit(c, steps, dt, p, m, v))
        assert srv.wait(-1, WAIT_S) == 0
        mix_bh = srv.result(tb, 20000)
        mix_direct = srv.result(td, 3000)
        st = srv.stats()
        assert st["completed"] == 8 and st["failed"] == 0
        assert st["peak_jobs"] >= 2  # the jobs overlapped on the GPU
    for a, b in zip(alone_bh, mix_bh):
        np.testing.assert_array_equal(a, b)
    for a, b in zip(alone_direct, mix_direct):
        np.testing.assert_array_equal(a, b)
    # tree job: bit-identical to a standalone handle
    ref = standalone(nb, target_bh[0], target_bh[1], dt, target_bh[2])
    np.testing.assert_array_equal(mix_bh[0], ref[0])
    np.testing.assert_array_equal(mix_bh[1], ref[1])
    # direct job: the standalone tiled kernel sums in another order
    ref = standalone(nb, target_direct[0], target_direct[1], dt, target_direct[2])
    np.testing.assert_allclose(mix_direct[0], ref[0], rtol=0, atol=1e-5)


def test_collision_jobs_match_standalone(gpu):
    """Jobs with collision = 1 are served (the collision update runs in the
    batched step after their integration): a tree job equals a standalone
    handle bit for bit, alone and next to a job without collisions."""
    nb = gpu
    dt = 1e-3
    c = jcfg(nb, 12000, True)
    c.collision = 1
    pos, vel, mass = job_state(12000, 31)
    state = (0.06 * pos, 10 * vel, mass)  # dense enough for contacts
    other = jcfg(nb, 30000, True)
    with nb.Server() as srv:
        jo = srv.submit(other, 40, dt, *[job_state(30000, 32)[i] for i in (0, 2, 1)])
        j = srv.submit(c, 25, dt, state[0], state[2], state[1])
        assert srv.wait(-1, WAIT_S) == 0
        got = srv.result(j, 12000)
    ref = standalone(nb, c, 25, dt, state)
    np.testing.assert_array_equal(got[0], ref[0])
    np.testing.assert_array_equal(got[1], ref[1])
    no_coll = standalone(nb, jcfg(nb, 12000, True), 25, dt, state)
    assert np.any(no_coll[1] != ref[1])  # the collisions changed the velocities


def test_snapshots_every_k_steps(gpu):
    nb = gpu
    dt = 1e-3
    cfg = jcfg(nb, 8000, True)
    state = job_state(8000, 9)
    events = []
    lock = threading.Lock()

    def on_event(job, event, value, pos, vel):
        with lock:
            events.append((job, event, value, pos, vel))

    with nb.Server(on_event=on_event, snapshot_every=10) as srv:
        j = srv.submit(cfg, 35, dt, state[0], state[2], state[1])
        j2 = srv.submit(jcfg(nb, 2000, False), 7, dt, *[job_state(2000, 3)[i] for i in (0, 2, 1)])
        assert srv.wait(-1, WAIT_S) == 0
    mine = [e for e in events if e[0] == j]
    assert [(e[1], e[2]) for e in mine] == [(0, 10), (0, 20), (0, 30), (1, 35)]
    for ev, step, pos, _ in [(e[1], e[2], e[3], e[4]) for e in mine]:
        ref = standalone(nb, cfg, step, dt, state)
        np.testing.assert_array_equal(pos, ref[0])
    other = [e for e in events if e[0] == j2]
    assert [(e[1], e[2]) for e in other] == [(1, 7)]


def test_admission_budget_and_slots(gpu):
    nb = gpu
    dt = 1e-3
    jobs = [(jcfg(nb, n, True), 12, job_state(n, 40 + n)) for n in (30000, 20000, 25000, 18000)]
    # footprints 15.5, 10.3, 12.9 and 9.3 MB: 16 MiB holds one job at a time
    with nb.Server(hbm_budget_bytes=16 << 20) as srv:
        ids = [srv.submit(c, s, dt, p, m, v) for c, s, (p, v, m) in jobs]
        assert srv.wait(-1, WAIT_S) == 0
        st = srv.stats()
        assert st["completed"] == 4
        assert st["peak_jobs"] == 1
        assert st["peak_bytes"] <= 16 << 20
        infos = [srv.info(i) for i in ids]
        # first come first served: admitted in submission order
        admits = [i["t_admit"] for i in infos]
        assert admits == sorted(admits)
        for (c, s, state), i in zip(jobs, ids):
            np.testing.assert_array_equal(srv.result(i, c.num_of_bodies)[0], standalone(nb, c, s, dt, state)[0])
    with nb.Server(max_jobs=2) as srv:
        ids = [srv.submit(c, s, dt, p, m, v) for c, s, (p, v, m) in jobs]
        assert srv.wait(-1, WAIT_S) == 0
        assert srv.stats()["peak_jobs"] <= 2
    # a job larger than the whole budget is refused, the others run
    with nb.Server(hbm_budget_bytes=8 << 20) as srv:
        big = srv.submit(jobs[0][0], 5, dt, jobs[0][2][0], jobs[0][2][2])
        small = srv.submit(jcfg(nb, 1000, False), 5, dt, *[job_state(1000, 1)[i] for i in (0, 2, 1)])
        assert srv.wait(big, WAIT_S) == 3  # NB_ERR_OUT_OF_MEMORY
        assert srv.wait(small, WAIT_S) == 0


def test_failed_job_is_isolated(gpu):
    nb = gpu
    dt = 1e-3
    good = (jcfg(nb, 6000, True), 20, job_state(6000, 77))
    with nb.Server() as srv:
        bad = srv.submit(jcfg(nb, 6000, True, cap=32), 20, dt, *[job_state(6000, 78)[i] for i in (0, 2, 1)])
        ok = srv.submit(good[0], good[1], dt, good[2][0], good[2][2], good[2][1])
        assert srv.wait(bad, WAIT_S) == 4  # NB_ERR_CELL_OVERFLOW
        assert srv.wait(ok, WAIT_S) == 0
        np.testing.assert_array_equal(srv.result(ok, 6000)[0], standalone(nb, *good[:2], dt, good[2])[0])
        st = srv.stats()
        assert st["failed"] == 1 and st["completed"] == 1


def test_generated_initial_conditions_and_validation(gpu):
    nb = gpu
    cfg = nb.default_config(num_of_bodies=5000, algo_config=nb.BARNES_HUT, theta=0.5, epsilon=0.01,
                            gravitational_constant=1.0, pos_config=nb.BALL_POS, vel_config=nb.CIRCULAR_Z_VEL,
                            mass_config=nb.MASS_EQUAL, starting_volume_radius=1.0, seed=11)
    pos, vel, mass = nb.generate_ic(cfg)
    with nb.Server() as srv:
        j = srv.submit(cfg, 15, 1e-3)  # the server generates the same initial conditions
        assert srv.wait(j, WAIT_S) == 0
        got = srv.result(j, 5000)
        with pytest.raises(nb.NbError) as e:
            srv.submit(jcfg(nb, 100, True, method=3), 5, 1e-3)
        assert e.value.status == 10
        with pytest.raises(nb.NbError):
            srv.submit(jcfg(nb, 100, True), 0, 1e-3)
    ref = standalone(nb, cfg, 15, 1e-3, (pos, vel, mass))
    np.testing.assert_array_equal(got[0], ref[0])


def test_snapshot_file_of_a_handle_and_of_a_job(gpu, tmp_path):
    nb = gpu
    cfg = jcfg(nb, 3000, True)
    state = job_state(3000, 21)
    with nb.Simulation(cfg) as s:
        s.set_state(state[0], state[2], state[1])
        s.step(1e-3, 4)
        p, v, _, m = s.get_state()
        path = tmp_path / "h.nbsnap"
        assert nb.load().nb_save_snapshot(s.h, str(path).encode(), 4, 4e-3) == 0
    step, t, p2, v2, m2 = nb.read_snapshot(path)
    assert step == 4 and abs(t - 4e-3) < 1e-15
    np.testing.assert_array_equal(p2, p)
    np.testing.assert_array_equal(v2, v)
    np.testing.assert_array_equal(m2, m)
    # a served job's snapshot, written from the callback, reads back as delivered
    got = {}

    def on_event(job, event, value, pos, vel):
        if event == nb.JOB_EVENT_SNAPSHOT and value == 10:
            nb.write_snapshot(tmp_path / "j.nbsnap", pos, state[2], step=value, time=value * 1e-3)
            got["pos"] = pos

    with nb.Server(on_event=on_event) as srv:
        j = srv.submit(cfg, 12, 1e-3, state[0], state[2], state[1])
        assert srv.wait(j, WAIT_S) == 0
    step, _, p3, _, _ = nb.read_snapshot(tmp_path / "j.nbsnap")
    assert step == 10
    np.testing.assert_array_equal(p3, got["pos"])
    np.testing.assert_array_equal(p3, standalone(nb, cfg, 10, 1e-3, state)[0])


def test_nonfinite_job_fails_alone(gpu):
    """A job with a NaN position fails with NB_ERR_NONFINITE; a job beside it
    is unaffected."""
    nb = gpu
    bad_state = job_state(4000, 31)
    bad_state[0][17, 1] = np.nan
    good = (jcfg(nb, 4000, True), 15, job_state(4000, 32))
    with nb.Server() as srv:
        bad = srv.submit(jcfg(nb, 4000, True), 15, 1e-3, bad_state[0], bad_state[2], bad_state[1])
        ok = srv.submit(good[0], good[1], 1e-3, good[2][0], good[2][2], good[2][1])
        assert srv.wait(bad, WAIT_S) == 7  # NB_ERR_NONFINITE
        assert srv.wait(ok, WAIT_S) == 0
        np.testing.assert_array_equal(srv.result(ok, 4000)[0], standalone(nb, *good[:2], 1e-3, good[2])[0])


def test_destroy_with_jobs_in_flight(gpu):
    """Destroying the server while jobs are queued and running cancels them
    and returns; nothing is left on the device."""
    nb = gpu
    srv = nb.Server(max_jobs=2)
    for k in range(6):
        n = 20000 + 1000 * k
        st = job_state(n, 50 + k)
        srv.submit(jcfg(nb, n, True), 300, 1e-3, st[0], st[2], st[1])
    time.sleep(0.05)
    t0 = time.time()
    srv.close()
    assert time.time() - t0 < 60
