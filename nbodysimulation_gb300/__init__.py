"""GB300 N-body step library: Python ctypes front-end of libnbgb.so.

The product is the C ABI in include/nbgb.h (libnbgb.so, CUDA for sm_103a);
this module binds it for tests, the benchmark and Python callers.  There is
no CPU fallback: if the shared library is missing or cannot load, `load()`
raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libnbgb.so")

# nb_status
OK, ERR_INVALID_ARGUMENT, ERR_CUDA, ERR_OUT_OF_MEMORY, ERR_CELL_OVERFLOW, ERR_DEPTH, ERR_SPIN_TIMEOUT, \
    ERR_NONFINITE, ERR_NO_DEVICE, ERR_STATE, ERR_UNSUPPORTED = range(11)
LEAPFROG, EULER, KDK_LEAPFROG = 1, 2, 3
SPHERE_POS, UNIFORM_POS, BALL_POS, NORMAL_SIGMA_POS = 0, 1, 2, 3
RANDOM_VEL, STARTING_OUT_VEL, STARTING_IN_VEL, FUNC_ZERO_VEL, TANGENT_XZ_VEL, CIRCULAR_Z_VEL = range(6)
BARNES_HUT, BRUTE_FORCE_GLOBAL, BRUTE_FORCE_LOCAL = 0, 1, 2
MASS_NORMAL_ABS, MASS_EQUAL, MASS_LOGNORMAL = 0, 1, 2
TREE_GEOMETRIC, TREE_REFERENCE = 0, 1
THETA_STANDARD, THETA_REFERENCE = 0, 1
PRECISION_FP32, PRECISION_COMPENSATED = 0, 1
FORCE_PLUMMER, FORCE_REFERENCE_QUIRK = 0, 1
DEBUG_BBOX, DEBUG_CHILDREN, DEBUG_NODE_POS, DEBUG_NODE_MASS, DEBUG_BODY_COUNT, DEBUG_SORTED, DEBUG_TREE_INFO, \
    DEBUG_DQ, DEBUG_NODE_QUAD = range(9)
MULTIPOLE_MONOPOLE, MULTIPOLE_QUADRUPOLE = 0, 1
STAGES = ("bbox", "build", "summarize", "sort", "force", "collision", "direct")
MAX_DEPTH = 64


class NbConfig(ctypes.Structure):
    """Mirror of `nb_config` (include/nbgb.h)."""

    _fields_ = [
        ("num_of_bodies", ctypes.c_int32),
        ("gravitational_constant", ctypes.c_float),
        ("starting_speed_mul", ctypes.c_float),
        ("starting_volume_radius", ctypes.c_float),
        ("number_of_massive_objects", ctypes.c_int32),
        ("massive_object_mass", ctypes.c_float),
        ("collision", ctypes.c_int32),
        ("pos_config", ctypes.c_int32),
        ("vel_config", ctypes.c_int32),
        ("algo_config", ctypes.c_int32),
        ("mass_mean", ctypes.c_float),
        ("mass_deviation", ctypes.c_float),
        ("numerical_method", ctypes.c_int32),
        ("max_octree_depth", ctypes.c_int32),
        ("theta", ctypes.c_float),
        ("epsilon", ctypes.c_float),
        ("simulation_speed_mul", ctypes.c_float),
        ("particle_size", ctypes.c_float),
        ("tree_semantics", ctypes.c_int32),
        ("theta_semantics", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("force_law", ctypes.c_int32),
        ("direct_epsilon", ctypes.c_float),
        ("cell_capacity", ctypes.c_int32),
        ("mass_config", ctypes.c_int32),
        ("pos_sigma", ctypes.c_float * 3),
        ("mass_lognormal_sigma", ctypes.c_float),
        ("seed", ctypes.c_uint64),
        ("device", ctypes.c_int32),
        ("multipole", ctypes.c_int32),
        ("reserved", ctypes.c_int32 * 6),
    ]


class NbDeviceView(ctypes.Structure):
    _fields_ = [("body_pm", ctypes.c_void_p), ("vel", ctypes.c_void_p), ("acc", ctypes.c_void_p),
                ("stream", ctypes.c_void_p), ("n", ctypes.c_int32)]


# every entry point of include/nbgb.h: name -> (argtypes, restype)
_P, _I, _F, _D, _SZ = ctypes.c_void_p, ctypes.c_int32, ctypes.c_float, ctypes.c_double, ctypes.c_size_t
SIGNATURES = {
    "nb_abi_version": ([], _I),
    "nb_status_string": ([_I], ctypes.c_char_p),
    "nb_config_default": ([ctypes.POINTER(NbConfig)], None),
    "nb_create": ([ctypes.POINTER(NbConfig), ctypes.POINTER(_P)], _I),
    "nb_destroy": ([_P], _I),
    "nb_get_config": ([_P, ctypes.POINTER(NbConfig)], _I),
    "nb_set_state": ([_P, _P, _P, _P, _I], _I),
    "nb_get_state": ([_P, _P, _P, _P, _P], _I),
    "nb_generate_ic": ([ctypes.POINTER(NbConfig), _P, _P, _P], _I),
    "nb_init_bodies": ([_P], _I),
    "nb_step": ([_P, _F, _I], _I),
    "nb_update": ([_P, _F], _I),
    "nb_step_async": ([_P, _F, _I], _I),
    "nb_synchronize": ([_P], _I),
    "nb_copy_vertices": ([_P, _P, _I], _I),
    "nb_get_stage_debug": ([_P, _I, _P, _SZ, ctypes.POINTER(_SZ)], _I),
    "nb_set_profiling": ([_P, _I], _I),
    "nb_get_timings": ([_P, _P, _I], _I),
    "nb_kernel_launches": ([_P], ctypes.c_int64),
    "nb_time_steps": ([_P, _F, _I, ctypes.POINTER(_F)], _I),
    "nb_get_work_counters": ([_P, _P], _I),
    "nb_debug_set_spin_cap": ([_P, _I], _I),
    "nb_get_device_view": ([_P, ctypes.POINTER(NbDeviceView)], _I),
    "nb_set_state_device": ([_P, _P, _P, _P], _I),
    "nb_get_state_device": ([_P, _P, _P], _I),
    "nb_force_error_probe": ([_P, _P, _I, ctypes.POINTER(_D), ctypes.POINTER(_D), _P], _I),
    "nb_diagnostics": ([_P, _I, _P], _I),
    "nb_last_error": ([_P], _I),
    "nb_last_error_message": ([_P], ctypes.c_char_p),
    "nb_host_alloc": ([_SZ], _P),
    "nb_host_free": ([_P], None),
    "nb_direct_accel_noalloc": ([_P, _I, _F, _F, _P, _P], _I),
    "nb_batch_create": ([_P, _I, ctypes.POINTER(_P)], _I),
    "nb_batch_destroy": ([_P], _I),
    "nb_batch_set_state": ([_P, _I, _P, _P, _P], _I),
    "nb_batch_get_state": ([_P, _I, _P, _P, _P, _P], _I),
    "nb_batch_step": ([_P, _F, _I], _I),
    "nb_batch_time_steps": ([_P, _F, _I, ctypes.POINTER(_F)], _I),
    "nb_batch_system_status": ([_P, _I], _I),
    "nb_batch_autotune": ([_P, ctypes.c_char_p, ctypes.POINTER(_I)], _I),
    "nb_batch_info": ([_P, _P], _I),
    "nb_batch_tree_shape": ([_P, _P], _I),
    "nb_batch_last_error_message": ([_P], ctypes.c_char_p),
    "nb_snapshot_write": ([ctypes.c_char_p, ctypes.c_int64, _D, _P, _P, _P, _I], _I),
    "nb_snapshot_read": ([ctypes.c_char_p, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(_D), _P, _P, _P, _I,
                          ctypes.POINTER(_I)], _I),
    "nb_save_snapshot": ([_P, ctypes.c_char_p, ctypes.c_int64, _D], _I),
    "nb_server_config_default": ([_P], None),
    "nb_server_create": ([_P, _P, _P, ctypes.POINTER(_P)], _I),
    "nb_server_submit": ([_P, ctypes.POINTER(NbConfig), _I, _F, _P, _P, _P, ctypes.POINTER(ctypes.c_int64)], _I),
    "nb_server_job_info": ([_P, ctypes.c_int64, _P], _I),
    "nb_server_wait": ([_P, ctypes.c_int64, _D], _I),
    "nb_server_result": ([_P, ctypes.c_int64, _P, _P], _I),
    "nb_server_get_stats": ([_P, _P], _I),
    "nb_server_destroy": ([_P], _I),
    "nb_server_last_error_message": ([_P], ctypes.c_char_p),
}
NOALLOC_MAX_BODIES = 65536

_lib = None


class NbError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{message} (status {status})")
        self.status = status


def load(path: str = LIB_PATH):
    """Load libnbgb.so (built by nbodysimulation_gb300.build).  Raises when absent."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise ImportError(f"libnbgb.so not built at {path}; run `python -m nbodysimulation_gb300.build`")
        L = ctypes.CDLL(path)
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def default_config(**kw) -> NbConfig:
    c = NbConfig()
    load().nb_config_default(ctypes.byref(c))
    for k, v in kw.items():
        if k == "pos_sigma":
            c.pos_sigma[:] = list(v)
        else:
            setattr(c, k, v)
    return c


def generate_ic(cfg: NbConfig):
    n = cfg.num_of_bodies
    pos = np.zeros((n, 3), np.float32)
    vel = np.zeros((n, 3), np.float32)
    mass = np.zeros(n, np.float32)
    st = load().nb_generate_ic(ctypes.byref(cfg), pos.ctypes.data, vel.ctypes.data, mass.ctypes.data)
    if st:
        raise NbError(st, "nb_generate_ic")
    return pos, vel, mass


def _f32(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a if shape is None else a.reshape(shape)


def _out(a, shape):
    """A float32 C-contiguous array of `shape` to write into: the caller's
    array `a` (reused, so its pages are already populated), or a new one."""
    if a is None:
        return np.zeros(shape, np.float32)
    if a.dtype != np.float32 or a.shape != shape or not a.flags.c_contiguous or not a.flags.writeable:
        raise ValueError(f"output array must be writeable C-contiguous float32 of shape {shape}")
    return a


class Simulation:
    """One system on the GPU: the handle of nb_create (CMyApp's buffers)."""

    def __init__(self, cfg: NbConfig | None = None, **kw):
        self.L = load()
        self.cfg = cfg if cfg is not None else default_config(**kw)
        h = ctypes.c_void_p()
        st = self.L.nb_create(ctypes.byref(self.cfg), ctypes.byref(h))
        if st:
            raise NbError(st, f"nb_create: {self.L.nb_status_string(st).decode()}")
        self.h = h
        self.n = self.cfg.num_of_bodies

    def close(self):
        if getattr(self, "h", None):
            self.L.nb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st, what):
        if st:
            msg = self.L.nb_last_error_message(self.h).decode()
            raise NbError(st, f"{what}: {msg or self.L.nb_status_string(st).decode()}")

    def set_state(self, pos, mass, vel=None):
        pos = _f32(pos, (-1,))
        mass = _f32(mass, (-1,))
        v = None if vel is None else _f32(vel, (-1,))
        self._check(self.L.nb_set_state(self.h, pos.ctypes.data, None if v is None else v.ctypes.data,
                                        mass.ctypes.data, self.n), "nb_set_state")

    def init_bodies(self):
        self._check(self.L.nb_init_bodies(self.h), "nb_init_bodies")

    def get_state(self, out=None):
        """(pos, vel, acc, mass); `out` = four arrays of those shapes to reuse."""
        o = out if out is not None else (None,) * 4
        pos, vel, acc = (_out(a, (self.n, 3)) for a in o[:3])
        mass = _out(o[3], (self.n,))
        self._check(self.L.nb_get_state(self.h, pos.ctypes.data, vel.ctypes.data, acc.ctypes.data,
                                        mass.ctypes.data), "nb_get_state")
        return pos, vel, acc, mass

    def positions(self, with_velocities=False, out=None):
        """Positions (N,3) -- what a snapshot or a renderer reads -- and, when
        asked, velocities.  `out` = the array (or the pair) to reuse: pages
        that the host has never touched cost several times the copy itself on
        their first use."""
        o = out if isinstance(out, (tuple, list)) else (out, None)
        pos = _out(o[0], (self.n, 3))
        vel = _out(o[1], (self.n, 3)) if with_velocities else None
        self._check(self.L.nb_get_state(self.h, pos.ctypes.data, None if vel is None else vel.ctypes.data, None,
                                        None), "nb_get_state")
        return (pos, vel) if with_velocities else pos

    def step(self, dt, nsteps=1, check=True):
        st = self.L.nb_step(self.h, dt, nsteps)
        if check:
            self._check(st, "nb_step")
        return st

    def update(self, frame_dt):
        self._check(self.L.nb_update(self.h, frame_dt), "nb_update")

    def step_async(self, dt, nsteps=1):
        self._check(self.L.nb_step_async(self.h, dt, nsteps), "nb_step_async")

    def synchronize(self):
        self._check(self.L.nb_synchronize(self.h), "nb_synchronize")

    def copy_vertices(self):
        out = np.zeros((self.n, 4), np.float32)
        self._check(self.L.nb_copy_vertices(self.h, out.ctypes.data, 0), "nb_copy_vertices")
        return out

    def stage_debug(self, which):
        need = ctypes.c_size_t(0)
        dummy = np.zeros(1, np.uint8)
        self.L.nb_get_stage_debug(self.h, which, dummy.ctypes.data, 0, ctypes.byref(need))
        dt = np.float32 if which in (DEBUG_BBOX, DEBUG_NODE_POS, DEBUG_NODE_MASS, DEBUG_DQ, DEBUG_NODE_QUAD) else np.int32
        out = np.zeros(need.value // 4, dt)
        self._check(self.L.nb_get_stage_debug(self.h, which, out.ctypes.data, need.value, None),
                    "nb_get_stage_debug")
        return out

    def set_profiling(self, on=True):
        self._check(self.L.nb_set_profiling(self.h, 1 if on else 0), "nb_set_profiling")

    def timings(self):
        ms = np.zeros(len(STAGES), np.float32)
        self._check(self.L.nb_get_timings(self.h, ms.ctypes.data, len(STAGES)), "nb_get_timings")
        return dict(zip(STAGES, ms.tolist()))

    def time_steps(self, dt, nsteps):
        """Device time (ms) of nsteps steps, CUDA events on the handle's stream."""
        ms = ctypes.c_float(0.0)
        self._check(self.L.nb_time_steps(self.h, dt, nsteps, ctypes.byref(ms)), "nb_time_steps")
        return ms.value

    def work_counters(self):
        """(interactions, cells opened, cell interactions) of the last nb_step call."""
        out = np.zeros(3, np.uint64)
        self._check(self.L.nb_get_work_counters(self.h, out.ctypes.data), "nb_get_work_counters")
        return int(out[0]), int(out[1]), int(out[2])

    def set_spin_cap(self, cap):
        """Test hook: cap the tree stages' bounded waits (0 = default)."""
        self._check(self.L.nb_debug_set_spin_cap(self.h, cap), "nb_debug_set_spin_cap")

    def kernel_launches(self):
        return int(self.L.nb_kernel_launches(self.h))

    def device_view(self):
        v = NbDeviceView()
        self._check(self.L.nb_get_device_view(self.h, ctypes.byref(v)), "nb_get_device_view")
        return v

    def force_error(self, sample):
        sample = np.ascontiguousarray(sample, np.int32)
        mx, rms = ctypes.c_double(), ctypes.c_double()
        per = np.zeros(len(sample), np.float64)
        self._check(self.L.nb_force_error_probe(self.h, sample.ctypes.data, len(sample), ctypes.byref(mx),
                                                ctypes.byref(rms), per.ctypes.data), "nb_force_error_probe")
        return mx.value, rms.value, per

    def diagnostics(self, with_potential=False):
        out = np.zeros(9, np.float64)
        self._check(self.L.nb_diagnostics(self.h, 1 if with_potential else 0, out.ctypes.data), "nb_diagnostics")
        keys = ("kinetic", "px", "py", "pz", "lx", "ly", "lz", "mass", "potential")
        return dict(zip(keys, out.tolist()))


class Batch:
    """Many independent systems advanced together (nb_batch_*): one launch per
    stage over all systems, one CUDA graph per step."""

    def __init__(self, cfgs):
        self.L = load()
        self.cfgs = list(cfgs)
        arr = (NbConfig * len(self.cfgs))(*self.cfgs)
        h = ctypes.c_void_p()
        st = self.L.nb_batch_create(ctypes.cast(arr, ctypes.c_void_p), len(self.cfgs), ctypes.byref(h))
        if st:
            raise NbError(st, f"nb_batch_create: {self.L.nb_status_string(st).decode()}")
        self.h = h
        self.ns = [c.num_of_bodies for c in self.cfgs]

    def close(self):
        if getattr(self, "h", None):
            self.L.nb_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __len__(self):
        return len(self.ns)

    def _check(self, st, what):
        if st:
            msg = self.L.nb_batch_last_error_message(self.h).decode()
            raise NbError(st, f"{what}: {msg or self.L.nb_status_string(st).decode()}")

    def set_state(self, k, pos, mass, vel=None):
        pos = _f32(pos, (-1,))
        mass = _f32(mass, (-1,))
        v = None if vel is None else _f32(vel, (-1,))
        self._check(self.L.nb_batch_set_state(self.h, k, pos.ctypes.data, None if v is None else v.ctypes.data,
                                              mass.ctypes.data), "nb_batch_set_state")

    def get_state(self, k, out=None):
        """System k's (pos, vel, acc, mass); `out` = four arrays to reuse."""
        n = self.ns[k]
        o = out if out is not None else (None,) * 4
        pos, vel, acc = (_out(a, (n, 3)) for a in o[:3])
        mass = _out(o[3], (n,))
        self._check(self.L.nb_batch_get_state(self.h, k, pos.ctypes.data, vel.ctypes.data, acc.ctypes.data,
                                              mass.ctypes.data), "nb_batch_get_state")
        return pos, vel, acc, mass

    def step(self, dt, nsteps=1, check=True):
        st = self.L.nb_batch_step(self.h, dt, nsteps)
        if check:
            self._check(st, "nb_batch_step")
        return st

    def time_steps(self, dt, nsteps):
        ms = ctypes.c_float(0.0)
        self._check(self.L.nb_batch_time_steps(self.h, dt, nsteps, ctypes.byref(ms)), "nb_batch_time_steps")
        return ms.value

    def system_status(self, k):
        return int(self.L.nb_batch_system_status(self.h, k))

    def autotune(self, cache_path=None):
        chosen = ctypes.c_int32(-1)
        path = None if cache_path is None else os.fsencode(cache_path)
        self._check(self.L.nb_batch_autotune(self.h, path, ctypes.byref(chosen)), "nb_batch_autotune")
        return chosen.value

    def tree_shape(self):
        """The tree stages' launch shape: force warps per block, percent of the
        resident force blocks, build chunk (0: default rule), top-level cap."""
        out = np.zeros(4, np.int32)
        self._check(self.L.nb_batch_tree_shape(self.h, out.ctypes.data), "nb_batch_tree_shape")
        keys = ("force_warps", "force_grid_pct", "build_chunk", "top_levels")
        return dict(zip(keys, (int(x) for x in out)))

    def info(self):
        out = np.zeros(8, np.int64)
        self._check(self.L.nb_batch_info(self.h, out.ctypes.data), "nb_batch_info")
        keys = ("systems", "bodies", "tree_systems", "direct_systems", "launches_per_step", "direct_variant",
                "launches", "interactions")
        return dict(zip(keys, (int(x) for x in out)))


class NbServerConfig(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("max_jobs", ctypes.c_int32), ("hbm_budget_bytes", ctypes.c_int64),
                ("snapshot_every", ctypes.c_int32), ("numerical_method", ctypes.c_int32),
                ("precision", ctypes.c_int32), ("multipole", ctypes.c_int32), ("direct_variant", ctypes.c_int32),
                ("reserved", ctypes.c_int32 * 7)]


class NbJobInfo(ctypes.Structure):
    _fields_ = [("state", ctypes.c_int32), ("status", ctypes.c_int32), ("steps", ctypes.c_int32),
                ("n", ctypes.c_int32), ("t_submit", ctypes.c_double), ("t_admit", ctypes.c_double),
                ("t_done", ctypes.c_double), ("bytes", ctypes.c_int64)]


class NbServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_int64), ("completed", ctypes.c_int64), ("failed", ctypes.c_int64),
                ("queued", ctypes.c_int64), ("running", ctypes.c_int64), ("rounds", ctypes.c_int64),
                ("bytes_in_use", ctypes.c_int64), ("peak_bytes", ctypes.c_int64), ("peak_jobs", ctypes.c_int32),
                ("pad", ctypes.c_int32), ("body_updates", ctypes.c_double), ("first_submit_s", ctypes.c_double),
                ("last_done_s", ctypes.c_double), ("latency_p50_s", ctypes.c_double),
                ("latency_p99_s", ctypes.c_double), ("latency_max_s", ctypes.c_double),
                ("latency_mean_s", ctypes.c_double)]


JOB_QUEUED, JOB_RUNNING, JOB_DONE, JOB_FAILED = range(4)
JOB_EVENT_SNAPSHOT, JOB_EVENT_DONE, JOB_EVENT_FAILED = range(3)
JOB_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
                          ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float), ctypes.c_int32)


def server_config(**kw) -> NbServerConfig:
    c = NbServerConfig()
    load().nb_server_config_default(ctypes.byref(c))
    for k, v in kw.items():
        setattr(c, k, v)
    return c


class Server:
    """Job server (nb_server_*): continuous batching of simulation jobs.

    on_event(job, event, value, pos, vel) is called from a library thread with
    numpy copies of the arrays (None where absent); without it, finished
    results are kept for result()."""

    def __init__(self, cfg: NbServerConfig | None = None, on_event=None, copy_arrays=True, **kw):
        self.L = load()
        self.cfg = cfg if cfg is not None else server_config(**kw)
        self._user_fn = on_event
        self._fn = None
        if on_event is not None:
            def _cb(user, job, event, value, pos, vel, n):
                p = v = None
                if copy_arrays and pos:
                    p = np.ctypeslib.as_array(pos, shape=(n, 3)).copy()
                if copy_arrays and vel:
                    v = np.ctypeslib.as_array(vel, shape=(n, 3)).copy()
                on_event(int(job), int(event), int(value), p, v)
            self._fn = JOB_FN(_cb)
        h = ctypes.c_void_p()
        fn_ptr = ctypes.cast(self._fn, ctypes.c_void_p) if self._fn is not None else None
        st = self.L.nb_server_create(ctypes.byref(self.cfg), fn_ptr, None, ctypes.byref(h))
        if st:
            raise NbError(st, f"nb_server_create: {self.L.nb_status_string(st).decode()}")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.nb_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st, what):
        if st:
            msg = self.L.nb_server_last_error_message(self.h).decode()
            raise NbError(st, f"{what}: {msg or self.L.nb_status_string(st).decode()}")

    def submit(self, cfg: NbConfig, steps, dt, pos=None, mass=None, vel=None):
        jid = ctypes.c_int64(-1)
        if pos is None:
            st = self.L.nb_server_submit(self.h, ctypes.byref(cfg), steps, dt, None, None, None, ctypes.byref(jid))
        else:
            p = _f32(pos, (-1,))
            m = _f32(mass, (-1,))
            v = None if vel is None else _f32(vel, (-1,))
            st = self.L.nb_server_submit(self.h, ctypes.byref(cfg), steps, dt, p.ctypes.data,
                                         None if v is None else v.ctypes.data, m.ctypes.data, ctypes.byref(jid))
        self._check(st, "nb_server_submit")
        return jid.value

    def info(self, job):
        out = NbJobInfo()
        self._check(self.L.nb_server_job_info(self.h, job, ctypes.byref(out)), "nb_server_job_info")
        return {k: getattr(out, k) for k, _ in NbJobInfo._fields_}

    def wait(self, job=-1, timeout=-1.0):
        """Returns the job's status (0 when it finished normally)."""
        return int(self.L.nb_server_wait(self.h, job, timeout))

    def result(self, job, n):
        pos = np.zeros((n, 3), np.float32)
        vel = np.zeros((n, 3), np.float32)
        self._check(self.L.nb_server_result(self.h, job, pos.ctypes.data, vel.ctypes.data), "nb_server_result")
        return pos, vel

    def stats(self):
        out = NbServerStats()
        self._check(self.L.nb_server_get_stats(self.h, ctypes.byref(out)), "nb_server_get_stats")
        return {k: getattr(out, k) for k, _ in NbServerStats._fields_ if k != "pad"}


def write_snapshot(path, pos, mass, vel=None, step=0, time=0.0):
    """Write one system's state in the snapshot format (nb_snapshot_write)."""
    p = _f32(pos, (-1,))
    m = _f32(mass, (-1,))
    v = None if vel is None else _f32(vel, (-1,))
    st = load().nb_snapshot_write(os.fsencode(path), int(step), float(time), p.ctypes.data,
                                  None if v is None else v.ctypes.data, m.ctypes.data, len(m))
    if st:
        raise NbError(st, f"nb_snapshot_write {path}")


def read_snapshot(path):
    """(step, time, pos[N,3], vel[N,3], mass[N]) of a snapshot file."""
    L = load()
    n = ctypes.c_int32(0)
    step = ctypes.c_int64(0)
    t = ctypes.c_double(0.0)
    st = L.nb_snapshot_read(os.fsencode(path), ctypes.byref(step), ctypes.byref(t), None, None, None, 0,
                            ctypes.byref(n))
    if st:
        raise NbError(st, f"nb_snapshot_read {path}")
    pos = np.zeros((n.value, 3), np.float32)
    vel = np.zeros((n.value, 3), np.float32)
    mass = np.zeros(n.value, np.float32)
    st = L.nb_snapshot_read(os.fsencode(path), ctypes.byref(step), ctypes.byref(t), pos.ctypes.data,
                            vel.ctypes.data, mass.ctypes.data, n.value, ctypes.byref(n))
    if st:
        raise NbError(st, f"nb_snapshot_read {path}")
    return step.value, t.value, pos, vel, mass
