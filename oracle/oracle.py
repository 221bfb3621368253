"""TEST INFRASTRUCTURE: ctypes front-end of the CPU oracle (nboracle.c).

Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg.  Arrays follow the reference's layout (packed float[3N] positions,
node index space bodies [0,N), cells (N, N+nodes), root N+nodes).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libnboracle.so")

SEM_REFERENCE, SEM_GEOMETRIC = 0, 1
CRIT_REFERENCE, CRIT_STANDARD = 0, 1
ARITH_REFERENCE, ARITH_FMA = 0, 1
LEAPFROG, EULER, KDK = 1, 2, 3
MAX_DEPTH = 64

_lib = None


def build() -> str:
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        i, f, d, lo = ctypes.c_int, ctypes.c_float, ctypes.c_double, ctypes.c_long
        sig = {
            "orc_bbox_exact": ([P, lo, P], None),
            "orc_bbox_sampled": ([P, i, P], None),
            "orc_root_cube": ([P, P], None),
            "orc_tree_build": ([i, P, i, i, P, P, P, P, P, P, P], i),
            "orc_tree_paths": ([P, i, i, i, P, P], i),
            "orc_saturate": ([i, i, i, i, P, P, P, P], i),
            "orc_sort": ([P, i, i, P], i),
            "orc_bh_thresholds": ([i, P, f, f, i, P], None),
            "orc_bh_force": ([P, P, P, i, i, P, f, f, i, i, P, i, i, i, P, P, P], i),
            "orc_quadrupoles": ([i, i, i, P, P, P, P], None),
            "orc_direct_fp32": ([P, P, i, f, f, i, i, P], None),
            "orc_direct_fp64": ([P, P, i, d, d, P, i, P], None),
            "orc_direct_quirk_global": ([P, P, i, f, P], None),
            "orc_direct_quirk_local": ([P, P, i, i, i, f, P], i),
            "orc_integrate": ([i, i, i, f, P, P, P, P, i], None),
            "orc_collision": ([P, P, i, i, i], i),
            "orc_copy_vertices": ([P, i, P], None),
            "orc_max_threads": ([], i),
            "orc_set_threads": ([i], None),
            "orc_generate_ic": ([i, ctypes.c_uint64, i, P, f, i, f, P, P], i),
            "orc_pipe_create": ([i, i], P),
            "orc_pipe_destroy": ([P], None),
            "orc_pipe_step": ([P, P, P, P, P, f, f, f, f, i, i, P, P], i),
            "orc_pipe_export": ([P, P, P, P], i),
            "orc_pipe_levels_of": ([P], i),
        }
        for name, (args, res) in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data if a is not None else None


def f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def bbox_exact(pos3):
    pos3 = f32(pos3).reshape(-1, 3)
    out = np.zeros(6, np.float32)
    lib().orc_bbox_exact(_p(pos3), pos3.shape[0], _p(out))
    return out


def bbox_sampled(p_buffer, wg):
    p_buffer = f32(p_buffer).ravel()
    out = np.zeros(6, np.float32)
    lib().orc_bbox_sampled(_p(p_buffer), wg, _p(out))
    return out


def root_cube(box6):
    box6 = f32(box6)
    out = np.zeros(4, np.float32)
    lib().orc_root_cube(_p(box6), _p(out))
    return out


def reference_nodes(n, cus=1, warpsize=16):
    """Cell budget of CMyApp::SetKernelConfig (src/MyApp.cpp:71-83)."""
    nodes = max(2 * n, 1024 * cus)
    while nodes & (warpsize - 1):
        nodes += 1
    return nodes


class Tree:
    """A tree in the reference's buffer layout."""

    def __init__(self, n, nodes):
        self.n, self.nodes = n, nodes
        total = n + nodes + 1
        self.pos = np.zeros(total * 3, np.float32)
        self.mass = np.zeros(total, np.float32)
        self.children = np.full(total * 8, -1, np.int32)
        self.body_count = np.zeros(total, np.int32)
        self.body_depth = np.zeros(n, np.int32)
        self.bottom = n + nodes
        self.max_depth = 1

    @property
    def root(self):
        return self.n + self.nodes


def tree_build(sem, pos3, mass, box6, nodes=None):
    pos3 = f32(pos3).reshape(-1, 3)
    n = pos3.shape[0]
    nodes = reference_nodes(n) if nodes is None else nodes
    t = Tree(n, nodes)
    t.pos[: 3 * n] = pos3.ravel()
    t.mass[:n] = f32(mass)
    bottom = ctypes.c_int(0)
    md = ctypes.c_int(0)
    box6 = f32(box6)
    rc = lib().orc_tree_build(sem, _p(pos3), n, nodes, _p(box6), _p(t.pos), _p(t.mass), _p(t.children),
                              _p(t.body_depth), ctypes.byref(bottom), ctypes.byref(md))
    t.bottom, t.max_depth, t.status = bottom.value, md.value, rc
    return t


def tree_paths(children, n, root, maxlen=MAX_DEPTH + 2):
    children = i32(children)
    paths = np.full((n, maxlen), -1, np.int8)
    depth = np.zeros(n, np.int32)
    found = lib().orc_tree_paths(_p(children), n, root, maxlen, _p(paths), _p(depth))
    return paths, depth, found


def saturate(t: Tree, compaction_bug=False):
    return lib().orc_saturate(1 if compaction_bug else 0, t.n, t.nodes, t.bottom, _p(t.pos), _p(t.mass),
                              _p(t.children), _p(t.body_count))


def sort_bodies(children, n, root):
    children = i32(children)
    out = np.full(n, -1, np.int32)
    k = lib().orc_sort(_p(children), n, root, _p(out))
    return out, k


def thresholds(criterion, box6, theta, eps, max_depth):
    dq = np.zeros(MAX_DEPTH, np.float32)
    lib().orc_bh_thresholds(criterion, _p(f32(box6)), theta, eps, max_depth, _p(dq))
    return dq


def quadrupoles(t: Tree):
    q = np.zeros((t.n + t.nodes + 1) * 6, np.float32)
    lib().orc_quadrupoles(t.n, t.nodes, t.bottom, _p(t.pos), _p(t.mass), _p(i32(t.children)), _p(q))
    return q


def bh_force(t: Tree, dq, eps, G, arith=ARITH_FMA, vote_width=32, order=None, skip_self=True,
             compensated=False, quad=None, stats=None):
    """Forces for the bodies of `order` (all bodies when None), walked in
    groups of `vote_width` consecutive entries.  `quad` (from quadrupoles())
    adds the cells' quadrupole terms; `stats` (int64[2]) receives the body and
    cell interaction counts."""
    acc = np.zeros(t.n * 3, np.float32)
    order = i32(order) if order is not None else None
    norder = 0 if order is None else len(order)
    q = f32(quad) if quad is not None else None
    rc = lib().orc_bh_force(_p(t.pos), _p(t.mass), _p(t.children), t.n, t.nodes, _p(f32(dq)), eps, G, arith,
                            vote_width, _p(order), norder, 1 if skip_self else 0, 1 if compensated else 0, _p(q),
                            _p(stats), _p(acc))
    return acc.reshape(-1, 3), rc


def direct_fp32(pos3, mass, eps, G, i0=0, i1=None):
    pos3 = f32(pos3).reshape(-1, 3)
    n = pos3.shape[0]
    i1 = n if i1 is None else i1
    acc = np.zeros((n, 3), np.float32)
    lib().orc_direct_fp32(_p(pos3), _p(f32(mass)), n, eps, G, i0, i1, _p(acc))
    return acc


def direct_fp64(pos3, mass, eps, G, targets=None):
    pos3 = f32(pos3).reshape(-1, 3)
    n = pos3.shape[0]
    tg = i32(targets) if targets is not None else None
    nt = n if targets is None else len(tg)
    acc = np.zeros((nt, 3), np.float64)
    lib().orc_direct_fp64(_p(pos3), _p(f32(mass)), n, eps, G, _p(tg), nt, _p(acc))
    return acc


def direct_quirk_global(pos3, mass, G):
    pos3 = f32(pos3).reshape(-1, 3)
    acc = np.zeros_like(pos3)
    lib().orc_direct_quirk_global(_p(pos3), _p(f32(mass)), pos3.shape[0], G, _p(acc))
    return acc


def direct_quirk_local(pos3, mass, G, wg=0, tile_schedule=False):
    pos3 = f32(pos3).reshape(-1, 3)
    acc = np.zeros_like(pos3)
    rc = lib().orc_direct_quirk_local(_p(pos3), _p(f32(mass)), pos3.shape[0], wg, 1 if tile_schedule else 0, G, _p(acc))
    if rc:
        raise ValueError("tile_schedule schedule needs n % wg == 0")
    return acc


def integrate(method, pos3, vel3, acc_new3, accs3, dt, primed=False):
    """Returns (pos, vel, accs) after one integrator update (copies)."""
    pos3 = f32(pos3).reshape(-1, 3).copy()
    vel3 = f32(vel3).reshape(-1, 3).copy()
    accs3 = f32(accs3).reshape(-1, 3).copy()
    acc_new3 = f32(acc_new3).reshape(-1, 3)
    lib().orc_integrate(method, 1 if primed else 0, pos3.shape[0], dt, _p(acc_new3), _p(accs3), _p(vel3),
                        _p(pos3), 3)
    return pos3, vel3, accs3


def collision(pos3, vel3, wg=0, tile_schedule=False):
    pos3 = f32(pos3).reshape(-1, 3)
    v = f32(vel3).reshape(-1, 3).copy()
    rc = lib().orc_collision(_p(pos3), _p(v), pos3.shape[0], wg, 1 if tile_schedule else 0)
    if rc:
        raise ValueError("tile_schedule schedule needs n % wg == 0")
    return v


def copy_vertices(pos3):
    pos3 = f32(pos3).reshape(-1, 3)
    out = np.zeros((pos3.shape[0], 4), np.float32)
    lib().orc_copy_vertices(_p(pos3), pos3.shape[0], _p(out))
    return out


def bh_step_forces(pos3, mass, theta, eps, G, sem=SEM_GEOMETRIC, criterion=CRIT_STANDARD, arith=ARITH_FMA,
                   vote_width=32, order="sorted", compensated=False, nodes=None, box=None, quadrupole=False):
    """bbox -> build -> summarise -> sort -> force, as the GPU library runs it.
    Returns (acc[N,3], tree, sorted)."""
    pos3 = f32(pos3).reshape(-1, 3)
    box = bbox_exact(pos3) if box is None else f32(box)
    t = tree_build(sem, pos3, mass, box, nodes)
    if t.status:
        raise RuntimeError(f"oracle tree build failed: {t.status}")
    rc = saturate(t)
    if rc:
        raise RuntimeError(f"oracle saturate failed: {rc}")
    srt, k = sort_bodies(t.children, t.n, t.root)
    dq = thresholds(criterion, box, theta, eps, t.max_depth)
    o = srt if order == "sorted" else (None if order is None else order)
    q = quadrupoles(t) if quadrupole else None
    acc, rc = bh_force(t, dq, eps, G, arith=arith, vote_width=vote_width, order=o, compensated=compensated, quad=q)
    if rc:
        raise RuntimeError(f"oracle force failed: {rc}")
    return acc, t, srt


# ---------------------------------------------------------------------------
# seeded initial conditions and the parallel whole step (nbpipeline.c)
# ---------------------------------------------------------------------------
POS_UNIFORM, POS_NORMAL_SIGMA = 1, 3
MASS_EQUAL, MASS_LOGNORMAL = 1, 2
PIPE_STAGES = ("bbox", "build", "summarize", "sort", "force", "integrate")


def generate_ic(n, seed, pos_mode=POS_NORMAL_SIGMA, sigma=(1.0, 1.0, 1.0), radius=1.0, mass_mode=MASS_EQUAL,
                mass_sigma=0.5):
    """Positions and masses of the library's seeded generator (the same
    bytes as nb_generate_ic for these modes), without the library."""
    pos = np.zeros((n, 3), np.float32)
    mass = np.zeros(n, np.float32)
    sg = np.asarray(sigma, np.float32)
    rc = lib().orc_generate_ic(n, seed, pos_mode, _p(sg), radius, mass_mode, mass_sigma, _p(pos), _p(mass))
    if rc:
        raise ValueError(f"orc_generate_ic: unsupported mode ({rc})")
    return pos, mass


class Pipeline:
    """One whole Barnes-Hut step (bbox, build, summarise, sort, force, Euler)
    on every host core, results equal to the sequential restatement.
    Geometric tree, standard criterion, vote width 32."""

    def __init__(self, n, nodes=None):
        self.n = n
        self.nodes = 2 * n if nodes is None else nodes
        self.h = lib().orc_pipe_create(n, self.nodes)
        if not self.h:
            raise MemoryError("orc_pipe_create failed")
        self.stage_s = np.zeros(6, np.float64)
        self.stats = np.zeros(2, np.int64)

    @property
    def levels(self):
        return lib().orc_pipe_levels_of(self.h)

    def step(self, pos, vel, acc, mass, theta, eps, G, dt, quadrupole=True, compensated=True):
        """Advances pos/vel (float32 [n,3], in place); acc receives the new
        accelerations.  Returns the stage seconds as a dict."""
        for a in (pos, vel, acc):
            assert a.dtype == np.float32 and a.flags.c_contiguous and a.size == 3 * self.n
        rc = lib().orc_pipe_step(self.h, _p(pos), _p(vel), _p(acc), _p(f32(mass)), theta, eps, G, dt,
                                 1 if quadrupole else 0, 1 if compensated else 0, _p(self.stage_s), _p(self.stats))
        if rc:
            raise RuntimeError(f"orc_pipe_step failed: {rc}")
        return dict(zip(PIPE_STAGES, self.stage_s.tolist()))

    def export(self):
        """(children rows, sorted order, bottom, max_depth) of the last step."""
        total = self.n + self.nodes + 1
        ch = np.empty(total * 8, np.int32)
        srt = np.empty(self.n, np.int32)
        info = np.zeros(2, np.int32)
        lib().orc_pipe_export(self.h, _p(ch), _p(srt), _p(info))
        return ch, srt, int(info[0]), int(info[1])

    def close(self):
        if self.h:
            lib().orc_pipe_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()
