"""TEST INFRASTRUCTURE: ctypes front-end of the reference emulator.

oracle/_ref/libnbref_wg<WG>.so holds the reference's own OpenCL C kernels
(compiled from the reference sources by oracle/ref/Makefile) on a coroutine
work-item runtime.  It exists only where the reference sources are present;
tests that need it skip elsewhere.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
def _recipe_reference_dir():
    """The reference sources: NBGB_REFERENCE_DIR, else the default that the
    build recipe (ref/Makefile, `REF ?= ...`) reads them from."""
    env = os.environ.get("NBGB_REFERENCE_DIR")
    if env:
        return env
    try:
        with open(os.path.join(HERE, "ref", "Makefile")) as f:
            for line in f:
                if line.startswith("REF ?="):
                    return line.split("?=", 1)[1].strip()
    except OSError:
        pass
    return ""


REF_SRC = _recipe_reference_dir()
WGS = (16, 64, 256)


def lib_path(wg):
    return os.path.join(HERE, "_ref", f"libnbref_wg{wg}.so")


def available() -> bool:
    return os.path.isdir(os.path.join(REF_SRC, "kernels")) or all(os.path.exists(lib_path(w)) for w in WGS)


def build():
    if not os.path.isdir(os.path.join(REF_SRC, "kernels")):
        return False
    subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref"), f"REF={REF_SRC}"], check=True)
    return True


_libs = {}


def lib(wg):
    if wg not in _libs:
        path = lib_path(wg)
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        P, i, f = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
        L.ref_create.restype = P
        L.ref_create.argtypes = [i, i]
        L.ref_destroy.argtypes = [P]
        L.ref_num_nodes.argtypes = [P]
        L.ref_num_nodes.restype = i
        L.ref_set_bodies.argtypes = [P, P, P, P, P]
        L.ref_set_boundary.argtypes = [P, P]
        L.ref_set_max_depth.argtypes = [P, i]
        L.ref_set_round_cap.argtypes = [ctypes.c_long]
        for name in ("ref_bbox_as_wired", "ref_init", "ref_build_tree", "ref_saturate_tree", "ref_collision"):
            getattr(L, name).argtypes = [P]
            getattr(L, name).restype = i
        L.ref_calculate_force.argtypes = [P, f, f, f, f, i]
        L.ref_calculate_force.restype = i
        L.ref_update_global.argtypes = [P, f, f, i]
        L.ref_update_global.restype = i
        L.ref_update_local.argtypes = [P, f, f, i]
        L.ref_update_local.restype = i
        L.ref_copy_vertices.argtypes = [P, P]
        L.ref_copy_vertices.restype = i
        L.ref_get.argtypes = [P, i, P]
        L.ref_get.restype = ctypes.c_long
        _libs[wg] = L
    return _libs[wg]


class RefSim:
    """The reference's buffers and kernels for N bodies at one work-group size."""

    POS, MASS, CHILDREN, BODY_COUNT, VEL, ACC, BOUNDARY, ERROR, BODY_DEPTH, BOTTOM, MAX_DEPTH = range(11)

    def __init__(self, n, wg=16, cus=1):
        self.L = lib(wg)
        self.n, self.wg = n, wg
        self.h = self.L.ref_create(n, cus)
        self.nodes = self.L.ref_num_nodes(self.h)

    def __del__(self):
        try:
            self.L.ref_destroy(self.h)
        except Exception:
            pass

    def set_bodies(self, pos3, mass, vel3=None, acc3=None):
        pos3 = np.ascontiguousarray(pos3, np.float32)
        mass = np.ascontiguousarray(mass, np.float32)
        v = None if vel3 is None else np.ascontiguousarray(vel3, np.float32)
        a = None if acc3 is None else np.ascontiguousarray(acc3, np.float32)
        self.L.ref_set_bodies(self.h, pos3.ctypes.data, None if v is None else v.ctypes.data, mass.ctypes.data,
                              None if a is None else a.ctypes.data)

    def set_boundary(self, box6):
        b = np.ascontiguousarray(box6, np.float32)
        self.L.ref_set_boundary(self.h, b.ctypes.data)

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"reference emulator: {what} returned {rc}")

    def bbox_as_wired(self):
        self._check(self.L.ref_bbox_as_wired(self.h), "bbox")
        return self.get(self.BOUNDARY, np.float32)[:6]

    def init(self):
        self._check(self.L.ref_init(self.h), "init")

    def build_tree(self):
        self._check(self.L.ref_build_tree(self.h), "build_tree")

    def saturate_tree(self):
        self._check(self.L.ref_saturate_tree(self.h), "saturate_tree")

    def calculate_force(self, theta, eps, G, dt, method):
        self._check(self.L.ref_calculate_force(self.h, theta, eps, G, dt, method), "calculate_force")

    def update_global(self, dt, G, method):
        self._check(self.L.ref_update_global(self.h, dt, G, method), "update")

    def update_local(self, dt, G, method):
        self._check(self.L.ref_update_local(self.h, dt, G, method), "update_local")

    def collision(self):
        self._check(self.L.ref_collision(self.h), "collision")

    def copy_vertices(self):
        out = np.zeros((self.n, 4), np.float32)
        self._check(self.L.ref_copy_vertices(self.h, out.ctypes.data), "copy_vertices")
        return out

    def get(self, which, dtype):
        nb = self.L.ref_get(self.h, which, None)
        a = np.zeros(nb // 4, dtype)
        self.L.ref_get(self.h, which, a.ctypes.data)
        return a

    def accelerations_via_leapfrog(self, theta, eps, G, kind="bh"):
        """Run a force kernel with method=Leapfrog, v=a=0 and dt=2: positions
        stay bit-identical (x + 0*dt) and v becomes exactly G*acc (acc*2*0.5),
        so every work-item sees step-start positions."""
        n = self.n
        z = np.zeros((n, 3), np.float32)
        pos = self.get(self.POS, np.float32)[: 3 * n].copy()
        mass = self.get(self.MASS, np.float32)[:n].copy()
        self.set_bodies(pos, mass, z, z)
        if kind == "bh":
            self.calculate_force(theta, eps, G, 2.0, 1)
        elif kind == "global":
            self.update_global(2.0, G, 1)
        elif kind == "local":
            self.update_local(2.0, G, 1)
        return self.get(self.VEL, np.float32).reshape(n, 3)
