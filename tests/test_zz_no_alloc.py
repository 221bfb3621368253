"""nb_direct_accel_noalloc: the all-pairs accelerations for callers that
cannot allocate device memory (their host owns the memory budget, or their
frame loop must stay out of the CUDA allocator).  Its scratch is a fixed
array inside the library, so this test checks it against the handle-based
path (nb_create / nb_step with NB_BRUTE_FORCE_LOCAL) and against the CPU
oracle's FP32 sum, on two calls in a row so the second call sees the scratch
the first one left behind; with softening and without it (eps = 0 skips the
self pair), and on the default stream and on a stream the caller created.

Named to be collected last: a failure here leaves every other test run."""
import ctypes
import glob
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def cudart():
    cands = ["libcudart.so.13", "libcudart.so"] + sorted(glob.glob("/usr/local/cuda/lib64/libcudart.so*"))
    for c in cands:
        try:
            L = ctypes.CDLL(c)
            L.cudaMalloc.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]
            L.cudaMemset.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t]
            L.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
            L.cudaFree.argtypes = [ctypes.c_void_p]
            L.cudaDeviceSynchronize.argtypes = []
            L.cudaStreamCreate.argtypes = [ctypes.POINTER(ctypes.c_void_p)]
            L.cudaStreamSynchronize.argtypes = [ctypes.c_void_p]
            L.cudaStreamDestroy.argtypes = [ctypes.c_void_p]
            return L
        except OSError:
            continue
    pytest.skip("libcudart not found")


def term_sums(pos, mass, G):
    """G * sum_j m_j |r_ij|^-2 per body (eps = 0): the sum of the magnitudes
    of the pair terms."""
    x = pos.astype(np.float64)
    out = np.zeros(len(x))
    for i0 in range(0, len(x), 512):
        d2 = np.sum((x[i0:i0 + 512, None, :] - x[None, :, :]) ** 2, axis=2)
        idx = np.arange(i0, min(len(x), i0 + 512))
        d2[idx - i0, idx] = np.inf
        out[i0:i0 + 512] = G * np.sum(mass[None, :] / d2, axis=1)
    return out


def rel_to_typical(a, b):
    scale = np.sqrt(np.mean(np.sum(b.astype(np.float64) ** 2, axis=1)))
    return float(np.max(np.linalg.norm(a.astype(np.float64) - b, axis=1)) / scale)


@pytest.mark.parametrize("n,eps,own_stream", [(5000, 0.05, False), (65536, 0.05, False), (4096, 0.0, False),
                                               (20000, 0.05, True)])
def test_noalloc_matches_handle_path_twice(gpu, oracle, n, eps, own_stream):
    nb = gpu
    L = nb.load()
    rng = np.random.default_rng(n)
    pos = rng.normal(size=(n, 3)).astype(np.float32)
    m = np.exp(0.5 * rng.normal(size=n))
    mass = (m / m.sum()).astype(np.float32)
    G = 1.0
    sim = nb.Simulation(num_of_bodies=n, algo_config=nb.BRUTE_FORCE_LOCAL, epsilon=eps, direct_epsilon=eps,
                        gravitational_constant=G)
    sim.set_state(pos, mass)
    sim.step(0.0, 1)  # dt = 0: accelerations only
    _, _, acc_ref, _ = sim.get_state()
    body = sim.device_view().body_pm  # float4 {x,y,z,m}, the same positions
    acc_orc = oracle.direct_fp32(pos, mass, eps, G)

    rt = cudart()
    out = ctypes.c_void_p()
    stream = ctypes.c_void_p()
    if own_stream:
        assert rt.cudaStreamCreate(ctypes.byref(stream)) == 0
    assert rt.cudaMalloc(ctypes.byref(out), 16 * n) == 0  # the caller's own output buffer
    try:
        host = np.zeros((n, 4), np.float32)
        for call in range(2):
            assert rt.cudaMemset(out, 0xFF, 16 * n) == 0  # poison: every entry must be written
            assert rt.cudaDeviceSynchronize() == 0
            st = L.nb_direct_accel_noalloc(body, n, eps, G, out, stream if own_stream else None)
            assert st == nb.OK, (call, st)
            assert rt.cudaMemcpy(host.ctypes.data, out, 16 * n, 2) == 0  # device to host
            assert np.all(np.isfinite(host))
            assert np.all(host[:, 3] == 0.0)
            err = rel_to_typical(host[:, :3], acc_ref)
            assert err < 2e-5, (call, err)
            if eps > 0.0:
                err = rel_to_typical(host[:, :3], acc_orc)
            else:
                # unsoftened, a close pair makes one body's |a| many times the
                # typical one: measure each body against the sum of its terms'
                # magnitudes, which bounds the rounding of both sums
                err = float(np.max(np.linalg.norm(host[:, :3] - acc_orc, axis=1) / term_sums(pos, mass, G)))
            assert err < 2e-5, (call, "oracle", err)
    finally:
        rt.cudaFree(out)
        if own_stream:
            rt.cudaStreamDestroy(stream)
    sim.close()


def test_noalloc_rejects_out_of_range(gpu):
    nb = gpu
    L = nb.load()
    rt = cudart()
    buf = ctypes.c_void_p()
    n = nb.NOALLOC_MAX_BODIES + 1
    assert rt.cudaMalloc(ctypes.byref(buf), 16 * n) == 0
    try:
        assert L.nb_direct_accel_noalloc(buf, n, 0.01, 1.0, buf, None) == nb.ERR_INVALID_ARGUMENT
        assert L.nb_direct_accel_noalloc(buf, 0, 0.01, 1.0, buf, None) == nb.ERR_INVALID_ARGUMENT
        misaligned = ctypes.c_void_p(buf.value + 4)
        assert L.nb_direct_accel_noalloc(misaligned, 16, 0.01, 1.0, buf, None) == nb.ERR_INVALID_ARGUMENT
    finally:
        rt.cudaFree(buf)
