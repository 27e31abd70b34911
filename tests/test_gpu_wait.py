"""Bounded host waits: a wait for the GPU that runs past qpc_set_wait_limit returns
QPC_ERR_TIMEOUT instead of blocking, and the handle stays usable afterwards.

The delay is made on the host, not on the GPU: a host function enqueued on the
handle's stream (cudaLaunchHostFunc) sleeps past a short limit, so the stream is
not done when the engine's next call waits for it.  No kernel is made to spin,
fault or hang."""
import ctypes
import threading
import time

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _cudart():
    """The CUDA runtime this process has loaded (the engine library links it)."""
    paths = []
    with open("/proc/self/maps") as fh:
        for line in fh:
            part = line.split()[-1]
            if "libcudart.so" in part and part not in paths:
                paths.append(part)
    for p in paths + ["libcudart.so.13", "libcudart.so"]:
        try:
            return ctypes.CDLL(p)
        except OSError:
            continue
    pytest.skip("no CUDA runtime library found")


def test_wait_limit_argument_checks(q):
    with pytest.raises(q.QpcError) as e:
        q.set_wait_limit(0.0)
    assert e.value.code == 1
    with pytest.raises(q.QpcError):
        q.set_wait_limit(float("nan"))


def test_wait_past_limit_returns_timeout(q):
    n_r, p, n_l, dt = 64, 6, 6, 0.05
    S, R, _, _, H = q.radial_setup(n_r, p, n_l, q.linear_knots(n_r, p, 0.0, 30.0))
    c0, _ = q.ground_state(S, H, n_l)
    prop = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, S, R, H, dt)
    prop.put(c0[None])
    n0 = prop.norm()[0]
    q.load()
    rt = _cudart()
    rt.cudaLaunchHostFunc.restype = ctypes.c_int
    rt.cudaLaunchHostFunc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    HOSTFN = ctypes.CFUNCTYPE(None, ctypes.c_void_p)
    done = threading.Event()

    def sleeper(_):
        time.sleep(1.5)
        done.set()

    cb = HOSTFN(sleeper)
    old = q.get_wait_limit()
    try:
        q.set_wait_limit(0.25)
        assert rt.cudaLaunchHostFunc(ctypes.c_void_p(prop.stream()), ctypes.cast(cb, ctypes.c_void_p), None) == 0
        t0 = time.perf_counter()
        with pytest.raises(q.QpcError) as e:
            prop.norm()
        waited = time.perf_counter() - t0
        assert e.value.code == 6, e.value          # QPC_ERR_TIMEOUT
        assert 0.2 < waited < 1.4, waited          # gave up at the limit, before the host function ended
    finally:
        assert done.wait(30)
        q.set_wait_limit(old)
    # the queued work completed; the handle is usable and its state unchanged
    assert abs(prop.norm()[0] - n0) < 1e-14 * n0
    prop.propagate()
    ref = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, S, R, H, dt)
    ref.put(c0[None])
    ref.propagate()
    assert rel_l2(prop.get(), ref.get()) < 1e-15
    prop.close()
    ref.close()
    del cb
