"""Request loop (hodlr_server_*) on the CPU: the scheduler in simulate mode
(no GPU work: builds and solves take a nominal time, x = b) and the byte
predictor.  The same scheduler drives the GPU engine in
tests/test_server_gpu.py."""
import os
import threading
import time

import numpy as np
import pytest

from hodlrnd_gb300 import _lib
from hodlrnd_gb300.kernels import Kernel
from hodlrnd_gb300.server import Server, predict_bytes


@pytest.fixture(scope="module", autouse=True)
def built_library():
    if not os.path.exists(_lib.LIB_PATH):
        from hodlrnd_gb300 import build
        build.build()


def cloud(n, ndim, seed):
    return np.random.default_rng(seed).uniform(0.0, 1.0, (n, ndim))


BOX3 = ([0.0] * 3, [1.0] * 3)
K = Kernel("inv_r", 1e-3, 1.0)


def test_predict_bytes_is_monotone_and_tracks_precision():
    small = predict_bytes(cloud(4000, 3, 1), BOX3, Nmax=64, eps_ACA=1e-8)
    big = predict_bytes(cloud(16000, 3, 1), BOX3, Nmax=64, eps_ACA=1e-8)
    assert 0 < small < big
    f64 = predict_bytes(cloud(16000, 3, 1), BOX3, Nmax=64, eps_ACA=1e-8, precision="fp64")
    f32 = predict_bytes(cloud(16000, 3, 1), BOX3, Nmax=64, eps_ACA=1e-8, precision="fp32_factors",
                        fp64_check=False)
    assert f32 < f64
    # with the FP64 check the FP64 factors are kept beside the FP32 ones
    f32c = predict_bytes(cloud(16000, 3, 1), BOX3, Nmax=64, eps_ACA=1e-8, precision="fp32_factors")
    assert f64 < f32c
    loose = predict_bytes(cloud(16000, 3, 1), BOX3, Nmax=64, eps_ACA=1e-4)
    assert loose <= f64


def test_single_request_round_trip():
    srv = Server(slots=2, simulate=True)
    b = np.random.default_rng(0).standard_normal(3000)
    t = srv.submit(cloud(3000, 3, 2), b, K, box=BOX3, eps_ACA=1e-8)
    x, r = srv.wait(t)
    assert np.array_equal(x, b)
    assert r["status"] == 0 and r["built"] == 1 and r["predicted_bytes"] > 0
    assert r["t_total_s"] >= r["t_build_s"]
    srv.close()


def test_resident_geometry_is_reused():
    srv = Server(slots=2, simulate=True)
    pts = cloud(5000, 3, 3)
    b = np.ones((5000, 2))
    x, r = srv.wait(srv.submit(pts, b, K, box=BOX3, key=11, eps_ACA=1e-8))
    assert r["built"] == 1
    x2, r2 = srv.wait(srv.submit(None, 2 * b, K, key=11, ndim=3, eps_ACA=1e-8))
    assert r2["built"] == 0 and np.array_equal(x2, 2 * b)
    st = srv.stats()
    assert st["resident"] == 1 and st["resident_hits"] == 1 and st["builds"] == 1
    srv.close()


def test_unknown_resident_key_fails_cleanly():
    srv = Server(slots=1, simulate=True)
    with pytest.raises(_lib.HodlrError) as e:
        srv.wait(srv.submit(None, np.ones(10), K, key=99, ndim=3))
    assert e.value.code == _lib.HODLR_ERR_STATE
    srv.close()


def test_budget_rejects_and_evicts_least_recently_used():
    pts = [cloud(6000, 3, 10 + i) for i in range(3)]
    need = max(predict_bytes(p, BOX3, Nmax=64, eps_ACA=1e-8) for p in pts)
    probe = Server(slots=1, simulate=True)
    kept = probe.wait(probe.submit(pts[0], np.ones(6000), K, box=BOX3, eps_ACA=1e-8))[1]["actual_bytes"]
    probe.close()
    assert 0 < kept < need  # the build's transient workspace is not kept
    # room for one build next to one resident geometry and a half
    budget = need + int(1.5 * kept)
    srv = Server(slots=1, memory_budget_bytes=budget, simulate=True)
    for i, p in enumerate(pts):
        srv.wait(srv.submit(p, np.ones(6000), K, box=BOX3, key=100 + i, eps_ACA=1e-8))
    st = srv.stats()
    assert st["evictions"] == 1 and st["resident"] == 2 and st["used_bytes"] <= budget
    # the first geometry was the least recently used one
    with pytest.raises(_lib.HodlrError) as e:
        srv.wait(srv.submit(None, np.ones(6000), K, key=100, ndim=3, eps_ACA=1e-8))
    assert e.value.code == _lib.HODLR_ERR_STATE
    x, r = srv.wait(srv.submit(None, np.ones(6000), K, key=102, ndim=3, eps_ACA=1e-8))
    assert r["built"] == 0
    tiny = Server(slots=1, memory_budget_bytes=need // 4, simulate=True)
    with pytest.raises(_lib.HodlrError) as e:
        tiny.wait(tiny.submit(pts[0], np.ones(6000), K, box=BOX3, eps_ACA=1e-8))
    assert e.value.code == _lib.HODLR_ERR_BUDGET
    srv.close()
    tiny.close()


def test_slots_bound_concurrency_and_everything_completes():
    srv = Server(slots=2, simulate=True)
    peak = [0]
    stop = threading.Event()

    def watch():
        while not stop.is_set():
            peak[0] = max(peak[0], srv.stats()["running"])
            time.sleep(0.0005)

    th = threading.Thread(target=watch)
    th.start()
    tickets = [srv.submit(cloud(20000, 2, i), np.full(20000, float(i)), K, box=([0.0] * 2, [1.0] * 2),
                          eps_ACA=1e-8) for i in range(8)]
    for i, t in enumerate(tickets):
        x, r = srv.wait(t)
        assert r["status"] == 0 and np.all(x == float(i))
    stop.set()
    th.join()
    assert 1 <= peak[0] <= 2
    st = srv.stats()
    assert st["completed"] == 8 and st["queued"] == 0 and st["running"] == 0
    srv.close()


def test_same_key_requests_run_one_at_a_time():
    srv = Server(slots=4, simulate=True)
    pts = cloud(8000, 3, 5)
    tickets = [srv.submit(pts if i == 0 else None, np.full(8000, float(i)), K, box=BOX3 if i == 0 else None,
                          key=42, ndim=3, eps_ACA=1e-8) for i in range(4)]
    res = [srv.wait(t) for t in tickets]
    assert [r["built"] for _, r in res] == [1, 0, 0, 0]
    assert all(np.all(x == float(i)) for i, (x, _) in enumerate(res))
    assert srv.stats()["builds"] == 1
    srv.close()


def test_wait_timeout_and_bad_ticket():
    srv = Server(slots=1, simulate=True)
    t = srv.submit(cloud(200000, 2, 1), np.ones(200000), K, box=([0.0] * 2, [1.0] * 2), eps_ACA=1e-8)
    with pytest.raises(TimeoutError):
        srv.wait(t, timeout=0.0)
    srv.wait(t)
    with pytest.raises(KeyError):
        srv.wait(t)
    srv.close()


def test_reuse_waits_behind_its_queued_build():
    """A request that reuses key K (no points) queued behind the request that
    builds K, while memory holds that build back, waits instead of failing."""
    big = cloud(120000, 2, 7)
    pts = cloud(6000, 3, 8)
    box2 = ([0.0] * 2, [1.0] * 2)
    need_big = predict_bytes(big, box2, Nmax=64, eps_ACA=1e-8)
    need = predict_bytes(pts, BOX3, Nmax=64, eps_ACA=1e-8)
    srv = Server(slots=2, memory_budget_bytes=max(need_big, need) + min(need_big, need) // 2, simulate=True)
    ta = srv.submit(big, np.ones(120000), K, box=box2, eps_ACA=1e-8)
    t1 = srv.submit(pts, np.ones(6000), K, box=BOX3, key=5, eps_ACA=1e-8)
    t2 = srv.submit(None, 2 * np.ones(6000), K, key=5, ndim=3, eps_ACA=1e-8)
    t3 = srv.submit(pts, 3 * np.ones(6000), K, box=BOX3, key=5, eps_ACA=1e-8)  # points given, still reused
    srv.wait(ta)
    r1, r2, r3 = srv.wait(t1)[1], srv.wait(t2)[1], srv.wait(t3)[1]
    assert (r1["built"], r2["built"], r3["built"]) == (1, 0, 0)
    assert srv.stats()["builds"] == 2
    srv.close()
