"""The simulation server (pcg_server_*): continuous batching of independent
requests on one GPU.

Each result must be the same alone and in the mix: every request is also run by
itself with pcg_solve, and the served field must agree within the FP32 tolerance
(1e-5 relative per substrate; the only difference is the order of floating-point
atomic sums in the ballots), with identical ballot counts.  Requests arrive while
others run, so admission happens between ticks of a running batch.  Also covered:
refusal of a request that can never fit the memory limit, waiting for memory held
by running requests, cancellation, a malformed request, and the statistics.
"""
import time

import numpy as np
import pytest

from physicore_gb300 import workloads as W
from test_gpu_golden import rel_err

pytestmark = pytest.mark.gpu

FP32_RTOL = 1e-5


def _problems(n=10, seed0=100):
    out = []
    for k in range(n):
        p = W.random_small(seed0 + k, max_side=40)
        out.append((p, 3 + (7 * k) % 29))
    return out


def _wait_all(server, count, timeout=60.0):
    got = []
    t0 = time.time()
    while len(got) < count and time.time() - t0 < timeout:
        got += server.poll(64, wait_ms=50)
    assert len(got) == count, f"{len(got)} of {count} requests came back"
    return {r["tag"]: r for r in got}


def test_served_results_equal_alone(pcg):
    probs = _problems()
    alone = []
    for p, steps in probs:
        s = W.apply(pcg.Solver(pcg.FP32), p, with_field=False)  # requests start from the initial conditions
        s.solve(steps)
        alone.append((s.get_field(), s.get_counts() if s.A else None))
        s.close()
    srv = pcg.Server(pcg.FP32, steps_per_tick=4, reserve_bytes=0)
    half = len(probs) // 2
    outs = {}

    def submit(k, p, steps):
        s = W.apply(pcg.Solver(pcg.FP32), p, initialize=False)
        if k % 2:  # odd requests: the server reads the field back before returning them
            nx, ny, nz = s.grid
            outs[k] = np.full((s.S, nz, ny, nx), np.nan, np.float32)
            srv.submit(s, steps, k, out=outs[k], layout=pcg.LAYOUT_PLANAR)
        else:
            srv.submit(s, steps, k)

    for k, (p, steps) in enumerate(probs[:half]):
        submit(k, p, steps)
    time.sleep(0.05)  # the first ones are running when the rest arrive
    for k, (p, steps) in enumerate(probs[half:], start=half):
        submit(k, p, steps)
    res = _wait_all(srv, len(probs))
    for k, (p, steps) in enumerate(probs):
        r = res[k]
        assert r["status"] == "done", r
        s = r["solver"]
        e = rel_err(s.get_field(), alone[k][0])
        assert e <= FP32_RTOL, f"{p['name']}: served vs alone {e:.3e}"
        if k in outs:
            assert np.array_equal(outs[k], s.get_field(layout=pcg.LAYOUT_PLANAR, dtype=np.float32)), k
        if alone[k][1] is not None:
            assert np.array_equal(s.get_counts(), alone[k][1]), p["name"]
        assert 0 <= r["t_submit"] <= r["t_admit"] <= r["t_done"]
        s.close()
    st = srv.stats()
    assert st["completed"] == len(probs) and st["failed"] == 0 and st["in_flight"] == 0
    assert st["vss"] == sum(steps * W.apply(pcg.Solver(pcg.FP32), p, initialize=False).voxels * len(p["D"])
                            for p, steps in probs)
    srv.close()


def test_refusal_wait_cancel_and_malformed(pcg):
    p, _ = _problems(1, 300)[0]
    probe = W.apply(pcg.Solver(pcg.FP32), p, initialize=False)
    need = probe.estimate_device_bytes()
    probe.close()
    # a limit below one request: refused at once
    srv = pcg.Server(pcg.FP32, memory_limit_bytes=need // 2, reserve_bytes=0)
    srv.submit(W.apply(pcg.Solver(pcg.FP32), p, initialize=False), 5, 1)
    r = _wait_all(srv, 1)[1]
    assert r["status"] == "refused" and r["t_admit"] < 0, r
    r["solver"].close()
    srv.close()
    # room for one request at a time: the second waits for the first
    srv = pcg.Server(pcg.FP32, memory_limit_bytes=int(need * 1.5), reserve_bytes=0, steps_per_tick=2)
    srv.submit(W.apply(pcg.Solver(pcg.FP32), p, initialize=False), 20, 1)
    srv.submit(W.apply(pcg.Solver(pcg.FP32), p, initialize=False), 20, 2)
    res = _wait_all(srv, 2)
    assert res[1]["status"] == res[2]["status"] == "done"
    assert res[2]["t_admit"] >= res[1]["t_done"] - 1e-3
    for r in res.values():
        r["solver"].close()
    # cancellation of a long request while it runs
    srv.submit(W.apply(pcg.Solver(pcg.FP32), p, initialize=False), 10 ** 9, 3)
    time.sleep(0.2)
    srv.cancel(3)
    r = _wait_all(srv, 1)[3]
    assert r["status"] == "cancelled", r
    r["solver"].close()
    # malformed: no substrates -> rejected at submit
    bad = pcg.Solver(pcg.FP32)
    bad.set_mesh(3, (0, 0, 0), (100, 100, 100), (20, 20, 20))
    with pytest.raises(pcg.PcgError):
        srv.submit(bad, 5, 4)
    # an initialised context is not a request
    init = W.apply(pcg.Solver(pcg.FP32), p)
    with pytest.raises(pcg.PcgError):
        srv.submit(init, 5, 5)
    st = srv.stats()
    assert st["cancelled"] == 1 and st["completed"] == 2
    srv.close()
