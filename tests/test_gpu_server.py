"""Served form: requests admitted while others run, advanced together, each
result identical to the same scene run alone and in agreement with the
oracle's run of that scene (src/sph.cpp:195-275 restated); the failure
path (injected on the host) fails every request, running or queued."""
import time

import numpy as np
import pytest

from _util import REL_TOL, rel_err

pytestmark = pytest.mark.gpu

FIELDS = ("pos", "vel", "rho", "prs")


def alone(sphx, s, pos, box, nsteps):
    with sphx.Scene(s, box, pos) as sc:
        sc.step(sphx.DT, nsteps)
        return sc.read()


def requests(sphx):
    scenes = sphx.batch_scenes(count=6, seed=11, nmin=300, nmax=5000)
    steps = [13, 4, 30, 9, 21, 7]
    return [(s, pos, box, k) for (s, pos, box), k in zip(scenes, steps)]


@pytest.mark.parametrize("budget", [None, 1])  # 1 byte: one scene resident at a time
def test_each_result_equals_alone(sphx_lib, budget):
    sphx = sphx_lib
    reqs = requests(sphx)
    with sphx.Server(budget_bytes=budget, steps_per_tick=5) as srv:
        tickets = []
        for k, (s, pos, box, n) in enumerate(reqs):
            tickets.append(srv.submit(s, box, pos, n))
            if k % 2 == 1:
                time.sleep(0.01)  # later requests arrive while earlier ones run
        for t in tickets:
            srv.wait(t, timeout=120)
        statuses = [srv.status(t) for t in tickets]
        results = [srv.result(t) for t in tickets]
        st = srv.stats()
    assert st.completed == len(reqs) and st.queued == 0 and st.live_scenes == 0
    for (s, pos, box, n), res, stt in zip(reqs, results, statuses):
        assert stt.state == sphx.Server.REQ_DONE and stt.steps_done == n
        assert stt.submit_s <= stt.admit_s <= stt.done_s
        ref = alone(sphx, s, pos, box, n)
        for f in FIELDS:
            assert np.array_equal(res[f], ref[f]), f


def test_overlap_in_the_mix(sphx_lib):
    """With room for all, later requests are admitted before earlier ones finish."""
    sphx = sphx_lib
    reqs = requests(sphx)
    with sphx.Server(steps_per_tick=2) as srv:
        tickets = [srv.submit(s, box, pos, n) for (s, pos, box, n) in reqs]
        for t in tickets:
            srv.wait(t, timeout=120)
        sts = [srv.status(t) for t in tickets]
        for t in tickets:
            srv.result(t)
    longest = max(range(len(reqs)), key=lambda k: reqs[k][3])
    others_admitted = [sts[k].admit_s for k in range(len(reqs)) if k != longest]
    assert max(others_admitted) < sts[longest].done_s


def test_served_results_vs_oracle(sphx_lib, port):
    """Served results against the oracle: one-step requests within the
    one-step tolerance on every field; requests of a few steps with positions
    within it too and velocities, densities and pressures within 1e-3 (chained
    steps let rounding grow, as in the multi-step parity tests)."""
    sphx = sphx_lib
    scenes = sphx.batch_scenes(count=8, seed=21, nmin=500, nmax=8000)
    steps = [1, 3, 1, 5, 2, 1, 4, 1]
    with sphx.Server(steps_per_tick=2) as srv:
        tickets = []
        for k, ((s, pos, box), n) in enumerate(zip(scenes, steps)):
            tickets.append(srv.submit(s, box, pos, n))
            if k == 3:
                time.sleep(0.01)
        for t in tickets:
            srv.wait(t, timeout=120)
        results = [srv.result(t) for t in tickets]
    for (s, pos, box), n, res in zip(scenes, steps, results):
        p, v, rho, prs = port.run(pos, None, sphx.args_array(s), sphx.DT, n, box=box.as_array())
        assert rel_err(res["pos"], p) < REL_TOL
        tol = REL_TOL if n == 1 else 1e-3
        assert rel_err(res["vel"], v) < tol
        assert rel_err(res["rho"], rho) < tol
        assert rel_err(res["prs"], prs) < tol


def test_failure_fails_running_and_queued_requests(sphx_lib):
    """A tick that fails (injected on the host, no GPU fault) stops the
    server: the running request and the one still queued behind the budget
    both end FAILED with the injected code, and waiting on the queued one
    returns that error at once instead of running out its timeout."""
    sphx = sphx_lib
    (s, pos, box), (s2, pos2, box2) = sphx.batch_scenes(count=2, seed=5, nmin=2000, nmax=3000)
    with sphx.Server(budget_bytes=1, steps_per_tick=1) as srv:
        running = srv.submit(s, box, pos, 100000)
        queued = srv.submit(s2, box2, pos2, 10)
        t0 = time.time()
        while srv.status(running).state != sphx.Server.REQ_RUNNING and time.time() - t0 < 60:
            time.sleep(0.005)
        assert srv.status(queued).state == sphx.Server.REQ_QUEUED
        srv.inject_failure(-2)
        t0 = time.time()
        for t in (running, queued):
            with pytest.raises(sphx.SphxError) as e:
                srv.wait(t, timeout=60)
            assert e.value.code == -2
            assert srv.status(t).state == sphx.Server.REQ_FAILED
        assert time.time() - t0 < 30
        with pytest.raises(sphx.SphxError):
            srv.submit(s2, box2, pos2, 1)  # a stopped server takes no requests
