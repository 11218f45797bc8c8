"""Served form: requests admitted while others run, advanced together, each
result identical to the same scene run alone."""
import time

import numpy as np
import pytest

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
