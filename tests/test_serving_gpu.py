"""Serving loop: jobs that arrive while others run are admitted between rounds
and share every launch (the engine's lock-step ticks); each job's streamed
populations equal the same job run alone (FP64: 1e-12; mixed: 1e-6)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def specs():
    from qca_gb300 import workloads as W
    rng = np.random.default_rng(5)
    out = []
    for k, (alg, n, d, iv, chi, steps) in enumerate([("2tdvp", 9, 1, range(1, 2), 8, 12), ("1tdvp", 8, 2, range(2, 4), 8, 10),
                                                    ("2tdvp", 12, 2, range(2, 5), 16, 11), ("2tdvp", 7, 3, range(2, 4), 8, 7),
                                                    ("1tdvp", 10, 1, range(1, 2), 16, 13)]):
        out.append(W.ChainSpec(n, d, iv, chi, W.product_probabilities(rng, n), alg, 0.05, 1e-9, steps))
    return out


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-6)])
def test_each_job_same_alone_and_in_the_mix(precision, tol):
    from qca_gb300.serving import Server
    ss = specs()
    arrivals = [0.0, 0.0, 1.5, 3.0, 3.5]  # virtual arrival times; one round per time unit
    mix = Server(precision, hbm_budget_bytes=8 << 30, stream_every=5, ticks_per_round=8)
    for s, a in zip(ss, arrivals):
        mix.submit(s, a)
    t = 0.0
    while mix.pending or mix.active:
        mix.round(now=t)
        t += 1.0
    assert len(mix.done) == len(ss) and mix.max_overlap >= 3
    by_id = {j.job_id: j for j in mix.done}
    for k, s in enumerate(ss):
        alone = Server(precision, hbm_budget_bytes=8 << 30, stream_every=5, ticks_per_round=5)
        alone.submit(s, 0.0)
        while alone.pending or alone.active:
            alone.round(now=1e9)
        a = alone.done[0].stream
        m = by_id[k].stream
        assert [x[0] for x in a] == [x[0] for x in m]
        for (sa, pa), (sm, pm) in zip(a, m):
            assert np.abs(pa - pm).max() < tol, (k, sa)


def test_admission_waits_for_memory():
    from qca_gb300.serving import Server
    ss = [specs()[0]] * 3  # equal footprints
    probe = Server("mixed", hbm_budget_bytes=8 << 30)
    f = probe.footprint(ss[0])
    srv = Server("mixed", hbm_budget_bytes=2 * f - 1, stream_every=100)  # room for one job at a time
    for s in ss:
        srv.submit(s, 0.0)
    srv.round(now=0.0)
    assert len(srv.active) == 1 and len(srv.pending) == 2
    while srv.pending or srv.active:
        srv.round(now=1e9)
        assert srv.used <= srv.budget and len(srv.active) <= 1
    assert len(srv.done) == 3


def test_failed_job_is_retired_and_the_others_complete():
    """A job whose state holds a NaN fails with QCA_ERR_NAN inside a round; the
    server retires it and the other jobs complete with their results alone."""
    from qca_gb300.serving import Server
    ss = specs()[:3]
    bad = specs()[2]
    bad.p = bad.p.copy()
    bad.p[3] = np.nan
    srv = Server("fp64", hbm_budget_bytes=8 << 30, stream_every=5)
    for s in ss + [bad]:
        srv.submit(s, 0.0)
    while srv.pending or srv.active:
        srv.round(now=1e9)
    assert len(srv.done) == 3 and len(srv.failed) == 1 and srv.failed[0].job_id == 3
    alone = Server("fp64", hbm_budget_bytes=8 << 30, stream_every=5)
    alone.submit(ss[1], 0.0)
    while alone.pending or alone.active:
        alone.round(now=1e9)
    got = {j.job_id: j for j in srv.done}[1].stream
    assert np.abs(got[-1][1] - alone.done[0].stream[-1][1]).max() < 1e-12


def test_mixed_failure_is_restarted_in_fp64():
    """On the mixed-precision server a job that fails numerically is restarted on an
    FP64 engine; a job that fails there too (a NaN in its initial state) is retired,
    and the other jobs complete in mixed precision."""
    from qca_gb300 import _lib
    from qca_gb300.serving import Server
    ss = specs()[:3]
    bad = specs()[2]
    bad.p = bad.p.copy()
    bad.p[3] = np.nan
    srv = Server("mixed", hbm_budget_bytes=8 << 30, stream_every=5)
    for s in ss + [bad]:
        srv.submit(s, 0.0)
    while srv.pending or srv.active:
        srv.round(now=1e9)
    assert len(srv.done) == 3 and all(not j.escalated for j in srv.done)
    assert len(srv.failed) == 1 and srv.failed[0].job_id == 3 and srv.failed[0].escalated
    assert srv.escalations == {_lib.QCA_ERR_NAN: 1} and srv.failures == {_lib.QCA_ERR_NAN: 1}
