"""Host-side logic that needs no GPU: the product's MPO / MPS builders against the
reference fixtures, and the C-ABI library's exported symbols."""
import ctypes
import os
import re

import numpy as np
import pytest

from qca_gb300 import _lib
from qca_gb300.tensor_networks import MPO, MPS, Rules, rule_from_mpo

from conftest import ROOT

RULES = [(1, 1, 2), (1, 2, 4), (1, 2, 5), (2, 1, 2), (2, 2, 4), (2, 2, 5), (3, 1, 2), (3, 2, 4), (3, 2, 5)]


@pytest.mark.parametrize("d,lo,hi", RULES)
def test_mpo_builder_matches_reference(golden, d, lo, hi):
    g = golden("mpo_rules.npz")
    W = MPO.hamiltonian_from_rules(Rules(6, range(lo, hi), d)).W
    key = f"d{d}_{lo}{hi}"
    assert np.array_equal(W[2], g[key + "_bulk"])
    assert np.array_equal(W[0], g[key + "_first"])
    assert np.array_equal(W[-1], g[key + "_last"])


@pytest.mark.parametrize("d,lo,hi", RULES)
def test_rule_recovered_from_plain_w_list(golden, d, lo, hi):
    g = golden("mpo_rules.npz")
    key = f"d{d}_{lo}{hi}"

    class Bare:  # what the reference's MPO exposes: only W
        W = [g[key + "_first"]] + [g[key + "_bulk"]] * 4 + [g[key + "_last"]]

    dist, interval = rule_from_mpo(Bare)
    # equivalent rules (e.g. [2,4) and [2,5) at distance 1) give the same H
    from oracle import qca_oracle as O
    a = O.sparse_rule_hamiltonian(7, dist, interval).toarray()
    b = O.sparse_rule_hamiltonian(7, d, range(lo, hi)).toarray()
    assert np.array_equal(a, b)


def test_mps_constructors_match_reference(golden):
    m = golden("measure_case.npz")
    A = MPS.from_vector(m["psi"])
    assert np.array_equal(np.array([a.shape for a in A.A]), m["from_vector_shapes"])
    assert np.abs(A.as_vector() - m["as_vector"]).max() < 1e-14
    p = m["prod_p"]
    v = MPS.from_density_distribution(p).as_vector()
    assert abs(np.linalg.norm(v) - 1.0) < 1e-14


def test_mps_npz_roundtrip(tmp_path):
    A = MPS.from_vector(np.random.default_rng(1).standard_normal(32) + 0j)
    path = tmp_path / "s.npz"
    A.write_to_file(str(path))
    B = MPS.from_file(str(path))
    for a, b in zip(A.A, B.A):
        assert np.array_equal(a, b)


def test_classical_evolution_blinker():
    from qca_gb300.algorithms import Algorithm
    rules = Rules(5, range(1, 2), 1)
    first = np.array([0.0, 0.0, 1.0, 0.0, 0.0])
    heat = Algorithm.classical_evolution(first, rules, 3)
    assert heat.shape == (3, 5)
    assert np.array_equal(heat[1], [0.0, 1.0, 1.0, 1.0, 0.0])


def _header_functions():
    src = open(os.path.join(ROOT, "include", "qca_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(qca_\w+)\s*\(", src, re.M)))


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    names = _header_functions()
    assert len(names) >= 20
    for name in names:
        assert hasattr(lib, name), name
    assert set(_lib.SIGNATURES) | {"qca_last_error", "qca_version"} == set(names)


def test_library_reports_errors_without_a_gpu():
    lib = _lib.load()
    out = ctypes.c_void_p()
    # invalid arguments are rejected before any device call
    st = lib.qca_exact_create(1, 1, 1, 2, 0, 30, ctypes.byref(out))
    assert st == _lib.QCA_ERR_INVALID
    assert b"invalid" in lib.qca_last_error()
    with pytest.raises(_lib.QcaError):
        _lib.check(st)


def test_footprint_estimates():
    size = ctypes.c_size_t()
    _lib.call("qca_exact_footprint", 24, _lib.QCA_PREC_FP64, 30, ctypes.byref(size))
    assert size.value >= 30 * 16 * (1 << 24)


def test_chain_footprint_grows_with_bond_cap():
    from qca_gb300.algorithms import chain_desc
    from qca_gb300 import workloads as W
    sizes = []
    for chi in (16, 64, 256):
        s = W.single_chain(40, 2, range(2, 4), chi, seed=1)
        mps = s.mps()
        d, keep = chain_desc(mps.A, s.mpo().W, "2tdvp", 0.05, chi, 1e-10)
        size = ctypes.c_size_t()
        _lib.call("qca_chain_footprint", ctypes.byref(d), _lib.QCA_PREC_MIXED, ctypes.byref(size))
        sizes.append(size.value)
    assert sizes[0] < sizes[1] < sizes[2]
    assert sizes[2] > 16 * sizes[0]


def test_poisson_trace_shape():
    from qca_gb300 import workloads as W
    jobs = W.poisson_jobs(rate=200.0, duration=2.0, seed=3)
    assert 300 < len(jobs) < 500
    assert all(12 <= j.spec.n <= 128 and j.spec.distance in (1, 2) for j in jobs)
    assert all(50 <= j.spec.steps <= 500 for j in jobs)


def _fake_serving(monkeypatch, fail=None):
    """The serving module with its engine faked on the host: every tick of every
    chain completes one local update; a chain completes a time step after
    ``ticks_per_step`` ticks; every engine call takes one second of a fake clock.
    ``fail`` maps a chain id to the tick at which that chain reports QCA_ERR_NAN."""
    fail = fail or {}
    from qca_gb300 import serving
    clock = {"t": 0.0}
    chains = {}
    calls = []
    ticks_per_step = 3

    class FakeEngine:
        def __init__(self, *a, **k):
            self.h = ctypes.c_void_p(1)

    def fake_call(name, *args):
        calls.append(name)
        if name == "qca_chain_footprint":
            args[2]._obj.value = 1000
        elif name == "qca_chain_add":
            fake_call.next_id += 1
            args[3]._obj.value = fake_call.next_id
            chains[fake_call.next_id] = {"done": 0, "todo": 0, "tick": 0}
        elif name == "qca_chain_schedule":
            chains[args[1]]["todo"] += args[2]
        elif name == "qca_engine_advance":
            ids = [args[1][i] for i in range(args[2])]
            failed = []
            for _ in range(args[3]):
                for cid in ids:
                    c = chains[cid]
                    if c.get("status"):
                        continue
                    c["ticks"] = c.get("ticks", 0) + 1
                    if fail.get(cid) == c["ticks"]:
                        c["status"] = serving._lib.QCA_ERR_NAN
                        failed.append(cid)
                        continue
                    if c["todo"] > 0:
                        c["tick"] += 1
                        if c["tick"] == ticks_per_step:
                            c["tick"] = 0
                            c["todo"] -= 1
                            c["done"] += 1
            clock["t"] += 1.0
            if failed:
                raise serving._lib.QcaError(serving._lib.QCA_ERR_NAN, f"chain {failed[0]}: non-finite values")
        elif name == "qca_engine_step_chains":
            c = chains[args[1][0]]
            if c.get("status"):
                raise serving._lib.QcaError(c["status"], f"chain {args[1][0]} failed in an earlier step (at tick {fail[args[1][0]]})")
        elif name == "qca_chain_progress":
            c = chains[args[1]]
            args[2][0], args[2][1], args[2][2], args[2][3] = c["done"], c["todo"], int(c["tick"] > 0), c.get("status", 0)
        elif name == "qca_chain_remove":
            del chains[args[1]]
    fake_call.next_id = 0
    monkeypatch.setattr(serving, "_Engine", FakeEngine)
    monkeypatch.setattr(serving._lib, "call", fake_call)
    monkeypatch.setattr(serving.time, "perf_counter", lambda: clock["t"])
    monkeypatch.setattr(serving.time, "sleep", lambda s: clock.__setitem__("t", clock["t"] + s))
    return serving, clock, calls


def test_serving_jobs_progress_at_their_own_pace(monkeypatch):
    """The serving loop's host logic with the engine faked: every admitted job has
    its next streaming interval scheduled, a round advances all of them by a few
    ticks, a short job finishes and leaves while a long one keeps running, and a
    job arriving later is admitted at the next round; a bounded run stops at its
    time limit."""
    from qca_gb300.workloads import ChainSpec
    serving, clock, calls = _fake_serving(monkeypatch)
    short = ChainSpec(n=6, distance=1, interval=range(1, 2), chi=4, p=np.full(6, 0.5), steps=2)
    long_ = ChainSpec(n=6, distance=1, interval=range(1, 2), chi=4, p=np.full(6, 0.5), steps=100)
    srv = serving.Server("mixed", hbm_budget_bytes=1 << 30, stream_every=4, max_resident=5, ticks_per_round=6)
    srv.submit(short, arrival=0.0)
    srv.submit(long_, arrival=0.0)
    srv.submit(short, arrival=1.5)
    srv.round(now=0.0)  # 6 ticks: the short job completes its 2 steps, the long one 2 of its first 4
    assert [j.job_id for j in srv.done] == [0]
    assert [j.job_id for j in srv.active] == [1] and srv.active[0].steps_done == 0
    srv.round(now=2.0)  # the late job joins; the long job reaches step 4 and streams
    assert [j.job_id for j in srv.done] == [0, 2]
    assert srv.active[0].steps_done == 4 and len(srv.active[0].stream) == 1
    rep = srv.run([], time_limit=3.5)
    assert rep["elapsed_s"] <= 3.5 + 1.0 and rep["jobs_done"] == 2 and rep["jobs_active"] == 1


def test_serving_retires_a_failed_job_with_the_engine_message(monkeypatch):
    """A job whose chain fails numerically is retired with the engine's account of
    the failure (status code and message) while the others complete; the report
    counts it by status and lists it with its specification."""
    from qca_gb300.workloads import ChainSpec
    serving, clock, calls = _fake_serving(monkeypatch, fail={2: 4})
    spec = ChainSpec(n=6, distance=1, interval=range(1, 2), chi=4, p=np.full(6, 0.5), steps=3)
    srv = serving.Server("mixed", hbm_budget_bytes=1 << 30, stream_every=2, max_resident=4, ticks_per_round=5,
                         escalate=False)
    for _ in range(3):
        srv.submit(spec, arrival=0.0)
    rep = srv.run([], time_limit=None)
    assert rep["jobs_done"] == 2 and rep["jobs_failed"] == 1 and rep["jobs_escalated"] == 0
    assert rep["failures_by_status"] == {str(serving._lib.QCA_ERR_NAN): 1}
    assert "chain 2: non-finite values" in rep["first_failure"]
    (f,) = rep["failed_jobs"]
    assert f["job"] == 1 and f["n"] == 6 and f["chi"] == 4 and f["algorithm"] == "2tdvp"
    assert "failed in an earlier step (at tick 4)" in f["error"]


def test_serving_restarts_a_failed_mixed_job_in_fp64(monkeypatch):
    """On the mixed-precision server a job whose chain fails numerically is restarted
    from its initial state on an FP64 engine (a second engine, created then), keeps
    its arrival time, and completes; the site updates of its failed attempt are not
    counted; the report counts the escalation by status."""
    from qca_gb300.workloads import ChainSpec
    serving, clock, calls = _fake_serving(monkeypatch, fail={2: 4})
    engines = []
    base = serving._Engine

    class Recording(base):
        def __init__(self, *a, **k):
            super().__init__(*a, **k)
            engines.append(a[0] if a else None)

    monkeypatch.setattr(serving, "_Engine", Recording)
    spec = ChainSpec(n=6, distance=1, interval=range(1, 2), chi=4, p=np.full(6, 0.5), steps=3)
    srv = serving.Server("mixed", hbm_budget_bytes=1 << 30, stream_every=2, max_resident=4, ticks_per_round=5)
    for _ in range(3):
        srv.submit(spec, arrival=0.0)
    rep = srv.run([], time_limit=None)
    assert rep["jobs_done"] == 3 and rep["jobs_failed"] == 0
    assert rep["jobs_escalated"] == 1 and rep["escalations_by_status"] == {str(serving._lib.QCA_ERR_NAN): 1}
    assert engines == [serving._lib.QCA_PREC_MIXED, serving._lib.QCA_PREC_FP64]
    (j,) = [j for j in srv.done if j.escalated]
    assert j.job_id == 1 and j.arrival == 0.0 and j.precision == serving._lib.QCA_PREC_FP64
    assert j.error is None and "failed in an earlier step" in j.mixed_error
    assert rep["site_updates"] == 3 * 3 * spec.site_updates_per_step()


@pytest.mark.parametrize("share", [1, 4])
def test_serving_light_jobs_take_extra_ticks(monkeypatch, share):
    """A job whose local updates cost far less than the costliest resident job's
    (chi 4 against chi 64) gets ``light_share`` times the ticks of a round, in a
    call of its own (the heavy job's chain is not in it), and finishes in fewer
    rounds; with a share of 1 both progress alike."""
    from qca_gb300.workloads import ChainSpec
    serving, clock, calls = _fake_serving(monkeypatch)
    advanced = []
    real = serving._lib.call

    def spy(name, *args):
        if name == "qca_engine_advance":
            advanced.append(([args[1][i] for i in range(args[2])], args[3]))
        return real(name, *args)

    monkeypatch.setattr(serving._lib, "call", spy)
    heavy = ChainSpec(n=6, distance=1, interval=range(1, 2), chi=64, p=np.full(6, 0.5), steps=3)
    light = ChainSpec(n=6, distance=1, interval=range(1, 2), chi=4, p=np.full(6, 0.5), steps=3)
    srv = serving.Server("mixed", hbm_budget_bytes=1 << 30, stream_every=10, max_resident=4, ticks_per_round=3,
                         light_share=share)
    srv.submit(heavy, arrival=0.0)
    srv.submit(light, arrival=0.0)
    srv.round(now=0.0)  # 3 ticks = 1 step for both; the light job gets 3 (share - 1) more ticks
    if share == 1:
        assert advanced == [([1, 2], 3)] and srv.done == []
    else:
        assert advanced == [([1, 2], 3), ([2], 9)]
        assert [j.job_id for j in srv.done] == [1] and srv.active[0].job_id == 0
    rep = srv.run([], time_limit=None)
    assert rep["jobs_done"] == 2


def test_bench_roofline_arithmetic():
    """bench.py's roofline object from per-class kernel statistics (the numbers of
    a recorded batched run): the GEMM class against the measured bf16 peak, the
    derived 3xTF32 ceiling, the whole-step rate, shares that sum to one, and a
    line that serialises to JSON."""
    import json
    import sys
    sys.path.insert(0, ROOT)
    import bench
    ms = 3 * 3476.8
    ks = {k: {"launches": 1000.0, "ms": 0.0, "flops": 0.0, "bytes": 0.0} for k in bench.KCLASS}
    ks["gemm"].update(ms=4373.0, flops=16.92e12 * 4.373)
    ks["svd"].update(ms=3387.0, flops=0.653e12 * 3.387)
    ks["lanczos_vec"].update(ms=880.0)
    ks["mpo_apply"].update(ms=584.0)
    ks["lanczos_exp"].update(ms=317.0)
    pk = {"hbm_gbs": 6800.3, "bf16_tflops": 1917.0, "bf16_tflops_sustained": 1700.0, "source": "measured"}
    r = bench.tdvp_roofline(ks, pk, 3, ms)
    assert r["kernel"] == "gemm" and r["bound"] == "tensor" and r["unit"] == "TFLOP/s"
    assert r["dominant_class"] == "gemm"
    assert abs(r["achieved"] - 16.92) < 1e-3
    assert abs(r["frac"] - 16.92 / 1917.0) < 1e-5
    assert abs(r["peak_3xtf32_derived"] - 319.5) < 0.1
    assert abs(r["frac_of_3xtf32"] - 16.92 / 319.5) < 1e-3
    assert abs(r["step_algorithmic_tflops"] - (16.92 * 4.373 + 0.653 * 3.387) / (ms / 1e3)) < 1e-3
    assert abs(sum(r["kernel_time_share"].values()) - 1.0) < 1e-3
    json.dumps(r)
    # no kernel time recorded: no division by zero
    empty = {k: {"launches": 0.0, "ms": 0.0, "flops": 0.0, "bytes": 0.0} for k in bench.KCLASS}
    json.dumps(bench.tdvp_roofline(empty, pk, 1, 0.0))


def test_chain_desc_packing_roundtrip():
    """chain_desc packs the MPS and MPO tensors concatenated in C order (the layout
    qca_chain_desc documents) with their bond arrays; unpack_mps inverts it."""
    from qca_gb300.algorithms import chain_desc, unpack_mps
    rng = np.random.default_rng(3)
    n = 5
    D = [1, 2, 4, 3, 2, 1]
    A = [rng.standard_normal((2, D[i], D[i + 1])) + 1j * rng.standard_normal((2, D[i], D[i + 1])) for i in range(n)]
    W = MPO.hamiltonian_from_rules(Rules(n, range(1, 2), 1)).W
    d, keep = chain_desc(A, W, "2tdvp", 0.05, 16, 1e-10)
    mps_bonds, mpo_bonds, mps, mpo = keep
    assert list(mps_bonds) == D
    assert list(mpo_bonds) == [W[0].shape[2]] + [w.shape[3] for w in W]
    assert d.n_sites == n and d.algorithm == _lib.QCA_ALGO_2TDVP and d.max_bond_dim == 16
    flat = mps.view(np.complex128)
    assert flat.size == sum(a.size for a in A)
    back = unpack_mps(flat, D)
    assert all(np.array_equal(x, y) for x, y in zip(back, A))
    # the MPO block of site i starts after the blocks of sites < i, C order
    off = 0
    for w in W:
        assert np.array_equal(mpo.view(np.complex128)[off:off + w.size].reshape(w.shape), w)
        off += w.size
    with pytest.raises(ValueError):
        chain_desc(A, W[:-1], "2tdvp", 0.05, 16, 1e-10)
    with pytest.raises(ValueError):
        chain_desc(A, W, "exact", 0.05, 16, 1e-10)


def test_serving_callbacks_run_on_a_completion_thread(monkeypatch):
    """Streamed populations reach the callback on the completion thread, in the
    order they were measured, all of them by the time run() returns; a callback
    that raises is recorded and the loop keeps serving."""
    import threading
    from qca_gb300.workloads import ChainSpec
    serving, clock, stepped = _fake_serving(monkeypatch)
    seen, threads = [], set()

    def on_pop(job_id, step, pop):
        threads.add(threading.get_ident())
        seen.append((job_id, step, pop.shape))
        if job_id == 1 and step == 2:
            raise RuntimeError("consumer failed")

    srv = serving.Server("mixed", hbm_budget_bytes=1 << 30, stream_every=1, max_resident=4,
                         on_populations=on_pop)
    spec = ChainSpec(n=5, distance=1, interval=range(1, 2), chi=4, p=np.full(5, 0.5), steps=3)
    for _ in range(2):
        srv.submit(spec, arrival=0.0)
    rep = srv.run([], time_limit=None)
    assert rep["jobs_done"] == 2
    assert seen == [(0, 1, (5,)), (1, 1, (5,)), (0, 2, (5,)), (1, 2, (5,)), (0, 3, (5,)), (1, 3, (5,))]
    assert threading.get_ident() not in threads and len(threads) == 1
    assert len(srv.callback_errors) == 1



def test_batched_workload_definition():
    """The benchmark's batched workload: 256 chains drawn from one seed with
    N ~ U{16..96}, distance in {1,2,3}, interval in {[1,1],[2,3],[2,4]}, bond cap in
    {32,64,128}, random product states, dt = 0.05; the same seed gives the same
    chains, each rank's seed its own."""
    from qca_gb300 import workloads as W
    a, b, c = W.chain_mix(256, seed=1000), W.chain_mix(256, seed=1000), W.chain_mix(256, seed=1001)
    assert len(a) == 256
    assert all(16 <= s.n <= 96 for s in a)
    assert {s.distance for s in a} == {1, 2, 3}
    assert {(s.interval.start, s.interval.stop) for s in a} == {(1, 2), (2, 4), (2, 5)}
    assert {s.chi for s in a} == {32, 64, 128}
    assert all(s.dt == 0.05 and s.algorithm == "2tdvp" and s.p.shape == (s.n,) for s in a)
    assert all(np.all((s.p >= 0) & (s.p <= 1)) for s in a)
    assert [(s.n, s.chi, s.distance) for s in a] == [(s.n, s.chi, s.distance) for s in b]
    assert all(np.array_equal(x.p, y.p) for x, y in zip(a, b))
    assert [(s.n, s.chi) for s in a] != [(s.n, s.chi) for s in c]
    assert sum(s.site_updates_per_step() for s in a) == sum(2 * (s.n - 1) for s in a)


def test_reference_sampler_is_bounded_and_models_the_caps():
    """bench.py's reference arm: a sample never runs past its budget by more than
    one update, counts the local updates it ran, and its cost model at the bond
    caps falls as the caps grow (dense n^3 problems)."""
    import sys
    import time
    sys.path.insert(0, ROOT)
    import bench
    from qca_gb300 import workloads as W
    specs = W.chain_mix(4, seed=1000, n_lo=8, n_hi=12, chis=(8, 16))
    rs = bench.RefSampler(specs, per_update_limit_s=1.0)
    t0 = time.perf_counter()
    done, used = rs.sample(1.5)
    assert done > 0 and used <= 1.5 + 1.0 and time.perf_counter() - t0 < 10.0
    assert rs.rate() > 0
    caps = rs.predicted_rate_at_caps()
    assert caps > 0
    rs16 = bench.RefSampler([W.ChainSpec(s.n, s.distance, s.interval, 64, s.p) for s in specs], 1.0)
    rs16.c, rs16.a = rs.c, rs.a
    assert rs16.predicted_rate_at_caps() < caps
