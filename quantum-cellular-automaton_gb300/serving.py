"""Continuous-batching serving loop for TDVP evolution jobs on one GPU.

A job is (rule, N, initial product state, dt, steps, bond cap, algorithm).
Jobs are admitted as device memory frees up: each chain's footprint comes from
``qca_chain_footprint`` (it grows as chi^2 N w) and the sum stays within the HBM
budget.  Admitted jobs get ``stream_every`` time steps scheduled on the engine
(``qca_chain_schedule``); every scheduling round runs a bounded number of
lock-step ticks (``qca_engine_advance``: one local update of every resident job
per tick, all jobs in the same grouped launches).  A job that completes its
scheduled steps idles only until the end of the round, where its populations are
measured and streamed and its next steps are scheduled, so long and short jobs,
and jobs of small and large bond dimension, progress at their own pace and new
jobs join at any round (continuous batching at local-update granularity).
<n_i> is streamed every ``stream_every`` steps and at the end of each job through
``on_populations(job_id, step, populations)`` on a completion thread, so user code
that consumes the populations overlaps with the next round on the GPU.  A job
that fails numerically (QCA_ERR_NAN / QCA_ERR_NOT_CONVERGED) does not stop the
others; on the mixed-precision server it is restarted from its initial state on a
plain FP64 engine (``escalate``, the default), elsewhere it is retired with its
error.

This replaces the reference's per-state driver loop (``quantum_game.py:28-119``:
one initial state at a time, measure every plot interval) with a multi-job
server; the per-job arithmetic is the same as a job run alone.
"""
from __future__ import annotations

import ctypes
import queue
import threading
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .algorithms import _Engine, chain_desc
from .workloads import ChainSpec, Job


@dataclass
class JobState:
    job_id: int
    spec: ChainSpec
    arrival: float
    admitted: float = 0.0
    finished: float = 0.0
    chain: int = -1
    steps_done: int = 0       # steps completed and streamed
    scheduled_to: int = 0     # step count the engine has been asked to reach
    bytes: int = 0
    error: str | None = None
    stream: list = field(default_factory=list)
    engine: object = None     # the _Engine holding the job's chain
    precision: int = 0
    escalated: bool = False   # restarted on the FP64 engine after a mixed failure
    mixed_error: str | None = None  # the engine's message of that mixed failure
    cost: float = 0.0         # relative cost of one local update (chi^3 w, x2 for two-site)


class Server:
    def __init__(self, precision: str = "mixed", hbm_budget_bytes: int = 150 << 30, stream_every: int = 10,
                 max_resident: int = 512, on_populations=None, ticks_per_round: int = 32,
                 escalate: bool = True, light_share: int = 4, light_ratio: float = 8.0) -> None:
        self.precision = _lib.QCA_PREC_MIXED if precision == "mixed" else _lib.QCA_PREC_FP64
        self.engine = _Engine(self.precision, hbm_budget_bytes)
        self.escalate = escalate and self.precision == _lib.QCA_PREC_MIXED
        self._fp64_engine = None                # created at the first escalation
        self.escalations: dict[int, int] = {}   # status code -> jobs restarted in FP64
        # Lock-step ticks last as long as the costliest resident local update, so a
        # job whose updates cost at most 1/light_ratio of the costliest one gets
        # light_share times the ticks of a round (the extra ticks in a call of their
        # own, short because no large job takes part); a job's arithmetic does not
        # depend on how its ticks are grouped.
        self.light_share = max(1, light_share)
        self.light_ratio = light_ratio
        self.budget = hbm_budget_bytes
        self.used = 0
        self.stream_every = stream_every
        self.max_resident = max_resident
        self.ticks_per_round = ticks_per_round
        self.on_populations = on_populations
        self._done_q: queue.Queue | None = None
        self._done_thread: threading.Thread | None = None
        self.callback_errors: list[BaseException] = []
        self.pending: deque[JobState] = deque()
        self.active: list[JobState] = []
        self.done: list[JobState] = []
        self.failed: list[JobState] = []
        self._next_id = 0
        self.site_updates = 0
        self.round_times: list[float] = []      # wall time of every scheduling round
        self.first_stream: list[float] = []     # arrival -> first streamed <n_i> per job
        self.max_overlap = 0                    # most jobs resident in one round
        self.failures: dict[int, int] = {}      # status code -> jobs retired with it
        self.first_failure: str | None = None   # the engine's message of the first failure

    # ------------------------------------------------------------------ requests
    def submit(self, spec: ChainSpec, arrival: float | None = None) -> int:
        js = JobState(self._next_id, spec, time.perf_counter() if arrival is None else arrival)
        self._next_id += 1
        self.pending.append(js)
        return js.job_id

    def footprint(self, spec: ChainSpec, precision: int | None = None) -> int:
        mps = spec.mps()
        d, keep = chain_desc(mps.A, spec.mpo().W, spec.algorithm, spec.dt, spec.chi, spec.eps)
        size = ctypes.c_size_t()
        _lib.call("qca_chain_footprint", ctypes.byref(d), self.precision if precision is None else precision,
                  ctypes.byref(size))
        return size.value

    def _schedule_next(self, js: JobState) -> None:
        target = min(js.spec.steps, js.steps_done + self.stream_every)
        if target > js.scheduled_to:
            _lib.call("qca_chain_schedule", js.engine.h, js.chain, target - js.scheduled_to)
            js.scheduled_to = target

    def _admit(self, now: float) -> None:
        while self.pending and self.pending[0].arrival <= now and len(self.active) < self.max_resident:
            js = self.pending[0]
            if js.engine is None:
                js.engine, js.precision = self.engine, self.precision
            need = self.footprint(js.spec, js.precision)
            if need > self.budget:
                raise _lib.AdmissionError(_lib.QCA_ERR_ADMISSION, f"job {js.job_id} needs {need} bytes > budget")
            if self.used + need > self.budget:
                break  # wait for memory to free up
            self.pending.popleft()
            mps = js.spec.mps()
            W = js.spec.mpo().W
            d, keep = chain_desc(mps.A, W, js.spec.algorithm, js.spec.dt, js.spec.chi, js.spec.eps)
            w = max(max(int(x.shape[2]), int(x.shape[3])) for x in W)  # MPO bonds: W[s, s', wl, wr]
            js.cost = float(js.spec.chi) ** 3 * w * (2.0 if js.spec.algorithm == "2tdvp" else 1.0)
            cid = ctypes.c_int(-1)
            _lib.call("qca_chain_add", js.engine.h, ctypes.byref(d), None, ctypes.byref(cid))
            js.chain = cid.value
            js.bytes = need
            js.admitted = now
            self.used += need
            self.active.append(js)
            self._schedule_next(js)

    def _progress(self, js: JobState) -> tuple[int, bool, int]:
        pr = (ctypes.c_longlong * 4)()
        _lib.call("qca_chain_progress", js.engine.h, js.chain, pr)
        return int(pr[0]), bool(pr[2]), int(pr[3])

    def _failure_message(self, js: JobState, status: int) -> str:
        """The engine's account of a failed chain (what failed, at which site): a
        step request on a failed chain returns its recorded error without running."""
        ids = (ctypes.c_int * 1)(js.chain)
        try:
            _lib.call("qca_engine_step_chains", js.engine.h, ids, 1, 1, None)
        except _lib.QcaError as e:
            return str(e)
        return f"status {status}"

    def _groups(self, jobs: list[JobState]) -> list[list[JobState]]:
        """Jobs by the engine that holds them (one grouped call per engine)."""
        g: dict[int, list[JobState]] = {}
        for j in jobs:
            g.setdefault(id(j.engine), []).append(j)
        return list(g.values())

    def _escalate(self, js: JobState, status: int) -> None:
        """Restart a job that failed on the mixed engine from its initial state on
        the FP64 engine; it keeps its arrival time (latency counts from there)."""
        _lib.call("qca_chain_remove", js.engine.h, js.chain)
        self.used -= js.bytes
        self.site_updates -= js.steps_done * js.spec.site_updates_per_step()  # redone in FP64
        self.escalations[status] = self.escalations.get(status, 0) + 1
        if self._fp64_engine is None:
            self._fp64_engine = _Engine(_lib.QCA_PREC_FP64, self.budget)
        js.engine, js.precision, js.escalated = self._fp64_engine, _lib.QCA_PREC_FP64, True
        js.mixed_error, js.error = js.error, None
        js.chain, js.bytes, js.steps_done, js.scheduled_to = -1, 0, 0, 0
        js.stream = []
        self.pending.appendleft(js)

    def _measure(self, jobs: list[JobState]) -> None:
        for group in self._groups(jobs):
            self._measure_group(group)

    def _measure_group(self, jobs: list[JobState]) -> None:
        ids = (ctypes.c_int * len(jobs))(*[j.chain for j in jobs])
        n_tot = sum(j.spec.n for j in jobs)
        pop = np.zeros(n_tot)
        _lib.call("qca_engine_measure", jobs[0].engine.h, ids, len(jobs), pop.ctypes.data_as(_lib._PD), None,
                  None, None, None)
        o = 0
        for j in jobs:
            p = pop[o:o + j.spec.n].copy()
            o += j.spec.n
            j.stream.append((j.steps_done, p))
            if self.on_populations:
                self._deliver(j.job_id, j.steps_done, p)

    def _retire(self, js: JobState, t: float, failed: bool = False) -> None:
        js.finished = t
        _lib.call("qca_chain_remove", js.engine.h, js.chain)
        self.used -= js.bytes
        (self.failed if failed else self.done).append(js)

    # ------------------------------------------------------------------ loop
    def _advance(self, group: list[JobState], ticks: int) -> None:
        """Up to ``ticks`` lock-step ticks over one engine's jobs; a numerical failure
        is recorded here and acted on from the jobs' progress."""
        ids = (ctypes.c_int * len(group))(*[j.chain for j in group])
        try:
            _lib.call("qca_engine_advance", group[0].engine.h, ids, len(group), ticks, None)
        except _lib.QcaError as e:
            if e.code not in (_lib.QCA_ERR_NAN, _lib.QCA_ERR_NOT_CONVERGED):
                raise
            if self.first_failure is None:
                self.first_failure = str(e)

    def round(self, now: float | None = None, ticks: int | None = None) -> bool:
        """Admit what has arrived, run up to ``ticks`` lock-step ticks over the
        resident jobs, stream the populations of jobs that reached their next
        streaming step, schedule their next steps and retire finished jobs.
        Returns False when idle."""
        now = time.perf_counter() if now is None else now
        t_round = time.perf_counter()
        self._admit(now)
        if not self.active:
            return bool(self.pending)
        self.max_overlap = max(self.max_overlap, len(self.active))
        nt = self.ticks_per_round if ticks is None else ticks
        for group in self._groups(self.active):
            self._advance(group, nt)
        if self.light_share > 1:
            top = max(j.cost for j in self.active)
            light = [j for j in self.active if j.cost * self.light_ratio <= top]
            for group in self._groups(light):
                self._advance(group, (self.light_share - 1) * nt)
        due, still = [], []
        t = time.perf_counter()
        for j in self.active:
            done, inside, status = self._progress(j)
            if status:
                j.error = self._failure_message(j, status)
                if self.escalate and not j.escalated:
                    self._escalate(j, status)
                    continue
                self.failures[status] = self.failures.get(status, 0) + 1
                self._retire(j, t, failed=True)
                continue
            if not inside and done >= j.scheduled_to and done > j.steps_done:
                self.site_updates += (done - j.steps_done) * j.spec.site_updates_per_step()
                j.steps_done = done
                due.append(j)
            still.append(j)
        self._measure(due)
        t = time.perf_counter()
        for j in due:
            if len(j.stream) == 1:
                self.first_stream.append(t - j.arrival)
        self.active = []
        for j in still:
            if j.steps_done >= j.spec.steps:
                self._retire(j, t)
            else:
                self._schedule_next(j)
                self.active.append(j)
        self.round_times.append(time.perf_counter() - t_round)
        return True

    # ------------------------------------------------------------------ completion thread
    def _deliver(self, job_id: int, step: int, populations: np.ndarray) -> None:
        if self._done_thread is None:
            self._done_q = queue.Queue()
            self._done_thread = threading.Thread(target=self._completions, name="qca-serving-completions",
                                                 daemon=True)
            self._done_thread.start()
        self._done_q.put((job_id, step, populations))

    def _completions(self) -> None:
        while True:
            item = self._done_q.get()
            if item is None:
                return
            try:
                self.on_populations(*item)
            except BaseException as e:  # kept for the caller; the loop keeps serving
                self.callback_errors.append(e)

    def close(self) -> None:
        """Wait until every streamed population has been handed to the callback."""
        if self._done_thread is not None:
            self._done_q.put(None)
            self._done_thread.join()
            self._done_thread = None
            self._done_q = None

    def run(self, jobs: list[Job], time_limit: float | None = None) -> dict:
        """Replay a request trace in real time (arrival offsets in seconds); with a
        time limit, no job is admitted after it and the rounds stop there."""
        t0 = time.perf_counter()
        for job in sorted(jobs, key=lambda j: j.arrival):
            self.submit(job.spec, t0 + job.arrival)
        while self.pending or self.active:
            now = time.perf_counter()
            if time_limit is not None and now - t0 > time_limit:
                break
            if not self.active and self.pending and self.pending[0].arrival > now:
                time.sleep(min(0.01, self.pending[0].arrival - now))
            self.round(now)
        elapsed = time.perf_counter() - t0
        self.close()
        return self.report(elapsed)

    def report(self, elapsed: float) -> dict:
        lat = np.array([j.finished - j.arrival for j in self.done]) if self.done else np.zeros(0)
        rt = np.array(self.round_times) if self.round_times else np.zeros(0)
        fs = np.array(self.first_stream) if self.first_stream else np.zeros(0)

        def pct(a, q):
            return float(np.percentile(a, q)) if a.size else None

        return {"jobs_done": len(self.done), "jobs_failed": len(self.failed),
                "failures_by_status": {str(k): v for k, v in self.failures.items()},
                "first_failure": self.first_failure,
                "jobs_escalated": sum(self.escalations.values()),
                "escalations_by_status": {str(k): v for k, v in self.escalations.items()},
                "failed_jobs": [{"job": j.job_id, "algorithm": j.spec.algorithm, "n": j.spec.n,
                                 "distance": j.spec.distance, "chi": j.spec.chi, "steps_done": j.steps_done,
                                 "error": j.error} for j in self.failed],
                "jobs_pending": len(self.pending),
                "jobs_active": len(self.active), "max_resident": self.max_overlap,
                "site_updates": self.site_updates, "elapsed_s": elapsed,
                "site_updates_per_s": self.site_updates / elapsed if elapsed > 0 else 0.0,
                "p50_latency_s": pct(lat, 50), "p99_latency_s": pct(lat, 99),
                "p50_round_s": pct(rt, 50), "p99_round_s": pct(rt, 99),
                "p50_first_stream_s": pct(fs, 50), "p99_first_stream_s": pct(fs, 99)}
