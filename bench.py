"""Benchmark of the GB300 time-evolution path: one JSON line on rank 0.

Workloads (``--workload``):
  batched (default)  256 independent 2TDVP chains in one engine, the batched
                     configuration: N ~ U{16..96}, distance in {1,2,3},
                     interval in {[1,1],[2,3],[2,4]}, bond cap in {32,64,128},
                     random product states, dt = 0.05, mixed precision.
                     One step = one TDVP time step of every chain.
                     Metric: site-updates/s (2(N-1) per chain per step).
  exact              2^24-amplitude exact evolution, distance 2, interval [2,3],
                     Krylov dimension 30, dt = 0.05 (amplitude-updates/s).
  single             single-chain 2TDVP, N = 64, distance 2, interval [2,3],
                     bond cap 256, cutoff 1e-10, dt = 0.05, mixed precision.

``--impl reference`` times the reference algorithm on the host cores instead:
the oracle's NumPy restatement of tdvp.py (dense effective Hamiltonian +
eigh, the reference's own cost profile) on a bounded sample of the same
workload.  Under torchrun every rank runs its own independent chains (weak
scaling, no data-path collective); only the timing uses a barrier and a max.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batched", choices=["batched", "exact", "single", "accuracy", "serving"])
    ap.add_argument("--serve-seconds", type=float, default=120.0)
    ap.add_argument("--serve-jobs", type=int, default=64)
    ap.add_argument("--serve-step-scale", type=int, default=10)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--chains", type=int, default=256)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--acc-chains", type=int, default=8,
                    help="chains of the batched mix re-run in mixed and FP64 precision for the accuracy leg")
    ap.add_argument("--acc-seconds", type=float, default=150.0,
                    help="wall-time bound of the accuracy leg's FP64 stepping")
    return ap.parse_args()


# --------------------------------------------------------------------------- helpers
class Dist:
    def __init__(self, gpus: int):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def peaks() -> dict:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"],
                "bf16_tflops_sustained": d.get("bf16_tflops_sustained", d["bf16_tflops"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "source": "fallback"}


KCLASS = ["gemm", "mpo_apply", "lanczos_vec", "lanczos_exp", "svd", "qr", "other"]


def kernel_stats(eng) -> dict:
    from qca_gb300 import _lib
    out = np.zeros(4 * len(KCLASS))
    _lib.call("qca_engine_kernel_stats", eng.h, out.ctypes.data_as(_lib._PD), 1)
    return {KCLASS[c]: {"launches": out[4 * c], "ms": out[4 * c + 1], "flops": out[4 * c + 2],
                        "bytes": out[4 * c + 3]} for c in range(len(KCLASS))}


# DRAM traffic of one tcgen05 GEMM launch against its algorithmic operand bytes, from
# one ncu capture (--set full) of the 201st gemm_umma_grouped launch of
# `bench.py --chains 16 --steps 1 --warmup 2 --no-e2e --no-cpu --acc-chains 0`
# on a GB300, the launch's work from the QCA_UMMA_LOG line of the same command
# (summary: profiles/gemm_umma_batched_16chains_mixed.md).  The operands are mostly
# L2 hits, so DRAM traffic is a fraction of the operand bytes; applied to the GEMM
# class's operand bytes per launch of the run at hand.
GEMM_DRAM_SAMPLE = {"dram_bytes": 1029888.0, "operand_bytes": 3183664.0, "useful_flops": 58133504.0}


def tdvp_roofline(ks: dict, pk: dict, steps: int, timed_ms: float) -> dict:
    """Roofline object of the TDVP workloads from the per-class kernel statistics.

    The tensor-core contraction class carries it (tensor bound; useful complex flops
    8 M N K per complex GEMM over its CUDA-event time) against the measured bf16
    dense peak.  Beside it: the ceiling of the 3xTF32 split derived from that peak
    (TF32 at half the bf16 rate, three TF32 MMAs per useful product), the whole
    step's algorithmic rate (all classes' flops over the timed region), the SVD
    class's FP32 rate (Golub-Van Loan count), and every class's time share."""
    dom = max(ks, key=lambda k: ks[k]["ms"])
    gemm, svd = ks["gemm"], ks["svd"]
    tflops = gemm["flops"] / (gemm["ms"] / 1e3) / 1e12 if gemm["ms"] > 0 else 0.0
    svd_tflops = svd["flops"] / (svd["ms"] / 1e3) / 1e12 if svd["ms"] > 0 else 0.0
    total_ms = sum(x["ms"] for x in ks.values())
    step_tflops = sum(x["flops"] for x in ks.values()) / (timed_ms / 1e3) / 1e12 if timed_ms > 0 else 0.0
    peak_3x = pk["bf16_tflops"] / 2.0 / 3.0
    per_launch = gemm["bytes"] / gemm["launches"] if gemm["launches"] > 0 else 0.0
    ratio = GEMM_DRAM_SAMPLE["dram_bytes"] / GEMM_DRAM_SAMPLE["operand_bytes"]
    return {"kernel": "gemm", "dominant_class": dom, "bound": "tensor",
            "achieved": round(tflops, 3), "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
            "frac": round(tflops / pk["bf16_tflops"], 5), "traffic": round(ratio * per_launch),
            "traffic_basis": "bytes per GEMM launch: operand bytes per launch of this run x the DRAM/operand "
                             f"ratio {ratio:.3f} of one ncu-captured tcgen05 launch (16-chain case)",
            "peak_source": f"{pk['source']} bf16 dense", "measured_kernel": "gemm",
            "peak_3xtf32_derived": round(peak_3x, 1), "frac_of_3xtf32": round(tflops / peak_3x, 4),
            "step_algorithmic_tflops": round(step_tflops, 3),
            "svd_achieved_tflops_fp32": round(svd_tflops, 3),
            "kernel_time_share": {k: round(v["ms"] / max(1e-9, total_ms), 4) for k, v in ks.items()},
            "kernel_ms_per_step": round(total_ms / max(1, steps), 3)}


def cuda_events():
    import torch
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def profiler_region(start: bool) -> None:
    """Bracket the timed region for ``ncu --profile-from-start off`` when
    QCA_PROFILE_REGION=1 (no effect otherwise)."""
    if os.environ.get("QCA_PROFILE_REGION") != "1":
        return
    import torch
    if start:
        torch.cuda.cudart().cudaProfilerStart()
    else:
        torch.cuda.cudart().cudaProfilerStop()


# ---------------------------------------------------------------- TDVP workloads
def build_specs(args, rank: int):
    from qca_gb300 import workloads as W
    if args.workload == "batched":
        return W.chain_mix(args.chains, seed=1000 + rank), "batched 2TDVP: %d chains, N~U{16..96}, d in {1,2,3}, " \
            "interval in {[1,1],[2,3],[2,4]}, chi in {32,64,128}, dt=0.05" % args.chains
    spec = W.single_chain(64, 2, range(2, 4), 256, seed=64 + rank, dt=0.05, eps=1e-10)
    return [spec], "single-chain 2TDVP: N=64, d=2, interval [2,3], chi=256, eps=1e-10, dt=0.05"


def add_chains(eng, specs, precision_code, stream=None):
    from qca_gb300 import _lib
    from qca_gb300.algorithms import chain_desc
    ids = []
    for s in specs:
        mps = s.mps()
        d, keep = chain_desc(mps.A, s.mpo().W, s.algorithm, s.dt, s.chi, s.eps)
        cid = ctypes.c_int(-1)
        _lib.call("qca_chain_add", eng.h, ctypes.byref(d), _lib.stream_handle(stream), ctypes.byref(cid))
        ids.append(cid.value)
    return ids


def get_mps(eng, cid, n):
    from qca_gb300 import _lib
    from qca_gb300.algorithms import unpack_mps
    b = np.zeros(n + 1, dtype=np.int32)
    _lib.call("qca_chain_bonds", eng.h, cid, b.ctypes.data_as(_lib._PI))
    size = sum(2 * int(b[i]) * int(b[i + 1]) for i in range(n))
    flat = np.zeros(size, dtype=np.complex128)
    _lib.call("qca_chain_get_mps", eng.h, cid, flat.view(np.float64).ctypes.data_as(_lib._PD),
              ctypes.c_size_t(2 * size), None)
    return unpack_mps(flat, [int(x) for x in b])


class RefSampler:
    """Bounded timing of the reference algorithm on the host cores: the oracle's
    restatement of tdvp.py (dense effective Hamiltonian + eigh per local update,
    the reference's own cost profile) evolving the chains of the workload in order
    from their product states.  ``sample(budget)`` runs local updates until the
    budget is used and never starts one whose predicted time (a + c n^3 for the
    local dimension n, calibrated on the updates run so far and on one eigh timed
    at start) exceeds what is left; a chain whose next update would not fit even a
    whole budget is retired and the next chain of the workload begins.  The
    sample therefore covers the cheap early updates of each chain, which makes the
    host rate an overestimate of the reference at the device run's bond
    dimensions."""

    def __init__(self, specs, per_update_limit_s: float):
        from oracle import qca_oracle as O
        self.O = O
        self.specs = specs
        self.limit = per_update_limit_s
        self.ci = -1
        self.done = 0
        self.used = 0.0
        self.retired = []
        self.max_bond = 0
        self.max_n = 0
        m = np.random.default_rng(0).standard_normal((768, 768))
        h = m + m.T
        t0 = time.perf_counter()
        np.linalg.eigh(h.astype(np.complex128))
        self.c = (time.perf_counter() - t0) / 768.0 ** 3
        self.a = 0.0
        self._next_chain()

    def _next_chain(self):
        self.ci += 1
        spec = self.specs[self.ci % len(self.specs)]
        W = self.O.build_mpo(self.O.Rules(spec.n, spec.interval, spec.distance))
        self.orc = self.O.TDVPOracle(self.O.mps_from_density_distribution(spec.p), W, spec.algorithm, spec.dt,
                                     spec.chi, spec.eps)
        self.it = self.orc.step_updates()

    def predict(self, n: int) -> float:
        return self.a + 1.2 * self.c * float(n) ** 3

    def sample(self, budget: float):
        done, used = 0, 0.0
        while used < budget:
            n = self.orc.upcoming_size()
            if self.predict(n) > self.limit:
                self.retired.append((self.ci, self.specs[self.ci % len(self.specs)].n, n))
                self._next_chain()
                continue
            if used + self.predict(n) > budget:
                break
            t0 = time.perf_counter()
            try:
                next(self.it)
                ok = True
            except StopIteration:
                self.it = self.orc.step_updates()
                ok = False
            dt = time.perf_counter() - t0
            used += dt
            if ok:
                done += 1
                self.max_n = max(self.max_n, n)
                self.max_bond = max(self.max_bond, max(a.shape[2] for a in self.orc.A))
                if n <= 64:
                    self.a = dt if self.a == 0.0 else min(self.a, dt)
                elif n >= 512:
                    self.c = max(self.c, (dt - self.a) / float(n) ** 3)
        self.done += done
        self.used += used
        return done, used

    def rate(self) -> float:
        return self.done / self.used if self.used > 0 else 0.0

    def predicted_rate_at_caps(self) -> float:
        """Site-updates/s the reference algorithm would reach on the whole workload
        with every bond at its cap min(2^i, 2^(N-i), chi), from the cost model
        a + c n^3 calibrated in this run: per 2TDVP time step each bond is one
        two-site update (dense problem n = 4 D_l D_r) and each inner site one
        backward single-site update (n = 2 D_l D_r).  A model, not a measurement:
        at chi = 128 one two-site update is a dense 65536^3 eigendecomposition."""
        t = 0.0
        su = 0
        for sp in self.specs:
            n = sp.n
            D = [min(2 ** min(i, 40), 2 ** min(n - i, 40), sp.chi) for i in range(n + 1)]
            for _ in range(2):  # right and left sweep
                for l in range(n - 1):
                    t += self.predict(4 * D[l] * D[l + 2])
                for s_ in range(1, n - 1):
                    t += self.predict(2 * D[s_] * D[s_ + 1])
            su += sp.site_updates_per_step()
        return su / t if t > 0 else 0.0

    def describe(self) -> str:
        return (f"{self.done} local updates of the reference algorithm (oracle restatement of tdvp.py: dense "
                f"effective Hamiltonian + eigh) in {self.used:.1f} s, evolving chains 0..{self.ci} of the workload "
                f"from their product states; bonds reached {self.max_bond}, largest local problem {self.max_n}; "
                f"{len(self.retired)} chain(s) retired when their next update was predicted to exceed "
                f"{self.limit:.0f} s; {int(os.environ.get('OMP_NUM_THREADS', os.cpu_count()))} BLAS threads")


def cpu_tdvp_sample(specs, budget_s: float):
    """(site-updates/s, description) of the reference algorithm on the host cores
    over a bounded sample of the workload (``RefSampler``)."""
    rs = RefSampler(specs, per_update_limit_s=min(5.0, budget_s / 3))
    rs.sample(budget_s)
    return rs.rate(), rs.describe() + (f"; cost model a + c n^3 at every bond's cap: "
                                       f"{rs.predicted_rate_at_caps():.3g} site-updates/s")


def run_tdvp(args, dist: Dist):
    import torch
    from qca_gb300 import _lib
    from qca_gb300.algorithms import _Engine
    torch.cuda.set_device(dist.local)
    prec = _lib.QCA_PREC_MIXED if args.precision == "mixed" else _lib.QCA_PREC_FP64
    specs, desc = build_specs(args, dist.rank)
    eng = _Engine(prec)
    ids = add_chains(eng, specs, prec)
    cids = (ctypes.c_int * len(ids))(*ids)
    su_per_step = sum(s.site_updates_per_step() for s in specs)
    # warm-up (bond dimensions grow from the product states)
    _lib.call("qca_engine_step_chains", eng.h, cids, len(ids), args.warmup, None)
    torch.cuda.synchronize()
    _lib.call("qca_engine_profile", eng.h, 1)
    kernel_stats(eng)  # reset
    clocks = Clocks(dist.local)
    dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    profiler_region(True)
    ev = [cuda_events()[0] for _ in range(args.steps + 1)]
    ev[0].record()
    for k in range(args.steps):  # one engine call per time step: per-step latencies
        _lib.call("qca_engine_step_chains", eng.h, cids, len(ids), 1, None)
        ev[k + 1].record()
    torch.cuda.synchronize()
    profiler_region(False)
    clk = clocks.stop()
    dist.barrier()
    step_ms = [ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)]
    ms = dist.max(ev[0].elapsed_time(ev[args.steps]))
    ks = kernel_stats(eng)
    _lib.call("qca_engine_profile", eng.h, 0)
    acc_idx = accuracy_subset(specs, args.acc_chains)
    acc_pops = measure_pops(eng, [ids[i] for i in acc_idx], [specs[i] for i in acc_idx]) if acc_idx else None
    total_su = dist.sum(su_per_step * args.steps)
    value = total_su / (ms / 1e3)
    bonds = []
    for cid, s in zip(ids, specs):
        b = np.zeros(s.n + 1, dtype=np.int32)
        _lib.call("qca_chain_bonds", eng.h, cid, b.ctypes.data_as(_lib._PI))
        bonds.append(int(b.max()))
    pk = peaks()
    launches = int(sum(v["launches"] for v in ks.values()))
    roofline = tdvp_roofline(ks, pk, args.steps, ms)
    # end to end through the public API with host buffers: upload the warmed-up
    # states (pinned host -> device), evolve, read the populations every step
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, specs, [get_mps(eng, cid, s.n) for cid, s in zip(ids, specs)], prec, dist)
    del eng
    acc = None
    if acc_idx:
        acc = accuracy_leg(args, [specs[i] for i in acc_idx], acc_pops, value)
    cpu = None
    if not args.no_cpu and dist.rank == 0:
        v, sample = cpu_tdvp_sample(specs, 15.0)
        cpu = {"value": round(v, 3), "unit": "site-updates/s", "cores": os.cpu_count(), "kind": "port",
               "sample": sample}
    line = {
        "metric": "site-updates/s", "value": round(value, 2), "unit": "site-updates/s", "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if args.precision == "mixed" else "f64", "data": "synthetic",
        "config": {"workload": desc, "precision": args.precision, "chains_per_gpu": len(specs),
                   "site_updates_per_step": su_per_step, "max_bond_dim_reached": max(bonds),
                   "l2": "working set larger than L2 (>= %.1f GB resident)" % (len(specs) * 0.01)},
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clk,
        "step_latency_ms": {"p50": round(float(np.percentile(step_ms, 50)), 2),
                            "p99": round(float(np.percentile(step_ms, 99)), 2)},
        "accuracy": acc,
    }
    if acc is not None:
        line["fp64"] = acc.pop("fp64")
    return line


def accuracy_subset(specs, count: int) -> list[int]:
    """Every (len/count)-th chain of the workload: a sample of its mix of lengths,
    rules and bond caps."""
    if count <= 0:
        return []
    stride = max(1, len(specs) // count)
    return list(range(0, len(specs), stride))[:count]


def measure_pops(eng, ids, specs) -> np.ndarray:
    from qca_gb300 import _lib
    n_tot = sum(s.n for s in specs)
    pop = np.zeros(n_tot)
    cids = (ctypes.c_int * len(ids))(*ids)
    _lib.call("qca_engine_measure", eng.h, cids, len(ids), pop.ctypes.data_as(_lib._PD), None, None, None, None)
    return pop


def accuracy_leg(args, specs, pops_batched, batched_value: float) -> dict:
    """The metric's accuracy condition and its FP64 leg on a sample of the timed
    chains: the same chains from the same product states through the same
    warm-up + timed steps, (a) with the mixed path alone (its populations are
    compared with the batched run's) and (b) with the plain FP64 path, <n_i>
    compared after every step; the FP64 path's site-updates/s over the timed
    steps is the metric's plain-FP64 rate."""
    import torch
    from qca_gb300 import _lib
    from qca_gb300.algorithms import _Engine
    series, rates, timed_steps = {}, {}, {}
    total = args.warmup + args.steps
    su_step = sum(s.site_updates_per_step() for s in specs)
    for name, prec in (("mixed", _lib.QCA_PREC_MIXED), ("fp64", _lib.QCA_PREC_FP64)):
        eng = _Engine(prec)
        ids = add_chains(eng, specs, prec)
        cids = (ctypes.c_int * len(ids))(*ids)
        rows, t_timed, t_all, n_timed = [], 0.0, 0.0, 0
        for step in range(total):
            if name == "fp64" and t_all > args.acc_seconds:
                break  # the plain FP64 path is slow on this part: bounded
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            _lib.call("qca_engine_step_chains", eng.h, cids, len(ids), 1, None)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            t_all += dt
            if step >= min(args.warmup, total - 1):
                t_timed += dt
                n_timed += 1
            rows.append(measure_pops(eng, ids, specs))
        series[name] = np.array(rows)
        if n_timed == 0:  # the budget ran out in the warm-up: rate over the steps run
            t_timed, n_timed = t_all, len(rows)
        rates[name] = su_step * n_timed / t_timed
        timed_steps[name] = n_timed
        del eng
    done = len(series["fp64"])
    dn = np.abs(series["mixed"][:done] - series["fp64"]).max(axis=1)
    within = [bool(x <= 1e-5) for x in dn]
    return {"max_dn_vs_fp64": float(dn.max()), "max_dn_by_step": [float(f"{x:.3g}") for x in dn],
            "steps_compared": done, "steps_run_mixed": total, "chains": len(specs),
            "bound": 1e-5, "within_bound_all_steps": all(within),
            "steps_within_bound_from_start": next((i for i, w in enumerate(within) if not w), len(within)),
            "chains_desc": [(s.n, s.distance, s.interval.stop - 1, s.chi) for s in specs],
            "batched_vs_alone_max_dn": float(np.abs(series["mixed"][-1] - pops_batched).max()),
            "fp64": {"site_updates_per_s": round(rates["fp64"], 2),
                     "measured_on": f"the {len(specs)} sampled chains, {timed_steps['fp64']} steps after the "
                                    f"warm-up (at most {args.acc_seconds:.0f} s of FP64 stepping)",
                     "mixed_same_chains_site_updates_per_s": round(rates["mixed"], 2),
                     "batched_mixed_over_fp64": round(batched_value / rates["fp64"], 2)}}


def run_e2e(args, specs, states, prec, dist: Dist):
    import torch
    from qca_gb300 import _lib
    from qca_gb300.algorithms import _Engine, chain_desc
    eng = _Engine(prec)
    n_tot = sum(s.n for s in specs)
    pop = np.zeros(n_tot)
    dpop = np.zeros(n_tot)
    sse = np.zeros(n_tot)
    bd = np.zeros(n_tot + len(specs))
    descs = [chain_desc(A, s.mpo().W, s.algorithm, s.dt, s.chi, s.eps) for s, A in zip(specs, states)]
    h2d = sum(k[2].nbytes + k[3].nbytes for _, k in descs)
    d2h = pop.nbytes + dpop.nbytes + sse.nbytes + bd.nbytes
    dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ids = []
    for d, _ in descs:
        cid = ctypes.c_int(-1)
        _lib.call("qca_chain_add", eng.h, ctypes.byref(d), None, ctypes.byref(cid))
        ids.append(cid.value)
    cids = (ctypes.c_int * len(ids))(*ids)
    t_add = time.perf_counter() - t0
    t_step = t_meas = 0.0
    for _ in range(args.steps):
        ta = time.perf_counter()
        _lib.call("qca_engine_step_chains", eng.h, cids, len(ids), 1, None)  # the first also initialises
        tb = time.perf_counter()
        _lib.call("qca_engine_measure", eng.h, cids, len(ids), pop.ctypes.data_as(_lib._PD),
                  dpop.ctypes.data_as(_lib._PD), sse.ctypes.data_as(_lib._PD), bd.ctypes.data_as(_lib._PD), None)
        t_step += tb - ta
        t_meas += time.perf_counter() - tb
    torch.cuda.synchronize()
    el = dist.max(time.perf_counter() - t0)
    su = dist.sum(sum(s.site_updates_per_step() for s in specs) * args.steps)
    del eng
    return {"value": round(su / el, 2), "unit": "site-updates/s", "h2d_bytes_per_step": int(h2d / args.steps),
            "d2h_bytes_per_step": int(d2h), "includes": "chain upload + TDVP init, every step: step + measure "
            "(populations, entropies, bond dims to host)",
            "phases_s": {"upload": round(t_add, 3), "init_and_steps": round(t_step, 3), "measure": round(t_meas, 3)}}


# ---------------------------------------------------------------- exact workload
def run_exact(args, dist: Dist):
    import torch
    import types
    from qca_gb300 import GpuExact, MPO, MPS, Rules
    from qca_gb300 import workloads as W
    torch.cuda.set_device(dist.local)
    n, d, lo, hi, dt, m = 24, 2, 2, 4, 0.05, 30
    p = W.product_probabilities(np.random.default_rng(2024 + dist.rank), n)
    H = MPO.hamiltonian_from_rules(Rules(n, range(lo, hi), d))
    a = GpuExact(MPS.from_density_distribution(p), H, types.SimpleNamespace(
        step_size=dt, algorithm="exact", precision=args.precision, krylov_dim=m))
    a.evolve(args.warmup)
    clocks = Clocks(dist.local)
    dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    profiler_region(True)
    e0, e1 = cuda_events()
    e0.record()
    a.evolve(args.steps)
    e1.record()
    torch.cuda.synchronize()
    profiler_region(False)
    clk = clocks.stop()
    ms = dist.max(e0.elapsed_time(e1))
    amps = dist.sum((1 << n) * args.steps)
    b = 16 if args.precision == "fp64" else 8
    alg_bytes = (4 * m + 1) * (1 << n) * b
    pk = peaks()
    gbs = alg_bytes / (ms / args.steps / 1e3) / 1e9
    # e2e: host state in, state out, through the public API
    psi = a.state_vector()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        a.set_state_vector(psi)
        a.do_time_step()
        psi = a.state_vector()
    el = time.perf_counter() - t0
    line = {
        "metric": "amplitude-updates/s", "value": round(amps / (ms / 1e3), 1), "unit": "amplitude-updates/s",
        "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32+f64", "data": "synthetic",
        "config": {"workload": "exact N=24, d=2, interval [2,3], Krylov 30, dt=0.05", "precision": args.precision,
                   "l2": "state 2^24 amplitudes x 30 Krylov vectors > L2"},
        "roofline": {"bound": "hbm", "achieved": round(gbs, 1), "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": round(gbs / pk["hbm_gbs"], 4), "traffic": None,
                     "note": "algorithmic bytes (4m+1) 2^N b per step over the whole step"},
        "e2e": {"value": round((1 << n) * args.steps / el, 1), "unit": "amplitude-updates/s",
                "h2d_bytes_per_step": 16 << n, "d2h_bytes_per_step": 16 << n},
        "gpu_launches": args.steps * (2 + 30 * 4), "clocks": clk, "cpu_baseline": None,
    }
    return line


# ---------------------------------------------------------------- reference arm
def run_reference(args, dist: Dist):
    if dist.rank != 0:
        return None
    from qca_gb300 import workloads as W
    from oracle import qca_oracle as O
    if args.workload == "exact":
        n = 20  # the dense/sparse CPU path at 2^24 takes minutes per step; sample 2^20
        p = W.product_probabilities(np.random.default_rng(2024), n)
        psi = O.product_state_vector(p)
        for _ in range(args.warmup):
            psi = O.exact_evolve(psi, n, 2, range(2, 4), 0.05, 1)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            psi = O.exact_evolve(psi, n, 2, range(2, 4), 0.05, 1)
        el = time.perf_counter() - t0
        v = (1 << n) * args.steps / el
        return {"impl": "reference", "metric": "amplitude-updates/s", "value": round(v, 1),
                "unit": "amplitude-updates/s", "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup,
                "higher_is_better": True, "config": {"workload": "exact, sampled at N=20 on the host"},
                "cpu_baseline": {"value": round(v, 1), "unit": "amplitude-updates/s", "cores": os.cpu_count(),
                                 "kind": "port", "sample": "sparse expm_multiply restatement at N=20"},
                "e2e": {"value": round(v, 1), "unit": "amplitude-updates/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
    specs, desc = build_specs(args, 0)
    # each step is a bounded sample of the workload (RefSampler): local updates of
    # the reference algorithm on the chains of the mix, at most 6 s per step
    rs = RefSampler(specs, per_update_limit_s=4.0)
    for _ in range(args.warmup):
        rs.sample(1.0)
    rs.done, rs.used = 0, 0.0
    per_step = []
    for _ in range(args.steps):
        d_, u_ = rs.sample(6.0)
        per_step.append(u_)
    v = rs.rate()
    return {"impl": "reference", "metric": "site-updates/s", "value": round(v, 3), "unit": "site-updates/s",
            "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(rs.used / max(1, args.steps) * 1e3, 2), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": desc},
            "cpu_baseline": {"value": round(v, 3), "unit": "site-updates/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": rs.describe(),
                             "model_rate_at_bond_caps": float(f"{rs.predicted_rate_at_caps():.3g}")},
            "e2e": {"value": round(v, 3), "unit": "site-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ---------------------------------------------------------------- accuracy and serving
def run_accuracy(args, dist: Dist):
    """Mixed precision against the FP64 path (pinned to the oracle at 1e-8) on
    chains of the batched mix: max |d<n_i>| over every step, discarded weight,
    bond dimensions, and the site-update rates of both paths on the same chains."""
    import torch
    from qca_gb300 import _lib
    from qca_gb300 import workloads as W
    from qca_gb300.algorithms import _Engine
    torch.cuda.set_device(dist.local)
    specs = [s for s in W.chain_mix(64, seed=1000 + dist.rank) if s.n <= 48][:args.chains if args.chains < 256 else 6]
    out = {}
    pops, rates, discs, bonds = {}, {}, {}, {}
    for name, prec in (("mixed", _lib.QCA_PREC_MIXED), ("fp64", _lib.QCA_PREC_FP64)):
        eng = _Engine(prec)
        ids = add_chains(eng, specs, prec)
        cids = (ctypes.c_int * len(ids))(*ids)
        n_tot = sum(s.n for s in specs)
        series = []
        t_step = 0.0
        for step in range(args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            _lib.call("qca_engine_step_chains", eng.h, cids, len(ids), 1, None)
            torch.cuda.synchronize()
            t_step += time.perf_counter() - t0
            pop = np.zeros(n_tot)
            _lib.call("qca_engine_measure", eng.h, cids, len(ids), pop.ctypes.data_as(_lib._PD), None, None, None,
                      None)
            series.append(pop)
        d = 0.0
        for cid in ids:
            st = np.zeros(2)
            _lib.call("qca_chain_stats", eng.h, cid, st.ctypes.data_as(_lib._PD))
            d = max(d, st[1])
        bm = 0
        for cid, s in zip(ids, specs):
            bb = np.zeros(s.n + 1, dtype=np.int32)
            _lib.call("qca_chain_bonds", eng.h, cid, bb.ctypes.data_as(_lib._PI))
            bm = max(bm, int(bb.max()))
        pops[name], discs[name], bonds[name] = np.array(series), d, bm
        rates[name] = sum(s.site_updates_per_step() for s in specs) * args.steps / t_step
        del eng
    dn = float(np.abs(pops["mixed"] - pops["fp64"]).max())
    return {"metric": "max|d<n_i>| mixed vs fp64", "value": dn, "unit": "population", "n_gpus": dist.world,
            "steps": args.steps, "higher_is_better": False, "data": "synthetic",
            "config": {"workload": f"{len(specs)} chains of the batched mix with N <= 48 "
                                   f"({[(s.n, s.distance, s.interval.stop - 1, s.chi) for s in specs]})",
                       "dt": specs[0].dt, "eps": specs[0].eps},
            "discarded_weight_last_step": {"mixed": discs["mixed"], "fp64": discs["fp64"]},
            "max_bond_dim": bonds, "site_updates_per_s": {k: round(v, 1) for k, v in rates.items()},
            "mixed_over_fp64_speedup": round(rates["mixed"] / rates["fp64"], 2)}


def serving_trace(args, rank: int):
    """A bounded slice of the serving configuration: the first ``--serve-jobs``
    requests of the Poisson(200/s) trace (1TDVP/2TDVP, N ~ U{12..128}, distance in
    {1,2}, bond cap in {16,...,256}, dt = 0.05) with their step counts (50-500)
    divided by ``--serve-step-scale`` so that the slice runs to completion."""
    from qca_gb300 import workloads as W
    jobs = W.poisson_jobs(rate=200.0, duration=60.0, seed=7 + rank)[:args.serve_jobs]
    for j in jobs:
        j.spec.steps = max(1, -(-j.spec.steps // args.serve_step_scale))
    return jobs


def run_serving(args, dist: Dist):
    """The serving loop on a bounded slice of the serving configuration, replayed
    in real time (arrivals at their trace offsets), once with the mixed path and
    once with the plain FP64 path on the same requests, each until every job is
    done or ``--serve-seconds`` have passed.  Reports completed jobs, p50/p99
    latency (arrival to last populations), site-updates/s of both paths and their
    ratio, and max|d<n_i>| between the two paths' streamed populations of the jobs
    both completed."""
    import torch
    from qca_gb300.serving import Server
    torch.cuda.set_device(dist.local)
    reps, streams = {}, {}
    for prec in ("mixed", "fp64"):
        jobs = serving_trace(args, dist.rank)
        srv = Server(prec, hbm_budget_bytes=150 << 30, stream_every=10, max_resident=args.chains,
                     ticks_per_round=32)
        reps[prec] = srv.run(jobs, time_limit=args.serve_seconds)
        streams[prec] = {j.job_id: j.stream for j in srv.done}
        del srv
    both = set(streams["mixed"]) & set(streams["fp64"])
    dn = 0.0
    for k in both:
        for (sa, pa), (sb, pb) in zip(streams["mixed"][k], streams["fp64"][k]):
            dn = max(dn, float(np.abs(pa - pb).max()))
    jobs = serving_trace(args, dist.rank)
    m, f = reps["mixed"], reps["fp64"]

    def summary(r):
        return {"site_updates_per_s": round(r["site_updates_per_s"], 1), "jobs_done": r["jobs_done"],
                "jobs_failed": r["jobs_failed"], "failures_by_status": r["failures_by_status"],
                "first_failure": r["first_failure"], "failed_jobs": r["failed_jobs"][:16],
                "jobs_escalated": r["jobs_escalated"], "escalations_by_status": r["escalations_by_status"],
                "jobs_unfinished": r["jobs_active"] + r["jobs_pending"],
                "p50_latency_s": r["p50_latency_s"], "p99_latency_s": r["p99_latency_s"],
                "p50_first_populations_s": r["p50_first_stream_s"],
                "p99_first_populations_s": r["p99_first_stream_s"], "max_resident_jobs": r["max_resident"],
                "p50_round_s": r["p50_round_s"], "elapsed_s": round(r["elapsed_s"], 1)}

    return {"metric": "site-updates/s", "value": round(m["site_updates_per_s"], 1), "unit": "site-updates/s",
            "n_gpus": dist.world, "higher_is_better": True, "data": "synthetic", "dtype": "f32+f64",
            "config": {"workload": f"serving: the first {len(jobs)} requests of the Poisson(200/s) trace "
                                   "(1TDVP/2TDVP, N~U{12..128}, d in {1,2}, chi in {16..256}, dt=0.05), step counts "
                                   f"50-500 divided by {args.serve_step_scale}, replayed in real time, HBM budget "
                                   "150 GB, <n_i> streamed every 10 steps",
                       "wall_limit_s_per_path": args.serve_seconds, "ticks_per_round": 32},
            "p50_latency_s": m["p50_latency_s"], "p99_latency_s": m["p99_latency_s"],
            "mixed": summary(m), "fp64": summary(f),
            "mixed_over_fp64": round(m["site_updates_per_s"] / f["site_updates_per_s"], 2)
            if f["site_updates_per_s"] > 0 else None,
            "accuracy": {"max_dn_vs_fp64": dn, "jobs_compared": len(both)}}


def main():
    args = parse()
    dist = Dist(args.gpus)
    if args.impl == "reference":
        line = run_reference(args, dist)
    elif args.workload == "accuracy":
        line = run_accuracy(args, dist)
    elif args.workload == "serving":
        line = run_serving(args, dist)
    elif args.workload == "exact":
        line = run_exact(args, dist)
    else:
        line = run_tdvp(args, dist)
    if dist.rank == 0 and line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
