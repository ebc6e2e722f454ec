"""Generate the golden fixtures in this directory from the reference implementation.

Run in a container where the reference checkout is available:

    python tests/golden/make_golden.py /path/to/quantum-cellular-automaton

It imports the reference's own classes (``tensor_networks``, ``algorithms``,
``lautils``) and records their outputs on seeded inputs.  The fixtures pin the
oracle (``oracle/qca_oracle.py``) and, through it, the CUDA path.  Nothing at
test time reads the reference checkout; only the ``.npz`` files travel.

Fixtures:
  mpo_rules.npz        W tensors of MPO.hamiltonian_from_rules for several rules
  exact_series.npz     Exact (dense U) populations after each recorded step
  tdvp_series.npz      TDVP populations / bond dims, unmodified and gauge-fixed
  qr_lapack.npz        numpy.linalg.qr outputs (complete and reduced) incl.
                       zero-padded and rank-deficient inputs
  measure_case.npz     MPS.measure outputs for a random MPS and a product state
  a1tdvp_series.npz    a1tdvp populations / bond dims (exact_exponential local evolution)
"""
from __future__ import annotations

import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load_reference(path: str):
    sys.argv = ["x"]  # the reference parses argv at import time (tensor_networks/mps.py:11)
    sys.path.insert(0, path)
    from tensor_networks import MPO, MPS  # noqa
    from parameters import Rules  # noqa
    from algorithms import Exact, TDVP  # noqa
    return types.SimpleNamespace(MPO=MPO, MPS=MPS, Rules=Rules, Exact=Exact, TDVP=TDVP)


RULES = [(1, 1, 2), (1, 2, 4), (1, 2, 5), (2, 1, 2), (2, 2, 4), (2, 2, 5), (3, 1, 2), (3, 2, 4), (3, 2, 5)]


def gen_mpo(ref):
    out = {}
    for d, lo, hi in RULES:
        r = ref.Rules(ncells=6, activation_interval=range(lo, hi), distance=d, periodic=False)
        W = ref.MPO.hamiltonian_from_rules(r).W
        key = f"d{d}_{lo}{hi}"
        out[key + "_bulk"] = W[2]
        out[key + "_first"] = W[0]
        out[key + "_last"] = W[-1]
    np.savez_compressed(os.path.join(HERE, "mpo_rules.npz"), **out)


def gen_exact(ref):
    out = {}
    cases = [
        # name, n, d, lo, hi, p, step_size (already multiplied by the plot interval), steps
        ("single8", 8, 1, 1, 2, [0.0] * 3 + [1.0] + [0.0] * 4, 0.1, 12),
        ("rand10", 10, 2, 2, 4, None, 0.05, 10),
    ]
    for name, n, d, lo, hi, p, dt, steps in cases:
        if p is None:
            th = np.random.default_rng(7).uniform(0, np.pi / 2, size=n)
            p = list(np.sin(th) ** 2)
        r = ref.Rules(ncells=n, activation_interval=range(lo, hi), distance=d, periodic=False)
        H = ref.MPO.hamiltonian_from_rules(r)
        psi0 = ref.MPS.from_density_distribution(p)
        args = types.SimpleNamespace(step_size=dt, algorithm="exact")
        alg = ref.Exact(psi_0=psi0, H=H, args=args)
        pops = np.zeros((steps + 1, n))
        bonds = np.zeros((steps + 1, n + 1))
        sse = np.zeros((steps + 1, n))
        dpop = np.zeros((steps + 1, n))
        for s in range(steps + 1):
            alg.measure(pops[s], dpop[s], sse[s], bonds[s])
            if s < steps:
                alg.do_time_step()
        out[name + "_p"] = np.array(p)
        out[name + "_meta"] = np.array([n, d, lo, hi, dt, steps])
        out[name + "_pop"] = pops
        out[name + "_dpop"] = dpop
        out[name + "_bonds"] = bonds
        out[name + "_final"] = alg._psi
    np.savez_compressed(os.path.join(HERE, "exact_series.npz"), **out)


def fixed_tdvp_class(TDVP):
    class FixedTDVP(TDVP):
        """Gauge-consistent variant: right environments rebuilt after tdvp.py:54."""

        def do_time_step(self):
            self._psi.make_site_canonical(0)
            for site in reversed(range(1, len(self._psi.A))):
                self._update_layer_H_eff(side="right", site=site)
            if self.args.algorithm == "2tdvp":
                self._sweep_right_2tdvp()
                self._sweep_left_2tdvp()
                return
            self._sweep_right()
            self._sweep_left()

    return FixedTDVP


TDVP_CASES = [
    # name, algorithm, n, d, lo, hi, p (None = random seed 11), dt, chi, eps, steps
    ("t2_single8", "2tdvp", 8, 1, 1, 2, [0.0] * 3 + [1.0] + [0.0] * 4, 0.1, 8, 1e-8, 8),
    ("t1_single8", "1tdvp", 8, 1, 1, 2, [0.0] * 3 + [1.0] + [0.0] * 4, 0.1, 8, 1e-8, 8),
    ("t2_rand7", "2tdvp", 7, 2, 2, 4, None, 0.05, 16, 1e-10, 6),
    ("t1_rand7", "1tdvp", 7, 2, 2, 4, None, 0.05, 6, 1e-10, 6),
    ("t2_rand9_d3", "2tdvp", 9, 3, 2, 5, None, 0.05, 6, 1e-6, 5),
]


def gen_tdvp(ref):
    out = {}
    Fixed = fixed_tdvp_class(ref.TDVP)
    for name, alg_name, n, d, lo, hi, p, dt, chi, eps, steps in TDVP_CASES:
        if p is None:
            th = np.random.default_rng(11).uniform(0, np.pi / 2, size=n)
            p = list(np.sin(th) ** 2)
        r = ref.Rules(ncells=n, activation_interval=range(lo, hi), distance=d, periodic=False)
        H = ref.MPO.hamiltonian_from_rules(r)
        for mode, cls in (("fixed", Fixed), ("ref", ref.TDVP)):
            psi0 = ref.MPS.from_density_distribution(p)
            args = types.SimpleNamespace(step_size=dt, algorithm=alg_name, max_bond_dim=chi, svd_epsilon=eps)
            alg = cls(psi_0=psi0, H=H, args=args)
            pops = np.zeros((steps + 1, n))
            dpop = np.zeros((steps + 1, n))
            sse = np.zeros((steps + 1, n))
            bonds = np.zeros((steps + 1, n + 1))
            for s in range(steps + 1):
                alg.measure(pops[s], dpop[s], sse[s], bonds[s])
                if s < steps:
                    alg.do_time_step()
            out[f"{name}_{mode}_pop"] = pops
            out[f"{name}_{mode}_dpop"] = dpop
            out[f"{name}_{mode}_sse"] = sse
            out[f"{name}_{mode}_bonds"] = bonds
        out[name + "_p"] = np.array(p)
        out[name + "_meta"] = np.array([n, d, lo, hi, dt, chi, eps, steps])
        out[name + "_alg"] = np.array(alg_name)
    np.savez_compressed(os.path.join(HERE, "tdvp_series.npz"), **out)


A1TDVP_CASES = [
    # name, n, d, lo, hi, p (None = random seed 13), dt, chi, eps, steps
    ("a1_single8", 8, 1, 1, 2, [0.0] * 3 + [1.0] + [0.0] * 4, 0.1, 8, 1e-3, 6),
    ("a1_rand8", 8, 2, 2, 4, None, 0.05, 8, 1e-4, 5),
]


def gen_a1tdvp(ref):
    """The reference's a1tdvp (tdvp.py:212-267) with its "exact_exponential" local
    evolution (the default "taylor" path calls np.math, absent from numpy 2):
    populations and bond dimensions after every step, measured like the driver."""
    out = {}
    for name, n, d, lo, hi, p, dt, chi, eps, steps in A1TDVP_CASES:
        if p is None:
            th = np.random.default_rng(13).uniform(0, np.pi / 2, size=n)
            p = list(np.sin(th) ** 2)
        r = ref.Rules(ncells=n, activation_interval=range(lo, hi), distance=d, periodic=False)
        H = ref.MPO.hamiltonian_from_rules(r)
        psi0 = ref.MPS.from_density_distribution(p)
        args = types.SimpleNamespace(step_size=dt, algorithm="a1tdvp", max_bond_dim=chi, svd_epsilon=eps,
                                     approximative_evolution_method="exact_exponential", taylor_steps=10)
        alg = ref.TDVP(psi_0=psi0, H=H, args=args)
        pops = np.zeros((steps + 1, n))
        dpop = np.zeros((steps + 1, n))
        sse = np.zeros((steps + 1, n))
        bonds = np.zeros((steps + 1, n + 1))
        for s_ in range(steps + 1):
            alg.measure(pops[s_], dpop[s_], sse[s_], bonds[s_])
            if s_ < steps:
                alg.do_time_step()
        out[f"{name}_ref_pop"] = pops
        out[f"{name}_ref_bonds"] = bonds
        out[name + "_p"] = np.array(p)
        out[name + "_meta"] = np.array([n, d, lo, hi, dt, chi, eps, steps])
    np.savez_compressed(os.path.join(HERE, "a1tdvp_series.npz"), **out)


def gen_qr():
    rng = np.random.default_rng(3)
    out = {}
    shapes = [(8, 3), (6, 6), (4, 7), (16, 5), (12, 12)]
    for k, (m, n) in enumerate(shapes):
        a = rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))
        if k == 3:  # zero-padded columns, as truncate_and_pad produces (mps.py:233-234)
            a[:, 3:] = 0
        if k == 4:  # rank deficient
            a[:, 6:] = a[:, :6] @ (rng.standard_normal((6, 6)) + 0j)
        for mode in ("reduced", "complete"):
            q, r = np.linalg.qr(a, mode=mode)
            out[f"a{k}"] = a
            out[f"a{k}_{mode}_q"] = q
            out[f"a{k}_{mode}_r"] = r
    np.savez_compressed(os.path.join(HERE, "qr_lapack.npz"), **out)


def gen_measure(ref):
    rng = np.random.default_rng(5)
    n = 7
    psi = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    psi /= np.linalg.norm(psi)
    mps = ref.MPS.from_vector(psi)
    out = {"psi": psi}
    pop, dpop, sse, bonds = np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(n + 1)
    mps.measure(pop, dpop, sse, bonds)
    out.update(pop=pop, dpop=dpop, sse=sse, bonds=bonds)
    p = [0.0, 1.0, 0.3, 0.5, 0.0, 0.9, 1.0]
    mps2 = ref.MPS.from_density_distribution(p)
    pop, dpop, sse, bonds = np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(n + 1)
    mps2.measure(pop, dpop, sse, bonds)
    out.update(prod_p=np.array(p), prod_pop=pop, prod_dpop=dpop, prod_sse=sse, prod_bonds=bonds)
    mps3 = ref.MPS.from_vector(psi)
    out["from_vector_shapes"] = np.array([a.shape for a in mps3.A])
    out["as_vector"] = mps3.as_vector()
    np.savez_compressed(os.path.join(HERE, "measure_case.npz"), **out)


GENERATORS = {"mpo": gen_mpo, "exact": gen_exact, "tdvp": gen_tdvp, "a1tdvp": gen_a1tdvp,
              "qr": lambda ref: gen_qr(), "measure": gen_measure}


def main() -> None:
    if len(sys.argv) < 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the reference checkout> [fixture ...]\n"
                 "fixtures: " + " ".join(GENERATORS) + " (default: all)")
    ref = load_reference(sys.argv[1])
    for name in sys.argv[2:] or list(GENERATORS):
        GENERATORS[name](ref)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
