"""Parity at the sizes of the benchmark configurations.

* Exact evolution at its full size (N = 24, 2^24 amplitudes, distance 2,
  interval [2,3], random product state, Krylov dimension 30, dt = 0.05) against
  the oracle's sparse restatement of algorithms/exact.py:27-28 for three steps
  (fixture ``exact24.npz``, made by ``tests/golden/make_exact24.py``): FP64
  within 1e-10, mixed within 1e-5.
* 2TDVP at the single-chain shape (N = 64, distance 2, interval [2,3], random
  product state, cutoff 1e-10, dt = 0.05) with the bond cap at 64, where the
  oracle's matrix-free restatement of tdvp.py (``TDVPKrylovOracle``) still runs
  in seconds per step: FP64 within 1e-8 with identical bond dimensions at every
  step, mixed within 1e-5.
* The plain 2TDVP configuration (N = 15, distance 1, interval [1,1], only the
  centre cell alive, bond cap 64, cutoff 1e-8, dt = 0.1, <n_i> recorded every 10
  steps; the first 200 of its 1000 steps, all 1000 with QCA_FULL_CONFIGS=1)
  against the FP64 exact state vector (2^15 amplitudes), itself pinned to the
  oracle over its first steps.  TDVP differs
  from the exact evolution by its integrator and truncation error only.
"""
import types

import numpy as np
import pytest

from oracle import qca_oracle as O

pytestmark = pytest.mark.gpu


def _exact(n, d, lo, hi, p, dt, precision, m=30):
    from qca_gb300 import GpuExact, MPO, MPS, Rules
    H = MPO.hamiltonian_from_rules(Rules(n, range(lo, hi), d))
    return GpuExact(MPS.from_density_distribution(p), H, types.SimpleNamespace(
        step_size=dt, algorithm="exact", precision=precision, krylov_dim=m))


def _tdvp(n, d, lo, hi, p, dt, chi, eps, precision, alg="2tdvp"):
    from qca_gb300 import GpuTDVP, MPO, MPS, Rules
    H = MPO.hamiltonian_from_rules(Rules(n, range(lo, hi), d))
    return GpuTDVP(MPS.from_density_distribution(p), H, types.SimpleNamespace(
        step_size=dt, algorithm=alg, max_bond_dim=chi, svd_epsilon=eps, precision=precision))


def _pop(alg, n):
    r = [np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(n + 1)]
    alg.measure(*r)
    return r[0], r[3]


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-5)])
def test_exact_n24_matches_oracle(golden, precision, tol):
    from qca_gb300 import _lib
    t = golden("exact24.npz")
    n, d, lo, hi, dt, steps = t["meta"]
    n, d, lo, hi, steps = int(n), int(d), int(lo), int(hi), int(steps)
    alg = _exact(n, d, lo, hi, t["p"], float(dt), precision)
    psi0 = O.product_state_vector(t["p"]) if precision == "fp64" else None
    for s in range(steps):
        alg.do_time_step()
        pop = np.zeros(n)
        rho = np.zeros((n, 2, 2), dtype=np.complex128)
        _lib.call("qca_exact_measure", alg._h, pop.ctypes.data_as(_lib._PD),
                  rho.view(np.float64).ctypes.data_as(_lib._PD), None)
        assert np.abs(pop - t["pop"][s]).max() < tol, (s, np.abs(pop - t["pop"][s]).max())
        assert np.abs(rho - t["rho"][s]).max() < tol, s
        if psi0 is not None:
            assert abs(np.vdot(psi0, alg.state_vector()) - t["overlap"][s]) < tol, s


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-8), ("mixed", 1e-5)])
def test_2tdvp_single_chain_shape_matches_krylov_oracle(precision, tol):
    n, d, lo, hi, dt, chi, eps, steps = 64, 2, 2, 4, 0.05, 64, 1e-10, 4
    p = np.sin(np.random.default_rng(64).uniform(0.0, np.pi / 2, size=n)) ** 2
    alg = _tdvp(n, d, lo, hi, p, dt, chi, eps, precision)
    orc = O.TDVPKrylovOracle(O.mps_from_density_distribution(p), O.build_mpo(O.Rules(n, range(lo, hi), d)),
                             "2tdvp", dt, chi, eps)
    for s in range(steps):
        alg.do_time_step()
        orc.step()
        pop, bonds = _pop(alg, n)
        want_bonds = [a.shape[1] for a in orc.A] + [1]
        want = O.measure([a.copy() for a in orc.A])[0]
        err = np.abs(pop - want).max()
        assert err < tol, (s, err)
        if precision == "fp64":
            assert list(bonds.astype(int)) == want_bonds, s
    assert max(a.shape[2] for a in orc.A) == chi  # the cap was reached


def test_2tdvp_plain_configuration_tracks_exact_state_vector():
    """The full 1000 steps take about 14 minutes in FP64 on one GB300 (FP64 runs at
    1/64 of the FP32 rate on this part), longer than a test suite should; the
    default covers the first 200 steps, QCA_FULL_CONFIGS=1 runs all 1000."""
    import os
    full = os.environ.get("QCA_FULL_CONFIGS") == "1"
    n, d, lo, hi, dt, chi, eps, steps, every = 15, 1, 1, 2, 0.1, 64, 1e-8, 1000 if full else 200, 10
    p = np.zeros(n)
    p[n // 2] = 1.0
    ex = _exact(n, d, lo, hi, p, dt, "fp64")
    td = _tdvp(n, d, lo, hi, p, dt, chi, eps, "fp64")
    # the exact path at N = 15 is pinned to the oracle over its first steps
    ex.evolve(5)
    ref = O.exact_evolve(O.product_state_vector(p), n, d, range(lo, hi), dt, 5)
    assert np.abs(ex.state_vector() - ref).max() < 1e-10
    ex.set_state_vector(O.product_state_vector(p))
    worst, worst_step = 0.0, 0
    for s in range(every, steps + 1, every):
        ex.evolve(every)
        td.evolve(every)
        e_pop, _ = _pop(ex, n)
        t_pop, _ = _pop(td, n)
        err = np.abs(e_pop - t_pop).max()
        if err > worst:
            worst, worst_step = err, s
    print(f"plain 2TDVP configuration: max|d<n_i>| vs exact = {worst:.3e} (step {worst_step})")
    assert worst < 1e-2, (worst, worst_step)
