"""Exact state-vector path on the GPU against the oracle and the reference's
own outputs.  Tolerances: max|d<n_i>| <= 1e-10 for the FP64 path (the target
bound for exact), <= 1e-5 for the mixed (complex64) path."""
import types

import numpy as np
import pytest

from oracle import qca_oracle as O

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-10
TOL_MIXED = 1e-5


def make(n, d, lo, hi, p, dt, precision="fp64", krylov=30):
    from qca_gb300 import GpuExact, MPO, MPS, Rules
    H = MPO.hamiltonian_from_rules(Rules(n, range(lo, hi), d))
    args = types.SimpleNamespace(step_size=dt, algorithm="exact", precision=precision, krylov_dim=krylov)
    return GpuExact(MPS.from_density_distribution(p), H, args)


def rows(n):
    return np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(n + 1)


@pytest.mark.parametrize("precision,tol", [("fp64", TOL_FP64), ("mixed", TOL_MIXED)])
@pytest.mark.parametrize("name", ["single8", "rand10"])
def test_exact_matches_reference_series(golden, name, precision, tol):
    e = golden("exact_series.npz")
    n, d, lo, hi, dt, steps = e[name + "_meta"]
    n, d, steps = int(n), int(d), int(steps)
    alg = make(n, d, int(lo), int(hi), e[name + "_p"], float(dt), precision)
    for s in range(steps + 1):
        pop, dpop, sse, bonds = rows(n)
        alg.measure(pop, dpop, sse, bonds)
        assert np.abs(pop - e[name + "_pop"][s]).max() < tol
        assert np.array_equal(dpop, e[name + "_dpop"][s])
        assert np.array_equal(bonds, e[name + "_bonds"][s])
        if s < steps:
            alg.do_time_step()
    if precision == "fp64":
        assert np.abs(alg.state_vector() - e[name + "_final"]).max() < TOL_FP64


@pytest.mark.parametrize("n", [13, 14, 16, 18])
@pytest.mark.parametrize("precision,tol", [("fp64", TOL_FP64), ("mixed", TOL_MIXED)])
def test_exact_multiphase_against_oracle(n, precision, tol):
    d, lo, hi, dt, steps = 2, 2, 4, 0.05, 4
    th = O.random_thetas(n, seed=n)
    p = np.sin(th) ** 2
    alg = make(n, d, lo, hi, p, dt, precision)
    alg.evolve(steps)
    ref = O.exact_evolve(O.product_state_vector(p), n, d, range(lo, hi), dt, steps)
    got = alg.state_vector()
    assert np.abs(O.populations_from_vector(got, n) - O.populations_from_vector(ref, n)).max() < tol
    if precision == "fp64":
        assert np.abs(got - ref).max() < TOL_FP64


def test_exact_large_step_is_substepped():
    n, d, lo, hi = 10, 1, 1, 2
    p = np.zeros(n)
    p[4] = 1.0
    alg = make(n, d, lo, hi, p, 3.0)
    alg.do_time_step()
    ref = O.exact_evolve(O.product_state_vector(p), n, d, range(lo, hi), 3.0, 1)
    assert np.abs(alg.state_vector() - ref).max() < TOL_FP64


def test_exact_krylov_breakdown_on_invariant_state():
    # all cells dead and the rule needs one alive neighbour: H|0...0> = 0
    n = 9
    alg = make(n, 1, 1, 2, np.zeros(n), 0.1)
    alg.evolve(3)
    v = alg.state_vector()
    assert abs(v[0] - 1.0) < 1e-14 and np.abs(v[1:]).max() < 1e-14


def test_exact_measure_density_matrices():
    n = 11
    p = np.sin(O.random_thetas(n, 3)) ** 2
    alg = make(n, 2, 2, 4, p, 0.05)
    alg.evolve(3)
    pop, dpop, sse, bonds = rows(n)
    alg.measure(pop, dpop, sse, bonds)
    A = O.mps_from_vector(alg.state_vector())
    rpop, rdpop, rsse, rbonds = O.measure(A)
    assert np.abs(pop - rpop).max() < 1e-12
    assert np.abs(sse - rsse).max() < 1e-9
    assert np.array_equal(bonds, rbonds)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 2e-5)])
def test_exact_n24_time_reversal(precision, tol):
    """Size-independent property at the 2^24-amplitude workload: evolving by +dt
    then -dt returns the initial state; the norm is conserved."""
    n, d, lo, hi, dt = 24, 2, 2, 4, 0.05
    p = np.sin(O.random_thetas(n, 2024)) ** 2
    alg = make(n, d, lo, hi, p, dt, precision)
    v0 = alg.state_vector()
    alg.evolve(3, dt)
    v1 = alg.state_vector()
    assert abs(np.linalg.norm(v1) - 1.0) < tol
    assert np.abs(v1 - v0).max() > 1e-4  # it moved
    alg.evolve(3, -dt)
    v2 = alg.state_vector()
    assert np.abs(v2 - v0).max() < tol
