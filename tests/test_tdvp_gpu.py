"""TDVP on the GPU against the reference's own outputs (gauge-consistent form,
golden fixtures from tests/golden/make_golden.py) and against the oracle.

Tolerances (the target bounds): FP64 plain path max|d<n_i>| <= 1e-8 with
identical truncated bond dimensions; mixed path max|d<n_i>| <= 1e-5 for 2TDVP.
Mixed 1TDVP is held to 5e-5: its bond growth uses the complement columns of a
complete QR (tdvp.py:74, 95) of nearly rank-deficient matrices, and below the
FP32 rounding floor those columns are set by rounding noise."""
import types

import numpy as np
import pytest

from oracle import qca_oracle as O

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-8
TOL_MIXED = 1e-5
TOL_MIXED_1TDVP = 5e-5
CASES = ["t2_single8", "t1_single8", "t2_rand7", "t1_rand7", "t2_rand9_d3"]


def make(alg_name, n, d, lo, hi, p, dt, chi, eps, precision="fp64", engine=None):
    from qca_gb300 import GpuTDVP, MPO, MPS, Rules
    H = MPO.hamiltonian_from_rules(Rules(n, range(lo, hi), d))
    args = types.SimpleNamespace(step_size=dt, algorithm=alg_name, max_bond_dim=chi, svd_epsilon=eps,
                                 precision=precision)
    return GpuTDVP(MPS.from_density_distribution(p), H, args, engine=engine)


def rows(n):
    return np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(n + 1)


def meta(t, name):
    n, d, lo, hi, dt, chi, eps, steps = t[name + "_meta"]
    return int(n), int(d), int(lo), int(hi), float(dt), int(chi), float(eps), int(steps)


@pytest.mark.parametrize("name", CASES)
def test_tdvp_fp64_matches_reference_fixed(golden, name):
    t = golden("tdvp_series.npz")
    n, d, lo, hi, dt, chi, eps, steps = meta(t, name)
    alg = make(str(t[name + "_alg"]), n, d, lo, hi, t[name + "_p"], dt, chi, eps)
    for s in range(steps + 1):
        pop, dpop, sse, bonds = rows(n)
        alg.measure(pop, dpop, sse, bonds)
        assert np.abs(pop - t[f"{name}_fixed_pop"][s]).max() < TOL_FP64, s
        assert np.array_equal(bonds, t[f"{name}_fixed_bonds"][s]), (s, bonds)
        assert np.abs(sse - t[f"{name}_fixed_sse"][s]).max() < 1e-6
        if s < steps:
            alg.do_time_step()


@pytest.mark.parametrize("name", CASES)
def test_tdvp_mixed_matches_reference_fixed(golden, name):
    t = golden("tdvp_series.npz")
    n, d, lo, hi, dt, chi, eps, steps = meta(t, name)
    alg_name = str(t[name + "_alg"])
    tol = TOL_MIXED if alg_name == "2tdvp" else TOL_MIXED_1TDVP
    alg = make(alg_name, n, d, lo, hi, t[name + "_p"], dt, chi, max(eps, 1e-6), "mixed")
    for s in range(steps + 1):
        pop, dpop, sse, bonds = rows(n)
        alg.measure(pop, dpop, sse, bonds)
        assert np.abs(pop - t[f"{name}_fixed_pop"][s]).max() < tol, s
        if s < steps:
            alg.do_time_step()


@pytest.mark.parametrize("alg_name", ["2tdvp", "1tdvp"])
def test_tdvp_state_matches_oracle_without_measurements(alg_name):
    n, d, lo, hi, dt, chi, eps, steps = 9, 2, 2, 4, 0.05, 12, 1e-9, 4
    p = np.sin(O.random_thetas(n, 77)) ** 2
    alg = make(alg_name, n, d, lo, hi, p, dt, chi, eps)
    W = O.build_mpo(O.Rules(n, range(lo, hi), d))
    orc = O.TDVPOracle(O.mps_from_density_distribution(p), W, alg_name, dt, chi, eps, fixed=True)
    alg.evolve(steps)
    for _ in range(steps):
        orc.step()
    got = alg.psi.as_vector()
    ref = O.mps_as_vector(orc.A)
    assert np.abs(got - ref).max() < TOL_FP64
    assert alg.bonds() == [a.shape[1] for a in orc.A] + [1]


def test_tdvp_batched_equals_alone():
    """Chains of different length, rule and bond cap stepped together in one engine
    give the same populations as each chain stepped alone."""
    from qca_gb300.algorithms import _Engine
    from qca_gb300 import _lib
    specs = [("2tdvp", 8, 1, 1, 2, 8), ("2tdvp", 11, 2, 2, 4, 16), ("1tdvp", 7, 2, 2, 4, 8), ("2tdvp", 6, 3, 2, 5, 8)]
    eng = _Engine(_lib.QCA_PREC_FP64)
    together = []
    for k, (a, n, d, lo, hi, chi) in enumerate(specs):
        p = np.sin(O.random_thetas(n, 100 + k)) ** 2
        together.append(make(a, n, d, lo, hi, p, 0.05, chi, 1e-9, engine=eng))
    import ctypes
    ids = (ctypes.c_int * len(together))(*[g._chain for g in together])
    _lib.call("qca_engine_step_chains", eng.h, ids, len(together), 3, None)
    for k, (a, n, d, lo, hi, chi) in enumerate(specs):
        p = np.sin(O.random_thetas(n, 100 + k)) ** 2
        alone = make(a, n, d, lo, hi, p, 0.05, chi, 1e-9)
        alone.evolve(3)
        r1, r2 = rows(n), rows(n)
        together[k].measure(*r1)
        alone.measure(*r2)
        assert np.abs(r1[0] - r2[0]).max() < 1e-12
        assert np.array_equal(r1[3], r2[3])


def test_tdvp_rejects_bad_arguments():
    from qca_gb300 import _lib
    with pytest.raises((ValueError, _lib.QcaError)):
        make("2tdvp", 6, 1, 1, 2, np.zeros(6), 0.1, 0, 1e-8)


@pytest.mark.parametrize("alg_name,tol", [("2tdvp", 5e-4), ("1tdvp", 1e-2)])
def test_tdvp_tracks_exact_evolution(alg_name, tol):
    """The benchmark configuration checked against the exact state vector
    (distance 1, interval [1,1], only the centre cell alive, dt = 0.1), at N = 10
    and full bond dimension: TDVP differs from the exact evolution only by its
    integrator error (a few 1e-5 for 2TDVP and 1e-3 for 1TDVP per unit time at
    this step size, measured on the reference)."""
    import types
    from qca_gb300 import GpuExact, MPO, MPS, Rules
    n, d, lo, hi, dt, steps = 10, 1, 1, 2, 0.1, 10
    p = np.zeros(n)
    p[n // 2] = 1.0
    H = MPO.hamiltonian_from_rules(Rules(n, range(lo, hi), d))
    ex = GpuExact(MPS.from_density_distribution(p), H, types.SimpleNamespace(step_size=dt, algorithm="exact"))
    td = make(alg_name, n, d, lo, hi, p, dt, 32, 1e-12)
    worst = 0.0
    for s in range(steps):
        ex.do_time_step()
        td.do_time_step()
        r1, r2 = rows(n), rows(n)
        ex.measure(*r1)
        td.measure(*r2)
        worst = max(worst, np.abs(r1[0] - r2[0]).max())
    assert worst < tol, worst


@pytest.mark.parametrize("alg_name", ["2tdvp", "1tdvp"])
def test_tdvp_mixed_tracks_fp64_at_large_bonds(alg_name):
    """A random MPS with bonds up to 48 (local problems with M = 4 D >= 96 take the
    tcgen05 contraction kernel): two mixed-precision steps agree with the FP64
    path (itself pinned to the reference).  The bond cap (96) is above what two
    steps reach.  On this random, highly entangled state the mixed 2TDVP differs
    from FP64 by 1.4e-5 after two steps with the tcgen05, the mma.sync and the FP32
    CUDA-core contraction kernels alike (set by the FP32 storage of the state):
    tolerance 3e-5.  1TDVP grows bonds from the complement columns of nearly
    rank-deficient complete QRs, which amplify contraction rounding (1e-6 to 3e-5
    depending on the kernel): tolerance 5e-5, as for its golden fixtures."""
    from qca_gb300 import GpuTDVP, MPO, MPS, Rules
    n, d, lo, hi, dt, chi = 14, 2, 2, 4, 0.05, 96
    rng = np.random.default_rng(77)
    dims = [min(2 ** min(i, n - i), 48) for i in range(n + 1)]
    A = [(rng.standard_normal((2, dims[i], dims[i + 1])) + 1j * rng.standard_normal((2, dims[i], dims[i + 1])))
         / np.sqrt(4.0 * dims[i]) for i in range(n)]
    env = np.ones((1, 1), dtype=np.complex128)
    for a in A:
        env = sum(a[s].conj().T @ env @ a[s] for s in range(2))
    A[0] = A[0] / np.sqrt(env[0, 0].real)
    H = MPO.hamiltonian_from_rules(Rules(n, range(lo, hi), d))
    res = []
    for prec in ("fp64", "mixed"):
        args = types.SimpleNamespace(step_size=dt, algorithm=alg_name, max_bond_dim=chi, svd_epsilon=1e-10,
                                     precision=prec)
        alg = GpuTDVP(MPS.from_tensors(A), H, args)
        alg.evolve(2)
        r = rows(n)
        alg.measure(*r)
        res.append(r)
    assert np.abs(res[0][0] - res[1][0]).max() < (3e-5 if alg_name == "2tdvp" else TOL_MIXED_1TDVP)



@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_1tdvp_long_chain(precision):
    """1TDVP on an 88-site chain (bond cap 16), one step from a product state,
    completes in both precisions within 2e-4 of the Krylov oracle.

    The bound is set by the algorithm, not the precision: 1TDVP's complement columns
    amplify rounding (a 1e-14 perturbation of the initial state moves the oracle's
    own populations by 1.5e-5 after one step at this size; measured GPU FP64
    deviation 3-6e-5).  The mixed case is the regression test of the Householder
    norm: with its squares taken in FP32 the residue columns of the rank-deficient
    complete QRs underflowed, the reflectors lost unitarity and the first left sweep
    failed with QCA_ERR_NAN."""
    n, chi = 88, 16
    p = np.sin(O.random_thetas(n, 5)) ** 2
    alg = make("1tdvp", n, 2, 1, 2, p, 0.05, chi, 1e-10, precision)
    alg.evolve(1)
    r = rows(n)
    alg.measure(*r)
    assert np.all(np.isfinite(r[0]))
    orc = O.TDVPKrylovOracle(O.mps_from_density_distribution(p), O.build_mpo(O.Rules(n, range(1, 2), 2)),
                             "1tdvp", 0.05, chi, 1e-10)
    orc.step()
    assert np.abs(r[0] - orc.measure()[0]).max() < 2e-4


@pytest.mark.parametrize("name", ["a1_single8", "a1_rand8"])
def test_a1tdvp_matches_reference(golden, name):
    """a1tdvp (tdvp.py:212-267) on the GPU against the reference's own run (fixture
    a1tdvp_series.npz, exact_exponential local evolution): populations within
    1e-8 and identical bond dimensions after every step, with the reference's
    measurements between the steps."""
    t = golden("a1tdvp_series.npz")
    n, d, lo, hi, dt, chi, eps, steps = t[name + "_meta"]
    n, d, lo, hi, chi, steps = int(n), int(d), int(lo), int(hi), int(chi), int(steps)
    alg = make("a1tdvp", n, d, lo, hi, t[name + "_p"], float(dt), chi, float(eps))
    for s in range(steps + 1):
        pop, dpop, sse, bonds = rows(n)
        alg.measure(pop, dpop, sse, bonds)
        assert np.abs(pop - t[name + "_ref_pop"][s]).max() < TOL_FP64, s
        assert np.array_equal(bonds, t[name + "_ref_bonds"][s]), (s, bonds)
        if s < steps:
            alg.do_time_step()
