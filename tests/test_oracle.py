"""The oracle against the reference's own outputs (golden fixtures made by
tests/golden/make_golden.py from the reference implementation), and against
properties of the dynamics that hold at any size: a real symmetric Hamiltonian,
unitary and time-reversible exact evolution, and 2TDVP at full bond dimension
tracking the exact evolution with its integrator's order."""
import numpy as np
import pytest
from scipy.linalg import expm as scipy_expm

from oracle import qca_oracle as O

RULES = [(1, 1, 2), (1, 2, 4), (1, 2, 5), (2, 1, 2), (2, 2, 4), (2, 2, 5), (3, 1, 2), (3, 2, 4), (3, 2, 5)]


@pytest.mark.parametrize("d,lo,hi", RULES)
def test_oracle_mpo_matches_reference(golden, d, lo, hi):
    g = golden("mpo_rules.npz")
    W = O.build_mpo(O.Rules(6, range(lo, hi), d))
    key = f"d{d}_{lo}{hi}"
    assert np.array_equal(W[2], g[key + "_bulk"])
    assert np.array_equal(W[0], g[key + "_first"])
    assert np.array_equal(W[-1], g[key + "_last"])


@pytest.mark.parametrize("d,lo,hi", RULES)
def test_oracle_matrix_free_equals_mpo(d, lo, hi):
    n = 7
    Hm = O.mpo_as_matrix(O.build_mpo(O.Rules(n, range(lo, hi), d)))
    Hs = O.sparse_rule_hamiltonian(n, d, range(lo, hi)).toarray()
    assert np.abs(Hm - Hs).max() == 0.0
    assert np.abs(Hs - Hs.T).max() == 0.0


@pytest.mark.parametrize("name", ["single8", "rand10"])
def test_oracle_exact_matches_reference(golden, name):
    e = golden("exact_series.npz")
    n, d, lo, hi, dt, steps = e[name + "_meta"]
    n, d, steps = int(n), int(d), int(steps)
    psi = O.product_state_vector(e[name + "_p"])
    for s in range(steps + 1):
        pop = O.populations_from_vector(psi, n)
        assert np.abs(pop - e[name + "_pop"][s]).max() < 1e-12
        psi = O.exact_evolve(psi, n, d, range(int(lo), int(hi)), float(dt), 1)


CASES = ["t2_single8", "t1_single8", "t2_rand7", "t1_rand7", "t2_rand9_d3"]


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("mode", ["fixed", "ref"])
def test_oracle_tdvp_matches_reference(golden, name, mode):
    t = golden("tdvp_series.npz")
    n, d, lo, hi, dt, chi, eps, steps = t[name + "_meta"]
    n, d, steps = int(n), int(d), int(steps)
    W = O.build_mpo(O.Rules(n, range(int(lo), int(hi)), d))
    orc = O.TDVPOracle(O.mps_from_density_distribution(t[name + "_p"]), W, str(t[name + "_alg"]), float(dt),
                       int(chi), float(eps), fixed=(mode == "fixed"))
    for s in range(steps + 1):
        pop, dpop, sse, bonds = orc.measure()
        assert np.abs(pop - t[f"{name}_{mode}_pop"][s]).max() < 1e-12
        assert np.array_equal(bonds, t[f"{name}_{mode}_bonds"][s])
        assert np.nanmax(np.abs(sse - t[f"{name}_{mode}_sse"][s])) < 1e-10
        if s < steps:
            orc.step()


def test_oracle_measure_matches_reference(golden):
    m = golden("measure_case.npz")
    pop, dpop, sse, b = O.measure(O.mps_from_vector(m["psi"]))
    assert np.abs(pop - m["pop"]).max() < 1e-14
    assert np.abs(sse - m["sse"]).max() < 1e-12
    assert np.array_equal(b, m["bonds"])
    A = O.mps_from_vector(m["psi"])
    assert np.array_equal(np.array([a.shape for a in A]), m["from_vector_shapes"])
    assert np.abs(O.mps_as_vector(A) - m["as_vector"]).max() < 1e-14


def test_oracle_qr_convention(golden):
    """numpy.linalg.qr (the call at mps.py:86) as the convention the device QR follows."""
    g = golden("qr_lapack.npz")
    for k in range(5):
        a = g[f"a{k}"]
        for mode in ("reduced", "complete"):
            q, r = np.linalg.qr(a, mode=mode)
            assert np.abs(q - g[f"a{k}_{mode}_q"]).max() < 1e-13
            assert np.abs(r - g[f"a{k}_{mode}_r"]).max() < 1e-13


def test_truncation_rule():
    s = np.array([1.0, 0.1, 1e-5, 1e-9, 1e-12])
    assert O.truncation_rank(s, 10, 1e-8) == 3
    assert O.truncation_rank(s, 2, 1e-8) == 2
    assert O.truncation_rank(s, 10, 1e-13) == 5


@pytest.mark.parametrize("d,lo,hi", RULES)
def test_oracle_hamiltonian_is_real_symmetric(d, lo, hi):
    """H = sum_i X_i P_i(neighbours) is a real symmetric 0/1 matrix for every rule."""
    H = O.sparse_rule_hamiltonian(7, d, range(lo, hi))
    assert abs(H - H.T).max() == 0
    assert np.all(np.isin(H.data, [0.0, 1.0]))


def test_oracle_exact_is_unitary_and_reversible():
    n, d, rule = 8, 2, range(2, 4)
    psi0 = O.product_state_vector(np.sin(O.random_thetas(n, 5)) ** 2)
    psi = O.exact_evolve(psi0, n, d, rule, 0.07, 3)
    assert abs(np.linalg.norm(psi) - 1.0) < 1e-12
    back = O.exact_evolve(psi, n, d, rule, -0.07, 3)
    assert np.abs(back - psi0).max() < 1e-10


def test_oracle_2tdvp_full_bond_tracks_exact():
    """At full bond dimension the gauge-consistent 2TDVP differs from the exact
    evolution only by its integrator error, which falls by about 2^3 when dt halves
    (distance 1, interval [1,1], centre cell alive, N = 6)."""
    n, d, lo, hi = 6, 1, 1, 2
    p = np.zeros(n)
    p[n // 2] = 1.0
    W = O.build_mpo(O.Rules(n, range(lo, hi), d))
    worst = {}
    for dt, steps in [(0.1, 5), (0.05, 10)]:
        orc = O.TDVPOracle(O.mps_from_density_distribution(p), W, "2tdvp", dt, 64, 1e-14, fixed=True)
        psi = O.product_state_vector(p)
        w = 0.0
        for _ in range(steps):
            orc.step()
            psi = O.exact_evolve(psi, n, d, range(lo, hi), dt, 1)
            w = max(w, np.abs(O.populations_from_vector(O.mps_as_vector(orc.A), n)
                              - O.populations_from_vector(psi, n)).max())
        worst[dt] = w
    assert worst[0.1] < 5e-5 and worst[0.05] < 5e-6
    assert worst[0.1] / worst[0.05] > 4.0


def test_heff_apply_is_the_transposed_assembled_matrix():
    """The matrix-free operator equals M^T of the reference's assembled effective
    Hamiltonian (tdvp.py:298-326 with lautils.py:80-81), for the 1-/2-site form and
    the bond form."""
    rng = np.random.default_rng(0)
    Dl, Dr, wl, wr = 3, 4, 5, 6
    cx = lambda *s: rng.standard_normal(s) + 1j * rng.standard_normal(s)  # noqa: E731
    L, R, W, x = cx(Dl, wl, Dl), cx(Dr, wr, Dr), cx(4, 4, wl, wr), cx(4, Dl, Dr)
    M = O._heff_site(L, R, W)
    assert np.abs(O.heff_apply(L, R, W, x).reshape(-1) - M.T @ x.reshape(-1)).max() < 1e-12
    Rb, xb = cx(Dr, wl, Dr), cx(Dl, Dr)
    K = O._keff_bond(L, Rb)
    assert np.abs(O.heff_apply(L, Rb, None, xb).reshape(-1) - K.T @ xb.reshape(-1)).max() < 1e-12


def test_krylov_expm_matches_dense_exponential():
    rng = np.random.default_rng(1)
    a = rng.standard_normal((60, 60)) + 1j * rng.standard_normal((60, 60))
    h = a + a.conj().T
    v = rng.standard_normal(60) + 1j * rng.standard_normal(60)
    want = scipy_expm(-1j * 0.3 * h) @ v
    got = O.krylov_expm(lambda x: h @ x, v, 0.3)
    assert np.abs(got - want).max() < 1e-11


@pytest.mark.parametrize("alg", ["2tdvp", "1tdvp"])
def test_krylov_tdvp_oracle_matches_dense_oracle(alg):
    """The matrix-free TDVP restatement (Lanczos local exponentials) used beyond the
    reach of the dense eigh gives the dense oracle's state and bond dimensions."""
    n = 9
    p = np.sin(O.random_thetas(n, 77)) ** 2
    W = O.build_mpo(O.Rules(n, range(2, 4), 2))
    a = O.TDVPOracle(O.mps_from_density_distribution(p), W, alg, 0.05, 12, 1e-9)
    b = O.TDVPKrylovOracle(O.mps_from_density_distribution(p), W, alg, 0.05, 12, 1e-9)
    for _ in range(3):
        a.step()
        b.step()
        assert [x.shape for x in a.A] == [x.shape for x in b.A]
    assert np.abs(O.mps_as_vector(a.A) - O.mps_as_vector(b.A)).max() < 1e-10


@pytest.mark.parametrize("name", ["a1_single8", "a1_rand8"])
def test_oracle_a1tdvp_matches_reference(golden, name):
    """The oracle's a1tdvp (tdvp.py:212-267, the reference's exact_exponential local
    evolution, its environments as the reference keeps them) reproduces the
    reference's populations and bond dimensions (fixture a1tdvp_series.npz)."""
    t = golden("a1tdvp_series.npz")
    n, d, lo, hi, dt, chi, eps, steps = t[name + "_meta"]
    n, d, lo, hi, chi, steps = int(n), int(d), int(lo), int(hi), int(chi), int(steps)
    orc = O.TDVPOracle(O.mps_from_density_distribution(t[name + "_p"]), O.build_mpo(O.Rules(n, range(lo, hi), d)),
                       "a1tdvp", float(dt), chi, float(eps), fixed=False)
    for s in range(steps + 1):
        pop, _, _, bonds = O.measure(orc.A)
        assert np.abs(pop - t[name + "_ref_pop"][s]).max() < 1e-12, s
        assert np.array_equal(bonds, t[name + "_ref_bonds"][s]), s
        if s < steps:
            orc.step()


def test_1tdvp_growth_from_product_states_is_ill_conditioned():
    """Characterises the reference algorithm, not an implementation: 1TDVP grows its
    bonds from the complement columns of complete QRs of rank-deficient site
    matrices (tdvp.py:65-105), and those columns are set by rounding-level residues,
    so a 1e-14 perturbation of the initial product state moves the populations
    after one step by orders of magnitude more (5.6e-7 at N = 20, about 1.5e-5 at
    N = 88), while 2TDVP passes it through at its own size.  This bounds how closely
    any two implementations of 1TDVP can agree on long chains."""
    n = 20
    p = np.sin(O.random_thetas(n, 5)) ** 2
    W = O.build_mpo(O.Rules(n, range(1, 2), 2))
    rng = np.random.default_rng(1)

    def run(alg, pert):
        A = O.mps_from_density_distribution(p)
        if pert:
            A = [a + pert * (rng.standard_normal(a.shape) + 1j * rng.standard_normal(a.shape)) for a in A]
        orc = O.TDVPKrylovOracle(A, W, alg, 0.05, 16, 1e-10)
        orc.step()
        return orc.measure()[0]

    assert np.abs(run("1tdvp", 0.0) - run("1tdvp", 1e-14)).max() > 1e-8
    assert np.abs(run("2tdvp", 0.0) - run("2tdvp", 1e-14)).max() < 1e-12
