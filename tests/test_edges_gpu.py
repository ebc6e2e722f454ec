"""Edge cases of the GPU paths against the oracle: the smallest chains (N = 2, 3,
4), rules whose neighbourhood reaches past both ends of the chain or starts at
zero live neighbours, a bond cap of 1 (the evolution stays a product state), and
state vectors of 4 to 32 amplitudes.  Bounds: FP64 1e-8 (TDVP state vectors, with
identical bond dimensions) and 1e-10 (exact populations); mixed 1e-5."""
import types

import numpy as np
import pytest

from oracle import qca_oracle as O

pytestmark = pytest.mark.gpu

SMALL = [(2, 1, 1, 2), (3, 1, 1, 2), (3, 2, 0, 2), (4, 3, 1, 3)]


def tdvp(alg_name, n, d, lo, hi, p, dt, chi, eps, precision="fp64"):
    from qca_gb300 import GpuTDVP, MPO, MPS, Rules
    H = MPO.hamiltonian_from_rules(Rules(n, range(lo, hi), d))
    args = types.SimpleNamespace(step_size=dt, algorithm=alg_name, max_bond_dim=chi, svd_epsilon=eps,
                                 precision=precision)
    return GpuTDVP(MPS.from_density_distribution(p), H, args)


@pytest.mark.parametrize("alg_name", ["2tdvp", "1tdvp"])
@pytest.mark.parametrize("n,d,lo,hi", SMALL)
def test_tdvp_small_chains_match_oracle(alg_name, n, d, lo, hi):
    dt, chi, eps, steps = 0.1, 8, 1e-12, 3
    p = np.sin(O.random_thetas(n, 40 + n)) ** 2
    alg = tdvp(alg_name, n, d, lo, hi, p, dt, chi, eps)
    orc = O.TDVPOracle(O.mps_from_density_distribution(p), O.build_mpo(O.Rules(n, range(lo, hi), d)), alg_name, dt,
                       chi, eps, fixed=True)
    alg.evolve(steps)
    for _ in range(steps):
        orc.step()
    assert np.abs(alg.psi.as_vector() - O.mps_as_vector(orc.A)).max() < 1e-8
    assert alg.bonds() == [a.shape[1] for a in orc.A] + [1]


@pytest.mark.parametrize("alg_name", ["2tdvp", "1tdvp"])
def test_tdvp_bond_cap_one_stays_a_product_state(alg_name):
    n, d, lo, hi, dt, eps, steps = 6, 1, 1, 2, 0.1, 1e-12, 3
    p = np.sin(O.random_thetas(n, 11)) ** 2
    alg = tdvp(alg_name, n, d, lo, hi, p, dt, 1, eps)
    orc = O.TDVPOracle(O.mps_from_density_distribution(p), O.build_mpo(O.Rules(n, range(lo, hi), d)), alg_name, dt,
                       1, eps, fixed=True)
    alg.evolve(steps)
    for _ in range(steps):
        orc.step()
    assert alg.bonds() == [1] * (n + 1)
    assert np.abs(alg.psi.as_vector() - O.mps_as_vector(orc.A)).max() < 1e-8


@pytest.mark.parametrize("n,d,lo,hi", SMALL)
def test_tdvp_small_chains_mixed(n, d, lo, hi):
    p = np.sin(O.random_thetas(n, 40 + n)) ** 2
    alg = tdvp("2tdvp", n, d, lo, hi, p, 0.1, 8, 1e-6, "mixed")
    orc = O.TDVPOracle(O.mps_from_density_distribution(p), O.build_mpo(O.Rules(n, range(lo, hi), d)), "2tdvp", 0.1,
                       8, 1e-6, fixed=True)
    alg.evolve(3)
    for _ in range(3):
        orc.step()
    got = O.populations_from_vector(alg.psi.as_vector(), n)
    ref = O.populations_from_vector(O.mps_as_vector(orc.A), n)
    assert np.abs(got - ref).max() < 1e-5


@pytest.mark.parametrize("n,d,lo,hi", SMALL + [(5, 2, 2, 4)])
def test_exact_small_state_vectors_match_oracle(n, d, lo, hi):
    from qca_gb300 import GpuExact, MPO, MPS, Rules
    p = np.sin(O.random_thetas(n, 60 + n)) ** 2
    H = MPO.hamiltonian_from_rules(Rules(n, range(lo, hi), d))
    alg = GpuExact(MPS.from_density_distribution(p), H, types.SimpleNamespace(step_size=0.1, algorithm="exact"))
    psi = O.product_state_vector(p)
    for _ in range(4):
        alg.do_time_step()
        psi = O.exact_evolve(psi, n, d, range(lo, hi), 0.1, 1)
        r = (np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(n + 1))
        alg.measure(*r)
        assert np.abs(r[0] - O.populations_from_vector(psi, n)).max() < 1e-10
