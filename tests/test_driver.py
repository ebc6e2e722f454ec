"""The driver loop (quantum_game.py:28-119) on the host, with oracle-backed
stand-ins for the GPU algorithms: measurement cadence, the exact path's scaled
step, file names and CSV / npz backups, several initial states in one run."""
import os
import types

import numpy as np
import pytest

from oracle import qca_oracle as O
from qca_gb300 import driver
from qca_gb300.algorithms import Algorithm
from qca_gb300.tensor_networks import MPO, MPS, Rules, rule_from_mpo


class OracleExact(Algorithm):
    def __init__(self, psi_0, H, args):
        super().__init__(psi_0, H, args)
        self.n = len(psi_0.A)
        self.d, self.iv = rule_from_mpo(H)
        self.psi = psi_0

    @property
    def psi(self):
        return MPS.from_vector(self.v)

    @psi.setter
    def psi(self, value):
        self.v = MPS(value.A).as_vector()

    def do_time_step(self):
        self.v = O.exact_evolve(self.v, self.n, self.d, self.iv, self.args.step_size, 1)

    def measure(self, population, d_population, single_site_entropy, bond_dims):
        p = O.populations_from_vector(self.v, self.n)
        population[:] = p
        d_population[:] = np.round(p)
        single_site_entropy[:] = 0.0
        bond_dims[:] = [min(2 ** i, 2 ** (self.n - i)) for i in range(self.n + 1)]


class OracleTDVP(OracleExact):
    def __init__(self, psi_0, H, args):
        super().__init__(psi_0, H, args)
        self.orc = O.TDVPOracle([np.array(a) for a in psi_0.A], [np.array(w) for w in H.W], args.algorithm,
                                args.step_size, args.max_bond_dim, args.svd_epsilon, fixed=True)

    def do_time_step(self):
        self.orc.step()
        self.v = O.mps_as_vector(self.orc.A)

    def measure(self, population, d_population, single_site_entropy, bond_dims):
        # mps.py:100-140, re-gauging the stored MPS like the reference
        pop, dpop, sse, bonds = O.measure(self.orc.A)
        population[:] = pop
        d_population[:] = dpop
        single_site_entropy[:] = sse
        bond_dims[:] = bonds


def make_args(algorithm):
    return types.SimpleNamespace(rules=Rules(6, range(1, 2), 1), algorithm=algorithm, step_size=0.1, num_steps=6,
                                 plot_step_interval=2, max_bond_dim=8, svd_epsilon=1e-10)


def test_driver_exact_cadence_files_and_names(tmp_path):
    args = make_args("exact")
    H = MPO.hamiltonian_from_rules(args.rules)
    p1 = np.zeros(6)
    p1[3] = 1.0
    p2 = np.sin(O.random_thetas(6, 9)) ** 2
    states = [MPS.from_density_distribution(p1), MPS.from_density_distribution(p2)]
    res = driver.run(args, states, H, out_dir=str(tmp_path), state_names=["single"], algorithm_cls=OracleExact)
    assert [r["name"] for r in res] == ["single6_112_01_exact", "16_112_01_exact"]
    assert args.step_size == 0.1  # not scaled in place
    for p, r in zip((p1, p2), res):
        psi = O.product_state_vector(p)
        for k in range(3):  # rows at t = 0, 2 dt, 4 dt: one step of 2 dt per measurement
            assert np.abs(r["population"][k] - O.populations_from_vector(psi, 6)).max() < 1e-12
            psi = O.exact_evolve(psi, 6, 1, range(1, 2), 0.2, 1)
    for suffix in ("population", "d_population", "single_site_entropy", "bond_dims"):
        rows = np.loadtxt(tmp_path / f"single6_112_01_exact-{suffix}.csv", delimiter=",")
        assert rows.shape[0] == 3  # every measured row, the last one included
    back = MPS.from_file(str(tmp_path / "single6_112_01_exact.npz"))
    assert len(back.A) == 6


def test_driver_tdvp_steps_every_step():
    args = make_args("2tdvp")
    H = MPO.hamiltonian_from_rules(args.rules)
    p = np.sin(O.random_thetas(6, 4)) ** 2
    res = driver.run(args, [MPS.from_density_distribution(p)], H, out_dir=None, algorithm_cls=OracleTDVP)
    assert res[0]["name"] == "06_112_01_2tdvp_8"
    orc = O.TDVPOracle(O.mps_from_density_distribution(p), O.build_mpo(O.Rules(6, range(1, 2), 1)), "2tdvp", 0.1, 8,
                       1e-10, fixed=True)
    for k in range(3):  # rows after 0, 2, 4 steps of dt
        got = res[0]["population"][k]
        assert np.abs(got - O.populations_from_vector(O.mps_as_vector(orc.A), 6)).max() < 1e-12
        orc.step()
        orc.step()


@pytest.mark.gpu
@pytest.mark.parametrize("algorithm", ["exact", "2tdvp", "1tdvp"])
def test_driver_over_gpu_algorithms_matches_oracle_run(tmp_path, algorithm):
    """The driver loop over GpuExact / GpuTDVP (the classes quantum_game.py:62-68
    would select) writes the same files under the same names as the run over the
    oracle-backed stand-ins, with the same observables: populations within 1e-8,
    identical rounded populations and bond dimensions."""
    args = make_args(algorithm)
    args.precision = "fp64"
    H = MPO.hamiltonian_from_rules(args.rules)
    p = np.sin(O.random_thetas(6, 21)) ** 2
    stand_in = OracleExact if algorithm == "exact" else OracleTDVP
    gpu_dir, ref_dir = tmp_path / "gpu", tmp_path / "ref"
    got = driver.run(args, [MPS.from_density_distribution(p)], H, out_dir=str(gpu_dir), state_names=["rand"])
    want = driver.run(args, [MPS.from_density_distribution(p)], H, out_dir=str(ref_dir), state_names=["rand"],
                      algorithm_cls=stand_in)
    assert got[0]["name"] == want[0]["name"]
    assert sorted(os.listdir(gpu_dir)) == sorted(os.listdir(ref_dir))
    assert np.abs(got[0]["population"] - want[0]["population"]).max() < 1e-8
    assert np.array_equal(got[0]["d_population"], want[0]["d_population"])
    if algorithm != "exact":
        assert np.array_equal(got[0]["bond_dims"], want[0]["bond_dims"])
    rows = np.loadtxt(gpu_dir / f"{got[0]['name']}-population.csv", delimiter=",")
    assert np.abs(rows - want[0]["population"]).max() < 1e-8
    back = MPS.from_file(str(gpu_dir / f"{got[0]['name']}.npz"))
    assert len(back.A) == 6
