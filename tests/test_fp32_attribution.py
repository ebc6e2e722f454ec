"""Where the mixed path's drift comes from, measured on the CPU with an FP32
emulation around the oracle (``tests/fp32_emulation.py``).

With exact splits, complex64 storage of tensors, environments and Krylov vectors
and complex64 products keep 2TDVP within 1e-6 of FP64 over ten steps (3.1e-7).
An error of 2.7e-6 in the Gram matrix of each split's isometric factor -- the
isometry a one-sided Jacobi in FP32 leaves at its rotation tolerance of 16 eps32
(measured on the device) -- with the other factor formed from that factor as on
the device, takes it to 1.3e-5, the level the device's mixed path shows.  One
Newton-Schulz polar step per split in complex64 brings it back to 9.3e-7.  So the
split's isometry, not the FP32 accumulation of the contractions, sets the mixed
path's drift, and a polar correction removes it."""
import numpy as np

from oracle import qca_oracle as O
from tests.fp32_emulation import FP32KrylovOracle


def _drift(isometry_error: float, polar: bool = False) -> float:
    n, chi = 14, 16
    rng = np.random.default_rng(3)
    p = np.sin(rng.uniform(0.0, np.pi / 2, n)) ** 2
    W = O.build_mpo(O.Rules(n, range(2, 4), 2))
    ref = O.TDVPKrylovOracle(O.mps_from_density_distribution(p), W, "2tdvp", 0.05, chi, 1e-10)
    emu = FP32KrylovOracle(O.mps_from_density_distribution(p), W, "2tdvp", 0.05, chi, 1e-10,
                           isometry_error=isometry_error, seed=1, polar=polar)
    dn = 0.0
    for _ in range(10):
        ref.step()
        emu.step()
        dn = max(dn, float(np.abs(ref.measure()[0] - emu.measure()[0]).max()))
    return dn


def test_fp32_storage_and_products_drift_below_1e6():
    assert _drift(0.0) < 1e-6


def test_split_isometry_error_dominates_and_a_polar_step_removes_it():
    base = _drift(0.0)
    broken = _drift(2.7e-6)
    fixed = _drift(2.7e-6, polar=True)
    assert broken > 10 * base
    assert fixed < broken / 5 and fixed < 2e-6
