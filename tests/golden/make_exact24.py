"""Generate ``exact24.npz``: the exact-evolution configuration at its full size
(N = 24 cells, 2^24 amplitudes, distance 2, interval [2,3], product state with
theta_i ~ U(0, pi/2) from numpy.random.default_rng(24), dt = 0.05) evolved for
three steps by the oracle's sparse restatement of algorithms/exact.py:27-28
(``expm_multiply`` on the matrix-free rule Hamiltonian, complex128; the same
restatement matches the reference's dense Exact to ~1e-15 at N <= 12, pinned by
``exact_series.npz``).  The state itself (268 MB) is not stored: the fixture keeps
the single-cell populations <n_i>, the 2x2 reduced density matrices and
<psi_0|psi_t> after every step, which the GPU path must reproduce.

Run from the repository root (needs ~20 GB of host memory, a few minutes):
    python tests/golden/make_exact24.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import qca_oracle as O  # noqa: E402

N, DIST, LO, HI, DT, STEPS, SEED = 24, 2, 2, 4, 0.05, 3, 24


def rho_single(psi: np.ndarray, n: int) -> np.ndarray:
    """rho_i[s, s'] = sum over the other cells of psi[.. s ..] conj(psi[.. s' ..])."""
    out = np.zeros((n, 2, 2), dtype=np.complex128)
    for i in range(n):
        t = psi.reshape(1 << i, 2, 1 << (n - 1 - i))
        out[i] = np.einsum("asb,atb->st", t, t.conj())
    return out


def main() -> None:
    theta = np.random.default_rng(SEED).uniform(0.0, np.pi / 2, size=N)
    p = np.sin(theta) ** 2
    psi0 = O.product_state_vector(p)
    psi = psi0
    pops, rhos, overlaps = [], [], []
    for _ in range(STEPS):
        psi = O.exact_evolve(psi, N, DIST, range(LO, HI), DT, 1)
        r = rho_single(psi, N)
        rhos.append(r)
        pops.append(r[:, 1, 1].real.copy())
        overlaps.append(np.vdot(psi0, psi))
    np.savez_compressed(os.path.join(HERE, "exact24.npz"), p=p, meta=np.array([N, DIST, LO, HI, DT, STEPS]),
                        pop=np.array(pops), rho=np.array(rhos), overlap=np.array(overlaps))
    print("wrote exact24.npz")


if __name__ == "__main__":
    main()
