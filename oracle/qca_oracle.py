"""CPU oracle for the quantum-game-of-life time-evolution path (TEST INFRASTRUCTURE).

This module is the checker, never the product: only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` may import it.  The CUDA library must never route through
it.

It restates, in plain NumPy/SciPy (complex128 throughout), the reference
algorithms of BenjaminDecker/quantum-cellular-automaton:

* the rule Hamiltonian H = sum_i X_i Pi_i, both matrix-free
  (``rule_flip_mask`` / ``apply_rule_hamiltonian``) and as the MPO produced by
  the state automaton of ``tensor_networks/mpo.py:54-200`` (``build_mpo``);
* the exact evolution of ``algorithms/exact.py:9-28`` with the propagator
  exp(-i pi/2 dt H) of ``lautils/lautils.py:44-54``;
* the MPS helpers of ``tensor_networks/mps.py`` (QR gauge moves, pad/truncate,
  vector conversion, measurement);
* 1-site and 2-site TDVP of ``algorithms/tdvp.py:10-365`` in the
  gauge-consistent ("fixed") form: after the canonicalisation at the start of
  each step (``tdvp.py:54``) the right environments are rebuilt.  The
  unmodified form (``fixed=False``) is kept for reporting the deviation.

Parity pinning: the golden fixtures in ``tests/golden`` were produced by the
reference itself (``tests/golden/make_golden.py`` imports it); the CPU tests
check this restatement against them.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import scipy.linalg
import scipy.sparse
import scipy.sparse.linalg

# --------------------------------------------------------------------------------------
# Rules and the matrix-free Hamiltonian
# --------------------------------------------------------------------------------------


@dataclass
class Rules:
    """Mirror of ``parameters/rules.py:1-6``; ``activation_interval`` is a Python range
    (upper bound excluded, ``parameters/parser.py:182``)."""
    ncells: int
    activation_interval: range
    distance: int
    periodic: bool = False


def rule_flip_mask(n: int, distance: int, interval: range) -> np.ndarray:
    """c[i, x] = 1 iff cell i of basis state x may flip.

    Cell i flips iff the number of alive cells j != i with |i-j| <= distance inside
    the chain lies in ``interval``; cells outside the chain are dead
    (``tensor_networks/mpo.py:179-198`` contracts dead virtual cells at both ends).
    Cell 0 is the most significant bit of x (``mps.py:194-208``).
    Returns a bool array of shape (n, 2**n).
    """
    x = np.arange(1 << n, dtype=np.int64)
    bits = [((x >> (n - 1 - j)) & 1) for j in range(n)]
    mask = np.zeros((n, 1 << n), dtype=bool)
    for i in range(n):
        count = np.zeros(1 << n, dtype=np.int64)
        for j in range(max(0, i - distance), min(n, i + distance + 1)):
            if j != i:
                count += bits[j]
        mask[i] = (count >= interval.start) & (count < interval.stop)
    return mask


def apply_rule_hamiltonian(psi: np.ndarray, n: int, distance: int, interval: range,
                           mask: np.ndarray | None = None) -> np.ndarray:
    """(H psi)[x] = sum_i c_i(x) psi[x xor bit_i]; H is real symmetric because c_i does
    not depend on bit i itself."""
    if mask is None:
        mask = rule_flip_mask(n, distance, interval)
    x = np.arange(1 << n, dtype=np.int64)
    out = np.zeros_like(psi)
    for i in range(n):
        partner = x ^ (1 << (n - 1 - i))
        out += np.where(mask[i], psi[partner], 0)
    return out


def sparse_rule_hamiltonian(n: int, distance: int, interval: range) -> scipy.sparse.csr_matrix:
    mask = rule_flip_mask(n, distance, interval)
    x = np.arange(1 << n, dtype=np.int64)
    rows, cols = [], []
    for i in range(n):
        sel = mask[i]
        rows.append(x[sel])
        cols.append((x ^ (1 << (n - 1 - i)))[sel])
    rows = np.concatenate(rows)
    cols = np.concatenate(cols)
    data = np.ones(rows.shape[0], dtype=np.float64)
    return scipy.sparse.csr_matrix((data, (rows, cols)), shape=(1 << n, 1 << n))


def exact_propagator(h_dense: np.ndarray, step_size: float) -> np.ndarray:
    """U = exp(-i pi/2 step H) by a full eigendecomposition (``lautils.py:44-54``)."""
    w, v = np.linalg.eigh(h_dense)
    return (np.exp(-1j * (np.pi / 2) * step_size * w) * v) @ v.conj().T


def exact_evolve(psi: np.ndarray, n: int, distance: int, interval: range, step_size: float,
                 steps: int) -> np.ndarray:
    """psi <- exp(-i pi/2 dt H)^steps psi with ``expm_multiply`` on the sparse rule H
    (restatement of ``exact.py:27-28``; agrees with the dense reference to ~1e-15)."""
    h = sparse_rule_hamiltonian(n, distance, interval).astype(np.complex128)
    a = (-1j * (np.pi / 2) * step_size) * h
    out = np.asarray(psi, dtype=np.complex128)
    for _ in range(steps):
        out = scipy.sparse.linalg.expm_multiply(a, out)
    return out


def populations_from_vector(psi: np.ndarray, n: int) -> np.ndarray:
    """<n_i> = sum_x |psi[x]|^2 bit_i(x) (cell 0 = most significant bit)."""
    prob = np.abs(psi) ** 2
    x = np.arange(1 << n, dtype=np.int64)
    return np.array([prob[((x >> (n - 1 - i)) & 1) == 1].sum() for i in range(n)])


def product_state_vector(p: np.ndarray) -> np.ndarray:
    """Tensor product of sqrt(1-p_i)|0> + sqrt(p_i)|1> with cell 0 as the most
    significant factor (``mps.py:34-52`` followed by ``mps.py:194-208``)."""
    v = np.ones(1, dtype=np.complex128)
    for pi in p:
        v = np.kron(v, np.array([math.sqrt(1.0 - pi), math.sqrt(pi)], dtype=np.complex128))
    return v


# --------------------------------------------------------------------------------------
# MPO from the rule automaton
# --------------------------------------------------------------------------------------

_P0 = np.array([[1.0, 0.0], [0.0, 0.0]])
_P1 = np.array([[0.0, 0.0], [0.0, 1.0]])
_SX = np.array([[0.0, 1.0], [1.0, 0.0]])
_ID = np.eye(2)


def _automaton_states(distance: int, interval: range):
    """Depth-first enumeration of the automaton states of ``mpo.py:90-149``.

    A state is (n0, n1, s): projectors onto |0>, |1> seen so far and whether the
    flip operator has been placed.  States are numbered in the order of first
    insertion; edges are (operator, target) and the final state is appended last
    with index -1 resolving to it.  The numbering must follow the reference's
    insertion order so that the W tensors agree entry by entry.
    """
    max_ops = 2 * distance
    index: dict[tuple[int, int, bool], int] = {}
    edges: list[list[tuple[np.ndarray, int]]] = []

    def visit(state: tuple[int, int, bool]) -> int:
        if state in index:
            return index[state]
        n0, n1, s = state
        if n0 + n1 + int(s) == max_ops + 1:
            return -1
        me = len(edges)
        index[state] = me
        edges.append([])
        if n0 + n1 == distance and not s:
            edges[me].append((_SX, visit((n0, n1, True))))
            return me
        if n0 + n1 + int(s) == 0:
            edges[me].append((_ID, 0))
        if n1 + 1 < interval.stop:
            edges[me].append((_P1, visit((n0, n1 + 1, s))))
        if n1 + (max_ops - (n0 + n1) - 1) >= interval.start:
            edges[me].append((_P0, visit((n0 + 1, n1, s))))
        return me

    visit((0, 0, False))
    edges.append([(_ID, -1)])  # final state loops on itself
    return edges


def build_mpo(rules: Rules) -> list[np.ndarray]:
    """W tensors (2, 2, w_left, w_right) of ``MPO.hamiltonian_from_rules``
    (``mpo.py:158-200``), open boundaries with ``distance`` dead cells contracted on
    both sides."""
    edges = _automaton_states(rules.distance, rules.activation_interval)
    w = len(edges)
    bulk = np.zeros((2, 2, w, w), dtype=np.complex128)
    for src, out in enumerate(edges):
        for op, dst in out:
            bulk[:, :, dst if dst >= 0 else w - 1, src] += op
    wl = [bulk] * rules.ncells
    dead = bulk[0, 0]  # <0|W|0>
    left = np.zeros((1, w))
    left[0, w - 1] = 1.0
    right = np.zeros((w, 1))
    right[0, 0] = 1.0
    for _ in range(rules.distance):
        left = left @ dead
        right = dead @ right
    wl = list(wl)
    wl[0] = np.einsum('lw,stwr->stlr', left, bulk)
    wl[-1] = np.einsum('stlw,wr->stlr', bulk, right)
    return wl


def mpo_as_matrix(W: list[np.ndarray]) -> np.ndarray:
    """Dense 2^N x 2^N matrix of an MPO (``mpo.py:202-228``)."""
    H = W[0]
    for Wi in W[1:]:
        H = np.tensordot(H, Wi, (3, 2)).transpose(0, 3, 1, 4, 2, 5)
        s = H.shape
        H = H.reshape(s[0] * s[1], s[2] * s[3], s[4], s[5])
    return np.trace(H, axis1=2, axis2=3)


# --------------------------------------------------------------------------------------
# MPS helpers (mps.py)
# --------------------------------------------------------------------------------------


def mps_from_density_distribution(p) -> list[np.ndarray]:
    """``mps.py:34-52``."""
    out = []
    for pi in p:
        a = np.zeros((2, 1, 1), dtype=np.complex128)
        a[0, 0, 0] = math.sqrt(1.0 - pi)
        a[1, 0, 0] = math.sqrt(pi)
        out.append(a)
    return out


def mps_from_vector(psi: np.ndarray) -> list[np.ndarray]:
    """``mps.py:54-73``: successive reduced QRs from the left."""
    A = []
    m = np.array(psi, dtype=np.complex128).reshape(2, -1)
    while m.shape[1] > 1:
        q, r = np.linalg.qr(m)
        A.append(q.reshape(-1, 2, r.shape[0]).transpose(1, 0, 2))
        m = r.reshape(r.shape[0] * 2, -1)
    A.append(m.reshape(-1, 2, 1).transpose(1, 0, 2))
    return A


def mps_as_vector(A: list[np.ndarray]) -> np.ndarray:
    """``mps.py:194-208``."""
    psi = A[0]
    for Ai in A[1:]:
        psi = np.tensordot(psi, Ai, (2, 1)).transpose(0, 2, 1, 3)
        s = psi.shape
        psi = psi.reshape(s[0] * s[1], s[2], s[3])
    return np.trace(psi, axis1=1, axis2=2)


def truncate_and_pad(t: np.ndarray, shape) -> np.ndarray:
    """``mps.py:226-236``."""
    idx = tuple(slice(0, min(a, b)) for a, b in zip(shape, t.shape))
    out = np.zeros(shape, dtype=t.dtype)
    out[idx] = t[idx]
    return out


def left_qr(A: np.ndarray, reduced: bool = True):
    """``mps.py:83-88``."""
    s = A.shape
    q, r = np.linalg.qr(A.reshape(s[0] * s[1], s[2]), mode='reduced' if reduced else 'complete')
    return q.reshape(s[0], s[1], -1), r


def right_qr(A: np.ndarray, reduced: bool = True):
    """``mps.py:90-98``."""
    q, r = left_qr(A.transpose(0, 2, 1), reduced)
    return q.transpose(0, 2, 1), r.T


def orthonormalize_left(A: list[np.ndarray], i: int) -> None:
    """``mps.py:146-164``."""
    shape = A[i].shape
    q, r = left_qr(A[i])
    q = truncate_and_pad(q, shape)
    r = truncate_and_pad(r, (shape[2], A[i + 1].shape[1]))
    A[i + 1] = np.tensordot(r, A[i + 1], (1, 1)).transpose(1, 0, 2)
    A[i] = q


def orthonormalize_right(A: list[np.ndarray], i: int) -> None:
    """``mps.py:166-181``."""
    shape = A[i].shape
    q, r = right_qr(A[i])
    q = truncate_and_pad(q, shape)
    r = truncate_and_pad(r, (A[i - 1].shape[2], shape[1]))
    A[i - 1] = np.tensordot(A[i - 1], r, (2, 0))
    A[i] = q


def make_site_canonical(A: list[np.ndarray], i: int) -> None:
    """``mps.py:184-192``."""
    for j in range(i):
        orthonormalize_left(A, j)
    for j in reversed(range(i + 1, len(A))):
        orthonormalize_right(A, j)


def measure(A: list[np.ndarray]):
    """``mps.py:100-140``; mutates the gauge of ``A`` exactly like the reference.

    Returns (population, rounded population, single-site entropy, bond dims).
    The entropy is -sum(lambda log2 lambda) over the eigenvalues of the 2x2 reduced
    density matrix with 0 log 0 = 0 (the reference evaluates -tr(rho logm(rho))/ln 2).
    """
    n = len(A)
    bond = np.array([A[i].shape[1] for i in range(n)] + [A[-1].shape[2]], dtype=np.int64)
    make_site_canonical(A, 0)
    pop = np.zeros(n)
    sse = np.zeros(n)
    for site in range(n):
        if site > 0:
            orthonormalize_left(A, site - 1)
        a = A[site]
        rho = np.tensordot(a, a.conj(), ((1, 2), (1, 2)))
        pop[site] = rho[1, 1].real
        lam = np.linalg.eigvalsh(rho)
        lam = lam[lam > 0]
        sse[site] = float(-(lam * np.log2(lam)).sum())
    return pop, np.round(pop), sse, bond


# --------------------------------------------------------------------------------------
# TDVP (tdvp.py)
# --------------------------------------------------------------------------------------


def _local_step(h: np.ndarray, v: np.ndarray, step: float) -> np.ndarray:
    """``lautils.timestep`` (``lautils.py:57-81``): v <- U^T v, U = exp(-i pi/2 step h)."""
    return np.tensordot(v, exact_propagator(h, step), (0, 0))


def _heff_site(L: np.ndarray, R: np.ndarray, W: np.ndarray) -> np.ndarray:
    """Dense effective Hamiltonian matrix of ``tdvp.py:298-310`` reshaped like
    ``tdvp.py:356-359``."""
    H = np.tensordot(W, L, (2, 1))
    H = np.tensordot(H, R, (2, 1)).transpose(0, 2, 4, 1, 3, 5)
    s = H.shape
    return H.reshape(s[0] * s[1] * s[2], s[3] * s[4] * s[5])


def _keff_bond(L: np.ndarray, R: np.ndarray) -> np.ndarray:
    """``tdvp.py:312-326`` reshaped like ``tdvp.py:179-182``."""
    K = np.tensordot(L, R, (1, 1)).transpose(0, 2, 1, 3)
    s = K.shape
    return K.reshape(s[0] * s[1], s[2] * s[3])


def _new_env(side: str, prev: np.ndarray, A: np.ndarray, W: np.ndarray) -> np.ndarray:
    """``tdvp.py:328-347``; env index order (ket, w, bra)."""
    if side == "left":
        t = np.tensordot(A.conj(), prev, (1, 2))
        t = np.tensordot(W, t, ((1, 2), (0, 3)))
        return np.tensordot(A, t, ((0, 1), (0, 3)))
    t = np.tensordot(A.conj(), prev, (2, 2))
    t = np.tensordot(W, t, ((1, 3), (0, 3)))
    return np.tensordot(A, t, ((0, 2), (0, 3)))


def _merge_w(Wl: np.ndarray, Wr: np.ndarray) -> np.ndarray:
    """``tdvp.py:281-284``."""
    W = np.tensordot(Wl, Wr, (3, 2)).transpose(0, 3, 1, 4, 2, 5)
    return W.reshape(Wl.shape[0] * Wr.shape[0], Wl.shape[1] * Wr.shape[1], Wl.shape[2], Wr.shape[3])


class TDVPOracle:
    """Restatement of ``algorithms/tdvp.py:10-365`` (``1tdvp`` / ``2tdvp``).

    ``fixed=True`` rebuilds the right environments after the canonicalisation at the
    start of each step (the gauge-consistent form the GPU path matches); ``fixed=False``
    reproduces the reference literally.
    """

    def __init__(self, A: list[np.ndarray], W: list[np.ndarray], algorithm: str, step_size: float,
                 max_bond_dim: int, svd_epsilon: float, fixed: bool = True) -> None:
        assert algorithm in ("1tdvp", "2tdvp", "a1tdvp")
        self.A = [np.array(a, dtype=np.complex128) for a in A]
        self.W = W
        self.algorithm = algorithm
        self.dt = step_size
        self.chi = max_bond_dim
        self.eps = svd_epsilon
        self.fixed = fixed
        n = len(self.A)
        make_site_canonical(self.A, n - 1)
        make_site_canonical(self.A, 0)
        self.L: list = [None] * n
        self.R: list = [None] * n
        self.max_bonds = [min(2 ** i, 2 ** (n - i), max_bond_dim) for i in range(n + 1)]
        self.target = list(self.max_bonds)
        for site in reversed(range(1, n)):
            make_site_canonical(self.A, site - 1)
            self._update_env("right", site)
        self._upcoming = self._pair_size(0) if algorithm == "2tdvp" else self._site_size(0)

    # environments -----------------------------------------------------------------
    def _env(self, side: str, site: int) -> np.ndarray:
        n = len(self.A)
        if (side == "left" and site < 0) or (side == "right" and site >= n):
            return np.ones((1, 1, 1))
        return self.L[site] if side == "left" else self.R[site]

    def _update_env(self, side: str, site: int) -> None:
        prev = site - 1 if side == "left" else site + 1
        e = _new_env(side, self._env(side, prev), self.A[site], self.W[site])
        if side == "left":
            self.L[site] = e
        else:
            self.R[site] = e

    def _refresh_right(self) -> None:
        for site in reversed(range(1, len(self.A))):
            self._update_env("right", site)

    # local evolutions -------------------------------------------------------------
    def _local_exp(self, L: np.ndarray, R: np.ndarray, W, v: np.ndarray, step: float) -> np.ndarray:
        """exp(-i pi/2 step H_eff) applied like ``lautils.timestep``: the dense
        effective Hamiltonian of ``tdvp.py:298-326`` (``W is None``: the bond
        matrix K_eff) and its full eigendecomposition, the reference's own method."""
        h = _keff_bond(L, R) if W is None else _heff_site(L, R, W)
        return _local_step(h, v.reshape(-1), step).reshape(v.shape)

    def _evolve_site(self, site: int, step: float) -> np.ndarray:
        return self._local_exp(self._env("left", site - 1), self._env("right", site + 1), self.W[site],
                               self.A[site], step)

    def _evolve_bond(self, bond: int, C: np.ndarray) -> np.ndarray:
        return self._local_exp(self._env("left", bond - 1), self._env("right", bond), None, C, -self.dt / 2)

    def _split(self, Al, Ar, L, R, Wl, Wr):
        """``tdvp.py:270-296``."""
        sl, sr = Al.shape, Ar.shape
        th = np.tensordot(Al, Ar, (2, 1)).transpose(0, 2, 1, 3).reshape(sl[0] * sr[0], sl[1], sr[2])
        th = self._local_exp(L, R, _merge_w(Wl, Wr), th, self.dt / 2)
        th = th.reshape(sl[0], sr[0], sl[1], sr[2]).transpose(0, 2, 1, 3).reshape(sl[0] * sl[1], sr[0] * sr[2])
        u, s, vh = np.linalg.svd(th, full_matrices=False)
        k = truncation_rank(s, self.chi, self.eps)
        Al_new = u.reshape(sl[0], sl[1], -1)[:, :, :k]
        Ar_new = vh.reshape(-1, sr[0], sr[2]).transpose(1, 0, 2)[:, :k, :]
        sk = s[:k] / np.linalg.norm(s[:k])
        return Al_new, sk, Ar_new

    # sweeps ------------------------------------------------------------------------
    def step(self) -> None:
        """``tdvp.py:50-63``."""
        for _ in self.step_updates():
            pass

    def upcoming_size(self) -> int:
        """Dimension of the next local problem of ``step_updates`` (the dense
        effective Hamiltonian is this size squared and its eigh costs the cube):
        4 D_l D_r for a 2TDVP bond update, 2 D_l D_r for a 1TDVP site update.
        Lets a timing harness skip an update it could not finish in its budget."""
        return self._upcoming

    def _pair_size(self, l: int) -> int:
        return 4 * self.A[l].shape[1] * self.A[l + 1].shape[2]

    def _site_size(self, s: int) -> int:
        return 2 * self.target[s] * self.target[s + 1]

    def step_updates(self):
        """One time step as a generator that yields after every local update
        (bond update for 2TDVP, site update for 1TDVP), for bounded timing;
        ``upcoming_size`` gives the size of the update the next ``next`` runs."""
        make_site_canonical(self.A, 0)
        if self.fixed:
            self._refresh_right()
        if self.algorithm == "2tdvp":
            yield from self._sweep_right_2()
            yield from self._sweep_left_2()
        else:
            if self.algorithm == "a1tdvp":
                self._new_target_bond_dims()
            yield from self._sweep_right_1()
            yield from self._sweep_left_1()

    def _new_target_bond_dims(self) -> None:
        """``tdvp.py:212-267`` (``a1tdvp``): the target bond dimensions of the next
        1TDVP step.  Left-canonical sweep with left environments; then, bond by bond
        from the right, the two-site tensor evolved by dt/2 (the reference's
        ``exact_exponential`` method, i.e. the local exponential of every other
        update) is split and the bond's target set to min{i : ||s[i:]|| < eps}
        (else the maximal bond dimension), clamped to [1, maximal]; the evolved
        tensor itself is discarded.  ``fixed`` rebuilds each right environment after
        the right gauge move, so that the next bond's effective Hamiltonian matches
        the tensors; the reference keeps the environments of the previous sweep."""
        n = len(self.A)
        for site in range(n - 1):
            make_site_canonical(self.A, site + 1)
            self._update_env("left", site)
        for bond in reversed(range(1, n)):
            Al, Ar = self.A[bond - 1], self.A[bond]
            sl, sr = Al.shape, Ar.shape
            th = np.tensordot(Al, Ar, (2, 1)).transpose(0, 2, 1, 3).reshape(sl[0] * sr[0], sl[1], sr[2])
            th = self._local_exp(self._env("left", bond - 2), self._env("right", bond + 1),
                                 _merge_w(self.W[bond - 1], self.W[bond]), th, self.dt / 2)
            th = th.reshape(sl[0], sr[0], sl[1], sr[2]).transpose(0, 2, 1, 3).reshape(sl[0] * sl[1], sr[0] * sr[2])
            s = np.linalg.svd(th, compute_uv=False)
            cap = min(self.max_bonds[bond], len(s))
            new = next((i for i in range(len(s)) if np.linalg.norm(s[i:]) < self.eps), cap)
            self.target[bond] = max(1, min(new, cap))
            make_site_canonical(self.A, bond - 1)
            if self.fixed:
                self._update_env("right", bond)

    def _sweep_right_2(self):
        n = len(self.A)
        for site in range(n - 1):
            Al, s, Ar = self._split(self.A[site], self.A[site + 1], self._env("left", site - 1),
                                    self._env("right", site + 2), self.W[site], self.W[site + 1])
            self.A[site] = Al
            self.A[site + 1] = np.tensordot(np.diag(s), Ar, (1, 1)).transpose(1, 0, 2)
            if site < n - 2:
                self._update_env("left", site)
                self.A[site + 1] = self._evolve_site(site + 1, -self.dt / 2)
            self._upcoming = self._pair_size(site + 1) if site < n - 2 else self._pair_size(n - 2)
            yield

    def _sweep_left_2(self):
        n = len(self.A)
        for site in reversed(range(1, n)):
            Al, s, Ar = self._split(self.A[site - 1], self.A[site], self._env("left", site - 2),
                                    self._env("right", site + 1), self.W[site - 1], self.W[site])
            self.A[site] = Ar
            self.A[site - 1] = np.tensordot(Al, np.diag(s), (2, 0))
            if site > 1:
                self._update_env("right", site)
                self.A[site - 1] = self._evolve_site(site - 1, -self.dt / 2)
            self._upcoming = self._pair_size(site - 2) if site > 1 else self._pair_size(0)
            yield

    def _sweep_right_1(self):
        """``tdvp.py:65-84``."""
        n = len(self.A)
        for site in range(n):
            tshape = (2, self.target[site], self.target[site + 1])
            new_a = self._evolve_site(site, self.dt / 2)
            if site == n - 1:
                self.A[site] = new_a
                self._upcoming = self._site_size(n - 1)
                yield
                continue
            q, c = left_qr(new_a, reduced=False)
            self.A[site] = truncate_and_pad(q, tshape)
            self._update_env("left", site)
            c = truncate_and_pad(c, (tshape[2], c.shape[1]))
            c = self._evolve_bond(site + 1, c)
            self.A[site + 1] = np.tensordot(c, self.A[site + 1], (1, 1)).transpose(1, 0, 2)
            self._upcoming = self._site_size(site + 1)
            yield

    def _sweep_left_1(self):
        """``tdvp.py:86-105``."""
        n = len(self.A)
        for site in reversed(range(n)):
            tshape = (2, self.target[site], self.target[site + 1])
            new_a = self._evolve_site(site, self.dt / 2)
            if site == 0:
                self.A[site] = new_a
                self._upcoming = self._site_size(0)
                yield
                continue
            q, c = right_qr(new_a, reduced=False)
            self.A[site] = truncate_and_pad(q, tshape)
            self._update_env("right", site)
            c = truncate_and_pad(c, (c.shape[0], tshape[1]))
            c = self._evolve_bond(site, c)
            self.A[site - 1] = np.tensordot(self.A[site - 1], c, (2, 0))
            self._upcoming = self._site_size(site - 1)
            yield

    def measure(self):
        return measure(self.A)


def heff_apply(L: np.ndarray, R: np.ndarray, W, x: np.ndarray) -> np.ndarray:
    """The operator the reference exponentiates, applied matrix free.

    ``lautils.timestep`` returns tensordot(v, U, (0, 0)) = U^T v with U built from
    the assembled matrix M[(s,a,c),(s',b,e)] = sum W[s,s',l,r] L[a,l,b] R[c,r,e]
    (``tdvp.py:298-310``; ``tdvp.py:312-326`` without W for the bond), so the
    operator is M^T:  y[s',b,e] = sum W[s,s',l,r] L[a,l,b] R[c,r,e] x[s,a,c].
    Environments are (ket, w, bra) as in ``tdvp.py:328-347``."""
    if W is None:
        t = np.tensordot(x, L, (0, 0))                  # [c, l, b]
        return np.tensordot(t, R, ((0, 1), (0, 1)))    # [b, e]
    t = np.tensordot(x, L, (1, 0))                      # [s, c, l, b]
    t = np.tensordot(W, t, ((0, 2), (0, 2)))            # [s', r, c, b]
    y = np.tensordot(t, R, ((1, 2), (1, 0)))            # [s', b, e]
    return y


def krylov_expm(apply, v: np.ndarray, tau: float, tol: float = 1e-14, mmax: int = 80) -> np.ndarray:
    """exp(-i tau H) v for a Hermitian H given as ``apply`` by Lanczos with full
    reorthogonalisation (complex128) and the small exponential from the
    eigendecomposition of the tridiagonal matrix; stops when the error estimate
    beta_m |(exp(-i tau T) e_1)_m| falls below tol.  Substitutes for the dense
    eigh of ``lautils.py:44-54`` where that is out of reach."""
    shape = v.shape
    v0 = v.reshape(-1).astype(np.complex128)
    nrm = np.linalg.norm(v0)
    if nrm == 0.0:
        return np.zeros(shape, dtype=np.complex128)
    V = [v0 / nrm]
    alpha: list[float] = []
    beta: list[float] = []
    c = np.ones(1, dtype=np.complex128)
    for j in range(min(mmax, v0.size)):
        w = apply(V[j].reshape(shape)).reshape(-1)
        alpha.append(float(np.real(np.vdot(V[j], w))))
        for _ in range(2):
            for u in V:
                w = w - np.vdot(u, w) * u
        b = float(np.linalg.norm(w))
        T = np.diag(alpha) + np.diag(beta, 1) + np.diag(beta, -1)
        ev, evec = np.linalg.eigh(T)
        c = evec @ (np.exp(-1j * tau * ev) * evec[0].conj())
        if b * abs(c[-1]) < tol or b < 1e-300 or j + 1 == v0.size:
            break
        beta.append(b)
        V.append(w / b)
    out = np.zeros_like(v0)
    for k in range(len(c)):
        out += c[k] * V[k]
    return (nrm * out).reshape(shape)


class TDVPKrylovOracle(TDVPOracle):
    """``TDVPOracle`` with the local exponentials computed matrix free by Lanczos
    (``heff_apply`` + ``krylov_expm``) instead of the dense effective Hamiltonian
    and its eigh: the same algorithm (sweeps, splits, truncation, QR moves) at
    bond dimensions where the reference's dense n x n problems (n = 4 D_l D_r) are
    out of reach.  Validated against ``TDVPOracle`` at small bonds."""

    def _local_exp(self, L, R, W, v, step):
        return krylov_expm(lambda x: heff_apply(L, R, W, x), v, (np.pi / 2) * step)


def truncation_rank(s: np.ndarray, max_bond_dim: int, epsilon: float) -> int:
    """``tdvp.py:290-292``: the first i with ||s[i:]||_2 < epsilon, capped at
    min(max_bond_dim, len(s)); when no i qualifies the cap is used."""
    cap = min(max_bond_dim, len(s))
    for i in range(len(s)):
        if np.linalg.norm(s[i:]) < epsilon:
            return min(i, cap)
    return cap


def random_thetas(n: int, seed: int) -> np.ndarray:
    """theta_i ~ U(0, pi/2) from ``numpy.random.default_rng(seed)``; p_i = sin^2 theta_i."""
    return np.random.default_rng(seed).uniform(0.0, np.pi / 2, size=n)
