"""Host-side tensor-network containers mirroring the reference's input producers.

* ``Rules`` mirrors ``parameters/rules.py:1-6``.
* ``MPO.hamiltonian_from_rules`` mirrors ``tensor_networks/mpo.py:158-200``: the
  rule Hamiltonian H = sum_i X_i Pi_i written as an MPO by a state automaton
  over (projectors onto |0>, projectors onto |1>, flip placed).  The states are
  numbered in depth-first insertion order, the order the reference uses, so
  the W tensors agree entry by entry with the reference's.
* ``MPS`` mirrors the constructors and vector conversions of
  ``tensor_networks/mps.py`` used by the drivers (``from_density_distribution``,
  ``from_vector``, ``as_vector``, npz I/O).

These run once per rule / initial state on the host; the device consumes the
``W`` and ``A`` lists they produce.  Both classes accept the reference's own
objects too (anything with ``.W`` / ``.A`` lists).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


@dataclass
class Rules:
    """``parameters/rules.py``; ``activation_interval`` is a ``range`` (upper bound
    excluded)."""
    ncells: int
    activation_interval: range
    distance: int
    periodic: bool = False


_PROJ0 = np.array([[1.0, 0.0], [0.0, 0.0]])
_PROJ1 = np.array([[0.0, 0.0], [0.0, 1.0]])
_FLIP = np.array([[0.0, 1.0], [1.0, 0.0]])
_EYE = np.eye(2)


class _Automaton:
    """Finite automaton whose accepted operator strings are the rule's flip terms
    (``mpo.py:54-149``).  Reading a site appends an operator: identity before the
    pattern starts, ``distance`` projectors, the flip, ``distance`` projectors,
    identity after the pattern ends.  A projector onto |1> is allowed while the
    count of |1> projectors stays below the interval's upper bound; a projector
    onto |0> only while enough positions remain to reach the lower bound."""

    def __init__(self, distance: int, interval: range) -> None:
        self.distance = distance
        self.interval = interval
        self.span = 2 * distance  # projectors per accepted string
        self.ids: dict[tuple[int, int, bool], int] = {}
        self.edges: list[list[tuple[np.ndarray, int]]] = []
        self._insert((0, 0, False))
        self.edges.append([(_EYE, -1)])  # accepting state, loops on itself

    def _insert(self, key: tuple[int, int, bool]) -> int:
        found = self.ids.get(key)
        if found is not None:
            return found
        zeros, ones, flipped = key
        if zeros + ones + flipped == self.span + 1:
            return -1  # complete pattern: the accepting state (numbered last)
        me = len(self.edges)
        self.ids[key] = me
        self.edges.append([])
        if zeros + ones == self.distance and not flipped:
            self.edges[me].append((_FLIP, self._insert((zeros, ones, True))))
            return me
        if zeros == ones == 0 and not flipped:
            self.edges[me].append((_EYE, 0))
        if ones + 1 < self.interval.stop:
            self.edges[me].append((_PROJ1, self._insert((zeros, ones + 1, flipped))))
        if ones + self.span - (zeros + ones) - 1 >= self.interval.start:
            self.edges[me].append((_PROJ0, self._insert((zeros + 1, ones, flipped))))
        return me

    def bulk_tensor(self) -> np.ndarray:
        w = len(self.edges)
        W = np.zeros((2, 2, w, w), dtype=np.complex128)
        for src, outs in enumerate(self.edges):
            for op, dst in outs:
                W[:, :, dst % w, src] += op
        return W


class MPO:
    """Matrix product operator: ``W[i]`` has shape (2, 2, w_i, w_{i+1})."""

    def __init__(self, Wlist: list[np.ndarray], rules: Rules | None = None) -> None:
        self.W = Wlist
        self.rules = rules

    @classmethod
    def hamiltonian_from_rules(cls, rules: Rules) -> "MPO":
        """``mpo.py:158-200``: one shared bulk tensor; the first and last site absorb
        ``distance`` dead (|0>) virtual cells each."""
        bulk = _Automaton(rules.distance, rules.activation_interval).bulk_tensor()
        w = bulk.shape[2]
        dead = bulk[0, 0].real  # <0|W|0>
        left = np.zeros((1, w))
        left[0, -1] = 1.0
        right = np.zeros((w, 1))
        right[0, 0] = 1.0
        for _ in range(rules.distance):
            left = left @ dead
            right = dead @ right
        Wlist = [bulk] * rules.ncells
        Wlist[0] = np.einsum("lw,abwr->ablr", left, bulk)
        Wlist[-1] = np.einsum("ablw,wr->ablr", bulk, right)
        return cls(Wlist, rules)

    def as_matrix(self) -> np.ndarray:
        """Dense 2^N x 2^N matrix (``mpo.py:219-228``), for small checks only."""
        H = self.W[0]
        for Wi in self.W[1:]:
            H = np.tensordot(H, Wi, (3, 2)).transpose(0, 3, 1, 4, 2, 5)
            s = H.shape
            H = H.reshape(s[0] * s[1], s[2] * s[3], s[4], s[5])
        return np.trace(H, axis1=2, axis2=3)


def rule_from_mpo(H) -> tuple[int, range]:
    """Recover (distance, activation interval) from an MPO built by
    ``hamiltonian_from_rules`` (either implementation): the bulk tensor is
    compared with the automaton tensor of every candidate rule."""
    rules = getattr(H, "rules", None)
    if rules is not None:
        return rules.distance, rules.activation_interval
    bulk = np.asarray(H.W[len(H.W) // 2])
    for distance in range(1, 9):
        for lo in range(0, 2 * distance + 1):
            for hi in range(lo + 1, 2 * distance + 2):
                cand = _Automaton(distance, range(lo, hi)).bulk_tensor()
                if cand.shape == bulk.shape and np.array_equal(cand, bulk):
                    return distance, range(lo, hi)
    raise ValueError("the MPO is not a rule Hamiltonian of MPO.hamiltonian_from_rules")


class MPS:
    """Matrix product state: ``A[i]`` has shape (2, D_i, D_{i+1}), complex128."""

    def __init__(self, Alist: list[np.ndarray]) -> None:
        self.A = Alist

    @classmethod
    def from_tensors(cls, Alist) -> "MPS":
        return cls([np.array(A, dtype=np.complex128) for A in Alist])

    @classmethod
    def from_density_distribution(cls, plist) -> "MPS":
        """``mps.py:34-52``: bond dimension 1, site i = sqrt(1-p_i)|0> + sqrt(p_i)|1>."""
        Alist = []
        for p in plist:
            a = np.zeros((2, 1, 1), dtype=np.complex128)
            a[0, 0, 0] = math.sqrt(1.0 - p)
            a[1, 0, 0] = math.sqrt(p)
            Alist.append(a)
        return cls(Alist)

    @classmethod
    def from_vector(cls, psi) -> "MPS":
        """``mps.py:54-73``: successive reduced QRs from the left."""
        Alist = []
        m = np.array(psi, dtype=np.complex128).reshape(2, -1)
        while m.shape[1] > 1:
            q, r = np.linalg.qr(m)
            Alist.append(q.reshape(-1, 2, r.shape[0]).transpose(1, 0, 2))
            m = r.reshape(r.shape[0] * 2, -1)
        Alist.append(m.reshape(-1, 2, 1).transpose(1, 0, 2))
        return cls(Alist)

    @classmethod
    def from_file(cls, path: str) -> "MPS":
        """``mps.py:75-80``."""
        with open(path, "rb") as f:
            d = np.load(f)
            return cls([d[f"arr_{i}"] for i in range(len(d.files))])

    def write_to_file(self, path: str) -> None:
        """``mps.py:142-144``."""
        with open(path, "wb") as f:
            np.savez(f, *self.A)

    def as_vector(self) -> np.ndarray:
        """``mps.py:194-208``."""
        psi = self.A[0]
        for Ai in self.A[1:]:
            psi = np.tensordot(psi, Ai, (2, 1)).transpose(0, 2, 1, 3)
            s = psi.shape
            psi = psi.reshape(s[0] * s[1], s[2], s[3])
        return np.trace(psi, axis1=1, axis2=2)

    def bond_dims(self) -> list[int]:
        return [a.shape[1] for a in self.A] + [self.A[-1].shape[2]]


def pack_tensors(tensors) -> np.ndarray:
    """Concatenate C-ordered complex128 tensors into one float64 array (re, im)."""
    flat = [np.ascontiguousarray(t, dtype=np.complex128).reshape(-1) for t in tensors]
    return np.ascontiguousarray(np.concatenate(flat)).view(np.float64)


def entropy_from_rho(rho: np.ndarray) -> float:
    """-tr(rho log2 rho) of a 2x2 density matrix with 0 log 0 = 0 (``mps.py:135-140``
    evaluates the same quantity through scipy's logm)."""
    lam = np.linalg.eigvalsh(rho)
    lam = lam[lam > 0]
    return float(-(lam * np.log2(lam)).sum())
