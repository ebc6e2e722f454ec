"""GPU drop-ins for the reference's ``Algorithm`` interface.

``Algorithm`` mirrors ``algorithms/algorithm.py:10-63``; ``GpuExact`` replaces
``algorithms/exact.py:9-28`` and ``GpuTDVP`` replaces ``algorithms/tdvp.py``
for ``--algorithm 1tdvp`` / ``2tdvp``.  Both take the reference's constructor
arguments ``(psi_0, H, args)``: ``psi_0`` is any object with an ``A`` list of
(2, D_i, D_{i+1}) tensors, ``H`` any object with a ``W`` list of
(2, 2, w_i, w_{i+1}) tensors, ``args`` any namespace with the reference's flag
names (``algorithm``, ``step_size``, ``max_bond_dim``, ``svd_epsilon``).  Two
optional fields select the GPU variant: ``precision`` ("fp64" = plain
complex128, "mixed" = complex64 storage with FP64 Krylov scalars, singular
values and norms) and ``krylov_dim`` (exact path, default 30).

All compute runs in ``libqca_gb300.so``; the state lives on the device.
"""
from __future__ import annotations

import ctypes
from abc import ABC, abstractmethod

import numpy as np

from . import _lib
from .tensor_networks import MPS, entropy_from_rho, pack_tensors, rule_from_mpo


def _precision(args) -> int:
    p = getattr(args, "precision", "fp64")
    if p in ("fp64", "plain", _lib.QCA_PREC_FP64):
        return _lib.QCA_PREC_FP64
    if p in ("mixed", "fp32", _lib.QCA_PREC_MIXED):
        return _lib.QCA_PREC_MIXED
    raise ValueError(f"unknown precision {p!r}")


class Algorithm(ABC):
    """``algorithms/algorithm.py:10-63``."""

    @abstractmethod
    def __init__(self, psi_0, H, args) -> None:
        self._H = H
        self.args = args

    @abstractmethod
    def do_time_step(self) -> None:
        ...

    @property
    @abstractmethod
    def psi(self) -> MPS:
        ...

    @psi.setter
    @abstractmethod
    def psi(self, value) -> None:
        ...

    @abstractmethod
    def measure(self, population, d_population, single_site_entropy, bond_dims) -> None:
        """Write <n_i>, round(<n_i>), the single-site entropy and the bond dimensions
        into the caller's rows (``algorithm.py:58-63`` -> ``mps.py:100-140``)."""

    @classmethod
    def classical_evolution(cls, first_column: np.ndarray, rules, plot_steps: int) -> np.ndarray:
        """Classical automaton shown beside the quantum heatmaps (``algorithm.py:34-56``):
        a cell flips when its count of alive neighbours lies in the interval; the
        first and last cell stay fixed."""
        n = len(first_column)
        heat = np.zeros((plot_steps, n))
        heat[0] = first_column
        heat[:, 0] = first_column[0]
        heat[:, -1] = first_column[-1]
        for step in range(1, plot_steps):
            prev = heat[step - 1]
            for site in range(n):
                total = 0.0
                for off in range(-rules.distance, rules.distance + 1):
                    if off and 0 <= site + off < n:
                        total += prev[site + off]
                heat[step, site] = 1.0 - prev[site] if total in rules.activation_interval else prev[site]
        return heat


class GpuExact(Algorithm):
    """Exact state-vector evolution on the GPU (``algorithms/exact.py:9-28``).

    The reference builds the dense U = exp(-i pi/2 dt H) once and multiplies; here
    each ``do_time_step`` applies exp(-i pi/2 dt H) to the resident 2^N amplitudes
    by a matrix-free Lanczos step (``krylov_dim`` vectors).  As in the reference,
    ``args.step_size`` is the step the driver already scaled by the plot interval
    (``quantum_game.py:70-73``).
    """

    def __init__(self, psi_0, H, args, stream=None) -> None:
        super().__init__(psi_0, H, args)
        self._lib = _lib.load()
        self._stream = _lib.stream_handle(stream)
        self.n = len(psi_0.A)
        self.distance, self.interval = rule_from_mpo(H)
        self.precision = _precision(args)
        self.krylov_dim = int(getattr(args, "krylov_dim", 30))
        h = ctypes.c_void_p()
        _lib.call("qca_exact_create", self.n, self.distance, self.interval.start, self.interval.stop,
                  self.precision, self.krylov_dim, ctypes.byref(h))
        self._h = h
        self.psi = psi_0

    def __del__(self) -> None:
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.qca_exact_destroy(h)
            self._h = None

    # state ------------------------------------------------------------------------
    def state_vector(self) -> np.ndarray:
        out = np.empty(1 << self.n, dtype=np.complex128)
        _lib.call("qca_exact_get_state", self._h, out.view(np.float64).ctypes.data_as(_lib._PD), self._stream)
        return out

    def set_state_vector(self, psi: np.ndarray) -> None:
        v = np.ascontiguousarray(psi, dtype=np.complex128)
        if v.shape != (1 << self.n,):
            raise ValueError(f"state vector must have 2^{self.n} amplitudes")
        _lib.call("qca_exact_set_state", self._h, v.view(np.float64).ctypes.data_as(_lib._PD), self._stream)

    @property
    def psi(self) -> MPS:
        return MPS.from_vector(self.state_vector())

    @psi.setter
    def psi(self, value) -> None:
        self.set_state_vector(value.as_vector() if hasattr(value, "as_vector") else MPS(value.A).as_vector())

    # evolution --------------------------------------------------------------------
    def do_time_step(self) -> None:
        _lib.call("qca_exact_step", self._h, float(self.args.step_size), 1, self._stream)

    def evolve(self, nsteps: int, step_size: float | None = None) -> None:
        dt = float(self.args.step_size if step_size is None else step_size)
        _lib.call("qca_exact_step", self._h, dt, int(nsteps), self._stream)

    def measure(self, population, d_population, single_site_entropy, bond_dims) -> None:
        n = self.n
        pop = np.zeros(n)
        rho = np.zeros((n, 2, 2), dtype=np.complex128)
        _lib.call("qca_exact_measure", self._h, pop.ctypes.data_as(_lib._PD),
                  rho.view(np.float64).ctypes.data_as(_lib._PD), self._stream)
        population[:] = pop
        d_population[:] = np.round(pop)
        for i in range(n):
            single_site_entropy[i] = entropy_from_rho(rho[i])
        # MPS.from_vector gives reduced-QR bond dimensions (mps.py:54-73)
        bond_dims[:] = [min(2 ** i, 2 ** (n - i)) for i in range(n + 1)]


class _Engine:
    """Owner of a ``qca_engine`` handle (many chains on one device)."""

    def __init__(self, precision: int, hbm_budget: int = 0) -> None:
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        _lib.call("qca_engine_create", precision, ctypes.c_size_t(hbm_budget), ctypes.byref(h))
        self.h = h
        self.precision = precision

    def __del__(self) -> None:
        h = getattr(self, "h", None)
        if h is not None and h.value:
            self.lib.qca_engine_destroy(h)
            self.h = None


def chain_desc(A: list, W: list, algorithm: str, step_size: float, max_bond_dim: int,
               svd_epsilon: float):
    """Build a ``qca_chain_desc`` (and keep its host arrays alive)."""
    n = len(A)
    if len(W) != n:
        raise ValueError("MPO and MPS lengths differ")
    if algorithm not in ("1tdvp", "2tdvp", "a1tdvp"):
        raise ValueError(f"algorithm {algorithm!r} is not a TDVP variant handled here")
    mps_bonds = np.array([a.shape[1] for a in A] + [A[-1].shape[2]], dtype=np.int32)
    mpo_bonds = np.array([w.shape[2] for w in W] + [W[-1].shape[3]], dtype=np.int32)
    mps = pack_tensors(A)
    mpo = pack_tensors(W)
    d = _lib.ChainDesc()
    d.n_sites = n
    d.mpo_bonds = mpo_bonds.ctypes.data_as(_lib._PI)
    d.mpo = mpo.ctypes.data_as(_lib._PD)
    d.mps_bonds = mps_bonds.ctypes.data_as(_lib._PI)
    d.mps = mps.ctypes.data_as(_lib._PD)
    d.algorithm = {"1tdvp": _lib.QCA_ALGO_1TDVP, "2tdvp": _lib.QCA_ALGO_2TDVP,
                   "a1tdvp": _lib.QCA_ALGO_A1TDVP}[algorithm]
    d.max_bond_dim = int(max_bond_dim)
    d.svd_epsilon = float(svd_epsilon)
    d.step_size = float(step_size)
    return d, (mps_bonds, mpo_bonds, mps, mpo)


def unpack_mps(flat: np.ndarray, bonds) -> list[np.ndarray]:
    out = []
    off = 0
    for i in range(len(bonds) - 1):
        size = 2 * bonds[i] * bonds[i + 1]
        out.append(flat[off:off + size].reshape(2, bonds[i], bonds[i + 1]).copy())
        off += size
    return out


class GpuTDVP(Algorithm):
    """1-site / 2-site TDVP on the GPU (``algorithms/tdvp.py:10-365``).

    The 2-site variant is the gauge-consistent form of the reference (right
    environments consistent with the tensors at the start of every sweep).
    ``a1tdvp`` is 1TDVP whose target bond dimensions are recomputed before every
    step from evolved two-site splits (``tdvp.py:212-267``, with the exact local
    exponential of the reference's ``exact_exponential`` method).
    """

    def __init__(self, psi_0, H, args, stream=None, engine: _Engine | None = None) -> None:
        super().__init__(psi_0, H, args)
        self._stream = _lib.stream_handle(stream)
        self.precision = _precision(args)
        self._engine = engine if engine is not None else _Engine(self.precision)
        self._W = [np.asarray(w, dtype=np.complex128) for w in H.W]
        self._chain = None
        self.psi = psi_0

    def _add(self, A) -> None:
        d, keep = chain_desc(A, self._W, self.args.algorithm, self.args.step_size, self.args.max_bond_dim,
                             self.args.svd_epsilon)
        cid = ctypes.c_int(-1)
        _lib.call("qca_chain_add", self._engine.h, ctypes.byref(d), self._stream, ctypes.byref(cid))
        del keep
        self._chain = cid.value

    def __del__(self) -> None:
        eng = getattr(self, "_engine", None)
        if eng is not None and self._chain is not None and eng.h is not None and eng.h.value:
            eng.lib.qca_chain_remove(eng.h, self._chain)
            self._chain = None

    @property
    def n(self) -> int:
        return len(self._W)

    def bonds(self) -> list[int]:
        b = np.zeros(self.n + 1, dtype=np.int32)
        _lib.call("qca_chain_bonds", self._engine.h, self._chain, b.ctypes.data_as(_lib._PI))
        return [int(x) for x in b]

    @property
    def psi(self) -> MPS:
        bonds = self.bonds()
        size = sum(2 * bonds[i] * bonds[i + 1] for i in range(self.n))
        flat = np.zeros(size, dtype=np.complex128)
        _lib.call("qca_chain_get_mps", self._engine.h, self._chain, flat.view(np.float64).ctypes.data_as(_lib._PD),
                  ctypes.c_size_t(2 * size), self._stream)
        return MPS(unpack_mps(flat, bonds))

    @psi.setter
    def psi(self, value) -> None:
        if self._chain is not None:
            _lib.call("qca_chain_remove", self._engine.h, self._chain)
            self._chain = None
        self._add([np.asarray(a, dtype=np.complex128) for a in value.A])

    def do_time_step(self) -> None:
        cid = (ctypes.c_int * 1)(self._chain)
        _lib.call("qca_engine_step_chains", self._engine.h, cid, 1, 1, self._stream)

    def evolve(self, nsteps: int) -> None:
        cid = (ctypes.c_int * 1)(self._chain)
        _lib.call("qca_engine_step_chains", self._engine.h, cid, 1, int(nsteps), self._stream)

    def measure(self, population, d_population, single_site_entropy, bond_dims) -> None:
        n = self.n
        pop, dpop, sse, bd = np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(n + 1)
        _lib.call("qca_chain_measure", self._engine.h, self._chain, pop.ctypes.data_as(_lib._PD),
                  dpop.ctypes.data_as(_lib._PD), sse.ctypes.data_as(_lib._PD), bd.ctypes.data_as(_lib._PD),
                  self._stream)
        population[:] = pop
        d_population[:] = dpop
        single_site_entropy[:] = sse
        bond_dims[:] = bd

    def stats(self) -> dict:
        s = np.zeros(2)
        _lib.call("qca_chain_stats", self._engine.h, self._chain, s.ctypes.data_as(_lib._PD))
        return {"krylov_max": int(s[0]), "discarded_weight": float(s[1])}


def algorithm_class(name: str):
    """``quantum_game.py:62-68``: the class for an ``--algorithm`` string."""
    if name == "exact":
        return GpuExact
    if name in ("1tdvp", "2tdvp", "a1tdvp"):
        return GpuTDVP
    raise ValueError(f"algorithm {name!r} is not provided by the GPU path")
