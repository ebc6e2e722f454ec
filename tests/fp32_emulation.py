"""FP32-rounding emulation of the mixed path's arithmetic around the oracle.

Test infrastructure, used to attribute the mixed path's drift against FP64: the
Krylov oracle (``oracle.qca_oracle.TDVPKrylovOracle``, the reference's 2TDVP with
Lanczos local exponentials) with

* site tensors, environments and Krylov vectors stored in complex64,
* effective-Hamiltonian products and environment updates computed in complex64
  (FP32 accumulation), Krylov projections in FP64, tolerance 1e-7 as on the device,
* optionally, a Hermitian error of a given size in the Gram matrix of every
  split's isometric factor: U -> U (I + E / 2), U^H U = I + E + O(E^2), which is
  what a one-sided Jacobi stopped at a rotation tolerance leaves behind,
* optionally, one Newton-Schulz polar step in complex64 that restores the
  isometry after the split (the correction proposed for the device).

The splits themselves are the oracle's FP64 SVDs; everything else follows
``algorithms/tdvp.py`` through the oracle.
"""
from __future__ import annotations

import numpy as np

from oracle import qca_oracle as O


def r32(x) -> np.ndarray:
    """Round to complex64 storage (kept in complex128 arrays)."""
    return np.asarray(x).astype(np.complex64).astype(np.complex128)


def krylov_expm_fp32(apply, v: np.ndarray, tau: float, tol: float = 1e-7, mmax: int = 40) -> np.ndarray:
    """exp(-i tau H) v with complex64 Krylov vectors and products, CGS twice with
    FP64 projections, stopping at the error estimate, at m = n, or at a beta_j at
    the FP32 rounding level of ||H v_j||."""
    shape = v.shape
    v0 = r32(v.reshape(-1))
    nrm = float(np.linalg.norm(v0))
    if nrm == 0.0:
        return np.zeros(shape, dtype=np.complex128)
    V = [r32(v0 / nrm)]
    alpha: list[float] = []
    beta: list[float] = []
    c = np.ones(1, dtype=np.complex128)
    for j in range(min(mmax, v0.size)):
        w = r32(apply(V[j].reshape(shape)).reshape(-1))
        a = 0.0
        for _ in range(2):
            h = np.array([np.vdot(u, w) for u in V])
            a += float(h[j].real)
            w = r32(w - sum(hk * u for hk, u in zip(h, V)))
        alpha.append(a)
        b = float(np.linalg.norm(w))
        T = np.diag(alpha) + np.diag(beta, 1) + np.diag(beta, -1)
        ev, evec = np.linalg.eigh(T)
        c = evec @ (np.exp(-1j * tau * ev) * evec[0].conj())
        scale = np.hypot(alpha[-1], beta[-1] if beta else 0.0)
        if b * abs(c[-1]) < tol or b <= 64 * 1.2e-7 * scale or len(alpha) >= v0.size:
            break
        beta.append(b)
        V.append(r32(w / b))
    out = sum(ck * vk for ck, vk in zip(c, V))
    return r32(nrm * out).reshape(shape)


class FP32KrylovOracle(O.TDVPKrylovOracle):
    """The Krylov oracle with the mixed path's FP32 storage and products, and an
    optional isometry error of size ``isometry_error`` in every split."""

    def __init__(self, *args, isometry_error: float = 0.0, seed: int = 0, polar: bool = False, **kw) -> None:
        self.isometry_error = isometry_error
        self.polar = polar
        self._rng = np.random.default_rng(seed)
        self._right = True
        super().__init__(*args, **kw)

    def _local_exp(self, L, R, W, v, step):
        L32 = np.asarray(L).astype(np.complex64)
        R32 = np.asarray(R).astype(np.complex64)
        W32 = None if W is None else np.asarray(W).astype(np.complex64)
        return krylov_expm_fp32(lambda x: O.heff_apply(L32, R32, W32, x.astype(np.complex64)).astype(np.complex128),
                                v, (np.pi / 2) * step)

    def _update_env(self, side: str, site: int) -> None:
        prev = site - 1 if side == "left" else site + 1
        e = O._new_env(side, np.asarray(self._env(side, prev)).astype(np.complex64),
                       self.A[site].astype(np.complex64), np.asarray(self.W[site]).astype(np.complex64))
        if side == "left":
            self.L[site] = e.astype(np.complex128)
        else:
            self.R[site] = e.astype(np.complex128)

    def _split(self, Al, Ar, L, R, Wl, Wr):
        """The oracle's split, then the device's arithmetic around it: the isometric
        factor U carries a Gram error (U -> U (I + E/2)), the other factor is formed
        from that U as on the device (U^H Theta, i.e. (I + E/2) times the exact one),
        and optionally both are corrected by one Newton-Schulz step
        M = (3I - U^H U) / 2: U <- U M, other <- M other."""
        a, sk, b = super()._split(Al, Ar, L, R, Wl, Wr)
        k = len(sk)
        if not self.isometry_error and not self.polar:
            return r32(a), sk, r32(b)
        c = np.complex64
        E = np.zeros((k, k))
        if self.isometry_error:
            R_ = self._rng.uniform(-1, 1, (k, k)) + 1j * self._rng.uniform(-1, 1, (k, k))
            E = (R_ + R_.conj().T) / 2 * self.isometry_error
        P = np.eye(k) + E / 2
        sa, sb = a.shape, b.shape
        if self._right:  # U = a (rows (s, l)), other = diag(sk) b (rows k)
            U = r32(a.reshape(-1, k) @ P)
            X = r32(P @ (sk[:, None] * b.transpose(1, 0, 2).reshape(k, -1)))
            if self.polar:
                U32 = U.astype(c)
                M = (3 * np.eye(k, dtype=c) - U32.conj().T @ U32) / 2
                U, X = r32(U32 @ M), r32(M @ X.astype(c))
            a = U.reshape(sa)
            b = (X / sk[:, None]).reshape(k, sb[0], sb[2]).transpose(1, 0, 2)
        else:  # U = b (rows k), other = a diag(sk)
            B = r32(P @ b.transpose(1, 0, 2).reshape(k, -1))
            Y = r32((a.reshape(-1, k) * sk[None, :]) @ P)
            if self.polar:
                B32 = B.astype(c)
                M = (3 * np.eye(k, dtype=c) - B32 @ B32.conj().T) / 2
                B, Y = r32(M @ B32), r32(Y.astype(c) @ M)
            b = B.reshape(k, sb[0], sb[2]).transpose(1, 0, 2)
            a = (Y / sk[None, :]).reshape(sa)
        return r32(a), sk, r32(b)

    def _sweep_right_2(self):
        self._right = True
        yield from super()._sweep_right_2()

    def _sweep_left_2(self):
        self._right = False
        yield from super()._sweep_left_2()

    def step(self) -> None:
        super().step()
        self.A = [r32(a) for a in self.A]
