"""Seeded synthetic workloads of the benchmark configurations.

The reference measures on no public dataset; these generators stand in for its
configurations with their shapes and value distributions:

* ``chain_mix`` — many independent chains: N ~ U{n_lo..n_hi}, (distance,
  interval) drawn from {1,2,3} x {[1,1], [2,3], [2,4]} (inclusive intervals,
  i.e. ranges [1,2), [2,4), [2,5)), bond caps from a list, random product
  states theta_i ~ U(0, pi/2) with p_i = sin^2 theta_i.
* ``single_chain`` — one chain with a given rule and product state.
* ``poisson_jobs`` — a Poisson request stream for the serving loop.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .tensor_networks import MPO, MPS, Rules

INTERVALS = [range(1, 2), range(2, 4), range(2, 5)]


@dataclass
class ChainSpec:
    n: int
    distance: int
    interval: range
    chi: int
    p: np.ndarray
    algorithm: str = "2tdvp"
    dt: float = 0.05
    eps: float = 1e-10
    steps: int = 200

    def mpo(self) -> MPO:
        return MPO.hamiltonian_from_rules(Rules(self.n, self.interval, self.distance))

    def mps(self) -> MPS:
        return MPS.from_density_distribution(self.p)

    def site_updates_per_step(self) -> int:
        return 2 * (self.n - 1) if self.algorithm == "2tdvp" else 2 * self.n


def product_probabilities(rng: np.random.Generator, n: int) -> np.ndarray:
    th = rng.uniform(0.0, np.pi / 2, size=n)
    return np.sin(th) ** 2


def chain_mix(count: int = 256, seed: int = 0, n_lo: int = 16, n_hi: int = 96, chis=(32, 64, 128),
              distances=(1, 2, 3), dt: float = 0.05, eps: float = 1e-10, steps: int = 200,
              algorithm: str = "2tdvp") -> list[ChainSpec]:
    """The batched configuration: ``count`` chains of uneven length, rule and cap."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(rng.integers(n_lo, n_hi + 1))
        d = int(rng.choice(distances))
        interval = INTERVALS[int(rng.integers(0, len(INTERVALS)))]
        chi = int(rng.choice(chis))
        out.append(ChainSpec(n, d, interval, chi, product_probabilities(rng, n), algorithm, dt, eps, steps))
    return out


def single_chain(n: int, distance: int, interval: range, chi: int, seed: int | None = 0, dt: float = 0.05,
                 eps: float = 1e-10, algorithm: str = "2tdvp", centre_only: bool = False) -> ChainSpec:
    if centre_only:
        p = np.zeros(n)
        p[n // 2] = 1.0
    else:
        p = product_probabilities(np.random.default_rng(seed), n)
    return ChainSpec(n, distance, interval, chi, p, algorithm, dt, eps)


@dataclass
class Job:
    arrival: float
    spec: ChainSpec


def poisson_jobs(rate: float = 200.0, duration: float = 60.0, seed: int = 0, n_lo: int = 12, n_hi: int = 128,
                 chis=(16, 32, 64, 128, 256), steps_lo: int = 50, steps_hi: int = 500, dt: float = 0.05,
                 eps: float = 1e-10) -> list[Job]:
    """The serving configuration: Poisson arrivals of 1TDVP / 2TDVP jobs with
    N ~ U{n_lo..n_hi}, distance in {1, 2}, intervals from the batched set."""
    rng = np.random.default_rng(seed)
    t = 0.0
    jobs = []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            break
        n = int(rng.integers(n_lo, n_hi + 1))
        d = int(rng.choice((1, 2)))
        interval = INTERVALS[int(rng.integers(0, len(INTERVALS)))]
        chi = int(rng.choice(chis))
        alg = "1tdvp" if rng.random() < 0.5 else "2tdvp"
        steps = int(rng.integers(steps_lo, steps_hi + 1))
        jobs.append(Job(t, ChainSpec(n, d, interval, chi, product_probabilities(rng, n), alg, dt, eps, steps)))
    return jobs
