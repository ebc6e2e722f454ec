"""The reference's driver loop (``quantum_game.py:28-119``) over the GPU algorithms.

For every initial state: build the algorithm chosen by ``args.algorithm``
(``quantum_game.py:62-68``), measure every ``plot_step_interval`` steps into the
rows of the population, rounded-population, single-site-entropy and bond-dimension
arrays (``algorithm.measure``, ``algorithm.py:58-63``), back the rows up to CSV
files and the state to an npz file after every measurement
(``quantum_game.py:92-115``), and step (``exact``: once per measurement with the
step size scaled by the interval, ``quantum_game.py:70-73``; TDVP: every step).
File names follow ``quantum_game.py:50-58``.  Plotting (``quantum_game.py:121-146``)
is not part of this package; the arrays are returned, and
``Algorithm.classical_evolution`` gives the classical automaton beside them.

Two deliberate differences: the CSV backups hold every measured row (the
reference's ``population[:plot_step]`` leaves out the row just measured, also in
the final files), and the exact path's scaled step size is computed per run
instead of being written back into ``args`` (where the reference scales it again
for every further initial state).
"""
from __future__ import annotations

import os
import types

import numpy as np

from .algorithms import algorithm_class


def run_name(args, state_name: str) -> str:
    """``quantum_game.py:50-58`` (the step size before the exact path's scaling)."""
    r = args.rules
    name = (f"{state_name}{r.ncells}_{r.distance}{r.activation_interval.start}{r.activation_interval.stop}_"
            f"{str(args.step_size).replace('.', '')}_{args.algorithm}")
    if args.algorithm != "exact":
        name += f"_{args.max_bond_dim}"
    return name


def run(args, initial_states, H, out_dir: str | None = "data", state_names=None, algorithm_cls=None,
        save_state: bool = True) -> list[dict]:
    """Evolve every initial state as the reference's ``QuantumGame.start`` does.

    ``args`` carries the reference's fields (``rules`` with ``ncells``,
    ``distance``, ``activation_interval``; ``algorithm``, ``step_size``,
    ``num_steps``, ``plot_step_interval``, ``max_bond_dim``, ``svd_epsilon``; the
    GPU fields ``precision`` / ``krylov_dim`` are optional).  ``out_dir`` = None
    writes no files.  Returns one dict per initial state with its name and the
    four observable arrays (``plot_steps`` rows each)."""
    names = list(state_names or [])
    interval = int(args.plot_step_interval)
    num_steps = int(args.num_steps)
    plot_steps = (num_steps + interval - 1) // interval
    n = args.rules.ncells
    cls = algorithm_cls or algorithm_class(args.algorithm)
    exact = args.algorithm == "exact"
    if out_dir is not None:
        os.makedirs(out_dir, exist_ok=True)
    results = []
    for index, psi_0 in enumerate(initial_states):
        population = np.zeros((plot_steps, n))
        d_population = np.zeros((plot_steps, n))
        single_site_entropy = np.zeros((plot_steps, n))
        bond_dims = np.zeros((plot_steps, n + 1))
        name = run_name(args, names[index] if index < len(names) else str(index))
        run_args = types.SimpleNamespace(**vars(args))
        run_args.step_size = args.step_size * interval if exact else args.step_size
        algorithm = cls(psi_0=psi_0, H=H, args=run_args)
        for step in range(num_steps):
            if step % interval == 0:
                k = step // interval
                algorithm.measure(population=population[k, :], d_population=d_population[k, :],
                                  single_site_entropy=single_site_entropy[k, :], bond_dims=bond_dims[k, :])
                if out_dir is not None:
                    base = os.path.join(out_dir, name)
                    for suffix, arr in (("population", population), ("d_population", d_population),
                                        ("single_site_entropy", single_site_entropy), ("bond_dims", bond_dims)):
                        np.savetxt(f"{base}-{suffix}.csv", arr[:k + 1, :], delimiter=",")
                    if save_state:
                        algorithm.psi.write_to_file(f"{base}.npz")
                if exact:
                    algorithm.do_time_step()
            if not exact:
                algorithm.do_time_step()
        results.append({"name": name, "population": population, "d_population": d_population,
                        "single_site_entropy": single_site_entropy, "bond_dims": bond_dims})
    return results
