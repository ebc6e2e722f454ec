"""Numerical failures come back as status codes through the C ABI (the reference's
convention is an ``assert``: tdvp.py:69-76, 177-178, 353-355).  Every failure here
is made on the host (a NaN in the uploaded MPS, a lowered Jacobi sweep limit); no
kernel is made to fault, and every device loop involved is bounded."""
import ctypes
import types

import numpy as np
import pytest

from oracle import qca_oracle as O

pytestmark = pytest.mark.gpu


def _chain(engine, n, p, chi=8, alg="2tdvp", precision="fp64", poison=False):
    from qca_gb300 import GpuTDVP, MPO, MPS, Rules
    H = MPO.hamiltonian_from_rules(Rules(n, range(2, 4), 2))
    psi = MPS.from_density_distribution(p)
    if poison:
        psi.A[n // 2] = psi.A[n // 2].copy()
        psi.A[n // 2][0, 0, 0] = np.nan
    args = types.SimpleNamespace(step_size=0.05, algorithm=alg, max_bond_dim=chi, svd_epsilon=1e-10,
                                 precision=precision)
    return GpuTDVP(psi, H, args, engine=engine)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("alg", ["2tdvp", "1tdvp"])
def test_nan_in_initial_state_returns_nan_status(precision, alg):
    """A NaN uploaded with qca_chain_add is reported by qca_engine_step_chains as
    QCA_ERR_NAN; a healthy chain stepped in the same call completes its step with
    the result it has alone, and the failed chain stays failed."""
    from qca_gb300 import _lib
    from qca_gb300.algorithms import _Engine
    prec = _lib.QCA_PREC_FP64 if precision == "fp64" else _lib.QCA_PREC_MIXED
    n = 8
    p = np.sin(O.random_thetas(n, 3)) ** 2
    eng = _Engine(prec)
    good = _chain(eng, n, p, alg=alg, precision=precision)
    bad = _chain(eng, n, p, alg=alg, precision=precision, poison=True)
    ids = (ctypes.c_int * 2)(good._chain, bad._chain)
    with pytest.raises(_lib.QcaError) as ei:
        _lib.call("qca_engine_step_chains", eng.h, ids, 2, 2, None)
    assert ei.value.code == _lib.QCA_ERR_NAN
    assert f"chain {bad._chain}" in str(ei.value)
    alone = _chain(None, n, p, alg=alg, precision=precision)
    alone.evolve(2)
    r1 = [np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(n + 1)]
    r2 = [np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(n + 1)]
    good.measure(*r1)
    alone.measure(*r2)
    assert np.abs(r1[0] - r2[0]).max() < 1e-12
    with pytest.raises(_lib.QcaError) as ei:
        bad.do_time_step()
    assert ei.value.code == _lib.QCA_ERR_NAN
    good.do_time_step()  # the healthy chain is unaffected


def _svd_sweeps(prec, Dl, Dr, theta, max_sweeps):
    import torch
    from qca_gb300 import _lib
    ct = torch.complex128 if prec == _lib.QCA_PREC_FP64 else torch.complex64
    nx = 2 * min(Dl, Dr)
    th = torch.from_numpy(theta).to(ct).cuda()
    Al = torch.zeros(2 * Dl * nx, dtype=ct, device="cuda")
    Ar = torch.zeros(2 * nx * Dr, dtype=ct, device="cuda")
    sv = torch.zeros(nx, dtype=torch.float64, device="cuda")
    k = ctypes.c_int(0)
    torch.cuda.synchronize()
    _lib.call("qca_test_svd_sweeps", prec, Dl, Dr, ctypes.c_void_p(th.data_ptr()), 100000, 0.0, max_sweeps,
              ctypes.c_void_p(Al.data_ptr()), ctypes.c_void_p(Ar.data_ptr()), ctypes.c_void_p(sv.data_ptr()),
              ctypes.byref(k), None)
    return k.value


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_svd_sweep_limit_returns_not_converged(precision):
    from qca_gb300 import _lib
    prec = _lib.QCA_PREC_FP64 if precision == "fp64" else _lib.QCA_PREC_MIXED
    Dl = Dr = 16
    rng = np.random.default_rng(11)
    theta = rng.standard_normal((4, Dl, Dr)) + 1j * rng.standard_normal((4, Dl, Dr))
    with pytest.raises(_lib.QcaError) as ei:
        _svd_sweeps(prec, Dl, Dr, theta, 1)
    assert ei.value.code == _lib.QCA_ERR_NOT_CONVERGED
    assert _svd_sweeps(prec, Dl, Dr, theta, 0) == 2 * Dl  # the default limit converges


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_svd_non_finite_input_returns_nan(precision):
    from qca_gb300 import _lib
    prec = _lib.QCA_PREC_FP64 if precision == "fp64" else _lib.QCA_PREC_MIXED
    Dl, Dr = 6, 5
    rng = np.random.default_rng(12)
    theta = rng.standard_normal((4, Dl, Dr)) + 1j * rng.standard_normal((4, Dl, Dr))
    theta[1, 2, 3] = np.inf
    with pytest.raises(_lib.QcaError) as ei:
        _svd_sweeps(prec, Dl, Dr, theta, 0)
    assert ei.value.code == _lib.QCA_ERR_NAN
