"""The two-site split (Householder QR, then one-sided Jacobi SVD of R^H on a
thread-block cluster) on its own, against numpy's complex128 SVD of the same
theta: singular values, the reconstruction A_l A_r = theta / ||theta||, the
isometry of A_l, and the truncation rule (tdvp.py:286-296).  Sizes run from the 2 x 2 product-state split
to 256 x 256 (bond dimension 128 on both sides), through both SVD kernels.
Tolerances: FP64 1e-12.  complex64 (mixed path): reconstruction and isometry
2e-5; singular values 1e-4 relative to the largest, since each column carries the
rounding of its few thousand FP32 rotations (about 2e-5 measured at 256 x 256)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = [(1, 1), (1, 2), (2, 1), (3, 5), (17, 9), (16, 16), (40, 50), (64, 64), (100, 100), (128, 128), (130, 60)]


def run_svd(prec, Dl, Dr, theta, chi=100000, eps=0.0):
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
    _lib.call("qca_test_svd", prec, Dl, Dr, ctypes.c_void_p(th.data_ptr()), chi, eps, ctypes.c_void_p(Al.data_ptr()),
              ctypes.c_void_p(Ar.data_ptr()), ctypes.c_void_p(sv.data_ptr()), ctypes.byref(k), None)
    kk = k.value
    Al = Al[: 2 * Dl * kk].cpu().numpy().astype(np.complex128).reshape(2, Dl, kk)
    Ar = Ar[: 2 * kk * Dr].cpu().numpy().astype(np.complex128).reshape(2, kk, Dr)
    return Al, Ar, sv.cpu().numpy(), kk


def theta_matrix(theta, Dl, Dr):
    # Theta[(s1, a), (s2, c)] = theta[s1 * 2 + s2][a][c]
    return theta.reshape(2, 2, Dl, Dr).transpose(0, 2, 1, 3).reshape(2 * Dl, 2 * Dr)


@pytest.mark.parametrize("prec_name", ["fp64", "mixed"])
@pytest.mark.parametrize("Dl,Dr", SIZES)
def test_svd_matches_numpy(prec_name, Dl, Dr):
    from qca_gb300 import _lib
    prec = _lib.QCA_PREC_FP64 if prec_name == "fp64" else _lib.QCA_PREC_MIXED
    tol = 1e-12 if prec_name == "fp64" else 2e-5
    tol_s = 1e-12 if prec_name == "fp64" else 1e-4
    rng = np.random.default_rng(Dl * 1000 + Dr)
    theta = rng.standard_normal((4, Dl, Dr)) + 1j * rng.standard_normal((4, Dl, Dr))
    if prec_name == "mixed":
        theta = theta.astype(np.complex64).astype(np.complex128)
    M = theta_matrix(theta, Dl, Dr)
    s_ref = np.linalg.svd(M, compute_uv=False)
    Al, Ar, sv, k = run_svd(prec, Dl, Dr, theta)
    nx = 2 * min(Dl, Dr)
    assert k == nx
    assert np.abs(sv - s_ref).max() <= tol_s * s_ref[0]
    # A_l A_r = Theta / ||Theta||_F
    R = np.einsum("sai,tic->satc", Al, Ar).reshape(2 * Dl, 2 * Dr)
    assert np.abs(R - M / np.linalg.norm(M)).max() <= tol
    U = Al.reshape(2 * Dl, k)
    assert np.abs(U.conj().T @ U - np.eye(k)).max() <= tol


@pytest.mark.parametrize("prec_name", ["fp64", "mixed"])
def test_svd_truncation_rule(prec_name):
    """k = min{i : ||s[i:]|| < eps} capped at chi, on a graded spectrum."""
    from qca_gb300 import _lib
    prec = _lib.QCA_PREC_FP64 if prec_name == "fp64" else _lib.QCA_PREC_MIXED
    Dl = Dr = 12
    rng = np.random.default_rng(5)
    n = 2 * Dl
    U, _ = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    V, _ = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    s = 10.0 ** (-0.5 * np.arange(n))
    M = (U * s) @ V.conj().T
    theta = M.reshape(2, Dl, 2, Dr).transpose(0, 2, 1, 3).reshape(4, Dl, Dr)
    eps = 0.5e-3 * np.linalg.norm(s)  # between the tails at i = 6 and 7, clear of both
    tail = np.sqrt(np.cumsum((s ** 2)[::-1])[::-1])
    k_ref = int(np.argmax(tail < eps))
    _, _, _, k = run_svd(prec, Dl, Dr, theta, eps=eps)
    assert k == k_ref
    _, _, _, k = run_svd(prec, Dl, Dr, theta, chi=3, eps=eps)
    assert k == min(3, k_ref)


@pytest.mark.parametrize("prec_name", ["fp64", "mixed"])
@pytest.mark.parametrize("D,decay", [(32, 0.3), (64, 0.15), (128, 0.08), (100, 0.12)])
def test_svd_graded_spectrum_converges(prec_name, D, decay):
    """Two-site matrices of TDVP have exponentially graded spectra (singular values
    spanning 1e-12 of the largest); one-sided Jacobi on them directly needs dozens
    of sweeps.  After the QR preconditioning the split converges within the sweep
    limit, A_l is an isometry to rounding and the kept singular values are
    accurate to rounding relative to the largest (FP64 1e-12; mixed: isometry 5e-6,
    set by the FP32 rotation tolerance of 16 eps32, reconstruction 2e-5, singular
    values 1e-5 of the largest)."""
    from qca_gb300 import _lib
    prec = _lib.QCA_PREC_FP64 if prec_name == "fp64" else _lib.QCA_PREC_MIXED
    rng = np.random.default_rng(D)
    n = 2 * D
    U, _ = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    V, _ = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    s = np.exp(-decay * np.arange(n))
    M = (U * s) @ V.conj().T
    M /= np.linalg.norm(M)
    theta = M.reshape(2, D, 2, D).transpose(0, 2, 1, 3).reshape(4, D, D)
    if prec_name == "mixed":
        theta = theta.astype(np.complex64).astype(np.complex128)
        M = theta_matrix(theta, D, D)
    tol_iso = 1e-12 if prec_name == "fp64" else 5e-6
    tol_rec = 1e-12 if prec_name == "fp64" else 2e-5
    tol_s = 1e-12 if prec_name == "fp64" else 1e-5
    Al, Ar, sv, k = run_svd(prec, D, D, theta)  # raises on QCA_ERR_NOT_CONVERGED
    ref = np.linalg.svd(M, compute_uv=False)
    assert np.abs(sv[:k] - ref[:k]).max() <= tol_s * ref[0]
    Ul = Al.reshape(n, k)
    assert np.abs(Ul.conj().T @ Ul - np.eye(k)).max() <= tol_iso
    R = np.einsum("sai,tic->satc", Al, Ar).reshape(n, n)
    assert np.linalg.norm(R - M / np.linalg.norm(M)) <= tol_rec + np.sqrt(np.sum(ref[k:] ** 2))
