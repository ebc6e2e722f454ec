"""The allocation-free exact step (qca_exact_step_noalloc) against the regular
exact step (qca_exact_step), through the C ABI.

Callers that may not allocate device memory (their device memory is owned by
their own pool, or they run latency-critical loops that cannot take
cudaMalloc's implicit synchronisation) use the allocation-free entry point; its
scratch is a static device array, so it must give the same state as the
allocating path, call after call, even though the array keeps the previous
call's contents.  Tolerance 1e-12 (both paths run the same FP64 kernels).
This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _handle(n, d, lo, hi, m):
    from qca_gb300 import _lib
    h = ctypes.c_void_p()
    _lib.call("qca_exact_create", n, d, lo, hi, _lib.QCA_PREC_FP64, m, ctypes.byref(h))
    return h


def _set(h, psi):
    from qca_gb300 import _lib
    v = np.ascontiguousarray(psi, dtype=np.complex128)
    _lib.call("qca_exact_set_state", h, v.view(np.float64).ctypes.data_as(_lib._PD), None)


def _get(h, n):
    from qca_gb300 import _lib
    out = np.empty(1 << n, dtype=np.complex128)
    _lib.call("qca_exact_get_state", h, out.view(np.float64).ctypes.data_as(_lib._PD), None)
    return out


def _dev(h):
    from qca_gb300 import _lib
    p = ctypes.c_void_p()
    _lib.call("qca_exact_state_device", h, ctypes.byref(p))
    return p


@pytest.mark.parametrize("n,d,lo,hi", [(12, 2, 2, 4), (14, 1, 1, 2)])
def test_noalloc_matches_exact_step_twice(n, d, lo, hi):
    from qca_gb300 import _lib
    m, dt = 30, 0.05
    rng = np.random.default_rng(n)
    psi = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    psi /= np.linalg.norm(psi)
    ref = _handle(n, d, lo, hi, m)
    src = _handle(n, d, lo, hi, m)   # holds the input state on the device
    dst = _handle(n, d, lo, hi, m)   # receives the output state
    try:
        _set(ref, psi)
        _set(src, psi)
        for call in range(2):
            _lib.call("qca_exact_step", ref, dt, 2, None)
            # in: src's state, out: dst's state; then feed the output back
            _lib.call("qca_exact_step_noalloc", n, d, lo, hi, m, dt, 2, _dev(src), _dev(dst), None)
            got = _get(dst, n)
            want = _get(ref, n)
            assert np.abs(got - want).max() < TOL, call
            _set(src, got)
    finally:
        for h in (ref, src, dst):
            _lib.load().qca_exact_destroy(h)


def test_noalloc_in_place_matches_exact_step_twice():
    """psi_in and psi_out may be the same buffer: the state is read into the
    scratch basis before the output is written."""
    from qca_gb300 import _lib
    n, d, lo, hi, m, dt = 12, 2, 2, 4, 30, 0.05
    rng = np.random.default_rng(3)
    psi = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    psi /= np.linalg.norm(psi)
    ref = _handle(n, d, lo, hi, m)
    buf = _handle(n, d, lo, hi, m)  # its device state is both input and output
    try:
        _set(ref, psi)
        _set(buf, psi)
        for call in range(2):
            _lib.call("qca_exact_step", ref, dt, 2, None)
            _lib.call("qca_exact_step_noalloc", n, d, lo, hi, m, dt, 2, _dev(buf), _dev(buf), None)
            assert np.abs(_get(buf, n) - _get(ref, n)).max() < TOL, call
    finally:
        for h in (ref, buf):
            _lib.load().qca_exact_destroy(h)


def test_noalloc_rejects_states_beyond_its_scratch():
    from qca_gb300 import _lib
    dummy = ctypes.c_void_p(1)
    st = _lib.load().qca_exact_step_noalloc(20, 2, 2, 4, 30, 0.05, 1, dummy, dummy, None)
    assert st == _lib.QCA_ERR_INVALID
    assert b"static scratch" in _lib.load().qca_last_error()
