"""Auxiliary behaviour of the operator on the GPU: pickling (the reference's
operator is picklable, mrrt/nufft/_nufft.py:405-407), and host-side
allocation-failure injection (no GPU fault: the library is told to report a
failed allocation without asking the device for it)."""
import pickle

import numpy as np
import pytest

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def _small():
    from mrrt.nufft_gb300.trajectories import complex_image, radial_2d

    omega = radial_2d(48, 96, golden=True)
    kw = dict(Nd=(48, 48), omega=omega, Jd=(6, 6), Kd=(96, 96), Ld=1024, precision="single")
    return kw, complex_image((48, 48), seed=5)


def test_pickle_round_trip_rebuilds_the_plan(gpu_lib):
    from mrrt.nufft_gb300 import NufftBase

    kw, x = _small()
    A = NufftBase(n_shift=(3.0, -2.0), **kw)
    B = pickle.loads(pickle.dumps(A))
    assert B.Nd == A.Nd and B.Kd == A.Kd and B.n_shift == A.n_shift and B.M == A.M
    np.testing.assert_array_equal(B.omega, A.omega)
    y_a, y_b = A.fft(x), B.fft(x)
    assert np.array_equal(y_a, y_b)
    assert np.array_equal(A.adj(y_a), B.adj(y_a))


def test_allocation_failure_is_reported_and_recoverable(gpu_lib):
    """Fail the k-th device allocation of plan construction, and of the first
    transform, for every k: each failing call returns GBN_ERR_NOMEM (raised
    as GbnError), nothing crashes, and with the injection off the same plan
    (or a new one) computes the right result."""
    from mrrt.nufft_gb300 import NufftBase, _lib
    from mrrt.nufft_gb300._lib import GBN_ERR_NOMEM, GbnError

    kw, x = _small()
    ref = NufftBase(**kw)
    y_ref = ref.fft(x)
    lib = _lib.load()
    seen_failure = False
    try:
        for k in range(64):
            lib.gbn_debug_fail_alloc(k)
            try:
                A = NufftBase(**kw)
            except GbnError as e:
                assert e.code == GBN_ERR_NOMEM, str(e)
                seen_failure = True
                continue
            # construction fitted in k allocations: the first transform makes the rest
            try:
                y = A.fft(x)
            except GbnError as e:
                assert e.code == GBN_ERR_NOMEM, str(e)
                seen_failure = True
                lib.gbn_debug_fail_alloc(-1)
                assert rel_l2(A.fft(x), y_ref) < 1e-6   # the same plan recovers
                continue
            lib.gbn_debug_fail_alloc(-1)
            assert rel_l2(y, y_ref) < 1e-6
            break
        else:
            pytest.fail("more than 64 allocations for a small plan")
    finally:
        lib.gbn_debug_fail_alloc(-1)
    assert seen_failure
