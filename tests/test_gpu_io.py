"""State upload and download through the C ABI (QubitVector::initialize_from_vector
and copy_to_vector, qubitvector.hpp:994-1041 / 1047-1077): a complex64 state
is filled from complex128 host data through a device staging slice and a
narrowing kernel, and read back through a widening kernel.  The round trip
must equal numpy's complex128 -> complex64 -> complex128 cast bit for bit,
for states of one slice and of several (2^26 amplitudes = 4 slices), and
from pinned as well as pageable host memory."""
import numpy as np
import pytest

from _pkg import pkg

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [3, 20, 26])
def test_c64_round_trip_is_the_rounding_cast(n):
    P = pkg()
    rng = np.random.default_rng(700 + n)
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    psi[:4] = [1e-40, -3.4e38, 1 + 2 ** -30, 0.1]
    with P.QubitVector(n, "single") as qv:
        qv.initialize_from_vector(psi)
        got = qv.copy_to_vector()
    want = psi.astype(np.complex64).astype(np.complex128)
    np.testing.assert_array_equal(got, want)


def test_c64_upload_from_pinned_memory():
    torch = pytest.importorskip("torch")
    P = pkg()
    n = 25
    t = torch.zeros(1 << n, dtype=torch.complex128, pin_memory=True)
    psi = t.numpy()
    rng = np.random.default_rng(9)
    psi[:] = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    with P.QubitVector(n, "single") as qv:
        qv.initialize_from_vector(psi)
        out = qv.copy_to_vector()
    np.testing.assert_array_equal(out, psi.astype(np.complex64).astype(np.complex128))


def test_c128_round_trip_exact_and_pure_state_dm():
    P = pkg()
    rng = np.random.default_rng(3)
    n = 12
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    with P.QubitVector(n, "double") as qv:
        qv.initialize_from_vector(psi)
        np.testing.assert_array_equal(qv.copy_to_vector(), psi)
    m = 5
    phi = rng.normal(size=1 << m) + 1j * rng.normal(size=1 << m)
    phi /= np.linalg.norm(phi)
    for precision in ("double", "single"):
        with P.DensityMatrix(m, precision) as dm:
            dm.initialize_from_vector(phi)
            rho = np.outer(phi, phi.conj())
            want = rho if precision == "double" else rho.astype(np.complex64).astype(np.complex128)
            np.testing.assert_allclose(dm.copy_to_matrix(), want, rtol=0, atol=1e-15)


def test_c64_download_into_pinned_memory():
    torch = pytest.importorskip("torch")
    P = pkg()
    n = 21
    rng = np.random.default_rng(12)
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    out = torch.zeros(1 << n, dtype=torch.complex128, pin_memory=True)
    with P.QubitVector(n, "single") as qv:
        qv.initialize_from_vector(psi)
        P._capi.check(P.lib().gbqv_copy_to_host(qv.handle, P._capi.C.c_void_p(out.data_ptr()), 1 << n), qv.handle)
    np.testing.assert_array_equal(out.numpy(), psi.astype(np.complex64).astype(np.complex128))


def test_c128_upload_from_pinned_memory_is_exact():
    torch = pytest.importorskip("torch")
    P = pkg()
    n = 21
    t = torch.zeros(1 << n, dtype=torch.complex128, pin_memory=True)
    psi = t.numpy()
    rng = np.random.default_rng(13)
    psi[:] = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    with P.QubitVector(n, "double") as qv:
        qv.initialize_from_vector(psi)
        np.testing.assert_array_equal(qv.copy_to_vector(), psi)
