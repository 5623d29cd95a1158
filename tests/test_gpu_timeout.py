"""The bounded-wait failure path of the tcgen05 complex128 kernel, made to
run on purpose without a GPU fault: with the test hook on, each CTA leaves
its first accumulator uncommitted, the epilogue's mbarrier wait gives up
after its 2 s bound, the CTA drains and returns, and the call reports
GBQV_ERR_TIMEOUT.  The context stays usable: the same gate afterwards
matches the oracle."""
import numpy as np
import pytest

from _pkg import pkg
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _haar(rng, d):
    z = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def test_stalled_pipeline_times_out_and_context_survives():
    P = pkg()
    L = P.lib()
    rng = np.random.default_rng(404)
    n = 16
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    psi /= np.linalg.norm(psi)
    u = _haar(rng, 16)
    q = [1, 5, 9, 14]
    with P.QubitVector(n) as qv:
        qv.initialize_from_vector(psi)
        assert L.gbqv_test_stall_tensor_pipeline(qv.handle, 1) == 0
        with pytest.raises(P.GBQVError) as e:
            qv.apply_matrix(q, u)
            qv.synchronize()
        assert e.value.code == 6, e.value  # GBQV_ERR_TIMEOUT
        assert "timed out" in str(e.value)
        assert L.gbqv_test_stall_tensor_pipeline(qv.handle, 0) == 0
        qv.initialize_from_vector(psi)
        qv.apply_matrix(q, u)
        got = qv.copy_to_vector()
    o = O.OracleQV(n, psi)
    o.apply_matrix(q, u)
    np.testing.assert_allclose(got, o.data, atol=1e-12, rtol=0)
