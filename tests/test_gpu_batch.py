"""Batched uneven instances in one persistent launch (gbqv_batch_*): per
instance <H> against the oracle and the single-instance adjoint engine, the
adjoint gradient against the single-instance engine, and the sampled shots bit-exact against the oracle for the same
RngEngine seed.  Instances span 3..13 qubits so that some fit one tile and
some need several tiles per run."""
import numpy as np
import pytest

from _pkg import pkg
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _engine_ansatz(adj, inst):
    kinds = {0: "rx", 1: "ry", 2: "rz", 3: "cx", 4: "cz", 5: "h"}
    gates = []
    for k, q0, q1, p in inst["gates"]:
        q = [q0, q1] if k in (3, 4) else [q0]
        gates.append((kinds[k], q, p if p >= 0 else None, None))
    return adj.Ansatz(inst["n"], gates)


def _oracle_state(inst):
    """The instance's ansatz applied gate by gate by the oracle (complex128)."""
    o = O.OracleQV(inst["n"])
    for k, q0, q1, p in inst["gates"]:
        if k in (0, 1, 2):
            o.apply_rotation([q0], k, inst["theta"][p])
        elif k == 3:
            o.apply_mcx([q0, q1])
        elif k == 4:
            o.apply_mcphase([q0, q1], -1.0)
        elif k == 5:
            o.apply_mcu([q0], O.u4(np.pi / 2, 0, np.pi, 0))
    return o


@pytest.mark.parametrize("precision,fp64,tol,gtol", [("double", False, 1e-11, 1e-9), ("double", True, 1e-11, 1e-9),
                                                     ("single", False, 2e-4, 2e-3)])
def test_batch_matches_single_instance_engine(precision, fp64, tol, gtol):
    """complex128 as float pairs (the default) and on the FP64 pipe, and
    complex64."""
    P = pkg()
    B, adj = P.batched, P.adjoint
    insts = B.config5_instances(10, seed=5, qmin=3, qmax=13, dmin=1, dmax=4, tmin=4, tmax=12, shots=300)
    b = B.Batch(precision)
    if fp64:
        b.set_fp64(True)
    for inst in insts:
        b.add(inst["n"], inst["gates"], inst["theta"], inst["terms"], inst["coeffs"], inst["shots"], inst["seed"])
    ms = b.run(want_grad=True)
    assert ms > 0
    for i, inst in enumerate(insts):
        e, g, s, lat = b.result(i)
        ans = _engine_ansatz(adj, inst)
        ham = adj.Hamiltonian(inst["terms"], inst["coeffs"])
        eng = adj.Engine(inst["n"], "double")
        e_ref, g_ref = eng.energy_and_grad(ans, inst["theta"], ham)
        eng.close()
        assert abs(e - e_ref) < tol * max(1, abs(e_ref)), (i, e, e_ref)
        np.testing.assert_allclose(g, g_ref, atol=gtol)
        assert lat > 0
        o = _oracle_state(inst)
        e_or = sum(c * o.expval_pauli(q, lab) for (q, lab), c in zip(inst["terms"], inst["coeffs"]))
        assert abs(e - e_or) < tol * max(1, abs(e_or)), (i, e, e_or)
        if precision == "double":
            want = o.sample_measure(O.uniforms(inst["seed"], inst["shots"]))
            np.testing.assert_array_equal(s, want)
    # a second run replays the captured graph and gives the same results
    e0 = b.result(0)[0]
    b.run(want_grad=True)
    assert b.result(0)[0] == e0
    b.close()


@pytest.mark.parametrize("precision,tol", [("double", 1e-12), ("single", 2e-5)])
def test_teams_match_single_cta_instances(precision, tol):
    """Instances run by two-CTA teams (tiles split, a barrier after each run,
    energy and gradient partial sums added atomically) give the results of
    the same instances on one CTA each; the shots are identical."""
    P = pkg()
    B = P.batched
    insts = B.config5_instances(12, seed=9, qmin=11, qmax=15, dmin=2, dmax=5, tmin=5, tmax=15, shots=256)
    out = []
    for teams in (0, 64):
        b = B.Batch(precision)
        b.set_teams(teams, 0.0)
        for inst in insts:
            b.add(inst["n"], inst["gates"], inst["theta"], inst["terms"], inst["coeffs"], inst["shots"], inst["seed"])
        b.run(want_grad=True)
        out.append([b.result(i) for i in range(len(insts))])
        b.close()
    for (e0, g0, s0, _), (e1, g1, s1, _) in zip(*out):
        assert abs(e0 - e1) < tol * max(1.0, abs(e0))
        np.testing.assert_allclose(g1, g0, atol=tol * 10)
        np.testing.assert_array_equal(s1, s0)
