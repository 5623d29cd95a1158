"""Noise models on the host, against the reference's own known-answer tests
(test/terra/reference/ref_pauli_noise.py, ref_reset_noise.py,
ref_kraus_noise.py; recorded in tests/golden/ref_noise_kats.json by
gen_ref_noise_kats.py): Pauli, reset and amplitude-damping errors on gates,
on reset and on measure; readout errors on single and 2-qubit measurements
(ref_readout_noise.py); noiseless resets of entangled qubits (ref_reset.py).

Each noise model is rebuilt through this package's noise API, and each
circuit is compiled by AerSimulator(method='density_matrix'): error
placement, the superoperators and Fusion.  The oracle's density matrix
applies every compiled op, and the distribution of the measured classical
bits must equal the reference's target counts / shots.  Also covered here:
where measure and reset errors go (before a measure, after a reset, per
qubit unless an error is given for exactly the op's qubits)."""
import json
from pathlib import Path

import numpy as np
import pytest

from _pkg import pkg
from oracle import oracle as O

_FIXTURE = json.loads((Path(__file__).parent / "golden" / "ref_noise_kats.json").read_text())
NOISE_KATS = _FIXTURE["cases"]
READOUT_KATS = _FIXTURE["readout_cases"]
RESET_KATS = _FIXTURE["reset_cases"]


def noise_model_of(P, calls):
    nm = P.NoiseModel()
    for c in calls:
        args = c["error"]["args"]
        if c["error"]["fn"] == "pauli_error":
            args = [[(label, p) for label, p in args[0]]] + args[1:]
        err = getattr(P, c["error"]["fn"])(*args, **c["error"]["kwargs"])
        if c["call"] == "add_all_qubit_quantum_error":
            nm.add_all_qubit_quantum_error(err, c["instructions"])
        else:
            nm.add_quantum_error(err, c["instructions"], c["qubits"])
    return nm


def circuit_of(P, case):
    qc = P.QuantumCircuit(case["num_qubits"], case["num_clbits"])
    for kind, name, qubits, params, clbits in case["ops"]:
        if kind == "gate":
            qc.append_gate(name, qubits, params)
        elif kind == "reset":
            qc.reset(qubits)
        else:
            qc.measure(qubits, clbits)
    return qc


def oracle_state(sim, qc):
    """The oracle's density matrix after the compiled op list, and the
    final measurements."""
    segments, meas, saves, _ = sim.compile(qc)
    o = O.OracleDM(qc.num_qubits)
    for _, nc in segments:
        for i, (t, _, q) in enumerate(nc.ops()):
            if t in (0, 1):  # gate, matrix
                o.apply_unitary_matrix(q, nc.op_matrix(i).reshape(-1))
            elif t == 2:
                o.apply_diagonal_unitary_matrix(q, nc.op_matrix(i))
            elif t == 3:
                o.apply_superop_matrix(q, nc.op_matrix(i))
            elif t == 5:
                o.apply_reset(q)
            elif t != 6:
                raise AssertionError(f"op type {t} in a compiled noisy circuit")
    return o, meas


def oracle_outcomes(sim, qc):
    """Distribution of the measured classical bits: the compiled op list
    applied by the oracle's density matrix."""
    o, meas = oracle_state(sim, qc)
    qubits = [q for m in meas for q in m.qubits]
    clbits = [c for m in meas for c in m.clbits]
    p = o.probabilities(qubits)
    out = np.zeros(1 << qc.num_clbits)
    for idx, v in enumerate(p):
        out[sum(((idx >> j) & 1) << c for j, c in enumerate(clbits))] += v
    return out


def kat_id(case):
    return f"{case['source'].split(':')[1]}[{case['index']}]"


def test_fixture_covers_gate_measure_and_reset_errors():
    names = {i for c in NOISE_KATS for call in c["noise"] for i in call["instructions"]}
    assert {"id", "x", "measure", "reset"} <= names
    fns = {call["error"]["fn"] for c in NOISE_KATS for call in c["noise"]}
    assert fns == {"pauli_error", "reset_error", "amplitude_damping_error"}


@pytest.mark.parametrize("fusion", [None, 1], ids=["unfused", "fused"])
@pytest.mark.parametrize("case", NOISE_KATS + RESET_KATS, ids=kat_id)
def test_reference_noise_kat(case, fusion):
    P = pkg()
    nm = noise_model_of(P, case["noise"])
    opts = dict(fusion_enable=False) if fusion is None else dict(fusion_threshold=fusion)
    sim = P.AerSimulator(method="density_matrix", noise_model=nm, **opts)
    got = oracle_outcomes(sim, circuit_of(P, case))
    want = np.zeros(1 << case["num_clbits"])
    for k, v in case["probabilities"].items():
        want[int(k)] = v
    np.testing.assert_allclose(got, want, atol=1e-12)


def superops(ops):
    return [(ins.kind, ins.name, list(ins.qubits)) for ins in ops]


def test_measure_errors_before_and_reset_errors_after():
    P = pkg()
    flip = P.pauli_error([("X", 0.5), ("I", 0.5)])
    flip2 = P.pauli_error([("XX", 0.5), ("II", 0.5)])
    nm = P.NoiseModel()
    nm.add_all_qubit_quantum_error(flip, ["measure", "reset"])
    nm.add_quantum_error(P.pauli_error([("Z", 0.5), ("I", 0.5)]), "reset", [2])
    nm.add_quantum_error(flip2, "measure", [0, 1])
    sim = P.AerSimulator(method="density_matrix", noise_model=nm)
    qc = P.QuantumCircuit(3, 3).h(0)
    qc.measure([0, 1], [0, 1])           # an error for exactly these qubits: one 2-qubit error, before
    qc.measure([1, 2], [1, 2])           # none for (1, 2): the all-qubit error per qubit
    qc.reset([1, 2])                     # per qubit: qubit 1 all-qubit, qubit 2 its own error
    got = superops(sim._with_noise(qc.data))
    assert got == [("gate", "h", [0]),
                   ("superop", "superop", [0, 1]), ("measure", "measure", [0, 1]),
                   ("superop", "superop", [1]), ("superop", "superop", [2]), ("measure", "measure", [1, 2]),
                   ("reset", "reset", [1, 2]), ("superop", "superop", [1]), ("superop", "superop", [2])]
    ops = sim._with_noise(qc.data)
    np.testing.assert_allclose(ops[-1].data, nm.error_for("reset", [2]).superop)
    np.testing.assert_allclose(ops[-2].data, flip.superop)
    # an error whose size differs from the instruction's is an error
    bad = P.NoiseModel()
    bad.add_all_qubit_quantum_error(flip2, "measure")
    with pytest.raises(ValueError, match="acts on 2 qubits"):
        P.AerSimulator(method="density_matrix", noise_model=bad)._with_noise(qc.data)


def test_final_measure_errors_come_after_saves():
    P = pkg()
    nm = P.NoiseModel()
    nm.add_all_qubit_quantum_error(P.pauli_error([("X", 0.25), ("I", 0.75)]), "measure")
    sim = P.AerSimulator(method="density_matrix", noise_model=nm, fusion_enable=False)
    qc = P.QuantumCircuit(2, 2).h(0)
    qc.save_density_matrix()
    qc.measure([0, 1], [0, 1])
    segments, meas, saves, _ = sim.compile(qc)
    # the save closes the first segment; the measure errors run after it
    assert [nc.num_ops() for _, nc in segments] == [1, 2]
    assert saves[0][0] == segments[0][0]
    assert [t for t, _, _ in segments[1][1].ops()] == [3, 3]
    # gate noise alone leaves the final measurements untouched
    nm2 = P.NoiseModel()
    nm2.add_all_qubit_quantum_error(P.pauli_error([("X", 0.25), ("I", 0.75)]), "h")
    segments, _, _, _ = P.AerSimulator(method="density_matrix", noise_model=nm2, fusion_enable=False).compile(
        P.QuantumCircuit(2, 2).h(0).measure([0, 1], [0, 1]))
    assert [[t for t, _, _ in nc.ops()] for _, nc in segments] == [[0, 3]]


def readout_model_of(P, calls):
    nm = P.NoiseModel()
    for c in calls:
        if c["call"] == "add_readout_error":
            nm.add_readout_error(P.ReadoutError(c["matrix"]), c["qubits"])
        else:
            nm.add_all_qubit_readout_error(P.ReadoutError(c["matrix"]))
    return nm


def ideal_memory(P, qc):
    """Distribution of the classical memory of the ideal circuit (oracle)."""
    sim = P.AerSimulator(method="statevector", fusion_enable=False)
    segments, meas, _, _ = sim.compile(qc)
    o = O.OracleQV(qc.num_qubits)
    for _, nc in segments:
        for i, (t, _, q) in enumerate(nc.ops()):
            o.apply_matrix(q, nc.op_matrix(i))
    qubits = [q for m in meas for q in m.qubits]
    clbits = [c for m in meas for c in m.clbits]
    out = np.zeros(1 << qc.num_clbits)
    for idx, v in enumerate(o.probabilities(qubits)):
        out[sum(((idx >> j) & 1) << c for j, c in enumerate(clbits))] += v
    return out, meas


@pytest.mark.parametrize("case", READOUT_KATS, ids=kat_id)
def test_reference_readout_kat(case):
    """The readout errors the simulator applies after the final measurements
    (which errors, over which classical bits, with which matrices), composed
    exactly over the ideal distribution, give the reference's target; the
    per-shot draws of the sampled path converge to it (200,000 shots)."""
    P = pkg()
    qc = circuit_of(P, case)
    sim = P.AerSimulator(noise_model=readout_model_of(P, case["noise"]))
    dist, meas = ideal_memory(P, qc)
    ro = sim._readout_ops(meas)
    assert ro
    exact = dist.copy()
    for bits, probs in ro:
        nxt = np.zeros_like(exact)
        for m, p in enumerate(exact):
            actual = sum(((m >> b) & 1) << j for j, b in enumerate(bits))
            cleared = m & ~sum(1 << b for b in bits)
            for read, q in enumerate(probs[actual]):
                nxt[cleared | sum(((read >> j) & 1) << b for j, b in enumerate(bits))] += p * q
        exact = nxt
    want = np.zeros(1 << case["num_clbits"])
    for k, v in case["probabilities"].items():
        want[int(k)] = v
    np.testing.assert_allclose(exact, want, atol=1e-12)
    shots = 200_000
    rng = np.random.default_rng(5)
    memory = rng.choice(dist.size, size=shots, p=dist)
    read = np.asarray(sim._readout_sampled(memory, ro, rng.random(shots * len(ro))))
    freq = np.bincount(read, minlength=want.size) / shots
    assert np.all(np.abs(freq - want) <= 5 * np.sqrt(want * (1 - want) / shots) + 1e-12)
