"""AerSimulator option handling on the host (AerBackend.set_option /
set_options, qiskit_aer/backends/aerbackend.py:623-658; AerSimulator
available_methods / available_devices / set_option,
qiskit_aer/backends/aer_simulator.py:877-935)."""
import pytest

from _pkg import pkg


def test_available_methods_and_devices():
    sim = pkg().AerSimulator()
    assert sim.available_methods() == ["statevector", "density_matrix", "unitary"]
    assert sim.available_devices() == ["GPU"]
    assert sim.name == "aer_simulator_statevector_gpu"


def test_set_options_and_defaults():
    P = pkg()
    sim = P.AerSimulator()
    nm = P.NoiseModel()
    sim.set_options(method="density_matrix", precision="single", fusion_threshold=3, seed_simulator=9,
                    noise_model=nm)
    assert (sim.method, sim.precision, sim.noise_model) == ("density_matrix", "single", nm)
    assert sim.options["fusion_threshold"] == 3 and sim.options["seed_simulator"] == 9
    assert sim.name == "aer_simulator_density_matrix_gpu"
    assert sim.fusion_config().threshold == 3
    # None restores the default
    sim.set_options(method=None, precision=None, fusion_threshold=None, noise_model=None)
    assert (sim.method, sim.precision, sim.noise_model) == ("statevector", "double", None)
    assert sim.options["fusion_threshold"] is None
    assert sim.fusion_config().threshold == 14


def test_invalid_options():
    sim = pkg().AerSimulator()
    with pytest.raises(ValueError, match="Invalid option shots_per_day"):
        sim.set_option("shots_per_day", 3)
    with pytest.raises(ValueError, match="Invalid simulation method stabilizer"):
        sim.set_options(method="stabilizer")
    with pytest.raises(ValueError, match="GPU only"):
        sim.set_options(device="CPU")
    with pytest.raises(ValueError, match="Invalid precision"):
        sim.set_options(precision="half")
    assert sim.method == "statevector"


def test_autotune_cache_option_replaces_the_tuner(tmp_path):
    sim = pkg().AerSimulator(autotune=True)
    first = sim.tuner()
    sim.set_options(autotune_cache=str(tmp_path / "t.json"))
    assert sim.tuner() is not first and sim.tuner().path == str(tmp_path / "t.json")


def test_run_options_apply_to_one_call_only():
    """Keyword options of run() override the simulator's options for that
    call (AerBackend.run's run_options, aerbackend.py:146-185) on a per-call
    copy: the simulator itself never changes, also when the run fails or
    while another thread runs with other options; unknown ones are ignored
    with a warning."""
    import threading

    P = pkg()
    nm = P.NoiseModel()
    seen = []
    gate = threading.Barrier(2, timeout=10)

    class Sim(P.AerSimulator):
        def _run(self, circuits, shots, seed, binds, memory):
            if shots in (21, 22):  # two concurrent calls meet here
                gate.wait()
            seen.append((self.method, self.precision, self.noise_model, self.options["fusion_threshold"], shots,
                         self._want_memory))
            if shots == 13:
                raise RuntimeError("boom")
            return "result"

    sim = Sim()
    qc = P.QuantumCircuit(1)
    assert sim.run(qc, shots=7, method="density_matrix", precision="single", noise_model=nm,
                   fusion_threshold=2) == "result"
    assert seen[-1][:5] == ("density_matrix", "single", nm, 2, 7)
    assert (sim.method, sim.precision, sim.noise_model, sim.options["fusion_threshold"]) == (
        "statevector", "double", None, None)
    with pytest.raises(RuntimeError):
        sim.run(qc, shots=13, method="unitary")
    assert sim.method == "statevector"
    with pytest.warns(UserWarning, match="blocking_qubits"):
        sim.run(qc, shots=1, blocking_qubits=20)
    assert seen[-1][0] == "statevector"
    with pytest.raises(ValueError, match="Invalid simulation method"):
        sim.run(qc, method="mps")
    assert sim.method == "statevector"
    # two threads on one simulator, each with its own overrides and memory flag
    t = threading.Thread(target=lambda: sim.run(qc, shots=21, method="density_matrix", memory=True))
    t.start()
    sim.run(qc, shots=22, precision="single")
    t.join()
    got = {r[4]: r for r in seen[-2:]}
    assert got[21][:2] == ("density_matrix", "double") and got[21][5] is True
    assert got[22][:2] == ("statevector", "single") and got[22][5] is False
    assert (sim.method, sim.precision, sim._want_memory) == ("statevector", "double", False)
