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
    call (AerBackend.run's run_options, aerbackend.py:146-185) and are
    restored afterwards, also when the run fails; unknown ones are ignored
    with a warning."""
    P = pkg()
    sim = P.AerSimulator()
    nm = P.NoiseModel()
    seen = []

    def fake_run(circuits, shots, seed, binds, memory):
        seen.append((sim.method, sim.precision, sim.noise_model, sim.options["fusion_threshold"], shots))
        if shots == 13:
            raise RuntimeError("boom")
        return "result"

    sim._run = fake_run
    qc = P.QuantumCircuit(1)
    assert sim.run(qc, shots=7, method="density_matrix", precision="single", noise_model=nm,
                   fusion_threshold=2) == "result"
    assert seen[-1] == ("density_matrix", "single", nm, 2, 7)
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
