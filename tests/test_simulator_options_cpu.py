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
