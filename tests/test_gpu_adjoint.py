"""Adjoint gradients (gbqv_adjoint_expval_grad / torch.autograd) against
parameter shift, central finite differences and the oracle's expectation
value.  complex128: relative error <= 1e-8 against parameter shift;
complex64: <= 2e-3 relative (float32 state)."""
import numpy as np
import pytest

from _pkg import pkg
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def oracle_energy(ansatz, theta, ham):
    o = O.OracleQV(ansatz.num_qubits)
    for ins in ansatz.instructions(theta):
        if ins.name in ("ry", "rx", "rz"):
            o.apply_rotation(ins.qubits, {"rx": 0, "ry": 1, "rz": 2}[ins.name], ins.params[0])
        elif ins.name in ("rxx", "ryy", "rzz", "rzx"):
            o.apply_rotation(ins.qubits, {"rxx": 3, "ryy": 4, "rzz": 5, "rzx": 6}[ins.name], ins.params[0])
        elif ins.name == "cx":
            o.apply_mcx(ins.qubits)
        elif ins.name == "h":
            o.apply_mcu(ins.qubits, O.u4(np.pi / 2, 0, np.pi, 0))
        elif ins.name == "x":
            o.apply_mcx(ins.qubits)
        elif ins.name == "swap":
            o.apply_mcswap(ins.qubits)
    return sum(c * o.expval_pauli(q, lab) for (q, lab), c in zip(ham.terms, ham.coeffs))


@pytest.mark.parametrize("precision", ["double", "single"])
def test_adjoint_vs_param_shift_and_oracle(precision):
    P = pkg()
    adj = P.adjoint
    rng = np.random.default_rng(11)
    n, layers = 8, 3
    ans = adj.hardware_efficient_ansatz(n, layers)
    ham = adj.random_hamiltonian(n, 30, rng)
    theta = rng.uniform(-np.pi, np.pi, ans.num_params)
    eng = adj.Engine(n, precision)
    e, g = eng.energy_and_grad(ans, theta, ham)
    ps = eng.param_shift_grad(ans, theta, ham)
    ps = np.array([ps[i] for i in range(ans.num_params)])
    rel = np.linalg.norm(g - ps) / np.linalg.norm(ps)
    e_or = oracle_energy(ans, theta, ham)
    if precision == "double":
        assert rel <= 1e-8, rel
        assert abs(e - e_or) < 1e-11
    else:
        assert rel <= 2e-3, rel
        assert abs(e - e_or) < 1e-4
    fd = eng.finite_diff_grad(ans, theta, ham, [0, 5, 17, ans.num_params - 1], h=1e-5 if precision == "double" else 1e-2)
    for i, v in fd.items():
        assert abs(v - g[i]) < (1e-7 if precision == "double" else 5e-2), (i, v, g[i])
    eng.close()


@pytest.mark.parametrize("precision,atol,etol", [("double", 1e-10, 1e-11), ("single", 2e-3, 1e-4)])
def test_permutation_runs_in_one_gather(precision, atol, etol):
    """Runs of CX, X and SWAP gates between the rotations, uncomputed in the
    sweep as one gather per state (their product is a linear map of the
    index bits plus a constant): gradients against parameter shift, energy
    against the oracle."""
    P = pkg()
    adj = P.adjoint
    rng = np.random.default_rng(21)
    n = 6
    gates = [("h", [q], None, None) for q in range(n)]
    p = 0
    perm_runs = ([("cx", [0, 3]), ("x", [2]), ("swap", [1, 4]), ("cx", [4, 0]), ("cx", [2, 5]), ("x", [5])],
                 [("swap", [0, 2]), ("cx", [5, 1]), ("cx", [1, 2]), ("cx", [2, 3]), ("swap", [3, 5])],
                 [("x", [0]), ("x", [4]), ("cx", [3, 4])])
    for run in perm_runs:
        for q in range(n):
            gates.append(("ry" if q % 2 else "rz", [q], p, None))
            p += 1
        gates += [(name, q, None, None) for name, q in run]
    gates.append(("rx", [2], p, None))
    ans = adj.Ansatz(n, gates)
    ham = adj.random_hamiltonian(n, 15, rng)
    theta = rng.uniform(-3, 3, ans.num_params)
    eng = adj.Engine(n, precision)
    e, g = eng.energy_and_grad(ans, theta, ham)
    ps = eng.param_shift_grad(ans, theta, ham)
    np.testing.assert_allclose(g, [ps[i] for i in range(ans.num_params)], atol=atol)
    assert abs(e - oracle_energy(ans, theta, ham)) < etol
    eng.close()


def test_all_generator_gates():
    P = pkg()
    adj = P.adjoint
    rng = np.random.default_rng(3)
    n = 5
    gates = [("h", [q], None, None) for q in range(n)]
    p = 0
    for name, k in (("rx", 1), ("ry", 1), ("rz", 1), ("rxx", 2), ("ryy", 2), ("rzz", 2), ("rzx", 2)):
        for _ in range(2):
            q = [int(x) for x in rng.choice(n, k, replace=False)]
            gates.append((name, q, p, None))
            p += 1
        gates.append(("cx", [0, 1], None, None))
    # a shared parameter on two gates
    gates.append(("ry", [3], 0, None))
    ans = adj.Ansatz(n, gates)
    ham = adj.random_hamiltonian(n, 12, rng)
    theta = rng.uniform(-3, 3, ans.num_params)
    eng = adj.Engine(n)
    e, g = eng.energy_and_grad(ans, theta, ham)
    ps = eng.param_shift_grad(ans, theta, ham)
    np.testing.assert_allclose(g, [ps[i] for i in range(ans.num_params)], atol=1e-10)
    assert abs(e - oracle_energy(ans, theta, ham)) < 1e-11
    eng.close()


def test_torch_autograd():
    torch = pytest.importorskip("torch")
    P = pkg()
    adj = P.adjoint
    rng = np.random.default_rng(5)
    n = 6
    ans = adj.hardware_efficient_ansatz(n, 2)
    ham = adj.random_hamiltonian(n, 10, rng)
    theta = torch.tensor(rng.uniform(-3, 3, ans.num_params), dtype=torch.float64, requires_grad=True)
    eng = adj.Engine(n)
    loss = adj.expval(theta, eng, ans, ham)
    loss.backward()
    ps = eng.param_shift_grad(ans, theta.detach().numpy(), ham)
    np.testing.assert_allclose(theta.grad.numpy(), [ps[i] for i in range(ans.num_params)], atol=1e-10)
    eng.close()
