// Test driver for include/gbqv_qubitvector.hpp: applies an op list read from
// stdin through the QubitVector-shaped C++ adapter and prints the results of
// the queries that follow, one per line.  tests/test_adapter_cpu.py compiles
// it (no GPU needed) and checks the error translation; tests/test_gpu_adapter.py
// runs it on the GPU and compares every printed value with the oracle.
//
// Input (whitespace separated):
//   header:  <kind: sv|dm> <precision: c128|c64> <num_qubits>
//   then records until "end":
//     matrix k q... (2^k x 2^k complex, column-major, as re im pairs)
//     diag k q... (2^k complex)
//     mcx k q...           mcu k q... (4 complex)      rotation k q... axis theta
//     pauli k q... label re im                         component k q... (2^k complex)
//     superop k q... (4^k x 4^k complex)               reset k q...
//     probs k q...         expval k q... label         probability outcome
//     norm                 normmat k q... (matrix)     normdiag k q... (2^k complex)
//     ket eps              sample count u...           state
//   outputs: "probs v0 v1 ...", "expval v", "probability v", "norm v",
//   "ket key re im ...", "sample i0 i1 ...", "state re im ...".
#include <iomanip>
#include <iostream>
#include <string>
#include <vector>

#include "gbqv_qubitvector.hpp"

using gbqv_aer::complex_t;
using gbqv_aer::cvector_t;
using gbqv_aer::reg_t;

template class gbqv_aer::QubitVector<double, GBQV_STATEVECTOR>;
template class gbqv_aer::QubitVector<float, GBQV_STATEVECTOR>;
template class gbqv_aer::QubitVector<double, GBQV_DENSITY_MATRIX>;
template class gbqv_aer::UnitaryMatrix<double>;

namespace {

reg_t read_qubits(std::istream &in) {
  size_t k;
  in >> k;
  reg_t q(k);
  for (auto &x : q) in >> x;
  return q;
}

cvector_t read_complex(std::istream &in, size_t count) {
  cvector_t v(count);
  for (auto &z : v) {
    double re, im;
    in >> re >> im;
    z = {re, im};
  }
  return v;
}

template <class QV>
int run(QV &qv, std::istream &in, bool density) {
  std::cout << std::setprecision(17);
  qv.set_omp_threads(4);
  qv.set_omp_threshold(14);
  qv.set_json_chop_threshold(1e-10);
  qv.set_sample_measure_index_size(10);
  qv.set_max_matrix_bits(5);
  qv.set_max_sampling_shots(0);
  reg_t gpus{0};
  qv.set_target_gpus(gpus);
  qv.cuStateVec_enable(false);
  if (qv.enable_batch(true)) return 4;
  qv.chunk_setup((int)qv.num_qubits(), (int)qv.num_qubits(), 0, 1);
  qv.initialize();
  std::string op;
  bool ended = false;
  while (in >> op) {
    if (op == "end") {
      ended = true;
      break;
    }
    if (op == "matrix") {
      reg_t q = read_qubits(in);
      const size_t D = 1ULL << q.size();
      cvector_t m = read_complex(in, D * D);
      if (density)
        qv.apply_unitary_matrix(q, m);
      else
        qv.apply_matrix(q, m);
    } else if (op == "diag") {
      reg_t q = read_qubits(in);
      qv.apply_diagonal_matrix(q, read_complex(in, 1ULL << q.size()));
    } else if (op == "mcx") {
      qv.apply_mcx(read_qubits(in));
    } else if (op == "mcu") {
      reg_t q = read_qubits(in);
      qv.apply_mcu(q, read_complex(in, 4));
    } else if (op == "rotation") {
      reg_t q = read_qubits(in);
      int axis;
      double theta;
      in >> axis >> theta;
      qv.apply_rotation(q, axis, theta);
    } else if (op == "pauli") {
      reg_t q = read_qubits(in);
      std::string label;
      double re, im;
      in >> label >> re >> im;
      qv.apply_pauli(q, label, complex_t(re, im));
    } else if (op == "component") {
      reg_t q = read_qubits(in);
      qv.initialize_component(q, read_complex(in, 1ULL << q.size()));
    } else if (op == "superop") {
      reg_t q = read_qubits(in);
      const size_t D = 1ULL << (2 * q.size());
      qv.apply_superop_matrix(q, read_complex(in, D * D));
    } else if (op == "reset") {
      qv.apply_reset(read_qubits(in));
    } else if (op == "probs") {
      const auto p = qv.probabilities(read_qubits(in));
      std::cout << "probs";
      for (double x : p) std::cout << ' ' << x;
      std::cout << '\n';
    } else if (op == "expval") {
      reg_t q = read_qubits(in);
      std::string label;
      in >> label;
      std::cout << "expval " << qv.expval_pauli(q, label) << '\n';
    } else if (op == "probability") {
      uint64_t k;
      in >> k;
      std::cout << "probability " << qv.probability(k) << '\n';
    } else if (op == "norm") {
      std::cout << "norm " << qv.norm() << '\n';
    } else if (op == "normmat") {
      reg_t q = read_qubits(in);
      const size_t D = 1ULL << q.size();
      std::cout << "norm " << qv.norm(q, read_complex(in, D * D)) << '\n';
    } else if (op == "normdiag") {
      reg_t q = read_qubits(in);
      std::cout << "norm " << qv.norm_diagonal(q, read_complex(in, 1ULL << q.size())) << '\n';
    } else if (op == "ket") {
      double eps;
      in >> eps;
      std::cout << "ket";
      for (const auto &kv : qv.vector_ket(eps)) std::cout << ' ' << kv.first << ' ' << kv.second.real() << ' ' << kv.second.imag();
      std::cout << '\n';
    } else if (op == "sample") {
      size_t count;
      in >> count;
      std::vector<double> u(count);
      for (auto &x : u) in >> x;
      std::cout << "sample";
      for (auto i : qv.sample_measure(u)) std::cout << ' ' << i;
      std::cout << '\n';
    } else if (op == "state") {
      const cvector_t v = qv.copy_to_vector();
      std::cout << "state";
      for (const auto &z : v) std::cout << ' ' << z.real() << ' ' << z.imag();
      std::cout << '\n';
    } else {
      std::cerr << "unknown record " << op << '\n';
      return 2;
    }
    if (!in) {
      std::cerr << "malformed record " << op << '\n';
      return 2;
    }
  }
  if (!ended) {
    std::cerr << "input ended without \"end\"\n";
    return 2;
  }
  qv.synchronize();
  return 0;
}

}  // namespace

int main() {
  std::string kind, precision;
  size_t n;
  if (!(std::cin >> kind >> precision >> n)) return 2;
  try {
    if (kind == "dm") {
      gbqv_aer::DensityMatrix<double> dm(n);
      return run(dm, std::cin, true);
    }
    if (precision == "c64") {
      gbqv_aer::QubitVector<float> qv(n);
      return run(qv, std::cin, false);
    }
    gbqv_aer::QubitVector<double> qv(n);
    return run(qv, std::cin, false);
  } catch (const std::invalid_argument &e) {
    std::cout << "invalid_argument: " << e.what() << '\n';
    return 3;
  } catch (const std::runtime_error &e) {
    std::cout << "runtime_error: " << e.what() << '\n';
    return 3;
  }
}
