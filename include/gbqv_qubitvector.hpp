// gbqv_qubitvector.hpp — header-only C++ adapter with the member surface of
// AER::QV::QubitVector<data_t> (src/simulators/statevector/qubitvector.hpp:61-651)
// and AER::QV::DensityMatrix<data_t> (src/simulators/density_matrix/
// densitymatrix.hpp:34-171), implemented over the C ABI of libgbqv.so
// (gbqv.h).  It is the `statevec_t` / `densmat_t` an Aer build would pass to
// Statevector::State<statevec_t> / DensityMatrix::State<densmat_t>
// (statevector_state.hpp:100-101); errors surface as std::runtime_error /
// std::invalid_argument like the reference's.  Only the types Aer already
// uses appear here (std::vector, std::complex, std::string).
#pragma once

#include <complex>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "gbqv.h"

namespace gbqv_aer {

using uint_t = uint64_t;
using reg_t = std::vector<uint_t>;
using complex_t = std::complex<double>;
using cvector_t = std::vector<complex_t>;

inline void check(int rc, gbqv_handle h) {
  if (rc == GBQV_OK) return;
  const std::string msg = gbqv_last_error(h);
  if (rc == GBQV_ERR_ARG || rc == GBQV_ERR_KIND) throw std::invalid_argument(msg);
  throw std::runtime_error(msg);
}

inline const gbqv_c128 *c(const cvector_t &v) { return reinterpret_cast<const gbqv_c128 *>(v.data()); }

// data_t = double -> complex128 state, float -> complex64 state
template <typename data_t = double, int Kind = GBQV_STATEVECTOR>
class QubitVector {
 public:
  QubitVector() = default;
  explicit QubitVector(size_t num_qubits) { set_num_qubits(num_qubits); }
  QubitVector(const QubitVector &) = delete;
  QubitVector &operator=(const QubitVector &) = delete;
  QubitVector(QubitVector &&o) noexcept : h_(std::exchange(o.h_, nullptr)), n_(o.n_) {}
  ~QubitVector() { gbqv_destroy(h_); }

  static std::string name() {
    return Kind == GBQV_STATEVECTOR ? "statevector_gb300"
           : Kind == GBQV_UNITARY   ? "unitary_gb300"
                                    : "density_matrix_gb300";
  }

  // ---- utility (qubitvector.hpp:913-1110) ----
  void set_num_qubits(size_t num_qubits) {
    gbqv_destroy(h_);
    h_ = nullptr;
    check(gbqv_create((int)num_qubits, sizeof(data_t) == 8 ? GBQV_C128 : GBQV_C64, Kind, &h_), nullptr);
    n_ = num_qubits;
  }
  uint_t num_qubits() const { return n_; }
  uint_t size() const {
    int v = 0;
    check(gbqv_num_vector_qubits(h_, &v), h_);
    return 1ULL << v;
  }
  void zero() { check(gbqv_zero(h_), h_); }
  void initialize() { check(gbqv_initialize(h_), h_); }
  void initialize_from_vector(const cvector_t &vec) {
    check(gbqv_initialize_from_vector(h_, c(vec), vec.size()), h_);
  }
  cvector_t copy_to_vector() const {
    cvector_t out(size());
    check(gbqv_copy_to_host(h_, reinterpret_cast<gbqv_c128 *>(out.data()), out.size()), h_);
    return out;
  }
  cvector_t move_to_vector() { return copy_to_vector(); }
  void checkpoint() { check(gbqv_checkpoint(h_), h_); }
  void revert(bool keep) { check(gbqv_revert(h_, keep ? 1 : 0), h_); }
  complex_t inner_product() const {
    gbqv_c128 z;
    check(gbqv_inner_product(h_, &z), h_);
    return {z.re, z.im};
  }

  // ---- gates (qubitvector.hpp:1298-1871) ----
  void apply_matrix(const reg_t &q, const cvector_t &mat) { check(gbqv_apply_matrix(h_, q.data(), (int)q.size(), c(mat)), h_); }
  void apply_diagonal_matrix(const reg_t &q, const cvector_t &d) {
    check(gbqv_apply_diagonal_matrix(h_, q.data(), (int)q.size(), c(d)), h_);
  }
  void apply_mcx(const reg_t &q) { check(gbqv_apply_mcx(h_, q.data(), (int)q.size()), h_); }
  void apply_mcy(const reg_t &q) { check(gbqv_apply_mcy(h_, q.data(), (int)q.size()), h_); }
  void apply_mcswap(const reg_t &q) { check(gbqv_apply_mcswap(h_, q.data(), (int)q.size()), h_); }
  void apply_mcphase(const reg_t &q, const complex_t phase) {
    check(gbqv_apply_mcphase(h_, q.data(), (int)q.size(), gbqv_c128{phase.real(), phase.imag()}), h_);
  }
  void apply_mcu(const reg_t &q, const cvector_t &mat) { check(gbqv_apply_mcu(h_, q.data(), (int)q.size(), c(mat)), h_); }
  void apply_rotation(const reg_t &q, int axis, double theta) {
    check(gbqv_apply_rotation(h_, q.data(), (int)q.size(), axis, theta), h_);
  }
  void apply_pauli(const reg_t &q, const std::string &pauli, const complex_t &coeff = 1) {
    check(gbqv_apply_pauli(h_, q.data(), (int)q.size(), pauli.c_str(), gbqv_c128{coeff.real(), coeff.imag()}), h_);
  }
  void apply_permutation_matrix(const reg_t &q, const std::vector<std::pair<uint_t, uint_t>> &pairs) {
    std::vector<uint64_t> flat;
    for (auto &p : pairs) flat.push_back(p.first), flat.push_back(p.second);
    check(gbqv_apply_permutation_matrix(h_, q.data(), (int)q.size(), flat.data(), (int)pairs.size()), h_);
  }
  void apply_multiplexer(const reg_t &ctrl, const reg_t &tgt, const cvector_t &mat) {
    check(gbqv_apply_multiplexer(h_, ctrl.data(), (int)ctrl.size(), tgt.data(), (int)tgt.size(), c(mat)), h_);
  }
  void apply_multi_swaps(const reg_t &q) { check(gbqv_apply_multi_swaps(h_, q.data(), (int)q.size()), h_); }

  // ---- reductions (qubitvector.hpp:1878-2347) ----
  double norm() const {
    double v;
    check(gbqv_norm(h_, &v), h_);
    return v;
  }
  double norm(const reg_t &q, const cvector_t &mat) const {
    double v;
    check(gbqv_norm_matrix(h_, q.data(), (int)q.size(), c(mat), &v), h_);
    return v;
  }
  std::vector<double> probabilities() const { return probabilities(reg_t{}); }
  std::vector<double> probabilities(const reg_t &q) const {
    std::vector<double> out(1ULL << (q.empty() ? n_ : q.size()));
    check(gbqv_probabilities(h_, q.data(), (int)q.size(), out.data()), h_);
    return out;
  }
  reg_t sample_measure(const std::vector<double> &rnds) const {
    reg_t out(rnds.size());
    check(gbqv_sample_measure(h_, rnds.data(), rnds.size(), out.data()), h_);
    return out;
  }
  double expval_pauli(const reg_t &q, const std::string &pauli, const complex_t initial_phase = 1.0) const {
    double v;
    check(gbqv_expval_pauli(h_, q.data(), (int)q.size(), pauli.c_str(),
                            gbqv_c128{initial_phase.real(), initial_phase.imag()}, &v), h_);
    return v;
  }

  // ---- density matrix (densitymatrix.hpp:265-542) ----
  void apply_superop_matrix(const reg_t &q, const cvector_t &mat) {
    check(gbqv_dm_apply_superop_matrix(h_, q.data(), (int)q.size(), c(mat)), h_);
  }
  void apply_unitary_matrix(const reg_t &q, const cvector_t &mat) {
    check(gbqv_dm_apply_unitary_matrix(h_, q.data(), (int)q.size(), c(mat)), h_);
  }
  void apply_diagonal_unitary_matrix(const reg_t &q, const cvector_t &d) {
    check(gbqv_dm_apply_diagonal_unitary_matrix(h_, q.data(), (int)q.size(), c(d)), h_);
  }
  void apply_cnot(uint_t a, uint_t b) { check(gbqv_dm_apply_cnot(h_, a, b), h_); }
  void apply_swap(uint_t a, uint_t b) { check(gbqv_dm_apply_swap(h_, a, b), h_); }
  void apply_x(uint_t q) { check(gbqv_dm_apply_x(h_, q), h_); }
  void apply_y(uint_t q) { check(gbqv_dm_apply_y(h_, q), h_); }
  void apply_phase(uint_t q, const complex_t &p) { check(gbqv_dm_apply_phase(h_, q, gbqv_c128{p.real(), p.imag()}), h_); }
  void apply_cphase(uint_t a, uint_t b, const complex_t &p) {
    check(gbqv_dm_apply_cphase(h_, a, b, gbqv_c128{p.real(), p.imag()}), h_);
  }
  void apply_toffoli(uint_t a, uint_t b, uint_t t) { check(gbqv_dm_apply_toffoli(h_, a, b, t), h_); }
  void apply_reset(const reg_t &q) { check(gbqv_dm_apply_reset(h_, q.data(), (int)q.size()), h_); }

  gbqv_handle handle() const { return h_; }

 private:
  gbqv_handle h_ = nullptr;
  size_t n_ = 0;
};

template <typename data_t = double>
using DensityMatrix = QubitVector<data_t, GBQV_DENSITY_MATRIX>;

// QV::UnitaryMatrix<data_t> (unitarymatrix.hpp): the unit of the unitary
// method; the QubitVector members act on the 2n-qubit vec(U), and
// initialize() sets the identity.
template <typename data_t = double>
class UnitaryMatrix : public QubitVector<data_t, GBQV_UNITARY> {
 public:
  using QubitVector<data_t, GBQV_UNITARY>::QubitVector;
  uint_t rows() const { return 1ULL << this->num_qubits(); }
  // column-major, as Utils::vectorize_matrix
  void initialize_from_matrix(const cvector_t &mat) { this->initialize_from_vector(mat); }
  cvector_t copy_to_matrix() const { return this->copy_to_vector(); }
  cvector_t move_to_matrix() { return this->copy_to_vector(); }
};

}  // namespace gbqv_aer
