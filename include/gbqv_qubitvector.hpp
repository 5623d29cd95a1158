// gbqv_qubitvector.hpp — header-only C++ adapter with the member surface of
// AER::QV::QubitVector<data_t> (src/simulators/statevector/qubitvector.hpp:61-651)
// and AER::QV::DensityMatrix<data_t> (src/simulators/density_matrix/
// densitymatrix.hpp:34-171), implemented over the C ABI of libgbqv.so
// (gbqv.h).  It is the `statevec_t` / `densmat_t` an Aer build would pass to
// Statevector::State<statevec_t> / DensityMatrix::State<densmat_t>
// (statevector_state.hpp:100-101); errors surface as std::runtime_error /
// std::invalid_argument like the reference's.  Only the types Aer already
// uses appear here (std::vector, std::complex, std::string, std::map);
// members whose arguments are Aer's own types (Operations::Op, RngEngine,
// AER::Vector) are templates, so the header compiles on its own and accepts
// Aer's types unchanged.
//
// Besides the gates and reductions, the class carries every configuration
// and chunk hook that the States and executors call on their register
// (qubitvector.hpp:100-170, 420-462; qubitvector_thrust.hpp:57-560).  The
// engine is one state on one GPU: OpenMP, chunk and batching knobs are kept
// and reported back (the CPU QubitVector also ignores most of them), a
// multi-chunk set-up is refused, and batched-shot hooks report "no batch"
// (enable_batch() is false), so Aer's executors take their per-state path;
// batched work goes through gbqv_execute_bound / gbqv_execute_segments.
#pragma once

#include <complex>
#include <cstdint>
#include <cstdio>
#include <map>
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
  QubitVector(QubitVector &&o) noexcept
      : h_(std::exchange(o.h_, nullptr)), n_(o.n_), omp_threads_(o.omp_threads_), omp_threshold_(o.omp_threshold_),
        chunk_index_(o.chunk_index_), json_chop_threshold_(o.json_chop_threshold_),
        sample_index_size_(o.sample_index_size_), max_matrix_bits_(o.max_matrix_bits_),
        max_sampling_shots_(o.max_sampling_shots_), target_gpus_(std::move(o.target_gpus_)) {}
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

  // QubitVector::probability(outcome) (qubitvector.hpp:302); DensityMatrix:
  // the diagonal entry (densitymatrix.hpp:530-534)
  double probability(uint_t outcome) const {
    double v;
    check(gbqv_probability(h_, outcome, &v), h_);
    return v;
  }
  // QubitVector::norm_diagonal (qubitvector.hpp:388-393): ||D psi||^2
  double norm_diagonal(uint_t qubit, const cvector_t &diag) const { return norm_diagonal(reg_t{qubit}, diag); }
  double norm_diagonal(const reg_t &q, const cvector_t &diag) const {
    const size_t D = 1ULL << q.size();
    if (diag.size() != D) throw std::invalid_argument("norm_diagonal: diagonal length must be 2^k");
    cvector_t mat(D * D, 0.0);
    for (size_t j = 0; j < D; ++j) mat[j + D * j] = diag[j];
    return norm(q, mat);
  }

  // ---- state set-up (qubitvector.hpp:143-145, 195-206, 856-899) ----
  // initialize_component: the qubits were reset to |0>; amplitude j of each
  // group becomes state[j] times the group's |0> amplitude, i.e. the matrix
  // whose first column is `state` and whose other columns are zero.
  void initialize_component(const reg_t &q, const cvector_t &state) {
    const size_t D = 1ULL << q.size();
    if (state.size() != D) throw std::invalid_argument("initialize_component: state length must be 2^k");
    cvector_t mat(D * D, 0.0);
    for (size_t j = 0; j < D; ++j) mat[j] = state[j];
    apply_matrix(q, mat);
  }
  template <typename T>
  void initialize_from_data(const std::complex<T> *data, size_t num_states) {
    if (num_states != size()) throw std::runtime_error("initialize_from_data: length does not match the state");
    cvector_t v(data, data + num_states);
    initialize_from_vector(v);
  }
  // AER::Vector (data(), size()) or std::vector of std::complex<T>, consumed
  template <class Vec>
  void move_from_vector(Vec &&vec) { initialize_from_data(vec.data(), vec.size()); }
  cvector_t vector() const { return copy_to_vector(); }
  // Utils::vec2ket(data, size, epsilon, 16): entries whose chopped magnitude
  // exceeds epsilon, keyed by the basis index in "0x" lowercase hex
  std::map<std::string, complex_t> vector_ket(double epsilon = 0) const {
    const cvector_t v = copy_to_vector();
    std::map<std::string, complex_t> out;
    auto chop = [epsilon](double x) { return std::abs(x) < epsilon ? 0.0 : x; };
    for (size_t k = 0; k < v.size(); ++k) {
      const complex_t z{chop(v[k].real()), chop(v[k].imag())};
      if (std::abs(z) > epsilon) {
        char key[24];
        std::snprintf(key, sizeof key, "0x%llx", (unsigned long long)k);
        out.emplace(key, z);
      }
    }
    return out;
  }
  // Statevector::State::required_memory_mb (qubitvector.hpp:110): the state
  // itself; per-handle scratch grows on demand
  size_t required_memory_mb(uint_t num_qubits) const {
    const uint_t vq = Kind == GBQV_STATEVECTOR ? num_qubits : 2 * num_qubits;
    return (size_t)((sizeof(std::complex<data_t>) << vq) >> 20);
  }
  void synchronize() { check(gbqv_synchronize(h_), h_); }

  // ---- configuration hooks (qubitvector.hpp:147-170, 420-462) ----
  void set_omp_threads(int n) {
    if (n > 0) omp_threads_ = (uint_t)n;
  }
  uint_t get_omp_threads() { return omp_threads_; }
  void set_omp_threshold(int n) {
    if (n > 0) omp_threshold_ = (uint_t)n;
  }
  uint_t get_omp_threshold() { return omp_threshold_; }
  void set_json_chop_threshold(double t) { json_chop_threshold_ = t; }
  double get_json_chop_threshold() { return json_chop_threshold_; }
  void set_sample_measure_index_size(int n) {
    check(gbqv_set_sample_measure_index_size(h_, n), h_);
    sample_index_size_ = n;
  }
  int get_sample_measure_index_size() { return sample_index_size_; }
  void set_max_matrix_bits(int64_t bits) { max_matrix_bits_ = bits; }
  void set_max_sampling_shots(int64_t shots) { max_sampling_shots_ = shots; }
  void set_num_threads_per_group(int) {}
  // cuStateVec is not used by this engine (qubitvector_thrust.hpp:90)
  void cuStateVec_enable(bool flg) {
    if (flg) throw std::invalid_argument("cuStateVec is not available in the GB300 engine");
  }
  // the engine runs on the current CUDA device; the list is kept
  void set_target_gpus(reg_t &t) { target_gpus_ = t; }
  const reg_t &target_gpus() const { return target_gpus_; }

  // ---- chunk and batch hooks (qubitvector.hpp:147-170, 322-362) ----
  uint_t chunk_setup(int chunk_bits, int num_qubits, uint_t chunk_index, uint_t num_local_chunks) {
    if (chunk_bits != num_qubits)
      throw std::runtime_error("the GB300 engine holds the whole state on one GPU: no multi-chunk set-up");
    chunk_index_ = chunk_index;
    return num_local_chunks;
  }
  uint_t chunk_setup(QubitVector &, const uint_t chunk_index) {
    chunk_index_ = chunk_index;
    return 0;
  }
  uint_t chunk_index() { return chunk_index_; }
  bool top_of_group() { return true; }
  bool fetch_chunk() const { return true; }
  void release_chunk(bool = true) const {}
  void enter_register_blocking(const reg_t &) {}
  void leave_register_blocking() {}
  bool support_global_indexing() { return false; }
  bool enable_batch(bool) const { return false; }
  bool batched_optimization_supported() { return false; }
  template <class... Args>
  void initialize_creg(Args &&...) {}
  template <class Op>
  void apply_bfunc(const Op &) {}
  void set_conditional(int64_t) {}
  template <class Op, class Rngs>
  void apply_roerror(const Op &, Rngs &) {}

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
  uint_t omp_threads_ = 1, omp_threshold_ = 14, chunk_index_ = 0;
  double json_chop_threshold_ = 0;
  int sample_index_size_ = 10;
  int64_t max_matrix_bits_ = 0, max_sampling_shots_ = 0;
  reg_t target_gpus_;
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
