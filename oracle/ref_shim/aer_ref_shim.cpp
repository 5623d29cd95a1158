// aer_ref_shim.cpp — project-written extern "C" wrapper around the
// reference's own QV::QubitVector<double>, QV::DensityMatrix<double> and
// QV::UnitaryMatrix<double>, compiled from the qiskit-aer sources by
// oracle/Makefile into oracle/_ref/libaerref.so.  TEST INFRASTRUCTURE ONLY:
// it generates the golden fixtures under tests/golden/ and pins the C
// restatement in oracle_qv.c; nothing in the engine links it.
#include "aer_prelude.hpp"
#include "simulators/density_matrix/densitymatrix.hpp"
#include "simulators/statevector/qubitvector.hpp"
#include "simulators/unitary/unitarymatrix.hpp"

#include <cstring>

using namespace AER;
using cd = std::complex<double>;

static reg_t to_reg(const uint64_t *q, int k) { return reg_t(q, q + k); }
static cvector_t to_cvec(const cd *m, uint64_t len) { return cvector_t(m, m + len); }

extern "C" {

void *ref_qv_create(int n, int threads) {
  auto *qv = new QV::QubitVector<double>(n);
  qv->set_omp_threads(threads);
  qv->initialize();
  return qv;
}
void ref_qv_destroy(void *h) { delete static_cast<QV::QubitVector<double> *>(h); }
void ref_qv_set(void *h, const cd *vec, uint64_t len) {
  auto *qv = static_cast<QV::QubitVector<double> *>(h);
  qv->initialize_from_vector(std::vector<cd>(vec, vec + len));
}
void ref_qv_get(void *h, cd *out) {
  auto *qv = static_cast<QV::QubitVector<double> *>(h);
  std::memcpy(out, qv->data(), sizeof(cd) * qv->size());
}
void ref_qv_apply_matrix(void *h, const uint64_t *q, int k, const cd *m) {
  static_cast<QV::QubitVector<double> *>(h)->apply_matrix(to_reg(q, k), to_cvec(m, 1ULL << (2 * k)));
}
void ref_qv_apply_diagonal(void *h, const uint64_t *q, int k, const cd *d) {
  static_cast<QV::QubitVector<double> *>(h)->apply_diagonal_matrix(to_reg(q, k), to_cvec(d, 1ULL << k));
}
void ref_qv_apply_mcx(void *h, const uint64_t *q, int k) { static_cast<QV::QubitVector<double> *>(h)->apply_mcx(to_reg(q, k)); }
void ref_qv_apply_mcy(void *h, const uint64_t *q, int k) { static_cast<QV::QubitVector<double> *>(h)->apply_mcy(to_reg(q, k)); }
void ref_qv_apply_mcswap(void *h, const uint64_t *q, int k) { static_cast<QV::QubitVector<double> *>(h)->apply_mcswap(to_reg(q, k)); }
void ref_qv_apply_mcphase(void *h, const uint64_t *q, int k, double re, double im) {
  static_cast<QV::QubitVector<double> *>(h)->apply_mcphase(to_reg(q, k), cd(re, im));
}
void ref_qv_apply_mcu(void *h, const uint64_t *q, int k, const cd *m) {
  static_cast<QV::QubitVector<double> *>(h)->apply_mcu(to_reg(q, k), to_cvec(m, 4));
}
void ref_qv_apply_rotation(void *h, const uint64_t *q, int k, int axis, double theta) {
  static_cast<QV::QubitVector<double> *>(h)->apply_rotation(to_reg(q, k), static_cast<QV::Rotation>(axis), theta);
}
void ref_qv_apply_pauli(void *h, const uint64_t *q, int k, const char *label, double re, double im) {
  static_cast<QV::QubitVector<double> *>(h)->apply_pauli(to_reg(q, k), std::string(label), cd(re, im));
}
void ref_qv_apply_permutation(void *h, const uint64_t *q, int k, const uint64_t *pairs, int np) {
  std::vector<std::pair<uint_t, uint_t>> p;
  for (int i = 0; i < np; ++i) p.emplace_back(pairs[2 * i], pairs[2 * i + 1]);
  static_cast<QV::QubitVector<double> *>(h)->apply_permutation_matrix(to_reg(q, k), p);
}
void ref_qv_apply_multiplexer(void *h, const uint64_t *c, int nc, const uint64_t *t, int nt, const cd *m) {
  uint64_t rows = 1ULL << (nc + nt), cols = 1ULL << nt;
  static_cast<QV::QubitVector<double> *>(h)->apply_multiplexer(to_reg(c, nc), to_reg(t, nt), to_cvec(m, rows * cols));
}
void ref_qv_apply_multi_swaps(void *h, const uint64_t *q, int k) {
  static_cast<QV::QubitVector<double> *>(h)->apply_multi_swaps(to_reg(q, k));
}
double ref_qv_norm(void *h) { return static_cast<QV::QubitVector<double> *>(h)->norm(); }
double ref_qv_norm_matrix(void *h, const uint64_t *q, int k, const cd *m) {
  return static_cast<QV::QubitVector<double> *>(h)->norm(to_reg(q, k), to_cvec(m, 1ULL << (2 * k)));
}
double ref_qv_expval_pauli(void *h, const uint64_t *q, int k, const char *label, double re, double im) {
  return static_cast<QV::QubitVector<double> *>(h)->expval_pauli(to_reg(q, k), std::string(label), cd(re, im));
}
void ref_qv_probabilities(void *h, const uint64_t *q, int k, double *out) {
  auto *qv = static_cast<QV::QubitVector<double> *>(h);
  std::vector<double> p = k == 0 ? qv->probabilities() : qv->probabilities(to_reg(q, k));
  std::memcpy(out, p.data(), sizeof(double) * p.size());
}
void ref_qv_sample_measure(void *h, const double *rnds, uint64_t shots, uint64_t *out) {
  auto *qv = static_cast<QV::QubitVector<double> *>(h);
  reg_t s = qv->sample_measure(std::vector<double>(rnds, rnds + shots));
  for (uint64_t i = 0; i < shots; ++i) out[i] = s[i];
}
void ref_qv_set_sample_index_size(void *h, int n) {
  static_cast<QV::QubitVector<double> *>(h)->set_sample_measure_index_size(n);
}
void ref_dm_set_sample_index_size(void *h, int n) {
  static_cast<QV::DensityMatrix<double> *>(h)->set_sample_measure_index_size(n);
}
void ref_qv_checkpoint(void *h) { static_cast<QV::QubitVector<double> *>(h)->checkpoint(); }
void ref_qv_inner_product(void *h, double *re, double *im) {
  cd z = static_cast<QV::QubitVector<double> *>(h)->inner_product();
  *re = z.real(); *im = z.imag();
}

// ---- density matrix ----
void *ref_dm_create(int n, int threads) {
  auto *dm = new QV::DensityMatrix<double>(n);
  dm->set_omp_threads(threads);
  dm->initialize();
  return dm;
}
void ref_dm_destroy(void *h) { delete static_cast<QV::DensityMatrix<double> *>(h); }
void ref_dm_set(void *h, const cd *vec, uint64_t len) {
  auto *dm = static_cast<QV::DensityMatrix<double> *>(h);
  dm->initialize_from_vector(std::vector<cd>(vec, vec + len));
}
void ref_dm_get(void *h, cd *out) {
  auto *dm = static_cast<QV::DensityMatrix<double> *>(h);
  std::memcpy(out, dm->data(), sizeof(cd) * dm->size());
}
void ref_dm_apply_superop(void *h, const uint64_t *q, int k, const cd *m) {
  static_cast<QV::DensityMatrix<double> *>(h)->apply_superop_matrix(to_reg(q, k), to_cvec(m, 1ULL << (4 * k)));
}
void ref_dm_apply_unitary(void *h, const uint64_t *q, int k, const cd *m) {
  static_cast<QV::DensityMatrix<double> *>(h)->apply_unitary_matrix(to_reg(q, k), to_cvec(m, 1ULL << (2 * k)));
}
void ref_dm_apply_diagonal_unitary(void *h, const uint64_t *q, int k, const cd *d) {
  static_cast<QV::DensityMatrix<double> *>(h)->apply_diagonal_unitary_matrix(to_reg(q, k), to_cvec(d, 1ULL << k));
}
void ref_dm_apply_cnot(void *h, uint64_t c, uint64_t t) { static_cast<QV::DensityMatrix<double> *>(h)->apply_cnot(c, t); }
void ref_dm_apply_swap(void *h, uint64_t a, uint64_t b) { static_cast<QV::DensityMatrix<double> *>(h)->apply_swap(a, b); }
void ref_dm_apply_x(void *h, uint64_t q) { static_cast<QV::DensityMatrix<double> *>(h)->apply_x(q); }
void ref_dm_apply_y(void *h, uint64_t q) { static_cast<QV::DensityMatrix<double> *>(h)->apply_y(q); }
void ref_dm_apply_phase(void *h, uint64_t q, double re, double im) {
  static_cast<QV::DensityMatrix<double> *>(h)->apply_phase(q, cd(re, im));
}
void ref_dm_apply_cphase(void *h, uint64_t a, uint64_t b, double re, double im) {
  static_cast<QV::DensityMatrix<double> *>(h)->apply_cphase(a, b, cd(re, im));
}
void ref_dm_apply_toffoli(void *h, uint64_t a, uint64_t b, uint64_t c) {
  static_cast<QV::DensityMatrix<double> *>(h)->apply_toffoli(a, b, c);
}
void ref_dm_apply_reset(void *h, const uint64_t *q, int k) {
  static_cast<QV::DensityMatrix<double> *>(h)->apply_reset(to_reg(q, k));
}
double ref_dm_expval_pauli(void *h, const uint64_t *q, int k, const char *label) {
  return static_cast<QV::DensityMatrix<double> *>(h)->expval_pauli(to_reg(q, k), std::string(label));
}
void ref_dm_probabilities(void *h, const uint64_t *q, int k, double *out) {
  auto *dm = static_cast<QV::DensityMatrix<double> *>(h);
  std::vector<double> p = k == 0 ? dm->probabilities() : dm->probabilities(to_reg(q, k));
  std::memcpy(out, p.data(), sizeof(double) * p.size());
}
void ref_dm_sample_measure(void *h, const double *rnds, uint64_t shots, uint64_t *out) {
  auto *dm = static_cast<QV::DensityMatrix<double> *>(h);
  reg_t s = dm->sample_measure(std::vector<double>(rnds, rnds + shots));
  for (uint64_t i = 0; i < shots; ++i) out[i] = s[i];
}

// ---- unitary (the fused-matrix builder of Fusion, fusion.hpp:159-174) ----
void *ref_um_create(int n) {
  auto *um = new QV::UnitaryMatrix<double>(n);
  um->initialize();
  return um;
}
void ref_um_destroy(void *h) { delete static_cast<QV::UnitaryMatrix<double> *>(h); }
void ref_um_apply_matrix(void *h, const uint64_t *q, int k, const cd *m) {
  static_cast<QV::UnitaryMatrix<double> *>(h)->apply_matrix(to_reg(q, k), to_cvec(m, 1ULL << (2 * k)));
}
void ref_um_apply_diagonal(void *h, const uint64_t *q, int k, const cd *d) {
  static_cast<QV::UnitaryMatrix<double> *>(h)->apply_diagonal_matrix(to_reg(q, k), to_cvec(d, 1ULL << k));
}
void ref_um_apply_mcx(void *h, const uint64_t *q, int k) { static_cast<QV::UnitaryMatrix<double> *>(h)->apply_mcx(to_reg(q, k)); }
void ref_um_apply_mcphase(void *h, const uint64_t *q, int k, double re, double im) {
  static_cast<QV::UnitaryMatrix<double> *>(h)->apply_mcphase(to_reg(q, k), cd(re, im));
}
void ref_um_apply_mcu(void *h, const uint64_t *q, int k, const cd *m) {
  static_cast<QV::UnitaryMatrix<double> *>(h)->apply_mcu(to_reg(q, k), to_cvec(m, 4));
}
void ref_um_get(void *h, cd *out) {
  auto *um = static_cast<QV::UnitaryMatrix<double> *>(h);
  std::memcpy(out, um->data(), sizeof(cd) * um->size());
}

// ---- VMatrix gate definitions (vmatrix_defs.hpp) ----
void ref_vmat_u3(double t, double p, double l, cd *out) { auto m = Linalg::VMatrix::u3(t, p, l); std::copy(m.begin(), m.end(), out); }
void ref_vmat_u4(double t, double p, double l, double g, cd *out) { auto m = Linalg::VMatrix::u4(t, p, l, g); std::copy(m.begin(), m.end(), out); }
void ref_vmat_rotation(int which, double t, cd *out) {
  cvector_t m;
  switch (which) {
    case 0: m = Linalg::VMatrix::rx(t); break;
    case 1: m = Linalg::VMatrix::ry(t); break;
    case 2: m = Linalg::VMatrix::rz(t); break;
    case 3: m = Linalg::VMatrix::rxx(t); break;
    case 4: m = Linalg::VMatrix::ryy(t); break;
    case 5: m = Linalg::VMatrix::rzz(t); break;
    case 6: m = Linalg::VMatrix::rzx(t); break;
    default: return;
  }
  std::copy(m.begin(), m.end(), out);
}
}  // extern "C"

// ---- RngEngine uniforms (src/framework/rng.hpp:65-67,96) ----
#include "framework/rng.hpp"
extern "C" void ref_uniforms(uint64_t seed, uint64_t count, double *out) {
  AER::RngEngine rng;
  rng.set_seed(seed);
  for (uint64_t i = 0; i < count; ++i) out[i] = rng.rand(0, 1);
}
