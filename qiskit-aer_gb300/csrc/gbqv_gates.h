// gbqv_gates.h — host-side gate algebra of the engine: the gate matrices of
// the reference (src/framework/linalg/matrix_utils/vmatrix_defs.hpp), Pauli
// masks (qubitvector.hpp:2235-2297) and superoperator construction
// (densitymatrix.hpp:265-281, smatrix_defs.hpp).  Matrices are column-major
// std::vector<std::complex<double>>.
#pragma once

#include <cmath>
#include <complex>
#include <cstdint>
#include <string>
#include <vector>

#include "gbqv_internal.h"

namespace gbqv {

struct PauliMasks {
  uint64_t x_mask = 0, z_mask = 0, num_y = 0, x_max = 0;
};

// pauli_masks_and_phase: label[N-1-i] acts on qubits[i].
inline PauliMasks pauli_masks(const reg_t &qubits, const char *label) {
  PauliMasks m;
  const size_t N = qubits.size();
  for (size_t i = 0; i < N; ++i) {
    const uint64_t bit = 1ULL << qubits[i];
    switch (label[N - 1 - i]) {
      case 'I': break;
      case 'X': m.x_mask += bit; m.x_max = std::max<uint64_t>(m.x_max, qubits[i]); break;
      case 'Z': m.z_mask += bit; break;
      case 'Y': m.x_mask += bit; m.x_max = std::max<uint64_t>(m.x_max, qubits[i]); m.z_mask += bit; ++m.num_y; break;
      default: throw Error(1, std::string("Invalid Pauli \"") + label[N - 1 - i] + "\".");
    }
  }
  return m;
}

// (-i)^num_y times c
inline cd add_y_phase(uint64_t num_y, cd c) {
  switch (num_y & 3) {
    case 1: return cd(c.imag(), -c.real());
    case 2: return cd(-c.real(), -c.imag());
    case 3: return cd(-c.imag(), c.real());
    default: return c;
  }
}

namespace gates {

using mat_t = std::vector<cd>;
constexpr cd I1(0.0, 1.0);

// index helper for column-major 2^k x 2^k
inline cd &at(mat_t &m, size_t dim, size_t r, size_t c) { return m[r + dim * c]; }

inline mat_t u3(double theta, double phi, double lam) {
  mat_t m(4);
  m[0] = std::cos(0.5 * theta);
  m[2] = -std::exp(I1 * lam) * std::sin(0.5 * theta);
  m[1] = std::exp(I1 * phi) * std::sin(0.5 * theta);
  m[3] = std::exp(I1 * (phi + lam)) * std::cos(0.5 * theta);
  return m;
}

inline mat_t u4(double theta, double phi, double lam, double gamma) {
  mat_t m(4);
  m[0] = std::exp(I1 * gamma) * std::cos(0.5 * theta);
  m[2] = -std::exp(I1 * (lam + gamma)) * std::sin(0.5 * theta);
  m[1] = std::exp(I1 * (phi + gamma)) * std::sin(0.5 * theta);
  m[3] = std::exp(I1 * (phi + lam + gamma)) * std::cos(0.5 * theta);
  return m;
}

inline mat_t u2(double phi, double lam) {
  mat_t m(4);
  const cd invsqrt2(1. / std::sqrt(2), 0.);
  m[0] = invsqrt2;
  m[2] = -std::exp(I1 * lam) * invsqrt2;
  m[1] = std::exp(I1 * phi) * invsqrt2;
  m[3] = std::exp(I1 * (phi + lam)) * invsqrt2;
  return m;
}

inline mat_t r(double theta, double phi) {
  mat_t m(4);
  m[0] = std::cos(0.5 * theta);
  m[2] = -I1 * std::exp(-I1 * phi) * std::sin(0.5 * theta);
  m[1] = -I1 * std::exp(I1 * phi) * std::sin(0.5 * theta);
  m[3] = std::cos(0.5 * theta);
  return m;
}

inline mat_t rx(double t) {
  mat_t m(4);
  m[0] = std::cos(0.5 * t);
  m[2] = -I1 * std::sin(0.5 * t);
  m[1] = m[2];
  m[3] = m[0];
  return m;
}

inline mat_t ry(double t) {
  mat_t m(4);
  m[0] = std::cos(0.5 * t);
  m[2] = -1.0 * std::sin(0.5 * t);
  m[1] = -m[2];
  m[3] = m[0];
  return m;
}

inline mat_t rz(double t) {
  mat_t m(4);
  m[0] = std::exp(-I1 * 0.5 * t);
  m[3] = std::exp(I1 * 0.5 * t);
  return m;
}

inline mat_t rz_diag(double t) { return {std::exp(-I1 * 0.5 * t), std::exp(I1 * 0.5 * t)}; }

inline mat_t rxx(double t) {
  mat_t m(16);
  const double c = std::cos(0.5 * t), s = std::sin(0.5 * t);
  at(m, 4, 0, 0) = c; at(m, 4, 0, 3) = -I1 * s;
  at(m, 4, 1, 1) = c; at(m, 4, 1, 2) = -I1 * s;
  at(m, 4, 2, 1) = -I1 * s; at(m, 4, 2, 2) = c;
  at(m, 4, 3, 0) = -I1 * s; at(m, 4, 3, 3) = c;
  return m;
}

inline mat_t ryy(double t) {
  mat_t m(16);
  const double c = std::cos(0.5 * t), s = std::sin(0.5 * t);
  at(m, 4, 0, 0) = c; at(m, 4, 0, 3) = I1 * s;
  at(m, 4, 1, 1) = c; at(m, 4, 1, 2) = -I1 * s;
  at(m, 4, 2, 1) = -I1 * s; at(m, 4, 2, 2) = c;
  at(m, 4, 3, 0) = I1 * s; at(m, 4, 3, 3) = c;
  return m;
}

inline mat_t rzz_diag(double t) {
  const cd ep = std::exp(I1 * 0.5 * t), em = std::exp(-I1 * 0.5 * t);
  return {em, ep, ep, em};
}

inline mat_t rzz(double t) {
  mat_t d = rzz_diag(t), m(16);
  for (int i = 0; i < 4; ++i) at(m, 4, i, i) = d[i];
  return m;
}

inline mat_t rzx(double t) {
  mat_t m(16);
  const double c = std::cos(0.5 * t), s = std::sin(0.5 * t);
  at(m, 4, 0, 0) = c; at(m, 4, 0, 2) = -I1 * s;
  at(m, 4, 1, 1) = c; at(m, 4, 1, 3) = I1 * s;
  at(m, 4, 2, 0) = -I1 * s; at(m, 4, 2, 2) = c;
  at(m, 4, 3, 1) = I1 * s; at(m, 4, 3, 3) = c;
  return m;
}

inline mat_t phase(double lam) { return {1.0, 0.0, 0.0, std::exp(I1 * lam)}; }

// Constant matrices of matrix_defs.hpp
inline mat_t X() { return {0.0, 1.0, 1.0, 0.0}; }
inline mat_t Y() { return {0.0, I1, -I1, 0.0}; }
inline mat_t Z() { return {1.0, 0.0, 0.0, -1.0}; }
inline mat_t H() { const double s = 1. / std::sqrt(2.); return {s, s, s, -s}; }
inline mat_t S() { return {1.0, 0.0, 0.0, I1}; }
inline mat_t SDG() { return {1.0, 0.0, 0.0, -I1}; }
inline mat_t T() { const double s = 1. / std::sqrt(2.); return {1.0, 0.0, 0.0, cd(s, s)}; }
inline mat_t TDG() { const double s = 1. / std::sqrt(2.); return {1.0, 0.0, 0.0, cd(s, -s)}; }
inline mat_t SX() { return {cd(0.5, 0.5), cd(0.5, -0.5), cd(0.5, -0.5), cd(0.5, 0.5)}; }
inline mat_t SXDG() { return {cd(0.5, -0.5), cd(0.5, 0.5), cd(0.5, 0.5), cd(0.5, -0.5)}; }
inline mat_t ECR() {
  // ECR = 1/sqrt(2) [[0, 1, 0, i], [1, 0, -i, 0], [0, i, 0, 1], [-i, 0, 1, 0]] (row-major)
  const double s = 1. / std::sqrt(2.);
  const cd rows[4][4] = {{0, s, 0, I1 * s}, {s, 0, -I1 * s, 0}, {0, I1 * s, 0, s}, {-I1 * s, 0, s, 0}};
  mat_t m(16);
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) at(m, 4, r, c) = rows[r][c];
  return m;
}

inline mat_t identity(size_t dim) {
  mat_t m(dim * dim);
  for (size_t i = 0; i < dim; ++i) m[i + dim * i] = 1.0;
  return m;
}

// vec(conj(U) (x) U) in the reference's layout (densitymatrix.hpp:265-281)
inline mat_t vmat2vsuperop(const cd *vmat, size_t dim) {
  mat_t ret(dim * dim * dim * dim);
  for (size_t i = 0; i < dim; ++i)
    for (size_t j = 0; j < dim; ++j)
      for (size_t k = 0; k < dim; ++k)
        for (size_t l = 0; l < dim; ++l)
          ret[dim * i + k + (dim * dim) * (dim * j + l)] = std::conj(vmat[i + dim * j]) * vmat[k + dim * l];
  return ret;
}

// SMatrix::reset(dim): |i><j| -> delta_ij |0><0| as a column-major superop.
inline mat_t reset_superop(int k) {
  const size_t dim = 1ULL << k, D = dim * dim;
  mat_t m(D * D);
  for (size_t i = 0; i < dim; ++i) m[0 + D * (i * (dim + 1))] = 1.0;
  return m;
}

}  // namespace gates
}  // namespace gbqv
