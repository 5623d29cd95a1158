/*
 * oracle_qv.c — TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement, in plain C99 + OpenMP, of the algorithms Qiskit Aer's
 * CPU simulators run for the statevector / density-matrix hot path.  It is
 * the checker that the CUDA engine is compared against and the CPU baseline
 * that bench.py times; the engine never calls it.  Only tests/,
 * __graft_entry__.smoke() and bench.py (cpu_baseline / --impl reference)
 * load it.
 *
 * Pinning: tests/test_oracle_golden.py checks every function here against
 * fixtures written by tests/golden/gen_golden.py from the reference's own
 * QubitVector<double> / DensityMatrix<double> compiled from its sources
 * (oracle/Makefile target _ref).
 *
 * Every function cites the reference member it restates (paths relative to
 * the qiskit-aer source tree).  Layout conventions: amplitude index bit q is
 * qubit q; matrices are column-major mat[row + DIM*col] with qubits[0] the
 * least-significant bit of the matrix index (src/simulators/statevector/
 * transformer.hpp:157-159, indexes.hpp:223-235).
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef double complex cplx;

static int g_threads = 1;
static int g_omp_threshold = 14; /* QubitVector omp_threshold_ (config.hpp:107) */

void orc_set_threads(int threads, int omp_threshold) {
  g_threads = threads > 0 ? threads : 1;
  g_omp_threshold = omp_threshold;
}

#define OMP_IF(n) if ((n) > g_omp_threshold && g_threads > 1) num_threads(g_threads)

/* index0: insert a zero bit at every sorted qubit position
 * (indexes.hpp:212-222). */
static inline uint64_t index0(const uint64_t *qs_sorted, int k, uint64_t i) {
  for (int j = 0; j < k; ++j) {
    const uint64_t lowbits = i & ((1ULL << qs_sorted[j]) - 1);
    i >>= qs_sorted[j];
    i <<= qs_sorted[j] + 1;
    i |= lowbits;
  }
  return i;
}

/* indexes: all 2^k indices of group i, bit j of the local index being
 * qubits[j] (indexes.hpp:237-258). */
static inline void indexes(const uint64_t *qs, const uint64_t *qs_sorted, int k, uint64_t i,
                           uint64_t *inds) {
  inds[0] = index0(qs_sorted, k, i);
  for (int j = 0; j < k; ++j) {
    const uint64_t n = 1ULL << j;
    const uint64_t bit = 1ULL << qs[j];
    for (uint64_t m = 0; m < n; ++m) inds[n + m] = inds[m] | bit;
  }
}

static void sort_qubits(const uint64_t *qs, int k, uint64_t *out) {
  memcpy(out, qs, sizeof(uint64_t) * k);
  for (int a = 1; a < k; ++a) {
    uint64_t v = out[a];
    int b = a - 1;
    while (b >= 0 && out[b] > v) { out[b + 1] = out[b]; --b; }
    out[b + 1] = v;
  }
}

/* Dense k-qubit matrix: Transformer::apply_matrix_n (transformer.hpp:151-171)
 * and apply_matrix_1 with its diagonal / anti-diagonal special cases
 * (transformer.hpp:173-232). */
static void apply_diag1(cplx *sv, int n, uint64_t q, const cplx *d);

void orc_apply_matrix(cplx *sv, int n, const uint64_t *qubits, int k, const cplx *mat) {
  const uint64_t DIM = 1ULL << k;
  const int64_t END = (int64_t)(1ULL << (n - k));
  uint64_t qs[64];
  sort_qubits(qubits, k, qs);
  if (k == 1) {
    const uint64_t q = qubits[0];
    if (mat[1] == 0.0 && mat[2] == 0.0) {
      cplx d[2] = {mat[0], mat[3]};
      apply_diag1(sv, n, q, d);
      return;
    }
    const uint64_t bit = 1ULL << q;
    if (mat[0] == 0.0 && mat[3] == 0.0) {
      if (mat[1] == 1.0 && mat[2] == 1.0) {
#pragma omp parallel for OMP_IF(n)
        for (int64_t i = 0; i < END; ++i) {
          uint64_t i0 = index0(qs, 1, i);
          cplx t = sv[i0]; sv[i0] = sv[i0 | bit]; sv[i0 | bit] = t;
        }
        return;
      }
      if (mat[2] == 0.0) {
#pragma omp parallel for OMP_IF(n)
        for (int64_t i = 0; i < END; ++i) {
          uint64_t i0 = index0(qs, 1, i);
          sv[i0 | bit] = mat[1] * sv[i0]; sv[i0] = 0.0;
        }
        return;
      }
      if (mat[1] == 0.0) {
#pragma omp parallel for OMP_IF(n)
        for (int64_t i = 0; i < END; ++i) {
          uint64_t i0 = index0(qs, 1, i);
          sv[i0] = mat[2] * sv[i0 | bit]; sv[i0 | bit] = 0.0;
        }
        return;
      }
#pragma omp parallel for OMP_IF(n)
      for (int64_t i = 0; i < END; ++i) {
        uint64_t i0 = index0(qs, 1, i);
        cplx c = sv[i0];
        sv[i0] = mat[2] * sv[i0 | bit]; sv[i0 | bit] = mat[1] * c;
      }
      return;
    }
#pragma omp parallel for OMP_IF(n)
    for (int64_t i = 0; i < END; ++i) {
      uint64_t i0 = index0(qs, 1, i);
      cplx c = sv[i0];
      sv[i0] = mat[0] * c + mat[2] * sv[i0 | bit];
      sv[i0 | bit] = mat[1] * c + mat[3] * sv[i0 | bit];
    }
    return;
  }
  /* per-thread index and cache tables of DIM entries (k <= 13) */
#pragma omp parallel OMP_IF(n)
  {
    uint64_t *inds = (uint64_t *)malloc(sizeof(uint64_t) * DIM);
    cplx *cache = (cplx *)malloc(sizeof(cplx) * DIM);
#pragma omp for
    for (int64_t i = 0; i < END; ++i) {
      indexes(qubits, qs, k, i, inds);
      for (uint64_t a = 0; a < DIM; ++a) { cache[a] = sv[inds[a]]; sv[inds[a]] = 0.0; }
      for (uint64_t a = 0; a < DIM; ++a)
        for (uint64_t b = 0; b < DIM; ++b) sv[inds[a]] += mat[a + DIM * b] * cache[b];
    }
    free(cache);
    free(inds);
  }
}

/* Transformer::apply_diagonal_matrix_1 (transformer.hpp:260-340). */
static void apply_diag1(cplx *sv, int n, uint64_t q, const cplx *d) {
  const int64_t END = (int64_t)(1ULL << (n - 1));
  const uint64_t bit = 1ULL << q;
  uint64_t qs[1] = {q};
  if (d[0] == 1.0) {
    if (d[1] == 1.0) return;
    if (d[1] == -I) {
#pragma omp parallel for OMP_IF(n)
      for (int64_t i = 0; i < END; ++i) {
        uint64_t k1 = index0(qs, 1, i) | bit;
        double c = cimag(sv[k1]);
        sv[k1] = CMPLX(c, creal(sv[k1]) * -1.);
      }
      return;
    }
    if (d[1] == I) {
#pragma omp parallel for OMP_IF(n)
      for (int64_t i = 0; i < END; ++i) {
        uint64_t k1 = index0(qs, 1, i) | bit;
        double c = cimag(sv[k1]);
        sv[k1] = CMPLX(c * -1., creal(sv[k1]));
      }
      return;
    }
    if (d[1] == 0.0) {
#pragma omp parallel for OMP_IF(n)
      for (int64_t i = 0; i < END; ++i) sv[index0(qs, 1, i) | bit] = 0.0;
      return;
    }
#pragma omp parallel for OMP_IF(n)
    for (int64_t i = 0; i < END; ++i) {
      uint64_t k1 = index0(qs, 1, i) | bit;
      sv[k1] *= d[1];
    }
    return;
  }
  if (d[1] == 1.0) {
    if (d[0] == 0.0) {
#pragma omp parallel for OMP_IF(n)
      for (int64_t i = 0; i < END; ++i) sv[index0(qs, 1, i)] = 0.0;
      return;
    }
#pragma omp parallel for OMP_IF(n)
    for (int64_t i = 0; i < END; ++i) sv[index0(qs, 1, i)] *= d[0];
    return;
  }
#pragma omp parallel for OMP_IF(n)
  for (int64_t i = 0; i < END; ++i) {
    uint64_t k0 = index0(qs, 1, i);
    sv[k0] *= d[0];
    sv[k0 | bit] *= d[1];
  }
}

/* Transformer::apply_diagonal_matrix (transformer.hpp:234-258): the entry is
 * picked by the bits of each index at the listed qubits; entries equal to 1
 * are skipped. */
void orc_apply_diagonal(cplx *sv, int n, const uint64_t *qubits, int k, const cplx *diag) {
  if (k == 1) { apply_diag1(sv, n, qubits[0], diag); return; }
  const int64_t END = (int64_t)(1ULL << n);
#pragma omp parallel for OMP_IF(n)
  for (int64_t i = 0; i < END; ++i) {
    uint64_t iv = 0;
    for (int j = 0; j < k; ++j)
      if ((uint64_t)i & (1ULL << qubits[j])) iv |= 1ULL << j;
    if (diag[iv] != 1.0) sv[i] *= diag[iv];
  }
}

/* Multi-controlled gates (qubitvector.hpp:1446-1612): the last qubit is the
 * target, pos0 = MASKS[N-1], pos1 = MASKS[N]. */
static void mc_pair(cplx *sv, int n, const uint64_t *qubits, int N, uint64_t *p0, uint64_t *p1,
                    uint64_t *base_qs) {
  (void)sv; (void)n;
  sort_qubits(qubits, N, base_qs);
  uint64_t ctrl = 0;
  for (int j = 0; j < N - 1; ++j) ctrl |= 1ULL << qubits[j];
  *p0 = ctrl;
  *p1 = ctrl | (1ULL << qubits[N - 1]);
}

void orc_apply_mcx(cplx *sv, int n, const uint64_t *qubits, int N) {
  uint64_t qs[64], p0, p1;
  mc_pair(sv, n, qubits, N, &p0, &p1, qs);
  const int64_t END = (int64_t)(1ULL << (n - N));
#pragma omp parallel for OMP_IF(n)
  for (int64_t i = 0; i < END; ++i) {
    uint64_t b = index0(qs, N, i);
    cplx t = sv[b | p0]; sv[b | p0] = sv[b | p1]; sv[b | p1] = t;
  }
}

void orc_apply_mcy(cplx *sv, int n, const uint64_t *qubits, int N) {
  uint64_t qs[64], p0, p1;
  mc_pair(sv, n, qubits, N, &p0, &p1, qs);
  const int64_t END = (int64_t)(1ULL << (n - N));
#pragma omp parallel for OMP_IF(n)
  for (int64_t i = 0; i < END; ++i) {
    uint64_t b = index0(qs, N, i);
    cplx c = sv[b | p0];
    sv[b | p0] = -I * sv[b | p1];
    sv[b | p1] = I * c;
  }
}

/* apply_mcswap: swaps pos0 = MASKS[N-1] and pos1 = pos0 + BITS[N-2]
 * (qubitvector.hpp:1539-1573). */
void orc_apply_mcswap(cplx *sv, int n, const uint64_t *qubits, int N) {
  uint64_t qs[64];
  sort_qubits(qubits, N, qs);
  uint64_t ctrl = 0;
  for (int j = 0; j < N - 2; ++j) ctrl |= 1ULL << qubits[j];
  const uint64_t p0 = ctrl | (1ULL << qubits[N - 2]);
  const uint64_t p1 = ctrl | (1ULL << qubits[N - 1]);
  const int64_t END = (int64_t)(1ULL << (n - N));
#pragma omp parallel for OMP_IF(n)
  for (int64_t i = 0; i < END; ++i) {
    uint64_t b = index0(qs, N, i);
    cplx t = sv[b | p0]; sv[b | p0] = sv[b | p1]; sv[b | p1] = t;
  }
}

void orc_apply_mcphase(cplx *sv, int n, const uint64_t *qubits, int N, cplx phase) {
  uint64_t qs[64], p0, p1;
  mc_pair(sv, n, qubits, N, &p0, &p1, qs);
  const int64_t END = (int64_t)(1ULL << (n - N));
#pragma omp parallel for OMP_IF(n)
  for (int64_t i = 0; i < END; ++i) sv[index0(qs, N, i) | p1] *= phase;
}

/* apply_mcu (qubitvector.hpp:1614-1720): diagonal and phase short cuts,
 * N == 1 falls back to the dense / diagonal single-qubit paths. */
void orc_apply_mcu(cplx *sv, int n, const uint64_t *qubits, int N, const cplx *mat) {
  if (mat[1] == 0.0 && mat[2] == 0.0) {
    if (mat[0] == 1.0) { orc_apply_mcphase(sv, n, qubits, N, mat[3]); return; }
    cplx d[2] = {mat[0], mat[3]};
    if (N == 1) { orc_apply_diagonal(sv, n, qubits, 1, d); return; }
    uint64_t qs[64], p0, p1;
    mc_pair(sv, n, qubits, N, &p0, &p1, qs);
    const int64_t END = (int64_t)(1ULL << (n - N));
#pragma omp parallel for OMP_IF(n)
    for (int64_t i = 0; i < END; ++i) {
      uint64_t b = index0(qs, N, i);
      sv[b | p0] = d[0] * sv[b | p0];
      sv[b | p1] = d[1] * sv[b | p1];
    }
    return;
  }
  if (N == 1) { orc_apply_matrix(sv, n, qubits, 1, mat); return; }
  uint64_t qs[64], p0, p1;
  mc_pair(sv, n, qubits, N, &p0, &p1, qs);
  const int64_t END = (int64_t)(1ULL << (n - N));
#pragma omp parallel for OMP_IF(n)
  for (int64_t i = 0; i < END; ++i) {
    uint64_t b = index0(qs, N, i);
    cplx c = sv[b | p0];
    sv[b | p0] = mat[0] * sv[b | p0] + mat[2] * sv[b | p1];
    sv[b | p1] = mat[1] * c + mat[3] * sv[b | p1];
  }
}

/* apply_permutation_matrix (qubitvector.hpp:1349-1434). */
void orc_apply_permutation(cplx *sv, int n, const uint64_t *qubits, int k, const uint64_t *pairs,
                           int npairs) {
  uint64_t qs[64];
  sort_qubits(qubits, k, qs);
  const int64_t END = (int64_t)(1ULL << (n - k));
#pragma omp parallel for OMP_IF(n)
  for (int64_t i = 0; i < END; ++i) {
    uint64_t inds[1024];
    indexes(qubits, qs, k, i, inds);
    for (int p = 0; p < npairs; ++p) {
      cplx t = sv[inds[pairs[2 * p]]];
      sv[inds[pairs[2 * p]]] = sv[inds[pairs[2 * p + 1]]];
      sv[inds[pairs[2 * p + 1]]] = t;
    }
  }
}

/* apply_multiplexer (qubitvector.hpp:1305-1340): targets then controls form
 * the index; block b of the stacked matrix acts when the controls read b. */
void orc_apply_multiplexer(cplx *sv, int n, const uint64_t *controls, int nc, const uint64_t *targets,
                           int nt, const cplx *mat) {
  uint64_t qubits[64], qs[64];
  for (int j = 0; j < nt; ++j) qubits[j] = targets[j];
  for (int j = 0; j < nc; ++j) qubits[nt + j] = controls[j];
  const int k = nt + nc;
  sort_qubits(qubits, k, qs);
  const uint64_t DIM = 1ULL << k, columns = 1ULL << nt, blocks = 1ULL << nc;
  const int64_t END = (int64_t)(1ULL << (n - k));
#pragma omp parallel for OMP_IF(n)
  for (int64_t i = 0; i < END; ++i) {
    uint64_t inds[1024];
    cplx cache[1024];
    indexes(qubits, qs, k, i, inds);
    for (uint64_t a = 0; a < DIM; ++a) { cache[a] = sv[inds[a]]; sv[inds[a]] = 0.0; }
    for (uint64_t b = 0; b < blocks; ++b)
      for (uint64_t r = 0; r < columns; ++r)
        for (uint64_t c = 0; c < columns; ++c)
          sv[inds[r + b * columns]] += mat[r + b * columns + DIM * c] * cache[b * columns + c];
  }
}

/* apply_multi_swaps (qubitvector.hpp:1842-1871). */
void orc_apply_multi_swaps(cplx *sv, int n, const uint64_t *qubits, int nq) {
  for (int i0 = 0; i0 < nq; i0 += 10) {
    int m = nq - i0 < 10 ? nq - i0 : 10;
    const uint64_t *q = qubits + i0;
    uint64_t qs[64];
    sort_qubits(q, m, qs);
    const uint64_t size = 1ULL << m;
    const int64_t END = (int64_t)(1ULL << (n - m));
#pragma omp parallel for OMP_IF(n)
    for (int64_t i = 0; i < END; ++i) {
      uint64_t inds[1024];
      cplx cache[1024];
      indexes(q, qs, m, i, inds);
      for (uint64_t a = 0; a < size; ++a) cache[a] = sv[inds[a]];
      for (uint64_t a = 0; a < size; ++a) {
        uint64_t pos = a;
        for (int j = 0; j < m; j += 2)
          if ((((pos >> j) & 1) ^ ((pos >> (j + 1)) & 1)) != 0) pos ^= (1ULL << j) | (1ULL << (j + 1));
        sv[inds[a]] = cache[pos];
      }
    }
  }
}

/* pauli_masks_and_phase (qubitvector.hpp:2235-2272); returns -1 on a bad
 * letter. */
static int pauli_masks(const uint64_t *qubits, int N, const char *pauli, uint64_t *x_mask,
                       uint64_t *z_mask, uint64_t *num_y, uint64_t *x_max) {
  *x_mask = *z_mask = *num_y = *x_max = 0;
  for (int i = 0; i < N; ++i) {
    const uint64_t bit = 1ULL << qubits[i];
    switch (pauli[N - 1 - i]) {
      case 'I': break;
      case 'X': *x_mask += bit; if (qubits[i] > *x_max) *x_max = qubits[i]; break;
      case 'Z': *z_mask += bit; break;
      case 'Y': *x_mask += bit; if (qubits[i] > *x_max) *x_max = qubits[i]; *z_mask += bit; ++*num_y; break;
      default: return -1;
    }
  }
  return 0;
}

/* add_y_phase: multiply by (-i)^num_y (qubitvector.hpp:2274-2297). */
static cplx add_y_phase(uint64_t num_y, cplx c) {
  switch (num_y & 3) {
    case 1: return CMPLX(cimag(c), -creal(c));
    case 2: return CMPLX(-creal(c), -cimag(c));
    case 3: return CMPLX(-cimag(c), creal(c));
    default: return c;
  }
}

static inline int parity(uint64_t v) { return __builtin_popcountll(v) & 1; }

/* QubitVector::norm (qubitvector.hpp:1878-1886). */
double orc_norm(const cplx *sv, int n) {
  const int64_t END = (int64_t)(1ULL << n);
  double acc = 0.0;
#pragma omp parallel for reduction(+ : acc) OMP_IF(n)
  for (int64_t i = 0; i < END; ++i) acc += creal(sv[i] * conj(sv[i]));
  return acc;
}

/* QubitVector::expval_pauli (qubitvector.hpp:2299-2347). */
int orc_expval_pauli(const cplx *sv, int n, const uint64_t *qubits, int N, const char *pauli,
                     cplx initial_phase, double *out) {
  uint64_t x_mask, z_mask, num_y, x_max;
  if (pauli_masks(qubits, N, pauli, &x_mask, &z_mask, &num_y, &x_max)) return -1;
  if (x_mask + z_mask == 0) { *out = orc_norm(sv, n); return 0; }
  const cplx phase = add_y_phase(num_y, initial_phase);
  double acc = 0.0;
  if (!x_mask) {
    const int64_t END = (int64_t)(1ULL << n);
#pragma omp parallel for reduction(+ : acc) OMP_IF(n)
    for (int64_t i = 0; i < END; ++i) {
      double v = creal(phase * sv[i] * conj(sv[i]));
      if (z_mask && parity((uint64_t)i & z_mask)) v = -v;
      acc += v;
    }
    *out = acc;
    return 0;
  }
  const uint64_t mask_u = ~((1ULL << (x_max + 1)) - 1);
  const uint64_t mask_l = (1ULL << x_max) - 1;
  const int64_t END = (int64_t)(1ULL << (n - 1));
#pragma omp parallel for reduction(+ : acc) OMP_IF(n)
  for (int64_t i = 0; i < END; ++i) {
    uint64_t i0 = (((uint64_t)i << 1) & mask_u) | ((uint64_t)i & mask_l);
    uint64_t i1 = i0 ^ x_mask;
    double v0 = creal(phase * sv[i1] * conj(sv[i0]));
    double v1 = creal(phase * sv[i0] * conj(sv[i1]));
    acc += (z_mask && parity(i0 & z_mask)) ? -v0 : v0;
    acc += (z_mask && parity(i1 & z_mask)) ? -v1 : v1;
  }
  *out = acc;
  return 0;
}

/* QubitVector::apply_pauli (qubitvector.hpp:2392-2433). */
int orc_apply_pauli(cplx *sv, int n, const uint64_t *qubits, int N, const char *pauli, cplx coeff) {
  uint64_t x_mask, z_mask, num_y, x_max;
  if (pauli_masks(qubits, N, pauli, &x_mask, &z_mask, &num_y, &x_max)) return -1;
  if (x_mask + z_mask == 0) return 0;
  const cplx phase = add_y_phase(num_y, coeff);
  if (!x_mask) {
    const int64_t END = (int64_t)(1ULL << n);
#pragma omp parallel for OMP_IF(n)
    for (int64_t i = 0; i < END; ++i) {
      if (z_mask && parity((uint64_t)i & z_mask)) sv[i] *= -1;
      sv[i] *= phase;
    }
    return 0;
  }
  const uint64_t mask_u = ~((1ULL << (x_max + 1)) - 1);
  const uint64_t mask_l = (1ULL << x_max) - 1;
  const int64_t END = (int64_t)(1ULL << (n - 1));
#pragma omp parallel for OMP_IF(n)
  for (int64_t i = 0; i < END; ++i) {
    uint64_t idx[2];
    idx[0] = (((uint64_t)i << 1) & mask_u) | ((uint64_t)i & mask_l);
    idx[1] = idx[0] ^ x_mask;
    cplx t = sv[idx[0]]; sv[idx[0]] = sv[idx[1]]; sv[idx[1]] = t;
    for (int j = 0; j < 2; ++j) {
      if (z_mask && parity(idx[j] & z_mask)) sv[idx[j]] *= -1;
      sv[idx[j]] *= phase;
    }
  }
  return 0;
}

/* QubitVector::probabilities(qubits) (qubitvector.hpp:2096-2143); k == 0
 * gives every basis probability (qubitvector.hpp:2089-2094). */
void orc_probabilities(const cplx *sv, int n, const uint64_t *qubits, int k, double *out) {
  if (k == 0) {
    const int64_t END = (int64_t)(1ULL << n);
#pragma omp parallel for OMP_IF(n)
    for (int64_t j = 0; j < END; ++j) out[j] = creal(sv[j] * conj(sv[j]));
    return;
  }
  uint64_t qs[64];
  sort_qubits(qubits, k, qs);
  const uint64_t DIM = 1ULL << k;
  const int64_t END = (int64_t)(1ULL << (n - k));
  for (uint64_t m = 0; m < DIM; ++m) out[m] = 0.0;
  if (k > 10) {
    /* registers wider than the per-thread tables below: one sequential
       pass, each amplitude added to its outcome's entry */
    const uint64_t N = 1ULL << n;
    for (uint64_t j = 0; j < N; ++j) {
      uint64_t m = 0;
      for (int b = 0; b < k; ++b) m |= ((j >> qubits[b]) & 1ULL) << b;
      out[m] += creal(sv[j] * conj(sv[j]));
    }
    return;
  }
#pragma omp parallel OMP_IF(n)
  {
    double priv[1024];
    for (uint64_t m = 0; m < DIM; ++m) priv[m] = 0.0;
#pragma omp for
    for (int64_t i = 0; i < END; ++i) {
      uint64_t inds[1024];
      indexes(qubits, qs, k, i, inds);
      for (uint64_t m = 0; m < DIM; ++m) priv[m] += creal(sv[inds[m]] * conj(sv[inds[m]]));
    }
#pragma omp critical
    for (uint64_t m = 0; m < DIM; ++m) out[m] += priv[m];
  }
}

/* QubitVector::sample_measure (qubitvector.hpp:2148-2228): block sums over
 * 2^index_size blocks, then a linear walk per shot.  Probabilities are read
 * through prob(k) so the density-matrix variant can reuse the walk. */
typedef double (*prob_fn)(const void *, uint64_t);
static double sv_prob(const void *p, uint64_t k) {
  const cplx *sv = (const cplx *)p;
  return creal(sv[k] * conj(sv[k]));
}

static void sample_generic(const void *data, prob_fn prob, int n, const double *rnds, uint64_t shots,
                           uint64_t *out, int index_size) {
  const int64_t END = (int64_t)(1ULL << n);
  const int64_t INDEX_END = (int64_t)(1ULL << index_size);
  if (END < INDEX_END) {
#pragma omp parallel for OMP_IF(n)
    for (int64_t i = 0; i < (int64_t)shots; ++i) {
      double rnd = rnds[i], p = 0.0;
      int64_t s;
      for (s = 0; s < END - 1; ++s) {
        p += prob(data, s);
        if (rnd < p) break;
      }
      out[i] = s;
    }
    return;
  }
  double *idxs = (double *)calloc(INDEX_END, sizeof(double));
  const uint64_t loop = END >> index_size;
#pragma omp parallel for OMP_IF(n)
  for (int64_t i = 0; i < INDEX_END; ++i) {
    uint64_t base = loop * i;
    double total = 0.0;
    for (uint64_t j = 0; j < loop; ++j) total += prob(data, base | j);
    idxs[i] = total;
  }
#pragma omp parallel for OMP_IF(n)
  for (int64_t i = 0; i < (int64_t)shots; ++i) {
    double rnd = rnds[i], p = 0.0;
    int64_t s = 0;
    for (int64_t j = 0; j < INDEX_END; ++j) {
      if (rnd < p + idxs[j]) break;
      p += idxs[j];
      s += loop;
    }
    for (; s < END - 1; ++s) {
      p += prob(data, s);
      if (rnd < p) break;
    }
    out[i] = s;
  }
  free(idxs);
}

void orc_sample_measure(const cplx *sv, int n, const double *rnds, uint64_t shots, uint64_t *out,
                        int index_size) {
  sample_generic(sv, sv_prob, n, rnds, shots, out, index_size);
}

/* checkpoint inner product <psi|ckpt> as QubitVector::inner_product computes
 * it: sum data[k] * conj(ckpt[k]) (qubitvector.hpp:1029-1041). */
void orc_inner_product(const cplx *sv, const cplx *ck, int n, double *re, double *im) {
  const int64_t END = (int64_t)(1ULL << n);
  double ar = 0.0, ai = 0.0;
#pragma omp parallel for reduction(+ : ar, ai) OMP_IF(n)
  for (int64_t i = 0; i < END; ++i) {
    cplx z = sv[i] * conj(ck[i]);
    ar += creal(z);
    ai += cimag(z);
  }
  *re = ar; *im = ai;
}

/* ---------------- density matrix (n qubits, 2n vector qubits) ---------------- */

/* DensityMatrix::expval_pauli (densitymatrix.hpp:445-496). */
int orc_dm_expval_pauli(const cplx *rho, int n, const uint64_t *qubits, int N, const char *pauli,
                        cplx initial_phase, double *out) {
  uint64_t x_mask, z_mask, num_y, x_max;
  if (pauli_masks(qubits, N, pauli, &x_mask, &z_mask, &num_y, &x_max)) return -1;
  const uint64_t nrows = 1ULL << n;
  double acc = 0.0;
  if (x_mask + z_mask == 0) {
    for (uint64_t i = 0; i < nrows; ++i) acc += creal(rho[i * (nrows + 1)]);
    *out = acc;
    return 0;
  }
  if (!x_mask) {
#pragma omp parallel for reduction(+ : acc) OMP_IF(2 * n)
    for (int64_t i = 0; i < (int64_t)nrows; ++i) {
      double v = creal(rho[(uint64_t)i * (nrows + 1)]);
      if (z_mask && parity((uint64_t)i & z_mask)) v = -v;
      acc += v;
    }
    *out = acc;
    return 0;
  }
  const cplx phase = add_y_phase(num_y, initial_phase);
  const uint64_t mask_u = ~((1ULL << (x_max + 1)) - 1);
  const uint64_t mask_l = (1ULL << x_max) - 1;
#pragma omp parallel for reduction(+ : acc) OMP_IF(2 * n)
  for (int64_t i = 0; i < (int64_t)(nrows >> 1); ++i) {
    uint64_t iv = (((uint64_t)i << 1) & mask_u) | ((uint64_t)i & mask_l);
    uint64_t im = (iv ^ x_mask) + nrows * iv;
    double v = 2 * creal(phase * rho[im]);
    if (z_mask && parity(iv & z_mask)) v = -v;
    acc += v;
  }
  *out = acc;
  return 0;
}

/* DensityMatrix::probability(outcome) = Re rho[k,k] (densitymatrix.hpp:516-520),
 * marginalised as QubitVector::probabilities(qubits) over the diagonal. */
void orc_dm_probabilities(const cplx *rho, int n, const uint64_t *qubits, int k, double *out) {
  const uint64_t nrows = 1ULL << n;
  if (k == 0) {
    for (uint64_t j = 0; j < nrows; ++j) out[j] = creal(rho[j * (nrows + 1)]);
    return;
  }
  const uint64_t DIM = 1ULL << k;
  for (uint64_t m = 0; m < DIM; ++m) out[m] = 0.0;
  for (uint64_t j = 0; j < nrows; ++j) {
    uint64_t m = 0;
    for (int b = 0; b < k; ++b)
      if (j & (1ULL << qubits[b])) m |= 1ULL << b;
    out[m] += creal(rho[j * (nrows + 1)]);
  }
}

static double dm_prob(const void *p, uint64_t k) {
  const cplx *rho = ((const cplx *const *)p)[0];
  const uint64_t nrows = ((const uint64_t *)p)[1];
  return creal(rho[k * (nrows + 1)]);
}

void orc_dm_sample_measure(const cplx *rho, int n, const double *rnds, uint64_t shots, uint64_t *out,
                           int index_size) {
  const void *ctx[2];
  ctx[0] = rho;
  ctx[1] = (const void *)(uintptr_t)(1ULL << n);
  sample_generic(ctx, dm_prob, n, rnds, shots, out, index_size);
}

/* ---------------- std::mt19937_64 + uniform_real_distribution ---------------- */
/* RngEngine::rand(0,1) (src/framework/rng.hpp:65-67,96) draws
 * std::uniform_real_distribution<double>(0,1) from std::mt19937_64; this is
 * the published MT19937-64 generator (Matsumoto & Nishimura) and the
 * libstdc++ generate_canonical step: one 64-bit draw converted to double and
 * scaled by 2^-64, clamped below 1. */
typedef struct { uint64_t mt[312]; int mti; } orc_mt64;

void orc_mt64_seed(orc_mt64 *s, uint64_t seed) {
  s->mt[0] = seed;
  for (int i = 1; i < 312; ++i)
    s->mt[i] = 6364136223846793005ULL * (s->mt[i - 1] ^ (s->mt[i - 1] >> 62)) + (uint64_t)i;
  s->mti = 312;
}

uint64_t orc_mt64_next(orc_mt64 *s) {
  static const uint64_t MAG[2] = {0ULL, 0xB5026F5AA96619E9ULL};
  const uint64_t UM = 0xFFFFFFFF80000000ULL, LM = 0x7FFFFFFFULL;
  if (s->mti >= 312) {
    int i;
    for (i = 0; i < 312 - 156; ++i) {
      uint64_t x = (s->mt[i] & UM) | (s->mt[i + 1] & LM);
      s->mt[i] = s->mt[i + 156] ^ (x >> 1) ^ MAG[x & 1ULL];
    }
    for (; i < 311; ++i) {
      uint64_t x = (s->mt[i] & UM) | (s->mt[i + 1] & LM);
      s->mt[i] = s->mt[i + (156 - 312)] ^ (x >> 1) ^ MAG[x & 1ULL];
    }
    uint64_t x = (s->mt[311] & UM) | (s->mt[0] & LM);
    s->mt[311] = s->mt[155] ^ (x >> 1) ^ MAG[x & 1ULL];
    s->mti = 0;
  }
  uint64_t x = s->mt[s->mti++];
  x ^= (x >> 29) & 0x5555555555555555ULL;
  x ^= (x << 17) & 0x71D67FFFEDA60000ULL;
  x ^= (x << 37) & 0xFFF7EEE000000000ULL;
  x ^= (x >> 43);
  return x;
}

/* Draw `count` uniforms in [0,1) from a fresh generator seeded with seed. */
void orc_uniforms(uint64_t seed, uint64_t count, double *out) {
  orc_mt64 s;
  orc_mt64_seed(&s, seed);
  for (uint64_t i = 0; i < count; ++i) {
    double r = (double)orc_mt64_next(&s) * 0x1p-64;
    if (r >= 1.0) r = nextafter(1.0, 0.0);
    out[i] = r;
  }
}
