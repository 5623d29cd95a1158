// gbqv_aerstate.cpp — the reference's C runtime API (contrib/runtime/
// aer_runtime_api.h:20-108, contrib/runtime/aer_runtime.cpp) implemented on
// the GB300 engine, so a C program written against Aer's imperative
// AerState interface links against libgbqv instead.  Semantics follow
// AerState (src/controllers/state_controller.hpp:81-387): configure
// ("method" = statevector, "device" = GPU, "precision" = double|single,
// "seed_simulator"), allocate qubits, initialize to |0...0>, apply gates with
// the statevector gate dispatch, measure (outcome drawn with
// std::discrete_distribution over the measured qubits' probabilities from
// the state's mt19937_64, then the state collapses and renormalises, as
// QubitVector::measure does), probabilities and amplitudes.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../include/aer_runtime_gb300.h"
#include "../../include/gbqv.h"
#include "gbqv_gates.h"
#include "gbqv_internal.h"

using namespace gbqv;


namespace {

struct AerStateGB {
  int precision = GBQV_C128;
  uint64_t seed = 0;
  bool seeded = false;
  uint_t num_qubits = 0;
  gbqv_handle h = nullptr;
  std::mt19937_64 rng;
};

void fail(AerStateGB *s, const char *what) {
  std::string msg = std::string("aer_state: ") + what + ": " + gbqv_last_error(s ? s->h : nullptr);
  throw std::runtime_error(msg);
}

void ok(AerStateGB *s, int rc, const char *what) {
  if (rc != GBQV_OK) fail(s, what);
}

// No exception leaves these C entry points: failures are recorded for
// gbqv_last_error(NULL) and the call returns (value-returning calls return
// 0 / NaN / NULL).
template <typename R, typename F>
R guarded(R on_error, F &&f) {
  try {
    return f();
  } catch (const std::exception &e) {
    set_last_error(nullptr, e.what());
    return on_error;
  }
}

template <typename F>
void guarded_void(F &&f) {
  try {
    f();
  } catch (const std::exception &e) {
    set_last_error(nullptr, e.what());
  }
}

AerStateGB *S(void *p) {
  if (!p) throw std::invalid_argument("aer_state: null state");
  return static_cast<AerStateGB *>(p);
}

gbqv_handle H(void *p) {
  AerStateGB *s = S(p);
  if (!s->h) throw std::runtime_error("aer_state: state is not initialized");
  return s->h;
}

void mcu(void *p, std::vector<uint64_t> q, const gates::mat_t &m) {
  ok(S(p), gbqv_apply_mcu(H(p), q.data(), (int)q.size(), reinterpret_cast<const gbqv_c128 *>(m.data())), "mcu");
}

void mcphase(void *p, std::vector<uint64_t> q, cd ph) {
  ok(S(p), gbqv_apply_mcphase(H(p), q.data(), (int)q.size(), gbqv_c128{ph.real(), ph.imag()}), "mcphase");
}

// One amplitude, read straight from device memory.
cd amplitude(void *p, uint_t outcome) {
  AerStateGB *s = S(p);
  int n = 0;
  ok(s, gbqv_num_vector_qubits(H(p), &n), "amplitude");
  if (outcome >= (1ULL << n)) throw std::invalid_argument("aer_state: outcome out of range");
  ok(s, gbqv_synchronize(H(p)), "amplitude");
  void *d = nullptr;
  ok(s, gbqv_device_data(H(p), &d), "amplitude");
  if (s->precision == GBQV_C128) {
    cd z;
    cuda_check(cudaMemcpy(&z, static_cast<cd *>(d) + outcome, sizeof(cd), cudaMemcpyDeviceToHost), "amplitude copy");
    return z;
  }
  std::complex<float> z;
  cuda_check(cudaMemcpy(&z, static_cast<std::complex<float> *>(d) + outcome, sizeof(z), cudaMemcpyDeviceToHost),
             "amplitude copy");
  return cd(z.real(), z.imag());
}

void diag1(void *p, uint64_t q, cd d1) {
  const gbqv_c128 d[2] = {{1.0, 0.0}, {d1.real(), d1.imag()}};
  ok(S(p), gbqv_apply_diagonal_matrix(H(p), &q, 1, d), "diagonal");
}

}  // namespace

extern "C" {

void *aer_state() { return guarded<void *>(nullptr, [] { return (void *)new AerStateGB; }); }

void aer_state_configure(void *state, char *key, char *value) {
  guarded_void([&] {
  AerStateGB *s = S(state);
  const std::string k(key ? key : ""), v(value ? value : "");
  if (s->h) throw std::runtime_error("aer_state: configure before initialize");
  if (k == "method") {
    if (v != "statevector" && v != "automatic") throw std::invalid_argument("aer_state: method must be statevector");
  } else if (k == "device") {
    if (v != "GPU") throw std::invalid_argument("aer_state: this engine runs on the GPU");
  } else if (k == "precision") {
    if (v == "double") s->precision = GBQV_C128;
    else if (v == "single") s->precision = GBQV_C64;
    else throw std::invalid_argument("aer_state: precision must be double or single");
  } else if (k == "seed_simulator") {
    s->seed = std::strtoull(v.c_str(), nullptr, 10);
    s->seeded = true;
  }
  // other AerState keys (threads, fusion, chunking) have no effect on one GPU
  });
}

uint_t aer_allocate_qubits(void *state, uint_t num_qubits) {
  return guarded<uint_t>(0, [&] {
    AerStateGB *s = S(state);
    if (s->h) throw std::runtime_error("aer_state: allocate qubits before initialize");
    const uint_t first = s->num_qubits;
    s->num_qubits += num_qubits;
    return first;
  });
}

void aer_state_initialize(void *state) {
  guarded_void([&] {
    AerStateGB *s = S(state);
    if (s->h) gbqv_destroy(s->h);
    s->h = nullptr;
    ok(s, gbqv_create((int)s->num_qubits, s->precision, GBQV_STATEVECTOR, &s->h), "initialize");
    s->rng.seed(s->seeded ? s->seed : std::random_device{}());
  });
}

void aer_state_finalize(void *state) {
  guarded_void([&] {
    AerStateGB *s = S(state);
    if (s->h) gbqv_destroy(s->h);
    delete s;
  });
}

// QubitVector::measure: probabilities of the measured qubits, an outcome from
// std::discrete_distribution (RngEngine::rand_int, rng.hpp:86-90), then the
// projector onto that outcome scaled by 1/sqrt(p) (measure_reset_update).
uint_t aer_apply_measure(void *state, uint_t *qubits, size_t num_qubits) {
  return guarded<uint_t>(0, [&] {
    AerStateGB *s = S(state);
    std::vector<uint64_t> q(qubits, qubits + num_qubits);
    std::vector<double> probs(1ULL << num_qubits);
    ok(s, gbqv_probabilities(H(state), q.data(), (int)q.size(), probs.data()), "measure");
    const uint_t outcome = std::discrete_distribution<size_t>(probs.begin(), probs.end())(s->rng);
    const double scale = 1.0 / std::sqrt(probs[outcome]);
    std::vector<gbqv_c128> d(probs.size(), gbqv_c128{0.0, 0.0});
    d[outcome] = gbqv_c128{scale, 0.0};
    ok(s, gbqv_apply_diagonal_matrix(H(state), q.data(), (int)q.size(), d.data()), "measure collapse");
    return outcome;
  });
}

double aer_probability(void *state, uint_t outcome) {
  return guarded<double>(NAN, [&] { return std::norm(amplitude(state, outcome)); });
}

_Complex double aer_amplitude(void *state, uint_t outcome) {
  return guarded<_Complex double>(NAN, [&] {
    const cd z = amplitude(state, outcome);
    _Complex double r;
    std::memcpy(&r, &z, sizeof(r));
    return r;
  });
}

_Complex double *aer_release_statevector(void *state) {
  return guarded<_Complex double *>(nullptr, [&] {
    AerStateGB *s = S(state);
    int n = 0;
    ok(s, gbqv_num_vector_qubits(H(state), &n), "release");
    const uint64_t len = 1ULL << n;
    auto *out = static_cast<_Complex double *>(std::malloc(sizeof(_Complex double) * len));
    if (!out) throw std::bad_alloc();
    ok(s, gbqv_copy_to_host(H(state), reinterpret_cast<gbqv_c128 *>(out), len), "release");
    gbqv_destroy(s->h);
    s->h = nullptr;
    return out;
  });
}

// ---- gates: Statevector::State::apply_gate (statevector_state.hpp:733-865) ----
void aer_apply_u3(void *s, uint_t q, double t, double p, double l) { guarded_void([&] { mcu(s, {q}, gates::u4(t, p, l, 0.)); }); }
void aer_apply_p(void *s, uint_t q, double l) { guarded_void([&] { mcphase(s, {q}, std::exp(cd(0, 1) * l)); }); }
void aer_apply_x(void *s, uint_t q) { guarded_void([&] { uint64_t qq = q; ok(S(s), gbqv_apply_mcx(H(s), &qq, 1), "x"); }); }
void aer_apply_y(void *s, uint_t q) { guarded_void([&] { uint64_t qq = q; ok(S(s), gbqv_apply_mcy(H(s), &qq, 1), "y"); }); }
void aer_apply_z(void *s, uint_t q) { guarded_void([&] { mcphase(s, {q}, -1.0); }); }
void aer_apply_h(void *s, uint_t q) { guarded_void([&] { mcu(s, {q}, gates::u4(M_PI / 2., 0., M_PI, 0.)); }); }
void aer_apply_s(void *s, uint_t q) { guarded_void([&] { diag1(s, q, cd(0., 1.)); }); }
void aer_apply_sdg(void *s, uint_t q) { guarded_void([&] { diag1(s, q, cd(0., -1.)); }); }
void aer_apply_t(void *s, uint_t q) { guarded_void([&] { const double r = 1. / std::sqrt(2); diag1(s, q, cd(r, r)); }); }
void aer_apply_tdg(void *s, uint_t q) { guarded_void([&] { const double r = 1. / std::sqrt(2); diag1(s, q, cd(r, -r)); }); }
void aer_apply_sx(void *s, uint_t q) { guarded_void([&] { mcu(s, {q}, gates::SX()); }); }
void aer_apply_rx(void *s, uint_t q, double t) { guarded_void([&] { mcu(s, {q}, gates::rx(t)); }); }
void aer_apply_ry(void *s, uint_t q, double t) { guarded_void([&] { mcu(s, {q}, gates::ry(t)); }); }
void aer_apply_rz(void *s, uint_t q, double t) { guarded_void([&] { mcu(s, {q}, gates::rz(t)); }); }
void aer_apply_cx(void *s, uint_t c, uint_t t) { guarded_void([&] { uint64_t qq[2] = {c, t}; ok(S(s), gbqv_apply_mcx(H(s), qq, 2), "cx"); }); }
void aer_apply_cy(void *s, uint_t c, uint_t t) { guarded_void([&] { uint64_t qq[2] = {c, t}; ok(S(s), gbqv_apply_mcy(H(s), qq, 2), "cy"); }); }
void aer_apply_cz(void *s, uint_t c, uint_t t) { guarded_void([&] { mcphase(s, {c, t}, -1.0); }); }
void aer_apply_cp(void *s, uint_t c, uint_t t, double l) { guarded_void([&] { mcphase(s, {c, t}, std::exp(cd(0, 1) * l)); }); }
void aer_apply_crx(void *s, uint_t c, uint_t t, double th) { guarded_void([&] { mcu(s, {c, t}, gates::rx(th)); }); }
void aer_apply_cry(void *s, uint_t c, uint_t t, double th) { guarded_void([&] { mcu(s, {c, t}, gates::ry(th)); }); }
void aer_apply_crz(void *s, uint_t c, uint_t t, double th) { guarded_void([&] { mcu(s, {c, t}, gates::rz(th)); }); }
void aer_apply_ch(void *s, uint_t c, uint_t t) { guarded_void([&] { mcu(s, {c, t}, gates::u4(M_PI / 2., 0., M_PI, 0.)); }); }
void aer_apply_swap(void *s, uint_t a, uint_t b) { guarded_void([&] { uint64_t qq[2] = {a, b}; ok(S(s), gbqv_apply_mcswap(H(s), qq, 2), "swap"); }); }
void aer_apply_ccx(void *s, uint_t a, uint_t b, uint_t c) {
  guarded_void([&] {
    uint64_t qq[3] = {a, b, c};
    ok(S(s), gbqv_apply_mcx(H(s), qq, 3), "ccx");
  });
}
void aer_apply_cswap(void *s, uint_t c, uint_t a, uint_t b) {
  guarded_void([&] {
    uint64_t qq[3] = {c, a, b};
    ok(S(s), gbqv_apply_mcswap(H(s), qq, 3), "cswap");
  });
}
void aer_apply_cu(void *s, uint_t c, uint_t t, double th, double ph, double la, double ga) {
  guarded_void([&] { mcu(s, {c, t}, gates::u4(th, ph, la, ga)); });
}

}  // extern "C"
