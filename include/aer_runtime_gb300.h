/*
 * aer_runtime_gb300.h — the imperative C runtime API of Qiskit Aer
 * (contrib/runtime/aer_runtime_api.h:20-108), served by libgbqv.so on a
 * GB300.  Same function names, arguments and meaning, so a C program written
 * against Aer's runtime relinks against libgbqv unchanged.  Differences:
 * "method" must be statevector and "device" GPU; errors do not throw — the
 * call returns (0 / NaN / NULL for value-returning calls) and
 * gbqv_last_error(NULL) holds the message.
 */
#ifndef AER_RUNTIME_GB300_H_
#define AER_RUNTIME_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#define GBQV_AER_COMPLEX _Complex double
#else
#include <complex.h>
#define GBQV_AER_COMPLEX double complex
#endif

typedef uint_fast64_t uint_t;

/* AerState lifetime (state_controller.hpp:81-387). */
void *aer_state(void);
void aer_state_initialize(void *state);
void aer_state_finalize(void *state);
void aer_state_configure(void *state, char *key, char *value);
uint_t aer_allocate_qubits(void *state, uint_t num_qubits);

/* Measurement and readout. */
uint_t aer_apply_measure(void *state, uint_t *qubits, size_t num_qubits);
double aer_probability(void *state, uint_t outcome);
GBQV_AER_COMPLEX aer_amplitude(void *state, uint_t outcome);
/* The full statevector in a malloc'ed buffer the caller frees; the state is
 * released. */
GBQV_AER_COMPLEX *aer_release_statevector(void *state);

/* Gates (Statevector::State::apply_gate, statevector_state.hpp:733-865). */
void aer_apply_u3(void *state, uint_t qubit, double theta, double phi, double lambda);
void aer_apply_p(void *state, uint_t qubit, double lambda);
void aer_apply_x(void *state, uint_t qubit);
void aer_apply_y(void *state, uint_t qubit);
void aer_apply_z(void *state, uint_t qubit);
void aer_apply_h(void *state, uint_t qubit);
void aer_apply_s(void *state, uint_t qubit);
void aer_apply_sdg(void *state, uint_t qubit);
void aer_apply_t(void *state, uint_t qubit);
void aer_apply_tdg(void *state, uint_t qubit);
void aer_apply_sx(void *state, uint_t qubit);
void aer_apply_rx(void *state, uint_t qubit, double theta);
void aer_apply_ry(void *state, uint_t qubit, double theta);
void aer_apply_rz(void *state, uint_t qubit, double theta);
void aer_apply_cx(void *state, uint_t ctrl_qubit, uint_t tgt_qubit);
void aer_apply_cy(void *state, uint_t ctrl_qubit, uint_t tgt_qubit);
void aer_apply_cz(void *state, uint_t ctrl_qubit, uint_t tgt_qubit);
void aer_apply_cp(void *state, uint_t ctrl_qubit, uint_t tgt_qubit, double lambda);
void aer_apply_crx(void *state, uint_t ctrl_qubit, uint_t tgt_qubit, double theta);
void aer_apply_cry(void *state, uint_t ctrl_qubit, uint_t tgt_qubit, double theta);
void aer_apply_crz(void *state, uint_t ctrl_qubit, uint_t tgt_qubit, double theta);
void aer_apply_ch(void *state, uint_t ctrl_qubit, uint_t tgt_qubit);
void aer_apply_swap(void *state, uint_t qubit0, uint_t qubit1);
void aer_apply_ccx(void *state, uint_t qubit0, uint_t qubit1, uint_t qubit2);
void aer_apply_cswap(void *state, uint_t ctrl_qubit, uint_t qubit0, uint_t qubit1);
void aer_apply_cu(void *state, uint_t ctrl_qubit, uint_t tgt_qubit, double theta, double phi, double lambda,
                  double gamma);

#ifdef __cplusplus
}
#endif
#undef GBQV_AER_COMPLEX

#endif /* AER_RUNTIME_GB300_H_ */
