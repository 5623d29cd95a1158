/*
 * gbqv.h — C ABI of the GB300 statevector / density-matrix engine (libgbqv.so).
 *
 * The engine replaces the `statevec_t` / `densmat_t` template argument that
 * Qiskit Aer's State classes are instantiated with: the member surface of
 * QV::QubitVector<T> (src/simulators/statevector/qubitvector.hpp:61-651),
 * its GPU twin QubitVectorThrust (qubitvector_thrust.hpp:57-560) and
 * QV::DensityMatrix<T> (src/simulators/density_matrix/densitymatrix.hpp:34-171).
 * Each entry point below names the reference member it stands in for.
 *
 * Conventions (all follow the reference):
 *   - A state of n qubits is 2^n amplitudes; amplitude index bit q is qubit q.
 *   - Matrices are column-major, mat[row + DIM*col], and qubits[0] is the
 *     least-significant bit of the matrix row/column index
 *     (transformer.hpp:157-159, indexes.hpp:223-235).
 *   - Multi-controlled gates take the target as the LAST qubit
 *     (qubitvector.hpp:1446-1720).
 *   - Pauli labels are read right to left: label[N-1-i] acts on qubits[i]
 *     (qubitvector.hpp:2235-2272).
 *   - A density matrix of n qubits is vec(rho) over 2n vector qubits,
 *     column-stacked: rho[i,j] sits at index i + 2^n * j
 *     (densitymatrix.hpp:265-323).
 *
 * Ownership and threading: a handle owns its device state and one CUDA
 * stream.  Inputs (qubit lists, matrices, uniforms) are host pointers that
 * are consumed before the call returns; outputs go to caller-owned host
 * buffers.  A handle is used by one thread at a time; different handles may
 * be used concurrently.  Calls that return a value synchronise the handle's
 * stream; others are asynchronous until gbqv_synchronize().
 *
 * Errors: every function returns GBQV_OK (0) or a positive error code and
 * never throws across the ABI (the reference throws std::runtime_error /
 * std::invalid_argument, qubitvector.hpp:698-747, 2266-2268).  The message
 * of the most recent failure on a handle is gbqv_last_error(handle); failures
 * that have no handle are reported by gbqv_last_error(NULL) (thread-local).
 */
#ifndef GBQV_H_
#define GBQV_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gbqv_state *gbqv_handle;
typedef struct gbqv_circuit *gbqv_circuit_t;
typedef struct gbqv_batch *gbqv_batch_t;

/* Interleaved complex double, layout-compatible with std::complex<double>. */
typedef struct {
  double re, im;
} gbqv_c128;

enum gbqv_status {
  GBQV_OK = 0,
  GBQV_ERR_ARG = 1,      /* bad size, null pointer, bad label, bad axis      */
  GBQV_ERR_QUBIT = 2,    /* qubit index out of range or repeated             */
  GBQV_ERR_CUDA = 3,     /* CUDA launch / runtime failure                    */
  GBQV_ERR_ALLOC = 4,    /* device memory could not be allocated             */
  GBQV_ERR_KIND = 5,     /* operation not valid for this state kind          */
  GBQV_ERR_TIMEOUT = 6   /* a bounded device-side wait gave up               */
};

enum gbqv_precision { GBQV_C64 = 0, GBQV_C128 = 1 };
/* GBQV_UNITARY: QV::UnitaryMatrix<T> (src/simulators/unitary/unitarymatrix.hpp),
 * the state of the unitary method: a 2^n x 2^n matrix stored column-major as
 * a vector of 2n qubits (row bits 0..n-1, column bits n..2n-1), starting as
 * the identity (UnitaryMatrix::initialize, unitarymatrix.hpp:236-247).  Gates
 * on qubits 0..n-1 give U <- G U (QubitUnitary::State::apply_gate,
 * unitary_state.hpp:414-545); copy_to_host returns the 4^n entries. */
enum gbqv_kind { GBQV_STATEVECTOR = 0, GBQV_DENSITY_MATRIX = 1, GBQV_UNITARY = 2 };

/* Rotation axes, QV::Rotation (qubitvector.hpp:50-59). */
enum gbqv_rotation {
  GBQV_ROT_X = 0, GBQV_ROT_Y = 1, GBQV_ROT_Z = 2,
  GBQV_ROT_XX = 3, GBQV_ROT_YY = 4, GBQV_ROT_ZZ = 5, GBQV_ROT_ZX = 6
};

/* ------------------------------------------------------------------ */
/* Library                                                              */
/* ------------------------------------------------------------------ */

/* ABI version of this header (major*10000 + minor*100 + patch). */
int gbqv_version(void);
/* Message of the last failure on h; h == NULL gives this thread's last
 * handle-less failure.  The pointer stays valid until the next call on h. */
const char *gbqv_last_error(gbqv_handle h);
/* Number of CUDA devices visible (0 when no GPU); never fails. */
int gbqv_device_count(void);
/* The uniform stream of RngEngine::rand(0, 1) after set_seed(seed)
 * (src/framework/rng.hpp:65-67, 96): std::uniform_real_distribution<double>
 * over std::mt19937_64.  These are the draws State::sample_measure consumes
 * (statevector_state.hpp:1016-1027); needs no GPU. */
int gbqv_uniforms(uint64_t seed, uint64_t count, double *out);
/* count draws of each of the streams seed0, seed0 + 1, .., seed0 + nstreams - 1
 * (mod 2^64) into out[s * count + i]: the per-shot streams of a circuit run
 * shot by shot (shot i seeded seed + i, circuit_executor.hpp:880-940). */
int gbqv_uniforms_streams(uint64_t seed0, uint64_t nstreams, uint64_t count, double *out);

/* ------------------------------------------------------------------ */
/* State lifetime — QubitVector(num_qubits) / set_num_qubits           */
/* (qubitvector.hpp:754-767, 913-967); QubitVectorThrust chunk_setup  */
/* + DeviceChunkContainer::Allocate (device_chunk_container.hpp:319). */
/* ------------------------------------------------------------------ */

/* n = number of qubits (a density matrix of n qubits holds 4^n entries). */
int gbqv_create(int num_qubits, int precision, int kind, gbqv_handle *out);
int gbqv_destroy(gbqv_handle h);
int gbqv_num_qubits(gbqv_handle h, int *out);
/* Number of vector qubits: n for a statevector, 2n for a density matrix. */
int gbqv_num_vector_qubits(gbqv_handle h, int *out);
int gbqv_synchronize(gbqv_handle h);
/* Device pointer of the amplitudes (complex<double> or complex<float>). */
int gbqv_device_data(gbqv_handle h, void **out);
/* The handle's cudaStream_t (every kernel of the handle runs on it), for
 * callers that order their own work or record events around the engine's
 * (the reference keeps its streams private, device_chunk_container.hpp:422). */
int gbqv_get_stream(gbqv_handle h, void **out);
/* Kernels this library has launched since load, all handles (a counter the
 * benchmark reads around its timed region). */
uint64_t gbqv_launch_count(void);

/* QubitVector::zero (qubitvector.hpp:973-979). */
int gbqv_zero(gbqv_handle h);
/* QubitVector::initialize -> |0...0>; DensityMatrix::initialize -> |0><0|
 * (qubitvector.hpp:1076-1080, densitymatrix.hpp:198-204). */
int gbqv_initialize(gbqv_handle h);
/* QubitVector::initialize_from_vector (qubitvector.hpp:1082-1110).  For a
 * density matrix a length-2^n vector is taken as a pure state and
 * vec(|psi><psi|) is stored (densitymatrix.hpp:206-226). */
int gbqv_initialize_from_vector(gbqv_handle h, const gbqv_c128 *vec, uint64_t len);
/* QubitVector::copy_to_vector / move_to_vector (qubitvector.hpp:1008-1050);
 * len must equal the number of stored amplitudes. */
int gbqv_copy_to_host(gbqv_handle h, gbqv_c128 *out, uint64_t len);
/* QubitVector::checkpoint / revert / inner_product
 * (qubitvector.hpp:994-1041): <state|checkpoint>. */
int gbqv_checkpoint(gbqv_handle h);
int gbqv_revert(gbqv_handle h, int keep);
int gbqv_inner_product(gbqv_handle h, gbqv_c128 *out);

/* ------------------------------------------------------------------ */
/* Gate application on the (vector) qubits of the state                */
/* ------------------------------------------------------------------ */

/* QubitVector::apply_matrix (qubitvector.hpp:1298-1303, transformer.hpp:89-232):
 * dense 2^k x 2^k column-major matrix, 1 <= k <= 13. */
int gbqv_apply_matrix(gbqv_handle h, const uint64_t *qubits, int k, const gbqv_c128 *mat);
/* QubitVector::apply_diagonal_matrix (qubitvector.hpp:1342-1347,
 * transformer.hpp:234-372): diag has 2^k entries, 1 <= k <= 20. */
int gbqv_apply_diagonal_matrix(gbqv_handle h, const uint64_t *qubits, int k, const gbqv_c128 *diag);
/* QubitVector::apply_mcx / apply_mcy / apply_mcswap (qubitvector.hpp:1446-1573). */
int gbqv_apply_mcx(gbqv_handle h, const uint64_t *qubits, int nq);
int gbqv_apply_mcy(gbqv_handle h, const uint64_t *qubits, int nq);
int gbqv_apply_mcswap(gbqv_handle h, const uint64_t *qubits, int nq);
/* QubitVector::apply_mcphase (qubitvector.hpp:1575-1612). */
int gbqv_apply_mcphase(gbqv_handle h, const uint64_t *qubits, int nq, gbqv_c128 phase);
/* QubitVector::apply_mcu (qubitvector.hpp:1614-1720): mat is 2x2 column-major. */
int gbqv_apply_mcu(gbqv_handle h, const uint64_t *qubits, int nq, const gbqv_c128 *mat);
/* QubitVector::apply_rotation (qubitvector.hpp:1722-1750), axis = gbqv_rotation. */
int gbqv_apply_rotation(gbqv_handle h, const uint64_t *qubits, int nq, int axis, double theta);
/* QubitVector::apply_pauli (qubitvector.hpp:2392-2433). */
int gbqv_apply_pauli(gbqv_handle h, const uint64_t *qubits, int nq, const char *label, gbqv_c128 coeff);
/* QubitVector::apply_permutation_matrix (qubitvector.hpp:1349-1434):
 * pairs = [a0, b0, a1, b1, ...] of local indices to swap, in order. */
int gbqv_apply_permutation_matrix(gbqv_handle h, const uint64_t *qubits, int k,
                                  const uint64_t *pairs, int npairs);
/* QubitVector::apply_multiplexer (qubitvector.hpp:1305-1340): mat is the
 * (2^nt * 2^nc) x 2^nt column-major stack of 2^nc blocks. */
int gbqv_apply_multiplexer(gbqv_handle h, const uint64_t *controls, int nc,
                           const uint64_t *targets, int nt, const gbqv_c128 *mat);
/* QubitVector::apply_multi_swaps (qubitvector.hpp:1842-1871): swaps qubit
 * pairs (q0,q1), (q2,q3), ... */
int gbqv_apply_multi_swaps(gbqv_handle h, const uint64_t *qubits, int nq);

/* ------------------------------------------------------------------ */
/* Reductions (FP64 accumulation in every precision)                    */
/* ------------------------------------------------------------------ */

/* QubitVector::norm (qubitvector.hpp:1878-1886); for a density matrix this is
 * the squared Frobenius norm of the stored vector, as in the reference. */
int gbqv_norm(gbqv_handle h, double *out);
/* QubitVector::norm(qubits, mat) (qubitvector.hpp:1888-2082): ||M psi||^2,
 * 1 <= k <= 13; the state is left as it is. */
int gbqv_norm_matrix(gbqv_handle h, const uint64_t *qubits, int k, const gbqv_c128 *mat, double *out);
/* QubitVector::probabilities() / probabilities(qubits)
 * (qubitvector.hpp:2089-2143); DensityMatrix uses the diagonal
 * (densitymatrix.hpp:516-520).  k == 0 means all qubits (out has 2^n);
 * otherwise out has 2^k entries for any 1 <= k <= n, outcome bit j = qubit
 * qubits[j]. */
int gbqv_probabilities(gbqv_handle h, const uint64_t *qubits, int k, double *out);
/* QubitVector::probability(outcome) (qubitvector.hpp:302, |psi_k|^2) and
 * DensityMatrix::probability (densitymatrix.hpp:530-534, Re rho[k, k]):
 * reads the one entry back. */
int gbqv_probability(gbqv_handle h, uint64_t outcome, double *out);
/* QubitVector::sample_measure (qubitvector.hpp:2148-2228): for each uniform
 * r in [0,1) the first basis index whose cumulative probability exceeds r,
 * with the cumulative sums formed in the reference's order (sequential sums
 * over 2^index_size blocks, then a sequential walk inside the block), so
 * that a uniform on a boundary resolves as in the reference.  A uniform at
 * or above the total of all block sums gives 2^n, as the reference's walk. */
int gbqv_sample_measure(gbqv_handle h, const double *rnds, uint64_t shots, uint64_t *out);
/* QubitVector::set_sample_measure_index_size (qubitvector.hpp:457): the
 * block count 2^index_size of the sampling walk (default 10, the
 * statevector_sample_measure_opt option). */
int gbqv_set_sample_measure_index_size(gbqv_handle h, int index_size);
/* QubitVector::expval_pauli (qubitvector.hpp:2299-2347) and
 * DensityMatrix::expval_pauli (densitymatrix.hpp:445-496). */
int gbqv_expval_pauli(gbqv_handle h, const uint64_t *qubits, int nq, const char *label,
                      gbqv_c128 initial_phase, double *out);
/* Many Pauli terms in one call: the loop of Base::apply_save_expval
 * (src/simulators/state.hpp:416-447) without one host round trip per term.
 * Term t acts on qubits[offsets[t] .. offsets[t+1]) with labels[t];
 * out[t] = <P_t>.  Returns sum_t coeffs[t] * out[t] in *total when non-NULL. */
int gbqv_expval_pauli_many(gbqv_handle h, int nterms, const uint64_t *qubits,
                           const int *offsets, const char *const *labels,
                           const double *coeffs, double *out, double *total);

/* Expectation values of up to 64 Pauli strings on a statevector that the
 * caller owns in device memory (state: 2^num_qubits complex<double> or
 * complex<float>, precision GBQV_C128 / GBQV_C64), for callers that cannot
 * allocate device memory: a framework whose allocator already owns the GPU's
 * memory, or a loop that must not pay the device synchronisation of
 * cudaMalloc / cudaFree.  No counterpart in the reference.  It allocates
 * nothing: its partial sums live in a static __device__ array of 78 KB that
 * every GPU loading the library holds until exit.  Terms as in
 * gbqv_expval_pauli_many; work is queued on `stream` (a cudaStream_t, NULL =
 * default stream) and the call returns once out / *total are written.  More
 * than 64 terms is GBQV_ERR_ARG.  The first call on a device looks up the
 * array's address (cudaGetSymbolAddress) with that device current: make it
 * before any stream capture.  The address is kept for the life of the
 * process; after a reset of the device (cudaDeviceReset) do not call this
 * entry point on that device again.  offsets[0] must be 0.  All calls share
 * the array: calls whose work overlaps on the GPU race; serialise them. */
int gbqv_expval_pauli_many_noalloc(const void *state, int num_qubits, int precision, int nterms,
                                   const uint64_t *qubits, const int *offsets, const char *const *labels,
                                   const double *coeffs, void *stream, double *out, double *total);

/* ------------------------------------------------------------------ */
/* Density-matrix surface (GBQV_DENSITY_MATRIX handles only)            */
/* ------------------------------------------------------------------ */

/* DensityMatrix::apply_superop_matrix (densitymatrix.hpp:284-288): a
 * 4^k x 4^k superoperator on qubits and qubits+n. */
int gbqv_dm_apply_superop_matrix(gbqv_handle h, const uint64_t *qubits, int k, const gbqv_c128 *mat);
/* DensityMatrix::apply_diagonal_superop_matrix (densitymatrix.hpp:290-295). */
int gbqv_dm_apply_diagonal_superop_matrix(gbqv_handle h, const uint64_t *qubits, int k,
                                          const gbqv_c128 *diag);
/* DensityMatrix::apply_unitary_matrix (densitymatrix.hpp:297-317): one 2k-qubit
 * superoperator for k <= 4, else U then conj(U) on the column qubits. */
int gbqv_dm_apply_unitary_matrix(gbqv_handle h, const uint64_t *qubits, int k, const gbqv_c128 *mat);
/* DensityMatrix::apply_diagonal_unitary_matrix (densitymatrix.hpp:319-325). */
int gbqv_dm_apply_diagonal_unitary_matrix(gbqv_handle h, const uint64_t *qubits, int k,
                                          const gbqv_c128 *diag);
/* DensityMatrix::apply_cnot / apply_swap / apply_x / apply_y / apply_phase /
 * apply_cphase / apply_toffoli (densitymatrix.hpp:331-440). */
int gbqv_dm_apply_cnot(gbqv_handle h, uint64_t ctrl, uint64_t trgt);
int gbqv_dm_apply_swap(gbqv_handle h, uint64_t q0, uint64_t q1);
int gbqv_dm_apply_x(gbqv_handle h, uint64_t q);
int gbqv_dm_apply_y(gbqv_handle h, uint64_t q);
int gbqv_dm_apply_phase(gbqv_handle h, uint64_t q, gbqv_c128 phase);
int gbqv_dm_apply_cphase(gbqv_handle h, uint64_t q0, uint64_t q1, gbqv_c128 phase);
int gbqv_dm_apply_toffoli(gbqv_handle h, uint64_t c0, uint64_t c1, uint64_t t);
/* DensityMatrix::apply_reset (densitymatrix.hpp:522-529). */
int gbqv_dm_apply_reset(gbqv_handle h, const uint64_t *qubits, int k);
/* Tr(rho), UnitaryMatrix::trace used by DensityMatrix (unitarymatrix.hpp). */
int gbqv_dm_trace(gbqv_handle h, gbqv_c128 *out);

/* ------------------------------------------------------------------ */
/* Circuits: op list, Aer's Fusion pass, execution                      */
/* ------------------------------------------------------------------ */
/* A circuit is the host-side op list that Aer's Circuit/Op hold
 * (src/framework/circuit.hpp, operations.hpp); the builder calls mirror
 * aer_compiler.py:_assemble_op (qiskit_aer/backends/aer_compiler.py:875-1020). */

int gbqv_circuit_create(int num_qubits, gbqv_circuit_t *out);
int gbqv_circuit_destroy(gbqv_circuit_t c);
/* A named gate of the statevector gate set (statevector_state.hpp:313-384),
 * params are the gate's real parameters. */
int gbqv_circuit_gate(gbqv_circuit_t c, const char *name, const uint64_t *qubits, int nq,
                      const double *params, int nparams);
/* "unitary" op (Operations::make_unitary) with a 2^k x 2^k column-major matrix. */
int gbqv_circuit_unitary(gbqv_circuit_t c, const uint64_t *qubits, int k, const gbqv_c128 *mat);
/* "diagonal" op (Operations::make_diagonal) with 2^k entries. */
int gbqv_circuit_diagonal(gbqv_circuit_t c, const uint64_t *qubits, int k, const gbqv_c128 *diag);
/* "superop" op (Operations::make_superop), 4^k x 4^k column-major. */
int gbqv_circuit_superop(gbqv_circuit_t c, const uint64_t *qubits, int k, const gbqv_c128 *mat);
/* "kraus" op: nk Kraus matrices of 2^k x 2^k, back to back. */
int gbqv_circuit_kraus(gbqv_circuit_t c, const uint64_t *qubits, int k, int nk, const gbqv_c128 *mats);
/* "reset" op. */
int gbqv_circuit_reset(gbqv_circuit_t c, const uint64_t *qubits, int k);
/* "barrier" op (ignored by fusion, Fusion::can_ignore fusion.hpp:120-129). */
int gbqv_circuit_barrier(gbqv_circuit_t c, const uint64_t *qubits, int k);
int gbqv_circuit_num_ops(gbqv_circuit_t c, int *out);
/* Op i: type (see gbqv_op_type), number of qubits, and its qubits (up to
 * max_qubits written); name is copied into name_buf (NUL-terminated). */
enum gbqv_op_type { GBQV_OP_GATE = 0, GBQV_OP_MATRIX = 1, GBQV_OP_DIAGONAL = 2,
                    GBQV_OP_SUPEROP = 3, GBQV_OP_KRAUS = 4, GBQV_OP_RESET = 5,
                    GBQV_OP_BARRIER = 6 };
int gbqv_circuit_op_info(gbqv_circuit_t c, int i, int *type, int *nq, uint64_t *qubits,
                         int max_qubits, char *name_buf, int name_len);
/* Matrix (MATRIX: 4^k entries; DIAGONAL: 2^k; SUPEROP: 16^k) of op i. */
int gbqv_circuit_op_matrix(gbqv_circuit_t c, int i, gbqv_c128 *out, uint64_t len);

/* Fusion configuration, Fusion::set_config (transpile/fusion.hpp:722-748)
 * with the per-method defaults of Executor::transpile_fusion
 * (simulators/circuit_executor.hpp:1228-1287). */
typedef struct {
  int method;          /* 0 = statevector, 1 = density_matrix                 */
  int enable;          /* fusion_enable (default 1)                           */
  int max_qubit;       /* fusion_max_qubit (statevector 5, density matrix 2)  */
  int threshold;       /* fusion_threshold (statevector 14, density matrix 7) */
  double cost_factor;  /* fusion_cost_factor (1.8)                            */
  int avx2_costs;      /* 1: CostBasedFusion AVX2 cost table (fusion.hpp:1119)*/
  int allow_superop;   /* set when the op set holds superop/kraus/reset       */
  int allow_kraus;
} gbqv_fusion_config;

/* Fills the defaults for method 0 = statevector, 1 = density_matrix. */
int gbqv_fusion_default_config(int method, gbqv_fusion_config *cfg);
/* Fusion::optimize_circuit (fusion.hpp:750-846) in place.  *applied gets the
 * "applied" metadata flag, *method_name (may be NULL) "unitary"/"superop"/
 * "kraus", written into a buffer of method_len bytes. */
int gbqv_circuit_fuse(gbqv_circuit_t c, const gbqv_fusion_config *cfg, int *applied,
                      char *method_name, int method_len);

/* Apply every op of c to the state (State::apply_ops, state.hpp:295-340),
 * dispatching gates as Statevector::State::apply_gate
 * (statevector_state.hpp:733-865) or DensityMatrix::State::apply_gate
 * (densitymatrix_state.hpp:641-850).  Runs of dense/diagonal ops are
 * scheduled into cache-blocked passes over HBM. */
int gbqv_execute(gbqv_handle h, gbqv_circuit_t c);

/* ------------------------------------------------------------------ */
/* Runtime parameter binding: one circuit, many parameter sets            */
/* ------------------------------------------------------------------ */
/* Gives parameter param_pos of gate op_index one value per binding: the
 * "parameterizations" table that Controller::execute expands with
 * runtime_parameter_bind_enable (src/controllers/controller_execute.hpp:
 * 104-131; the Python side builds it in qiskit_aer/backends/aerbackend.py:
 * 96-144).  Every call on a circuit passes the same nbind; values[j] is
 * binding j's value.  Out-of-range positions are GBQV_ERR_ARG with the
 * reference's messages.  Bound gates are left out of Fusion. */
int gbqv_circuit_bind_param(gbqv_circuit_t c, int op_index, int param_pos, int nbind, const double *values);
int gbqv_circuit_num_bindings(gbqv_circuit_t c, int *out);

/* Runs bindings [first, first + count) of a bound circuit of n qubits at
 * once, the work the batched-shots executor does for parameter bindings on
 * a GPU (src/simulators/batch_shots_executor.hpp:152-314, ops converted by
 * transpile/batch_converter.hpp:54-200).  h holds a stack of 2^b states of n
 * qubits (h has n + b qubits, 2^b >= count): state j, amplitudes
 * [j 2^n, (j + 1) 2^n), starts in |0...0> and ends as binding first + j
 * applied to it; states j >= count are zero.  Gates with bound parameters
 * run as per-binding matrices inside cache-blocked passes.  The circuit must
 * be unitary (gates, unitary, diagonal, barrier): GBQV_ERR_KIND otherwise. */
int gbqv_execute_bound(gbqv_handle h, gbqv_circuit_t c, uint64_t first, uint64_t count);

/* <P_t> on each of the first nseg states of such a stack (states of
 * 2^state_qubits amplitudes, terms on qubits below state_qubits, laid out as
 * in gbqv_expval_pauli_many): out[t * nseg + s] = <psi_s|P_t|psi_s>
 * (QubitVector::expval_pauli per state, qubitvector.hpp:2299-2347). */
int gbqv_expval_pauli_segments(gbqv_handle h, int state_qubits, uint64_t nseg, int nterms, const uint64_t *qubits,
                               const int *offsets, const char *const *labels, double *out);
/* QubitVector::sample_measure (qubitvector.hpp:2148-2228) on states first ..
 * first + nseg - 1 of such a stack, each exactly as a state of its own:
 * state first + s draws with rnds[s * shots .. (s + 1) * shots) into
 * out[s * shots ..] (indices within the state). */
int gbqv_sample_measure_segments(gbqv_handle h, int state_qubits, uint64_t first, uint64_t nseg,
                                 const double *rnds, uint64_t shots, uint64_t *out);

/* Batched shots of a circuit that cannot be measure-sampled (mid-circuit
 * measurements, resets, classically conditioned ops): shot s of a group is
 * state s of such a stack, the work QubitVectorThrust's batched-shots hooks
 * do (apply_batched_measure / apply_batched_reset,
 * src/simulators/statevector/qubitvector_thrust.hpp:2251-2448, conditions
 * through set_batched_system_conditional, :2568).  The classical memory and
 * each shot's RNG stay with the caller.
 *
 * initialize_segments: states 0..count-1 to |0...0>, the rest zero.
 * execute_segments: the unitary ops of c (n qubits, n <= the handle's) on
 *   every state of the stack at once (no size match needed).
 * probabilities_segments: out[s * 2^k + v] = the probability of outcome v
 *   (bit j on qubits[j], k <= state_qubits) in state s
 *   (QubitVector::probabilities, qubitvector.hpp:2089-2143, per state).
 * draw_segments: for registers of k >= 10 qubits, the probabilities and
 *   each state's outcome drawn on the device (RngEngine::rand_int,
 *   rng.hpp:94-96, with the uniform u[s]; u[s] < 0 draws nothing and gives
 *   outcome 0xffffffff): outcome[s] and its probability prob[s].  Parallel
 *   sums: an outcome can differ from the sequential draw only when u[s] lies
 *   within a few ulps of a cumulative boundary.
 * collapse_segments: State::measure_reset_update (statevector_state.hpp:
 *   936-1011) per state: the amplitude of outcome meas_state[s] times
 *   scale[s] (1/sqrt(p)) moves to outcome final_state[s] (the measured value
 *   for a measurement, 0 for a reset), the others become 0;
 *   meas_state[s] = 0xffffffff leaves state s untouched.
 * apply_matrix_segments: a k <= 4 qubit matrix (column-major) on the states
 *   whose mask[s] is non-zero (a classically conditioned gate). */
int gbqv_initialize_segments(gbqv_handle h, int state_qubits, uint64_t count);
int gbqv_execute_segments(gbqv_handle h, gbqv_circuit_t c);
int gbqv_probabilities_segments(gbqv_handle h, int state_qubits, uint64_t nseg, const uint64_t *qubits, int k,
                                double *out);
int gbqv_draw_segments(gbqv_handle h, int state_qubits, uint64_t nseg, const uint64_t *qubits, int k,
                       const double *u, uint32_t *outcome, double *prob);
int gbqv_collapse_segments(gbqv_handle h, int state_qubits, uint64_t nseg, const uint64_t *qubits, int k,
                           const uint32_t *meas_state, const uint32_t *final_state, const double *scale);
int gbqv_apply_matrix_segments(gbqv_handle h, int state_qubits, uint64_t nseg, const uint64_t *qubits, int k,
                               const gbqv_c128 *mat, const uint8_t *mask);

/* Sampled Kraus noise on a stack of shots (the statevector method's Kraus
 * noise, State::apply_kraus, src/simulators/statevector/
 * statevector_state.hpp:1112-1156, one shot per state).
 *
 * rdm_segments: out[(s D + a) D + b] = rho_s[a][b] = sum over the other
 *   qubits of x_a conj(x_b) in state s (D = 2^k, k <= 3, bit j of a on
 *   qubits[j]): the caller gets every operator's probability
 *   ||K psi_s||^2 = tr(K^dag K rho_s), the QubitVector::norm(qubits, mat)
 *   of apply_kraus (qubitvector.hpp:1878-2082), from one pass.
 * kraus_segments: state s gets mats[branch[s]] (m <= 255 column-major
 *   matrices) with every entry times scale[s] (1/sqrt(p), as apply_kraus
 *   scales the chosen matrix); branch[s] = 255 leaves state s untouched. */
int gbqv_rdm_segments(gbqv_handle h, int state_qubits, uint64_t nseg, const uint64_t *qubits, int k,
                      gbqv_c128 *out);
int gbqv_kraus_segments(gbqv_handle h, int state_qubits, uint64_t nseg, const uint64_t *qubits, int k,
                        const gbqv_c128 *mats, int m, const uint8_t *branch, const double *scale);

/* Adjoint-method gradient of E(theta) = <psi(theta)|H|psi(theta)>, psi =
 * c applied to |0...0>.  No counterpart in the reference (Aer has no gradient
 * code); it extends the statevector surface for the torch.autograd wrapper.
 * param_of_op[i] is -1 for a fixed op, else the index of the parameter that
 * replaces params[0] of gate i, which must be rx, ry, rz, rxx, ryy, rzz or
 * rzx (U = exp(-i theta P / 2)).  H = sum_t coeffs[t] P_t with the Pauli
 * terms laid out as in gbqv_expval_pauli_many.  Writes E to *energy and
 * dE/dparams to grad[0..nparams).  Uses two state buffers (the handle's and
 * one scratch buffer of the same size); on return the handle holds the
 * state after the first op (the end point of the reverse sweep). */
int gbqv_adjoint_expval_grad(gbqv_handle h, gbqv_circuit_t c, const int *param_of_op, const double *params,
                             int nparams, int nterms, const uint64_t *qubits, const int *offsets,
                             const char *const *labels, const double *coeffs, double *energy, double *grad);

/* ------------------------------------------------------------------ */
/* Batches of independent instances of uneven size in one launch        */
/* (the role of the batched-shots / parameter-bind executor,            */
/* src/simulators/batch_shots_executor.hpp:39-314, which batches        */
/* equal-size states only).                                             */
/* ------------------------------------------------------------------ */

/* Gate kinds of a batch instance: 0 RX, 1 RY, 2 RZ (rotations reading
 * params[param_of_gate[i]]), 3 CX, 4 CZ (control, target), 5 H. */
int gbqv_batch_create(int precision, gbqv_batch_t *out);
int gbqv_batch_destroy(gbqv_batch_t b);
/* Add an instance: num_qubits <= 30; ngates gates with kinds[i], qubits
 * [2*i, 2*i+1] (the second is ignored for 1-qubit kinds); a Hamiltonian laid
 * out as in gbqv_expval_pauli_many; `shots` samples from the RngEngine stream
 * of `seed` (gbqv_uniforms).  *index receives the instance number. */
int gbqv_batch_add(gbqv_batch_t b, int num_qubits, int ngates, const int *kinds, const uint64_t *qubits,
                   const int *param_of_gate, const double *params, int nparams, int nterms, const uint64_t *tq,
                   const int *toffsets, const char *const *labels, const double *coeffs, uint64_t shots,
                   uint64_t seed, int *index);
/* Teams: the costliest instances (at most max_team_instances <= 64, cost =
 * gates x 2^qubits at least min_cost_fraction of the largest, spanning two or
 * more tiles) run on two CTAs each, splitting every run's tiles and meeting at
 * a bounded barrier after each run (GBQV_ERR_TIMEOUT if one gives up).  Set
 * before the first gbqv_batch_run; default 64 and 0.5. */
int gbqv_batch_set_teams(gbqv_batch_t b, int max_team_instances, double min_cost_fraction);
/* Complex128 batches: on != 0 runs the gates, the Hamiltonian and the
 * generator sums in FP64; the default holds the states as pairs of floats
 * (~48-bit arithmetic on the FP32 pipe, 16 bytes per amplitude like
 * complex128, errors near 1e-14), with energies, gradients and sampling
 * probabilities accumulated in double.  Set before the first
 * gbqv_batch_run. */
int gbqv_batch_set_fp64(gbqv_batch_t b, int on);
/* Run every instance in one persistent kernel launch (captured once as a CUDA
 * graph and replayed on later calls): forward pass, `shots` samples of the
 * final state, E = <H>, and with want_grad the adjoint gradient dE/dparams.
 * *elapsed_ms gets the device time of the launch. */
int gbqv_batch_run(gbqv_batch_t b, int want_grad, double *elapsed_ms);
/* Results of instance i (any pointer may be NULL); latency = device time
 * from the instance's start to its end inside the launch. */
int gbqv_batch_result(gbqv_batch_t b, int i, double *energy, double *grad, int nparams, uint64_t *samples,
                      uint64_t shots, double *latency_ms);

/* Test hook of the failure path (no reference counterpart).  enable = 1:
 * later complex128 dense gates on the tcgen05 kernel withhold the commit of
 * each CTA's first accumulator, so that tile's epilogue waits on an mbarrier
 * that nothing completes; its bounded wait gives up after 2 s, the CTA
 * drains its copies and MMAs, frees its tensor memory and returns, and the
 * next synchronising call fails with GBQV_ERR_TIMEOUT (the state's contents
 * are then invalid).  enable = 0 restores normal operation.  No GPU fault is
 * involved: it exercises the same bounded waits that guard a real stall. */
int gbqv_test_stall_tensor_pipeline(gbqv_handle h, int enable);

/* Execution policy for gbqv_execute (no reference counterpart: Aer applies
 * one op per pass).  blocking = 0 applies one kernel per op; 1 (default)
 * schedules runs of small ops into cache-blocked passes whose tile is held
 * in registers; 2 the same passes with the tile swept in shared memory op by
 * op.  Bound execution (gbqv_execute_bound) always uses runs, mode 2 picks
 * the shared-memory form there too. */
int gbqv_set_blocking(gbqv_handle h, int blocking);

/* Tile of the cache-blocked runs (no reference counterpart; Aer's nearest
 * knob is its configured cache-blocking qubit count, cacheblocking.hpp:
 * 130-131): a run's ops act inside tiles of 2^tile_qubits amplitudes, one
 * read and write of the state per run.  0 (default) = 12 qubits at
 * complex128, 13 at complex64; otherwise 10..12 / 10..13.  Smaller tiles
 * hold fewer ops per run; the autotuner picks it per workload by timing. */
int gbqv_set_run_tile_qubits(gbqv_handle h, int tile_qubits);

/* Register-tile runs compiled for their op sequence (no reference
 * counterpart; Aer's GPU path interprets every gate the same way).  A run
 * whose structure (ops, qubits, matrix offsets) recurs — the same circuit
 * over new parameter bindings — is compiled once by NVRTC into a kernel with
 * every op's bits fixed, the matrices staying data; results are those of the
 * interpreting kernel.  mode 0: never; 1 (default): from a structure's
 * second execution on (the first runs the interpreting kernel; compiling
 * takes about a second); 2: from the first.  Without NVRTC the interpreting
 * kernel runs. */
int gbqv_set_run_jit(gbqv_handle h, int mode);

/* Host check of the specialised-run source generator: generates the kernel
 * of a synthetic run using every op kind and compiles it with NVRTC for
 * sm_103a (no GPU needed).  0 on success; 1 when it did not compile, with
 * NVRTC's log in `log` (up to cap - 1 bytes, NUL-terminated); GBQV_ERR_ARG
 * when NVRTC is not available. */
int gbqv_run_jit_compile_check(int double_precision, char *log, size_t cap);

/* Process-wide counts of specialised run kernels compiled and launched. */
int gbqv_run_jit_counts(uint64_t *compiled, uint64_t *launched);

/* Arithmetic of complex128 dense gates on 4 or 5 qubits (no reference
 * counterpart).  1 (default): exact digit slices on the tensor cores, error
 * <= ~1e-13 of (row max x group max) per gate (4-qubit gates on tcgen05 with
 * TMEM accumulators for states of >= 11 vector qubits, otherwise warp-level
 * mma.sync); 2: the same digit slices on mma.sync only; 0: native FP64 FMAs
 * (the reference's arithmetic, 1.2 TFLOP/s on GB300).  On a complex64 state
 * the same setting selects, for 4-qubit dense gates on >= 11 vector qubits,
 * tcgen05 products in split precision (3xTF32, fp32 accumulation; value 1)
 * or fp32 FMAs (0 or 2).  At complex128 a non-zero value also lets the
 * runs compiled for their op sequence (gbqv_set_run_jit) hold their register
 * amplitudes as float pairs (~48 significant bits on the FP32 pipe); 0 keeps
 * them in FP64.  Other values return GBQV_ERR_ARG.  A tcgen05 kernel whose bounded pipeline wait gave up makes
 * the next synchronising call return GBQV_ERR_TIMEOUT. */
int gbqv_set_tensor_c128(gbqv_handle h, int enable);

#ifdef __cplusplus
}
#endif

#endif /* GBQV_H_ */
