// gbqv_internal.h — declarations shared by the host side of libgbqv
// (gbqv_capi.cpp, gbqv_circuit.cpp) and the CUDA kernels (gbqv_kernels.cu).
// Nothing here crosses the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <complex>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

struct gbqv_state;

namespace gbqv {

using cd = std::complex<double>;
using reg_t = std::vector<uint64_t>;

// Thrown inside the library, turned into a status code at the C ABI.
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

void cuda_check(cudaError_t e, const char *what);
// Number of kernels launched by the library (incremented after each launch).
uint64_t launch_count();

// Limits of the kernels.
constexpr int kMaxQubits = 40;         // 2^40 c64 = 8 TB: capped by memory anyway
constexpr int kMaxDenseParamK = 5;     // dense k <= 5: matrix passed as kernel parameter
constexpr int kMaxDenseK = 13;         // dense k <= 13: matrix in device memory, group in smem
constexpr int kMaxDiagK = 10;          // diagonal entries passed as kernel parameter
constexpr int kMaxPermPairs = 1024;
constexpr int kReduceBlocks = 152 * 4; // 4 CTAs per SM on a GB300
constexpr int kReduceThreads = 256;
constexpr int kMaxTerms = 4096;        // Pauli terms per reduction launch

// Per-handle device state.  Scratch buffers grow on demand and live until
// the handle is destroyed.
struct Device {
  int n = 0;            // vector qubits (2 * logical for a density matrix)
  int nq = 0;           // logical qubits
  bool dbl = true;      // complex128 (true) or complex64 (false)
  bool density = false;
  bool unitary = false;     // UnitaryMatrix: 2 nq vector qubits, identity at initialisation
  int blocking = 1;         // 0 one kernel per op, 1 register-tile runs, 2 shared-memory runs
  int run_tile_bits = 0;    // tile qubits of the cache-blocked runs (0: 12 at complex128, 13 at complex64)
  int tensor_c128 = 1;      // complex128 dense k = 4, 5: 0 FP64 cores, 1 tensor (tcgen05 for k = 4), 2 mma.sync only
  int sample_index_size = 10;  // QubitVector::sample_measure_index_size_ (2^this blocks)
  int *tc_status = nullptr; // device word raised by a tcgen05 kernel whose bounded wait gave up
  int tc_test_stall = 0;    // test hook: the tcgen05 complex128 kernel withholds its first tile's commit
  int run_jit = 1;          // register-tile runs compiled for their op sequence: 0 never, 1 from a run's second use, 2 always
  // tcgen05 kernel: 128-byte-swizzled TMA descriptors of the state viewed as
  // rows of 8 amplitudes, box height 2^(L-3) for run length L = 7..12; built
  // on first use, dropped when the state buffer changes
  const void *tmap_state = nullptr;
  unsigned tmap_ok = 0;  // bit L-7: tmap[L-7] is valid
  alignas(128) unsigned char tmap[6][128];  // CUtensorMap storage (128-byte aligned)
  void *state = nullptr;
  void *ckpt = nullptr;
  cudaStream_t stream = nullptr;
  // scratch
  double *partials = nullptr; size_t partials_cap = 0;   // reduction partials
  double *results = nullptr;  size_t results_cap = 0;    // reduction outputs (device)
  double *h_results = nullptr; size_t h_results_cap = 0; // pinned host mirror
  void *mat = nullptr; size_t mat_cap = 0;               // large matrices
  void *aux = nullptr; size_t aux_cap = 0;               // sampling / probabilities
  void *aux2 = nullptr; size_t aux2_cap = 0;
  void *probs = nullptr; size_t probs_cap = 0;           // sampling: every outcome's probability
  uint64_t amps() const { return 1ULL << n; }
  size_t amp_bytes() const { return dbl ? 16 : 8; }
};

void *grow(void *&buf, size_t &cap, size_t bytes);
Device &device_of(gbqv_state *h);
// Records the message for gbqv_last_error(h) (h == nullptr: thread-local).
void set_last_error(gbqv_state *h, const std::string &msg);

// ---- launchers (gbqv_kernels.cu); all are asynchronous on dev.stream ----
void launch_dense(Device &dev, const reg_t &qubits, const cd *mat);
void launch_diagonal(Device &dev, const reg_t &qubits, const cd *diag);
// mc kinds: 0 = X, 1 = Y, 2 = phase (mat[0] = phase), 3 = U (mat = 2x2),
// 4 = diagonal U (mat[0], mat[1]), 5 = SWAP of the last two qubits
void launch_mc(Device &dev, const reg_t &qubits, int kind, const cd *mat);
void launch_swaps(Device &dev, const reg_t &qubits, const std::vector<std::pair<uint32_t, uint32_t>> &pairs);
void launch_pauli(Device &dev, uint64_t x_mask, uint64_t z_mask, uint64_t x_max, cd phase);
void launch_dm_y(Device &dev, uint64_t q);
void launch_scale(Device &dev, cd s);
void launch_set_basis(Device &dev, uint64_t index, cd value); // zero + one entry
void launch_set_identity(Device &dev);                         // unitary: vec(I) over 2 nq qubits
// complex64 states: state[offset, +count) <- narrow(src) / dst <- widen(state[offset, +count));
// src and dst are device buffers of complex128
void launch_narrow(Device &dev, const void *src, uint64_t offset, uint64_t count);
void launch_copy_in(Device &dev, const void *src, uint64_t offset, uint64_t count);  // complex128 states
void launch_widen(Device &dev, uint64_t offset, uint64_t count, void *dst);

// Reductions: write results into dev.results[0..count) (device), async.
void reduce_norm(Device &dev);                                   // 1 value
void reduce_norm_matrix(Device &dev, const reg_t &qubits, const cd *mat); // 1 value
struct PauliTerm { uint64_t x_mask, z_mask, x_max; double ph_re, ph_im; int diag_only; };
void reduce_expval(Device &dev, const std::vector<PauliTerm> &terms); // terms.size() values
void reduce_dm_expval(Device &dev, const std::vector<PauliTerm> &terms);
void reduce_inner_product(Device &dev);                          // 2 values (re, im)
void reduce_probabilities(Device &dev, const reg_t &qubits);     // 2^k values
void reduce_dm_trace(Device &dev);                               // 2 values
// Probabilities of every basis state into a device buffer of 2^nq doubles.
void probabilities_all(Device &dev, double *d_out);
// Sampling: rnds/out are device buffers of `shots` entries.  amp_offset /
// nbits (>= 0) sample the 2^nbits-amplitude statevector starting at that
// amplitude (one state of a stack) instead of the whole state.
void sample_measure(Device &dev, const double *d_rnds, uint64_t shots, uint64_t *d_out, uint64_t amp_offset = 0,
                    int nbits = -1);

// Adjoint gradients: out = sum_t c_t P_t src (one pass), and
// <lam|P|psi> into dev.results[2*slot .. 2*slot+1] (re, im).
struct HamTerm { uint64_t x_mask, z_mask; double re, im; };
void ham_apply(Device &dev, const void *src, void *dst, const std::vector<HamTerm> &terms);
// One 1-qubit sweep step on a complex128 state held as float pairs (16
// bytes per amplitude; adjoint_to_pairs / adjoint_from_pairs convert in
// place): with slot >= 0 first results[2 slot..] = <lam| phase X^gx Z^gz
// |psi> (generator on bit q), then, with apply, psi <- m psi and lam <- m lam
// (m column-major, form 0 general, 1 real, 2 diagonal).
// Up to 3 consecutive 1-qubit sweep steps on distinct qubits in one pass
// (psi, lam as complex64 / complex128, or as float pairs): per step the
// inverse matrix (column-major, form 0 general, 1 real, 2 diagonal), the
// generator bits (on the step's qubit) and phase, and the result slot (-1:
// no inner product).
struct AdjStepHost {
  int q = 0, form = 0;
  bool gx = false, gz = false;
  cd m[4];
  cd phase = 1.0;
  int slot = -1;
};
void adjoint_steps(Device &dev, void *psi, void *lam, const std::vector<AdjStepHost> &steps, bool pairs);
// A product of CX, X and SWAP gates as one gather pass, out[y] = in[src(y)]:
// src(y) = y ^ c ^ (xor of d[k] over the qubits q[k] whose bit is set in y).
struct LinearGatherHost {
  std::vector<int> q;
  std::vector<uint64_t> d;
  uint64_t c = 0;
};
void gather_linear(Device &dev, const void *in, void *out, const LinearGatherHost &g);
void adjoint_to_pairs(Device &dev, void *a);
void adjoint_from_pairs(Device &dev, void *a);
// lam = H psi with psi and lam as float pairs (complex128 adjoint sweep).
void ham_apply_pairs(Device &dev, const void *src, void *dst, const std::vector<HamTerm> &terms);
void adjoint_step_pairs(Device &dev, void *psi, void *lam, int q, const cd *m, int form, bool gx, bool gz, cd phase,
                        int slot, bool apply);
void reduce_pauli_inner(Device &dev, const void *lam, const void *psi, uint64_t x_mask, uint64_t z_mask, cd phase,
                        int slot);

// Fused-run (cache-blocked) execution: a run of dense/diagonal ops whose
// qubits all lie inside one tile of `tile_bits` vector qubits.
struct RunOp {
  int kind;       // 0 dense, 1 diagonal, 2 multi-controlled X (last qubit the target; no matrix)
  reg_t qubits;
  std::vector<cd> mat;
  // Bound runs (runtime parameter binding): one matrix per binding, binding
  // j at [j * mat size, (j + 1) * mat size); empty for an op that all
  // bindings share (its matrix is `mat`).
  std::vector<cd> bmat;
};
// A run over a stack of bound states: state j holds binding first + j, at
// amplitudes [j 2^state_bits, (j + 1) 2^state_bits); states j >= count are
// padding and are left untouched.
struct RunBound {
  int state_bits;
  uint64_t first, count;
};
// complex128 dense gates of 4 / 5 qubits on the tensor cores (exact digit
// slices, gbqv_ozaki.h): tcgen05 + TMEM for 4 qubits (gbqv_tc.cu), warp-level
// mma.sync for 5 qubits and for tensor mode 2.
bool tensor_dense_available(const Device &dev, int k);
void launch_dense_tensor(Device &dev, const reg_t &qubits, const cd *mat);
bool tc_dense_available(const Device &dev, int k);
void launch_dense_tc(Device &dev, const reg_t &qubits, const cd *mat);
void tc_matrix4(const cd *mat, uint16_t *planes, int *rowkey);
// Shared by the tcgen05 kernels (gbqv_tc.cu, gbqv_tc64.cu): tile run
// geometry, the swizzled TMA descriptor of the state for run length L
// (CUtensorMap, 128 bytes), the SM count.
void tc_tile_geometry(const reg_t &qubits, uint64_t *hoff, uint32_t *roff, uint16_t *zl, uint32_t &nruns,
                      uint32_t &runbytes, uint32_t amp_bytes);
bool tc_tensor_map(Device &dev, uint32_t L, void *out);
bool tc_runs_map(Device &dev, const reg_t &qubits, uint32_t L, void *out, uint32_t &rank, uint32_t &nreq,
                 uint32_t *row_off);
int sm_count();
// complex128 dense 5-qubit gates on tcgen05 (gbqv_tc.cu): usable when the
// highest target lies above the tile's run bits
bool tc5_usable(const Device &dev, const reg_t &qubits);
void launch_dense_tc5(Device &dev, const reg_t &qubits, const cd *mat);
// complex64 dense 4-qubit gates on tcgen05 (3xTF32, gbqv_tc64.cu)
bool tc64_dense_available(const Device &dev, int k);
void launch_dense_tc64(Device &dev, const reg_t &qubits, const cd *mat);
// Device word that a bounded wait of a tcgen05 kernel sets when it gives up;
// sync() turns it into GBQV_ERR_TIMEOUT.
int *tc_status_word(Device &dev);

// Group geometry shared by the kernels: lowmask[j] = 2^(sorted qubit j) - 1;
// offs[i] = the amplitude offset of local index i (qubits[j] = bit j of i).
void sorted_masks(const reg_t &qubits, uint64_t *lowmask);
void local_offsets(const reg_t &qubits, uint64_t *offs);
// Counts a launch and turns a launch error into an exception.
void check_launch(const char *what);

// Dispatch rules of the reference members, shared by the C ABI and the
// circuit executor (gbqv_capi.cpp).
void apply_matrix_impl(Device &dev, const reg_t &q, const cd *mat);
void apply_diag_impl(Device &dev, const reg_t &q, const cd *diag);
void apply_mcu_impl(Device &dev, const reg_t &q, const cd *mat);
reg_t superop_qubits(const Device &d, const reg_t &q);
void dm_unitary(Device &d, const reg_t &q, const cd *mat);
void dm_diag_unitary(Device &d, const reg_t &q, const cd *diag);

// Tile geometry of the run kernel for this state: tile qubits (m), the low
// qubits every tile contains (c), the matrix pool size in complex128 units,
// and the longest run.
int run_tile_qubits(const Device &dev);
int run_low_qubits(const Device &dev);
size_t run_pool_bytes(const Device &dev);
int run_max_ops();
void launch_run(Device &dev, const std::vector<const RunOp *> &ops, const RunBound *bound = nullptr);
// The register-tile form of a run (gbqv_runreg.cu), given the tile qubits
// (ascending) and the length c of their contiguous low prefix; false when the
// run has an op it does not take or the tile is too small.
// NVRTC found (the specialised runs of gbqv_runreg.cu can be compiled), and
// the host check of their source generator (0: compiled; log on failure).
bool run_jit_available();
void run_jit_counts(uint64_t &compiled, uint64_t &launched);
int run_jit_compile_check(bool dbl, std::string &log);
bool launch_run_reg(Device &dev, const std::vector<const RunOp *> &ops, const std::vector<int> &tile_qubits, int c,
                    const RunBound *bound);
// Bytes of per-binding matrices one bound run may hold per binding.
size_t run_bound_pool_bytes(const Device &dev);
// Every state of a stack of 2^state_bits-amplitude states: |0...0> for the
// first `count`, zero for the rest.
void launch_set_basis_segments(Device &dev, int state_bits, uint64_t count);
// Expectation values of `terms` on each of the first nseg states of a stack
// of 2^state_bits-amplitude states, into dev.results[t * nseg + s].
void reduce_expval_segments(Device &dev, const std::vector<PauliTerm> &terms, int state_bits, uint64_t nseg);

// batched shots (gbqv_shots.cu): per-state probabilities (nseg 2^k values
// in dev.results), collapse and a masked matrix over a stack of states
int seg_max_measure_qubits();
int seg_max_matrix_qubits();
void reduce_probabilities_segments(Device &dev, const reg_t &qubits, int state_bits, uint64_t nseg);
void launch_collapse_segments(Device &dev, const reg_t &qubits, int state_bits, uint64_t nseg, const uint32_t *meas,
                              const uint32_t *fin, const double *scale);
void launch_matrix_segments(Device &dev, const reg_t &qubits, int state_bits, uint64_t nseg, const cd *mat,
                            const uint8_t *mask);
void draw_segments(Device &dev, const reg_t &qubits, int state_bits, uint64_t nseg, const double *u,
                   uint32_t *outcome, double *prob);
// sampled Kraus noise: per-state reduced density matrices of k <= 3 qubits
// (nseg 4^k values in dev.results) and the chosen operator per state
int seg_max_kraus_qubits();
void reduce_rdm_segments(Device &dev, const reg_t &qubits, int state_bits, uint64_t nseg);
void launch_kraus_segments(Device &dev, const reg_t &qubits, int state_bits, uint64_t nseg, const cd *mats, int m,
                           const uint8_t *branch, const double *scale);

}  // namespace gbqv
