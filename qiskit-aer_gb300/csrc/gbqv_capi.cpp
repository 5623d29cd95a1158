// gbqv_capi.cpp — the C ABI of libgbqv (include/gbqv.h): handle lifetime,
// argument checks and the reference's per-member dispatch rules, on top of
// the kernels in gbqv_kernels.cu.  No exception crosses the ABI.
#include "../../include/gbqv.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <random>
#include <string>

#include "gbqv_internal.h"
#include "gbqv_gates.h"

struct gbqv_state {
  gbqv::Device dev;
  std::string err;
  uint64_t *io = nullptr;  // device staging for shots / samples / large outputs
  size_t io_cap = 0;
};

namespace gbqv {

void cuda_check(cudaError_t e, const char *what) {
  if (e != cudaSuccess) {
    cudaGetLastError();  // clear a non-sticky error
    const int code = (e == cudaErrorMemoryAllocation) ? GBQV_ERR_ALLOC : GBQV_ERR_CUDA;
    throw Error(code, std::string(what) + ": " + cudaGetErrorString(e));
  }
}

void *grow(void *&buf, size_t &cap, size_t bytes) {
  if (bytes <= cap && buf) return buf;
  if (buf) cudaFree(buf);
  buf = nullptr;
  cap = 0;
  const size_t want = std::max<size_t>(bytes, 4096);
  cuda_check(cudaMalloc(&buf, want), "scratch allocation");
  cap = want;
  return buf;
}

}  // namespace gbqv

namespace {
thread_local std::string g_err;
}

namespace gbqv {
Device &device_of(gbqv_state *h) { return h->dev; }
void set_last_error(gbqv_state *h, const std::string &msg) { (h ? h->err : g_err) = msg; }
}  // namespace gbqv

using namespace gbqv;

namespace {

template <typename F>
int guard(gbqv_handle h, F &&f) {
  try {
    f();
    return GBQV_OK;
  } catch (const Error &e) {
    (h ? h->err : g_err) = e.what();
    return e.code;
  } catch (const std::bad_alloc &) {
    (h ? h->err : g_err) = "host allocation failed";
    return GBQV_ERR_ALLOC;
  } catch (const std::exception &e) {
    (h ? h->err : g_err) = e.what();
    return GBQV_ERR_ARG;
  }
}

#define REQUIRE(cond, code, msg) \
  do {                           \
    if (!(cond)) throw Error(code, msg); \
  } while (0)

void need_handle(gbqv_handle h) {
  if (!h) throw Error(GBQV_ERR_ARG, "null state handle");
}

// QubitVector::check_qubit semantics (qubitvector.hpp:698-747) plus the
// distinctness every gate assumes.
reg_t check_qubits(const uint64_t *qubits, int k, int limit, const char *what, int kmin = 1) {
  REQUIRE(k >= kmin, GBQV_ERR_ARG, std::string(what) + ": too few qubits");
  REQUIRE(qubits || k == 0, GBQV_ERR_ARG, std::string(what) + ": null qubit list");
  reg_t q(qubits, qubits + k);
  for (int i = 0; i < k; ++i) {
    REQUIRE(q[i] < (uint64_t)limit, GBQV_ERR_QUBIT,
            std::string(what) + ": qubit index " + std::to_string(q[i]) + " out of range for " +
                std::to_string(limit) + " qubits");
    for (int j = 0; j < i; ++j)
      REQUIRE(q[i] != q[j], GBQV_ERR_QUBIT, std::string(what) + ": repeated qubit " + std::to_string(q[i]));
  }
  return q;
}

const cd *as_cd(const gbqv_c128 *p) { return reinterpret_cast<const cd *>(p); }
cd as_cd(gbqv_c128 z) { return cd(z.re, z.im); }

}  // namespace

namespace gbqv {

// Raises GBQV_ERR_TIMEOUT when a tcgen05 kernel's bounded wait gave up since
// the last check (the word is cleared for the next launches).
void check_tc_status(Device &dev) {
  if (!dev.tc_status) return;
  int word = 0;
  cuda_check(cudaMemcpyAsync(&word, dev.tc_status, sizeof(int), cudaMemcpyDeviceToHost, dev.stream), "status read");
  cuda_check(cudaStreamSynchronize(dev.stream), "stream synchronize");
  if (word) {
    cuda_check(cudaMemsetAsync(dev.tc_status, 0, sizeof(int), dev.stream), "status reset");
    throw Error(GBQV_ERR_TIMEOUT, "a tensor-core pipeline wait timed out; the results of that gate are invalid");
  }
}

int *tc_status_word(Device &dev) {
  if (!dev.tc_status) {
    cuda_check(cudaMalloc(&dev.tc_status, sizeof(int)), "status allocation");
    cuda_check(cudaMemsetAsync(dev.tc_status, 0, sizeof(int), dev.stream), "status reset");
  }
  return dev.tc_status;
}

void sync(Device &dev) {
  cuda_check(cudaStreamSynchronize(dev.stream), "stream synchronize");
  check_tc_status(dev);
}

// Copies n doubles of dev.results into out (host) and waits.
void read_results(Device &dev, double *out, size_t n) {
  if (dev.h_results_cap < n * sizeof(double)) {
    if (dev.h_results) cudaFreeHost(dev.h_results);
    dev.h_results = nullptr;
    dev.h_results_cap = 0;
    cuda_check(cudaMallocHost(&dev.h_results, std::max<size_t>(n * sizeof(double), 4096)), "pinned allocation");
    dev.h_results_cap = std::max<size_t>(n * sizeof(double), 4096);
  }
  cuda_check(cudaMemcpyAsync(dev.h_results, dev.results, n * sizeof(double), cudaMemcpyDeviceToHost, dev.stream),
             "result copy");
  sync(dev);
  std::memcpy(out, dev.h_results, n * sizeof(double));
}

}  // namespace gbqv

namespace {

void require_density(Device &dev, const char *what) {
  REQUIRE(dev.density, GBQV_ERR_KIND, std::string(what) + " needs a density-matrix state");
}

}  // namespace

namespace gbqv {

// Dense matrix with the single-qubit short cuts of apply_matrix_1
// (transformer.hpp:173-232): diagonal -> diagonal kernel, X -> exchange.
void apply_matrix_impl(Device &dev, const reg_t &q, const cd *mat) {
  if (q.size() == 1) {
    if (mat[1] == 0.0 && mat[2] == 0.0) {
      cd d[2] = {mat[0], mat[3]};
      if (d[0] == 1.0 && d[1] == 1.0) return;
      launch_diagonal(dev, q, d);
      return;
    }
    if (mat[0] == 0.0 && mat[3] == 0.0 && mat[1] == 1.0 && mat[2] == 1.0) {
      launch_mc(dev, q, 0, nullptr);
      return;
    }
  }
  REQUIRE((int)q.size() <= kMaxDenseK, GBQV_ERR_ARG, "apply_matrix supports at most 13 qubits");
  if (tensor_dense_available(dev, (int)q.size())) {
    launch_dense_tensor(dev, q, mat);
    return;
  }
  if (tc64_dense_available(dev, (int)q.size())) {
    launch_dense_tc64(dev, q, mat);
    return;
  }
  launch_dense(dev, q, mat);
}

void apply_diag_impl(Device &dev, const reg_t &q, const cd *diag) {
  bool identity = true;
  for (size_t i = 0; i < (1ULL << q.size()); ++i) identity &= diag[i] == 1.0;
  if (identity) return;
  launch_diagonal(dev, q, diag);
}

// QubitVector::apply_mcu (qubitvector.hpp:1614-1720)
void apply_mcu_impl(Device &dev, const reg_t &q, const cd *mat) {
  if (mat[1] == 0.0 && mat[2] == 0.0) {
    if (mat[0] == 1.0) {
      cd ph = mat[3];
      launch_mc(dev, q, 2, &ph);
      return;
    }
    cd d[2] = {mat[0], mat[3]};
    if (q.size() == 1) {
      apply_diag_impl(dev, q, d);
      return;
    }
    launch_mc(dev, q, 4, d);
    return;
  }
  if (q.size() == 1) {
    apply_matrix_impl(dev, q, mat);
    return;
  }
  launch_mc(dev, q, 3, mat);
}

}  // namespace gbqv

namespace {

std::vector<PauliTerm> make_terms(Device &dev, int nterms, const uint64_t *qubits, const int *offsets,
                                  const char *const *labels, int limit) {
  std::vector<PauliTerm> terms;
  terms.reserve(nterms);
  for (int t = 0; t < nterms; ++t) {
    const int k = offsets[t + 1] - offsets[t];
    REQUIRE(k >= 0, GBQV_ERR_ARG, "expval_pauli_many: offsets must be non-decreasing");
    reg_t q = check_qubits(qubits + offsets[t], k, limit, "expval_pauli", 0);
    REQUIRE(labels[t] && (int)std::strlen(labels[t]) == k, GBQV_ERR_ARG, "Pauli label length must equal qubit count");
    PauliMasks m = pauli_masks(q, labels[t]);
    const cd ph = add_y_phase(m.num_y, cd(1.0, 0.0));
    terms.push_back(PauliTerm{m.x_mask, m.z_mask, m.x_max, ph.real(), ph.imag(), m.x_mask == 0});
  }
  (void)dev;
  return terms;
}

}  // namespace

// ============================== library ==============================

extern "C" int gbqv_version(void) { return 1 * 10000 + 0 * 100 + 0; }

extern "C" const char *gbqv_last_error(gbqv_handle h) { return h ? h->err.c_str() : g_err.c_str(); }

extern "C" int gbqv_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

extern "C" int gbqv_uniforms(uint64_t seed, uint64_t count, double *out) {
  return guard(nullptr, [&] {
    REQUIRE(out || count == 0, GBQV_ERR_ARG, "null output");
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> dist(0.0, 1.0);
    for (uint64_t i = 0; i < count; ++i) out[i] = dist(rng);
  });
}

extern "C" int gbqv_uniforms_streams(uint64_t seed0, uint64_t nstreams, uint64_t count, double *out) {
  return guard(nullptr, [&] {
    REQUIRE(out || nstreams * count == 0, GBQV_ERR_ARG, "null output");
    for (uint64_t s = 0; s < nstreams; ++s) {
      std::mt19937_64 rng(seed0 + s);
      std::uniform_real_distribution<double> dist(0.0, 1.0);
      for (uint64_t i = 0; i < count; ++i) out[s * count + i] = dist(rng);
    }
  });
}

// ============================== lifetime ==============================

extern "C" int gbqv_create(int num_qubits, int precision, int kind, gbqv_handle *out) {
  return guard(nullptr, [&] {
    REQUIRE(out, GBQV_ERR_ARG, "null output handle");
    *out = nullptr;
    REQUIRE(precision == GBQV_C64 || precision == GBQV_C128, GBQV_ERR_ARG, "precision must be GBQV_C64 or GBQV_C128");
    REQUIRE(kind == GBQV_STATEVECTOR || kind == GBQV_DENSITY_MATRIX || kind == GBQV_UNITARY, GBQV_ERR_ARG,
            "unknown state kind");
    const int nvec = kind == GBQV_STATEVECTOR ? num_qubits : 2 * num_qubits;
    REQUIRE(num_qubits >= 1 && nvec <= kMaxQubits, GBQV_ERR_ARG,
            "number of qubits out of range: " + std::to_string(num_qubits));
    int ndev = 0;
    cuda_check(cudaGetDeviceCount(&ndev), "no CUDA device");
    REQUIRE(ndev > 0, GBQV_ERR_CUDA, "no CUDA device visible");
    auto s = std::make_unique<gbqv_state>();
    Device &d = s->dev;
    d.nq = num_qubits;
    d.n = nvec;
    d.dbl = precision == GBQV_C128;
    d.density = kind == GBQV_DENSITY_MATRIX;
    d.unitary = kind == GBQV_UNITARY;
    cuda_check(cudaStreamCreateWithFlags(&d.stream, cudaStreamNonBlocking), "stream creation");
    const size_t bytes = d.amps() * d.amp_bytes();
    cudaError_t e = cudaMalloc(&d.state, bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      cudaStreamDestroy(d.stream);
      size_t free_b = 0, total_b = 0;
      cudaMemGetInfo(&free_b, &total_b);
      throw Error(GBQV_ERR_ALLOC, "cannot allocate " + std::to_string(bytes) + " bytes of device memory (" +
                                      std::to_string(free_b) + " free)");
    }
    if (d.unitary)
      launch_set_identity(d);
    else
      launch_set_basis(d, 0, cd(1.0, 0.0));
    *out = s.release();
  });
}

extern "C" int gbqv_destroy(gbqv_handle h) {
  if (!h) return GBQV_OK;
  Device &d = h->dev;
  cudaStreamSynchronize(d.stream);
  for (void *p : {d.state, d.ckpt, (void *)d.partials, (void *)d.results, d.mat, d.aux, d.aux2, d.probs, (void *)h->io,
                  (void *)d.tc_status})
    if (p) cudaFree(p);
  if (d.h_results) cudaFreeHost(d.h_results);
  cudaStreamDestroy(d.stream);
  cudaGetLastError();
  delete h;
  return GBQV_OK;
}

extern "C" int gbqv_num_qubits(gbqv_handle h, int *out) {
  return guard(h, [&] { need_handle(h); *out = h->dev.nq; });
}

extern "C" int gbqv_num_vector_qubits(gbqv_handle h, int *out) {
  return guard(h, [&] { need_handle(h); *out = h->dev.n; });
}

extern "C" int gbqv_synchronize(gbqv_handle h) {
  return guard(h, [&] { need_handle(h); sync(h->dev); });
}

extern "C" int gbqv_device_data(gbqv_handle h, void **out) {
  return guard(h, [&] { need_handle(h); *out = h->dev.state; });
}

extern "C" int gbqv_get_stream(gbqv_handle h, void **out) {
  return guard(h, [&] { need_handle(h); REQUIRE(out, GBQV_ERR_ARG, "null output"); *out = (void *)h->dev.stream; });
}

extern "C" uint64_t gbqv_launch_count(void) { return launch_count(); }

extern "C" int gbqv_zero(gbqv_handle h) {
  return guard(h, [&] {
    need_handle(h);
    cuda_check(cudaMemsetAsync(h->dev.state, 0, h->dev.amps() * h->dev.amp_bytes(), h->dev.stream), "zero");
  });
}

extern "C" int gbqv_initialize(gbqv_handle h) {
  return guard(h, [&] {
    need_handle(h);
    if (h->dev.unitary)
      launch_set_identity(h->dev);
    else
      launch_set_basis(h->dev, 0, cd(1.0, 0.0));
  });
}

namespace {
// complex64 states from / to pageable host memory move through a device
// staging slice of kChunk complex128 values (256 MB): copy engine for the
// host <-> device leg, a kernel for the precision change.  One stream orders
// each copy after the kernel that used the slice before it.
constexpr uint64_t kChunk = 1ULL << 24;

// The device address of page-locked (pinned or registered) host memory, or
// nullptr for ordinary pageable memory.  A kernel reads or writes pinned
// host memory directly over the CPU-GPU link at the link's rate.
const void *pinned_device_view(const void *host) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

void upload(Device &d, const cd *src, uint64_t offset, uint64_t count) {
  if (d.dbl && count >= (1ULL << 20)) {
    if (const void *dv = pinned_device_view(src)) {  // SMs pull the pinned pages at the link's rate
      launch_copy_in(d, dv, offset, count);
      return;
    }
  }
  if (d.dbl) {
    cuda_check(cudaMemcpyAsync(reinterpret_cast<cd *>(d.state) + offset, src, count * sizeof(cd),
                               cudaMemcpyHostToDevice, d.stream),
               "state upload");
    return;
  }
  if (const void *dv = pinned_device_view(src)) {  // one pass: read the host data, write complex64
    launch_narrow(d, dv, offset, count);
    return;
  }
  void *stage = grow(d.aux2, d.aux2_cap, std::min(count, kChunk) * sizeof(cd));
  for (uint64_t o = 0; o < count; o += kChunk) {
    const uint64_t c = std::min(kChunk, count - o);
    cuda_check(cudaMemcpyAsync(stage, src + o, c * sizeof(cd), cudaMemcpyHostToDevice, d.stream), "state upload");
    launch_narrow(d, stage, offset + o, c);
  }
}
}  // namespace

extern "C" int gbqv_initialize_from_vector(gbqv_handle h, const gbqv_c128 *vec, uint64_t len) {
  return guard(h, [&] {
    need_handle(h);
    Device &d = h->dev;
    REQUIRE(vec, GBQV_ERR_ARG, "null vector");
    if (len == d.amps()) {
      upload(d, as_cd(vec), 0, len);
    } else if (d.density && len == (1ULL << d.nq)) {
      // pure state -> vec(|psi><psi|) = conj(psi) (x) psi, column by column
      const uint64_t dim = len;
      std::vector<cd> col(dim);
      const cd *psi = as_cd(vec);
      for (uint64_t j = 0; j < dim; ++j) {
        const cd cj = std::conj(psi[j]);
        for (uint64_t i = 0; i < dim; ++i) col[i] = cj * psi[i];
        upload(d, col.data(), j * dim, dim);
        sync(d);
      }
    } else {
      throw Error(GBQV_ERR_ARG, "initialize_from_vector: input vector is incorrect length. Expected: " +
                                    std::to_string(d.amps()) + " Received: " + std::to_string(len));
    }
    sync(d);
  });
}

extern "C" int gbqv_copy_to_host(gbqv_handle h, gbqv_c128 *out, uint64_t len) {
  return guard(h, [&] {
    need_handle(h);
    Device &d = h->dev;
    REQUIRE(out, GBQV_ERR_ARG, "null output buffer");
    REQUIRE(len == d.amps(), GBQV_ERR_ARG, "copy_to_host: length must equal the number of stored amplitudes");
    if (d.dbl) {
      cuda_check(cudaMemcpyAsync(out, d.state, len * sizeof(cd), cudaMemcpyDeviceToHost, d.stream), "state download");
      sync(d);
      return;
    }
    if (const void *dv = pinned_device_view(out)) {
      launch_widen(d, 0, len, const_cast<void *>(dv));
      sync(d);
      return;
    }
    void *stage = grow(d.aux2, d.aux2_cap, std::min(len, kChunk) * sizeof(cd));
    for (uint64_t o = 0; o < len; o += kChunk) {
      const uint64_t c = std::min(kChunk, len - o);
      launch_widen(d, o, c, stage);
      cuda_check(cudaMemcpyAsync(out + o, stage, c * sizeof(cd), cudaMemcpyDeviceToHost, d.stream), "state download");
    }
    sync(d);
  });
}

extern "C" int gbqv_checkpoint(gbqv_handle h) {
  return guard(h, [&] {
    need_handle(h);
    Device &d = h->dev;
    const size_t bytes = d.amps() * d.amp_bytes();
    if (!d.ckpt) cuda_check(cudaMalloc(&d.ckpt, bytes), "checkpoint allocation");
    cuda_check(cudaMemcpyAsync(d.ckpt, d.state, bytes, cudaMemcpyDeviceToDevice, d.stream), "checkpoint copy");
  });
}

extern "C" int gbqv_revert(gbqv_handle h, int keep) {
  return guard(h, [&] {
    need_handle(h);
    Device &d = h->dev;
    REQUIRE(d.ckpt, GBQV_ERR_ARG, "QubitVector: checkpoint must exist for inner_product() or revert()");
    if (keep) {
      cuda_check(cudaMemcpyAsync(d.state, d.ckpt, d.amps() * d.amp_bytes(), cudaMemcpyDeviceToDevice, d.stream),
                 "revert copy");
    } else {
      sync(d);
      cudaFree(d.state);
      d.state = d.ckpt;
      d.ckpt = nullptr;
    }
  });
}

extern "C" int gbqv_inner_product(gbqv_handle h, gbqv_c128 *out) {
  return guard(h, [&] {
    need_handle(h);
    Device &d = h->dev;
    REQUIRE(d.ckpt, GBQV_ERR_ARG, "QubitVector: checkpoint must exist for inner_product() or revert()");
    reduce_inner_product(d);
    double r[2];
    read_results(d, r, 2);
    out->re = r[0];
    out->im = r[1];
  });
}

// ============================== gates ==============================

extern "C" int gbqv_apply_matrix(gbqv_handle h, const uint64_t *qubits, int k, const gbqv_c128 *mat) {
  return guard(h, [&] {
    need_handle(h);
    reg_t q = check_qubits(qubits, k, h->dev.n, "apply_matrix");
    REQUIRE(mat, GBQV_ERR_ARG, "null matrix");
    apply_matrix_impl(h->dev, q, as_cd(mat));
  });
}

extern "C" int gbqv_apply_diagonal_matrix(gbqv_handle h, const uint64_t *qubits, int k, const gbqv_c128 *diag) {
  return guard(h, [&] {
    need_handle(h);
    reg_t q = check_qubits(qubits, k, h->dev.n, "apply_diagonal_matrix");
    REQUIRE(diag, GBQV_ERR_ARG, "null diagonal");
    REQUIRE(k <= kMaxDiagK, GBQV_ERR_ARG, "apply_diagonal_matrix supports at most 10 qubits");
    apply_diag_impl(h->dev, q, as_cd(diag));
  });
}

extern "C" int gbqv_apply_mcx(gbqv_handle h, const uint64_t *qubits, int nq) {
  return guard(h, [&] {
    need_handle(h);
    launch_mc(h->dev, check_qubits(qubits, nq, h->dev.n, "apply_mcx"), 0, nullptr);
  });
}

extern "C" int gbqv_apply_mcy(gbqv_handle h, const uint64_t *qubits, int nq) {
  return guard(h, [&] {
    need_handle(h);
    launch_mc(h->dev, check_qubits(qubits, nq, h->dev.n, "apply_mcy"), 1, nullptr);
  });
}

extern "C" int gbqv_apply_mcswap(gbqv_handle h, const uint64_t *qubits, int nq) {
  return guard(h, [&] {
    need_handle(h);
    launch_mc(h->dev, check_qubits(qubits, nq, h->dev.n, "apply_mcswap", 2), 5, nullptr);
  });
}

extern "C" int gbqv_apply_mcphase(gbqv_handle h, const uint64_t *qubits, int nq, gbqv_c128 phase) {
  return guard(h, [&] {
    need_handle(h);
    cd ph = as_cd(phase);
    launch_mc(h->dev, check_qubits(qubits, nq, h->dev.n, "apply_mcphase"), 2, &ph);
  });
}

extern "C" int gbqv_apply_mcu(gbqv_handle h, const uint64_t *qubits, int nq, const gbqv_c128 *mat) {
  return guard(h, [&] {
    need_handle(h);
    REQUIRE(mat, GBQV_ERR_ARG, "null matrix");
    apply_mcu_impl(h->dev, check_qubits(qubits, nq, h->dev.n, "apply_mcu"), as_cd(mat));
  });
}

extern "C" int gbqv_apply_rotation(gbqv_handle h, const uint64_t *qubits, int nq, int axis, double theta) {
  return guard(h, [&] {
    need_handle(h);
    reg_t q = check_qubits(qubits, nq, h->dev.n, "apply_rotation");
    switch (axis) {
      case GBQV_ROT_X: apply_mcu_impl(h->dev, q, gates::rx(theta).data()); break;
      case GBQV_ROT_Y: apply_mcu_impl(h->dev, q, gates::ry(theta).data()); break;
      case GBQV_ROT_Z: apply_mcu_impl(h->dev, q, gates::rz(theta).data()); break;
      case GBQV_ROT_XX: REQUIRE(nq == 2, GBQV_ERR_ARG, "rxx acts on 2 qubits"); apply_matrix_impl(h->dev, q, gates::rxx(theta).data()); break;
      case GBQV_ROT_YY: REQUIRE(nq == 2, GBQV_ERR_ARG, "ryy acts on 2 qubits"); apply_matrix_impl(h->dev, q, gates::ryy(theta).data()); break;
      case GBQV_ROT_ZZ: REQUIRE(nq == 2, GBQV_ERR_ARG, "rzz acts on 2 qubits"); apply_diag_impl(h->dev, q, gates::rzz_diag(theta).data()); break;
      case GBQV_ROT_ZX: REQUIRE(nq == 2, GBQV_ERR_ARG, "rzx acts on 2 qubits"); apply_matrix_impl(h->dev, q, gates::rzx(theta).data()); break;
      default: throw Error(GBQV_ERR_ARG, "QubitVector::invalid rotation axis.");
    }
  });
}

extern "C" int gbqv_apply_pauli(gbqv_handle h, const uint64_t *qubits, int nq, const char *label, gbqv_c128 coeff) {
  return guard(h, [&] {
    need_handle(h);
    reg_t q = check_qubits(qubits, nq, h->dev.n, "apply_pauli", 0);
    REQUIRE(label && (int)std::strlen(label) == nq, GBQV_ERR_ARG, "Pauli label length must equal qubit count");
    PauliMasks m = pauli_masks(q, label);
    if (m.x_mask + m.z_mask == 0) return;
    launch_pauli(h->dev, m.x_mask, m.z_mask, m.x_max, add_y_phase(m.num_y, as_cd(coeff)));
  });
}

extern "C" int gbqv_apply_permutation_matrix(gbqv_handle h, const uint64_t *qubits, int k, const uint64_t *pairs,
                                             int npairs) {
  return guard(h, [&] {
    need_handle(h);
    reg_t q = check_qubits(qubits, k, h->dev.n, "apply_permutation_matrix");
    REQUIRE(k <= 10, GBQV_ERR_ARG, "apply_permutation_matrix supports at most 10 qubits");
    REQUIRE(npairs >= 0 && npairs <= kMaxPermPairs && (pairs || npairs == 0), GBQV_ERR_ARG, "bad permutation pairs");
    std::vector<std::pair<uint32_t, uint32_t>> p;
    for (int i = 0; i < npairs; ++i) {
      REQUIRE(pairs[2 * i] < (1ULL << k) && pairs[2 * i + 1] < (1ULL << k), GBQV_ERR_ARG, "permutation index out of range");
      p.emplace_back((uint32_t)pairs[2 * i], (uint32_t)pairs[2 * i + 1]);
    }
    if (!p.empty()) launch_swaps(h->dev, q, p);
  });
}

extern "C" int gbqv_apply_multiplexer(gbqv_handle h, const uint64_t *controls, int nc, const uint64_t *targets, int nt,
                                      const gbqv_c128 *mat) {
  return guard(h, [&] {
    need_handle(h);
    REQUIRE(mat, GBQV_ERR_ARG, "null matrix");
    reg_t all(targets, targets + nt);
    all.insert(all.end(), controls, controls + nc);
    reg_t q = check_qubits(all.data(), nt + nc, h->dev.n, "apply_multiplexer");
    REQUIRE(nt >= 1 && nt + nc <= kMaxDenseK, GBQV_ERR_ARG, "apply_multiplexer supports at most 13 qubits");
    // Block-diagonal expansion of the stacked matrix (qubitvector.hpp:1316-1331):
    // full[i + b*cols, j + b*cols] = mat[i + b*cols + DIM*j].
    const uint64_t DIM = 1ULL << (nt + nc), cols = 1ULL << nt, blocks = 1ULL << nc;
    std::vector<cd> full(DIM * DIM, cd(0, 0));
    const cd *m = as_cd(mat);
    for (uint64_t b = 0; b < blocks; ++b)
      for (uint64_t i = 0; i < cols; ++i)
        for (uint64_t j = 0; j < cols; ++j) full[(i + b * cols) + DIM * (j + b * cols)] = m[i + b * cols + DIM * j];
    launch_dense(h->dev, q, full.data());
  });
}

extern "C" int gbqv_apply_multi_swaps(gbqv_handle h, const uint64_t *qubits, int nq) {
  return guard(h, [&] {
    need_handle(h);
    reg_t q = check_qubits(qubits, nq, h->dev.n, "apply_multi_swaps", 2);
    REQUIRE(nq % 2 == 0, GBQV_ERR_ARG, "apply_multi_swaps takes qubit pairs");
    // each (q[2i], q[2i+1]) is a SWAP; the pairs are disjoint so they commute
    for (int i = 0; i < nq; i += 2) launch_mc(h->dev, reg_t{q[i], q[i + 1]}, 5, nullptr);
  });
}

// ============================== reductions ==============================

extern "C" int gbqv_norm(gbqv_handle h, double *out) {
  return guard(h, [&] {
    need_handle(h);
    reduce_norm(h->dev);
    read_results(h->dev, out, 1);
  });
}

extern "C" int gbqv_norm_matrix(gbqv_handle h, const uint64_t *qubits, int k, const gbqv_c128 *mat, double *out) {
  return guard(h, [&] {
    need_handle(h);
    reg_t q = check_qubits(qubits, k, h->dev.n, "norm");
    REQUIRE(k <= kMaxDenseK, GBQV_ERR_ARG, "norm(qubits, mat) supports at most 13 qubits");
    reduce_norm_matrix(h->dev, q, as_cd(mat));
    read_results(h->dev, out, 1);
  });
}

extern "C" int gbqv_probabilities(gbqv_handle h, const uint64_t *qubits, int k, double *out) {
  return guard(h, [&] {
    need_handle(h);
    Device &d = h->dev;
    REQUIRE(out, GBQV_ERR_ARG, "null output");
    const int limit = d.density ? d.nq : d.n;
    if (k == 0) {
      const uint64_t count = 1ULL << limit;
      grow(reinterpret_cast<void *&>(h->io), h->io_cap, count * sizeof(double));
      probabilities_all(d, reinterpret_cast<double *>(h->io));
      cuda_check(cudaMemcpyAsync(out, h->io, count * sizeof(double), cudaMemcpyDeviceToHost, d.stream),
                 "probabilities copy");
      sync(d);
      return;
    }
    reg_t q = check_qubits(qubits, k, limit, "probabilities");
    reduce_probabilities(d, q);
    read_results(d, out, 1ULL << k);
  });
}

extern "C" int gbqv_probability(gbqv_handle h, uint64_t outcome, double *out) {
  return guard(h, [&] {
    need_handle(h);
    Device &d = h->dev;
    REQUIRE(out, GBQV_ERR_ARG, "null output");
    const int limit = d.density ? d.nq : d.n;
    REQUIRE(limit >= 64 || outcome < (1ULL << limit), GBQV_ERR_QUBIT, "outcome out of range");
    // the amplitude (or diagonal entry rho[k, k] of vec(rho)) is read back alone
    const uint64_t idx = d.density ? outcome * ((1ULL << d.nq) + 1) : outcome;
    const size_t amp = d.dbl ? 16 : 8;
    unsigned char buf[16] = {0};
    cuda_check(cudaMemcpyAsync(buf, static_cast<const unsigned char *>(d.state) + idx * amp, amp,
                               cudaMemcpyDeviceToHost, d.stream),
               "probability copy");
    sync(d);
    double re, im;
    if (d.dbl) {
      std::memcpy(&re, buf, 8);
      std::memcpy(&im, buf + 8, 8);
    } else {
      float r, i;
      std::memcpy(&r, buf, 4);
      std::memcpy(&i, buf + 4, 4);
      re = r;
      im = i;
    }
    *out = d.density ? re : re * re + im * im;
  });
}

extern "C" int gbqv_set_sample_measure_index_size(gbqv_handle h, int index_size) {
  return guard(h, [&] {
    need_handle(h);
    REQUIRE(index_size >= 1 && index_size <= 24, GBQV_ERR_ARG, "sample_measure index size must be 1..24");
    h->dev.sample_index_size = index_size;
  });
}

extern "C" int gbqv_sample_measure(gbqv_handle h, const double *rnds, uint64_t shots, uint64_t *out) {
  return guard(h, [&] {
    need_handle(h);
    Device &d = h->dev;
    if (shots == 0) return;
    REQUIRE(rnds && out, GBQV_ERR_ARG, "null shot buffers");
    grow(reinterpret_cast<void *&>(h->io), h->io_cap, shots * 16);
    double *d_r = reinterpret_cast<double *>(h->io);
    uint64_t *d_o = h->io + shots;
    cuda_check(cudaMemcpyAsync(d_r, rnds, shots * sizeof(double), cudaMemcpyHostToDevice, d.stream), "uniform upload");
    sample_measure(d, d_r, shots, d_o);
    cuda_check(cudaMemcpyAsync(out, d_o, shots * sizeof(uint64_t), cudaMemcpyDeviceToHost, d.stream), "sample copy");
    sync(d);
  });
}

extern "C" int gbqv_sample_measure_segments(gbqv_handle h, int state_qubits, uint64_t first, uint64_t nseg,
                                            const double *rnds, uint64_t shots, uint64_t *out) {
  return guard(h, [&] {
    need_handle(h);
    Device &d = h->dev;
    REQUIRE(!d.density && !d.unitary, GBQV_ERR_KIND, "sample_measure_segments: statevector stacks only");
    REQUIRE(state_qubits >= 1 && state_qubits <= d.n && first + nseg <= (d.amps() >> state_qubits), GBQV_ERR_ARG,
            "sample_measure_segments: the states do not fit the handle's vector");
    if (shots == 0 || nseg == 0) return;
    REQUIRE(rnds && out, GBQV_ERR_ARG, "null shot buffers");
    const uint64_t total = shots * nseg;
    grow(reinterpret_cast<void *&>(h->io), h->io_cap, total * 16);
    double *d_r = reinterpret_cast<double *>(h->io);
    uint64_t *d_o = h->io + total;
    cuda_check(cudaMemcpyAsync(d_r, rnds, total * sizeof(double), cudaMemcpyHostToDevice, d.stream),
               "uniform upload");
    for (uint64_t s = 0; s < nseg; ++s)  // each state sampled exactly as a state of its own
      sample_measure(d, d_r + s * shots, shots, d_o + s * shots, (first + s) << state_qubits, state_qubits);
    cuda_check(cudaMemcpyAsync(out, d_o, total * sizeof(uint64_t), cudaMemcpyDeviceToHost, d.stream), "sample copy");
    sync(d);
  });
}

extern "C" int gbqv_expval_pauli(gbqv_handle h, const uint64_t *qubits, int nq, const char *label,
                                 gbqv_c128 initial_phase, double *out) {
  return guard(h, [&] {
    need_handle(h);
    Device &d = h->dev;
    const int limit = d.density ? d.nq : d.n;
    reg_t q = check_qubits(qubits, nq, limit, "expval_pauli", 0);
    REQUIRE(label && (int)std::strlen(label) == nq, GBQV_ERR_ARG, "Pauli label length must equal qubit count");
    PauliMasks m = pauli_masks(q, label);
    const cd ph = add_y_phase(m.num_y, as_cd(initial_phase));
    std::vector<PauliTerm> t{PauliTerm{m.x_mask, m.z_mask, m.x_max, ph.real(), ph.imag(), m.x_mask == 0}};
    if (m.x_mask + m.z_mask == 0) t[0].ph_re = 1.0, t[0].ph_im = 0.0;  // norm() / trace
    if (d.density)
      reduce_dm_expval(d, t);
    else
      reduce_expval(d, t);
    read_results(d, out, 1);
  });
}

extern "C" int gbqv_expval_pauli_many(gbqv_handle h, int nterms, const uint64_t *qubits, const int *offsets,
                                      const char *const *labels, const double *coeffs, double *out, double *total) {
  return guard(h, [&] {
    need_handle(h);
    Device &d = h->dev;
    REQUIRE(nterms >= 0 && offsets && labels, GBQV_ERR_ARG, "bad term arrays");
    const int limit = d.density ? d.nq : d.n;
    std::vector<double> vals(nterms);
    for (int t0 = 0; t0 < nterms; t0 += kMaxTerms) {
      const int cnt = std::min(kMaxTerms, nterms - t0);
      std::vector<PauliTerm> terms = make_terms(d, cnt, qubits, offsets + t0, labels + t0, limit);
      if (d.density)
        reduce_dm_expval(d, terms);
      else
        reduce_expval(d, terms);
      read_results(d, vals.data() + t0, cnt);
    }
    if (out) std::copy(vals.begin(), vals.end(), out);
    if (total) {
      double s = 0.0;
      for (int t = 0; t < nterms; ++t) s += (coeffs ? coeffs[t] : 1.0) * vals[t];
      *total = s;
    }
  });
}

extern "C" int gbqv_expval_pauli_segments(gbqv_handle h, int state_qubits, uint64_t nseg, int nterms,
                                          const uint64_t *qubits, const int *offsets, const char *const *labels,
                                          double *out) {
  return guard(h, [&] {
    need_handle(h);
    Device &d = h->dev;
    REQUIRE(!d.density, GBQV_ERR_KIND, "expval_pauli_segments: statevector stacks only");
    REQUIRE(nterms >= 0 && offsets && labels && out, GBQV_ERR_ARG, "bad term arrays");
    REQUIRE(state_qubits >= 1 && state_qubits <= d.n && nseg >= 1 && nseg <= (d.amps() >> state_qubits),
            GBQV_ERR_ARG, "expval_pauli_segments: the states do not fit the handle's vector");
    // keep one launch's partial sums bounded: terms x states per launch
    const uint64_t per_launch = std::max<uint64_t>(1, (1ULL << 22) / nseg);
    const int step = (int)std::min<uint64_t>((uint64_t)kMaxTerms, per_launch);
    std::vector<double> vals;
    for (int t0 = 0; t0 < nterms; t0 += step) {
      const int cnt = std::min(step, nterms - t0);
      std::vector<PauliTerm> terms = make_terms(d, cnt, qubits, offsets + t0, labels + t0, state_qubits);
      reduce_expval_segments(d, terms, state_qubits, nseg);
      vals.resize((size_t)cnt * nseg);
      read_results(d, vals.data(), vals.size());
      std::copy(vals.begin(), vals.end(), out + (size_t)t0 * nseg);
    }
  });
}

// ============================== batched shots ==============================

namespace {
void check_stack(const Device &d, int state_qubits, uint64_t nseg, const char *what) {
  REQUIRE(!d.density && !d.unitary, GBQV_ERR_KIND, std::string(what) + ": statevector stacks only");
  REQUIRE(state_qubits >= 1 && state_qubits <= d.n && nseg >= 1 && nseg <= (d.amps() >> state_qubits), GBQV_ERR_ARG,
          std::string(what) + ": the states do not fit the handle's vector");
}
}  // namespace

extern "C" int gbqv_initialize_segments(gbqv_handle h, int state_qubits, uint64_t count) {
  return guard(h, [&] {
    need_handle(h);
    check_stack(h->dev, state_qubits, std::max<uint64_t>(count, 1), "initialize_segments");
    launch_set_basis_segments(h->dev, state_qubits, count);
  });
}

extern "C" int gbqv_probabilities_segments(gbqv_handle h, int state_qubits, uint64_t nseg, const uint64_t *qubits,
                                           int k, double *out) {
  return guard(h, [&] {
    need_handle(h);
    Device &d = h->dev;
    check_stack(d, state_qubits, nseg, "probabilities_segments");
    reg_t q = check_qubits(qubits, k, state_qubits, "probabilities_segments");
    REQUIRE(k <= seg_max_measure_qubits() && out, GBQV_ERR_ARG, "probabilities_segments: 1..30 qubits, an output");
    reduce_probabilities_segments(d, q, state_qubits, nseg);
    read_results(d, out, nseg << k);
  });
}

extern "C" int gbqv_draw_segments(gbqv_handle h, int state_qubits, uint64_t nseg, const uint64_t *qubits, int k,
                                  const double *u, uint32_t *outcome, double *prob) {
  return guard(h, [&] {
    need_handle(h);
    Device &d = h->dev;
    check_stack(d, state_qubits, nseg, "draw_segments");
    reg_t q = check_qubits(qubits, k, state_qubits, "draw_segments");
    REQUIRE(k >= 10 && k <= seg_max_measure_qubits() && u && outcome && prob, GBQV_ERR_ARG,
            "draw_segments: 10..30 qubits, uniforms and two outputs");
    for (uint64_t s = 0; s < nseg; ++s)
      REQUIRE(u[s] < 1.0, GBQV_ERR_ARG, "draw_segments: uniforms must lie below 1");
    draw_segments(d, q, state_qubits, nseg, u, outcome, prob);
    check_tc_status(d);
  });
}

extern "C" int gbqv_collapse_segments(gbqv_handle h, int state_qubits, uint64_t nseg, const uint64_t *qubits, int k,
                                      const uint32_t *meas_state, const uint32_t *final_state, const double *scale) {
  return guard(h, [&] {
    need_handle(h);
    Device &d = h->dev;
    check_stack(d, state_qubits, nseg, "collapse_segments");
    reg_t q = check_qubits(qubits, k, state_qubits, "collapse_segments");
    REQUIRE(k <= seg_max_measure_qubits() && meas_state && final_state && scale, GBQV_ERR_ARG,
            "collapse_segments: 1..30 qubits and three per-state arrays");
    const uint32_t D = 1u << k;
    for (uint64_t s = 0; s < nseg; ++s)
      REQUIRE(meas_state[s] == 0xffffffffu || (meas_state[s] < D && final_state[s] < D), GBQV_ERR_ARG,
              "collapse_segments: outcome of state " + std::to_string(s) + " out of range");
    launch_collapse_segments(d, q, state_qubits, nseg, meas_state, final_state, scale);
  });
}

extern "C" int gbqv_apply_matrix_segments(gbqv_handle h, int state_qubits, uint64_t nseg, const uint64_t *qubits,
                                          int k, const gbqv_c128 *mat, const uint8_t *mask) {
  return guard(h, [&] {
    need_handle(h);
    Device &d = h->dev;
    check_stack(d, state_qubits, nseg, "apply_matrix_segments");
    reg_t q = check_qubits(qubits, k, state_qubits, "apply_matrix_segments");
    REQUIRE(k <= seg_max_matrix_qubits() && mat && mask, GBQV_ERR_ARG,
            "apply_matrix_segments: 1..4 qubits, a matrix and a mask");
    launch_matrix_segments(d, q, state_qubits, nseg, reinterpret_cast<const cd *>(mat), mask);
  });
}

extern "C" int gbqv_rdm_segments(gbqv_handle h, int state_qubits, uint64_t nseg, const uint64_t *qubits, int k,
                                 gbqv_c128 *out) {
  return guard(h, [&] {
    need_handle(h);
    Device &d = h->dev;
    check_stack(d, state_qubits, nseg, "rdm_segments");
    reg_t q = check_qubits(qubits, k, state_qubits, "rdm_segments");
    REQUIRE(k <= seg_max_kraus_qubits() && out, GBQV_ERR_ARG, "rdm_segments: 1..3 qubits, an output");
    reduce_rdm_segments(d, q, state_qubits, nseg);
    const size_t D = 1ULL << k, E = D * D;
    std::vector<double> v(nseg * E);
    read_results(d, v.data(), v.size());
    // the packed values (diagonal; real part above, imaginary part below it)
    // to full Hermitian matrices
    for (uint64_t s = 0; s < nseg; ++s) {
      const double *e = v.data() + s * E;
      gbqv_c128 *r = out + s * E;
      for (size_t a = 0; a < D; ++a) {
        r[a * D + a] = gbqv_c128{e[a * D + a], 0.0};
        for (size_t b = a + 1; b < D; ++b) {
          r[a * D + b] = gbqv_c128{e[a * D + b], e[b * D + a]};
          r[b * D + a] = gbqv_c128{e[a * D + b], -e[b * D + a]};
        }
      }
    }
  });
}

extern "C" int gbqv_kraus_segments(gbqv_handle h, int state_qubits, uint64_t nseg, const uint64_t *qubits, int k,
                                   const gbqv_c128 *mats, int m, const uint8_t *branch, const double *scale) {
  return guard(h, [&] {
    need_handle(h);
    Device &d = h->dev;
    check_stack(d, state_qubits, nseg, "kraus_segments");
    reg_t q = check_qubits(qubits, k, state_qubits, "kraus_segments");
    REQUIRE(k <= seg_max_kraus_qubits() && mats && branch && scale, GBQV_ERR_ARG,
            "kraus_segments: 1..3 qubits, matrices and two per-state arrays");
    REQUIRE(m >= 1 && m <= 255, GBQV_ERR_ARG, "kraus_segments: 1..255 operators");
    for (uint64_t s = 0; s < nseg; ++s)
      REQUIRE(branch[s] == 0xff || branch[s] < m, GBQV_ERR_ARG,
              "kraus_segments: operator of state " + std::to_string(s) + " out of range");
    launch_kraus_segments(d, q, state_qubits, nseg, reinterpret_cast<const cd *>(mats), m, branch, scale);
  });
}

// ============================== density matrix ==============================

namespace gbqv {
reg_t superop_qubits(const Device &d, const reg_t &q) {
  reg_t s = q;
  for (uint64_t x : q) s.push_back(x + d.nq);
  return s;
}
}  // namespace gbqv

extern "C" int gbqv_dm_apply_superop_matrix(gbqv_handle h, const uint64_t *qubits, int k, const gbqv_c128 *mat) {
  return guard(h, [&] {
    need_handle(h);
    require_density(h->dev, "apply_superop_matrix");
    reg_t q = check_qubits(qubits, k, h->dev.nq, "apply_superop_matrix");
    REQUIRE(2 * k <= 10 && mat, GBQV_ERR_ARG, "apply_superop_matrix supports at most 5 qubits");
    apply_matrix_impl(h->dev, superop_qubits(h->dev, q), as_cd(mat));
  });
}

extern "C" int gbqv_dm_apply_diagonal_superop_matrix(gbqv_handle h, const uint64_t *qubits, int k,
                                                     const gbqv_c128 *diag) {
  return guard(h, [&] {
    need_handle(h);
    require_density(h->dev, "apply_diagonal_superop_matrix");
    reg_t q = check_qubits(qubits, k, h->dev.nq, "apply_diagonal_superop_matrix");
    REQUIRE(2 * k <= kMaxDiagK && diag, GBQV_ERR_ARG, "apply_diagonal_superop_matrix supports at most 5 qubits");
    apply_diag_impl(h->dev, superop_qubits(h->dev, q), as_cd(diag));
  });
}

namespace gbqv {
// DensityMatrix::apply_unitary_matrix (densitymatrix.hpp:297-317)
void dm_unitary(Device &d, const reg_t &q, const cd *mat) {
  const size_t k = q.size(), dim = 1ULL << k;
  if (k > 4) {
    REQUIRE(k <= (size_t)kMaxDenseK, GBQV_ERR_ARG, "apply_unitary_matrix supports at most 13 qubits");
    apply_matrix_impl(d, q, mat);
    std::vector<cd> c(mat, mat + dim * dim);
    for (auto &z : c) z = std::conj(z);
    reg_t cq;
    for (uint64_t x : q) cq.push_back(x + d.nq);
    apply_matrix_impl(d, cq, c.data());
    return;
  }
  apply_matrix_impl(d, superop_qubits(d, q), gates::vmat2vsuperop(mat, dim).data());
}

void dm_diag_unitary(Device &d, const reg_t &q, const cd *diag) {
  const size_t dim = 1ULL << q.size();
  std::vector<cd> s(dim * dim);
  for (size_t i = 0; i < dim; ++i)
    for (size_t j = 0; j < dim; ++j) s[i * dim + j] = std::conj(diag[i]) * diag[j];
  apply_diag_impl(d, superop_qubits(d, q), s.data());
}
}  // namespace gbqv

extern "C" int gbqv_dm_apply_unitary_matrix(gbqv_handle h, const uint64_t *qubits, int k, const gbqv_c128 *mat) {
  return guard(h, [&] {
    need_handle(h);
    require_density(h->dev, "apply_unitary_matrix");
    REQUIRE(mat, GBQV_ERR_ARG, "null matrix");
    dm_unitary(h->dev, check_qubits(qubits, k, h->dev.nq, "apply_unitary_matrix"), as_cd(mat));
  });
}

extern "C" int gbqv_dm_apply_diagonal_unitary_matrix(gbqv_handle h, const uint64_t *qubits, int k,
                                                     const gbqv_c128 *diag) {
  return guard(h, [&] {
    need_handle(h);
    require_density(h->dev, "apply_diagonal_unitary_matrix");
    REQUIRE(diag && k <= 5, GBQV_ERR_ARG, "apply_diagonal_unitary_matrix supports at most 5 qubits");
    dm_diag_unitary(h->dev, check_qubits(qubits, k, h->dev.nq, "apply_diagonal_unitary_matrix"), as_cd(diag));
  });
}

namespace {
void dm_perm(gbqv_handle h, const reg_t &q, const std::vector<std::pair<uint32_t, uint32_t>> &pairs, const char *what) {
  need_handle(h);
  require_density(h->dev, what);
  reg_t qq = check_qubits(q.data(), (int)q.size(), h->dev.nq, what);
  launch_swaps(h->dev, superop_qubits(h->dev, qq), pairs);
}
}  // namespace

// Permutation tables of densitymatrix.hpp:331-413.
extern "C" int gbqv_dm_apply_cnot(gbqv_handle h, uint64_t c, uint64_t t) {
  return guard(h, [&] { dm_perm(h, {c, t}, {{1, 3}, {4, 12}, {5, 15}, {6, 14}, {7, 13}, {9, 11}}, "apply_cnot"); });
}

extern "C" int gbqv_dm_apply_swap(gbqv_handle h, uint64_t a, uint64_t b) {
  return guard(h, [&] { dm_perm(h, {a, b}, {{1, 2}, {4, 8}, {5, 10}, {6, 9}, {7, 11}, {13, 14}}, "apply_swap"); });
}

extern "C" int gbqv_dm_apply_x(gbqv_handle h, uint64_t q) {
  return guard(h, [&] { dm_perm(h, {q}, {{0, 3}, {1, 2}}, "apply_x"); });
}

extern "C" int gbqv_dm_apply_toffoli(gbqv_handle h, uint64_t a, uint64_t b, uint64_t c) {
  return guard(h, [&] {
    dm_perm(h, {a, b, c},
            {{3, 7}, {11, 15}, {19, 23}, {24, 56}, {25, 57}, {26, 58}, {27, 63}, {28, 60}, {29, 61}, {30, 62},
             {31, 59}, {35, 39}, {43, 47}, {51, 55}},
            "apply_toffoli");
  });
}

extern "C" int gbqv_dm_apply_y(gbqv_handle h, uint64_t q) {
  return guard(h, [&] {
    need_handle(h);
    require_density(h->dev, "apply_y");
    check_qubits(&q, 1, h->dev.nq, "apply_y");
    launch_dm_y(h->dev, q);
  });
}

extern "C" int gbqv_dm_apply_phase(gbqv_handle h, uint64_t q, gbqv_c128 phase) {
  return guard(h, [&] {
    need_handle(h);
    require_density(h->dev, "apply_phase");
    check_qubits(&q, 1, h->dev.nq, "apply_phase");
    const cd ph = as_cd(phase);
    cd d[4] = {1.0, ph, std::conj(ph), 1.0};
    apply_diag_impl(h->dev, {q, q + h->dev.nq}, d);
  });
}

extern "C" int gbqv_dm_apply_cphase(gbqv_handle h, uint64_t q0, uint64_t q1, gbqv_c128 phase) {
  return guard(h, [&] {
    need_handle(h);
    require_density(h->dev, "apply_cphase");
    reg_t qq{q0, q1};
    check_qubits(qq.data(), 2, h->dev.nq, "apply_cphase");
    const cd ph = as_cd(phase), iph = std::conj(ph);
    std::vector<cd> d(16, cd(1.0, 0.0));
    d[3] = d[7] = d[11] = ph;
    d[12] = d[13] = d[14] = iph;
    apply_diag_impl(h->dev, superop_qubits(h->dev, qq), d.data());
  });
}

extern "C" int gbqv_dm_apply_reset(gbqv_handle h, const uint64_t *qubits, int k) {
  return guard(h, [&] {
    need_handle(h);
    require_density(h->dev, "apply_reset");
    reg_t q = check_qubits(qubits, k, h->dev.nq, "apply_reset");
    REQUIRE(2 * k <= 10, GBQV_ERR_ARG, "apply_reset supports at most 5 qubits");
    apply_matrix_impl(h->dev, superop_qubits(h->dev, q), gates::reset_superop(k).data());
  });
}

extern "C" int gbqv_dm_trace(gbqv_handle h, gbqv_c128 *out) {
  return guard(h, [&] {
    need_handle(h);
    require_density(h->dev, "trace");
    reduce_dm_trace(h->dev);
    double r[2];
    read_results(h->dev, r, 2);
    out->re = r[0];
    out->im = r[1];
  });
}

extern "C" int gbqv_set_tensor_c128(gbqv_handle h, int enable) {
  return guard(h, [&] {
    need_handle(h);
    REQUIRE(enable >= 0 && enable <= 2, GBQV_ERR_ARG, "tensor mode must be 0, 1 or 2");
    h->dev.tensor_c128 = enable;
  });
}

extern "C" int gbqv_test_stall_tensor_pipeline(gbqv_handle h, int enable) {
  return guard(h, [&] {
    need_handle(h);
    h->dev.tc_test_stall = enable ? 1 : 0;
  });
}

extern "C" int gbqv_set_run_tile_qubits(gbqv_handle h, int tile_qubits) {
  return guard(h, [&] {
    need_handle(h);
    const int hi = h->dev.dbl ? 12 : 13;
    REQUIRE(tile_qubits == 0 || (tile_qubits >= 10 && tile_qubits <= hi), GBQV_ERR_ARG,
            "run tile qubits must be 0 (default) or 10.." + std::to_string(hi));
    h->dev.run_tile_bits = tile_qubits;
  });
}

extern "C" int gbqv_set_run_jit(gbqv_handle h, int mode) {
  return guard(h, [&] {
    need_handle(h);
    REQUIRE(mode >= 0 && mode <= 2, GBQV_ERR_ARG, "run compile mode must be 0, 1 or 2");
    h->dev.run_jit = mode;
  });
}

extern "C" int gbqv_run_jit_counts(uint64_t *compiled, uint64_t *launched) {
  return guard(nullptr, [&] {
    REQUIRE(compiled && launched, GBQV_ERR_ARG, "null output");
    run_jit_counts(*compiled, *launched);
  });
}

extern "C" int gbqv_run_jit_compile_check(int double_precision, char *log, size_t cap) {
  std::string l = "NVRTC is not available";
  int rc = 0;
  const int g = guard(nullptr, [&] {
    REQUIRE(run_jit_available(), GBQV_ERR_ARG, l);
    rc = run_jit_compile_check(double_precision != 0, l);
  });
  if (log && cap) {
    const size_t k = std::min(cap - 1, l.size());
    std::memcpy(log, l.data(), k);
    log[k] = '\0';
  }
  return g ? g : rc;
}

extern "C" int gbqv_set_blocking(gbqv_handle h, int blocking) {
  return guard(h, [&] {
    need_handle(h);
    REQUIRE(blocking >= 0 && blocking <= 2, GBQV_ERR_ARG, "blocking mode must be 0, 1 or 2");
    h->dev.blocking = blocking;
  });
}
