// gbqv_circuit.cpp — host side of circuit execution: the op list, the gate
// dispatch of the reference's State classes, Aer's Fusion transpiler pass
// restated (src/transpile/fusion.hpp), and the executor that drives the
// kernels (with cache-blocked runs of dense/diagonal ops).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <set>
#include <string>
#include <unordered_map>
#include <unordered_set>

#include "../../include/gbqv.h"
#include "gbqv_gates.h"
#include "gbqv_internal.h"

using namespace gbqv;

namespace {
constexpr int OP_NOP = -1;

struct Op {
  int type = GBQV_OP_GATE;
  std::string name;
  reg_t qubits;
  std::vector<double> params;
  std::vector<cd> mat;                 // MATRIX 4^k, DIAGONAL 2^k, SUPEROP 16^k (column-major)
  std::vector<std::vector<cd>> kraus;  // KRAUS
  // Runtime parameter binding (controller_execute.hpp:104-131): binding j's
  // parameters at [j * params.size(), (j + 1) * params.size()); empty when
  // every binding uses `params` (which then hold binding 0's values).
  std::vector<double> bparams;
};
}  // namespace

struct gbqv_circuit {
  int num_qubits = 0;
  int nbind = 0;  // number of parameter bindings (0: none)
  std::vector<Op> ops;
  uint64_t version = 0;  // bumped by every change of ops or bindings
  // bound execution: the run form of every op, built once per version
  uint64_t bound_version = UINT64_MAX;
  std::vector<Op> bound_ops;
  std::vector<RunOp> bound_conv;
  std::vector<char> bound_runnable;
};

namespace {

// Errors of circuit calls go to gbqv_last_error(NULL); gbqv_execute reports
// on the state handle.
template <typename F>
int guard(F &&f, gbqv_state *h = nullptr) {
  try {
    f();
    return GBQV_OK;
  } catch (const Error &e) {
    set_last_error(h, e.what());
    return e.code;
  } catch (const std::exception &e) {
    set_last_error(h, e.what());
    return GBQV_ERR_ARG;
  }
}

#define REQUIRE(cond, code, msg) \
  do {                           \
    if (!(cond)) throw Error(code, msg); \
  } while (0)

reg_t check_q(const gbqv_circuit *c, const uint64_t *qubits, int k, int kmin = 1) {
  REQUIRE(c, GBQV_ERR_ARG, "null circuit");
  REQUIRE(k >= kmin && (qubits || k == 0), GBQV_ERR_ARG, "bad qubit list");
  reg_t q(qubits, qubits + k);
  for (int i = 0; i < k; ++i) {
    REQUIRE(q[i] < (uint64_t)c->num_qubits, GBQV_ERR_QUBIT, "qubit index " + std::to_string(q[i]) + " out of range");
    for (int j = 0; j < i; ++j) REQUIRE(q[i] != q[j], GBQV_ERR_QUBIT, "repeated qubit " + std::to_string(q[i]));
  }
  return q;
}

// ------------------------------------------------------------------------
// Statevector gate set and its primitives
// (Statevector::State::gateset_ / apply_gate, statevector_state.hpp:313-384, 733-865)
// ------------------------------------------------------------------------
enum class P { NONE, MCX, MCY, MCPHASE, MCU, MATRIX, DIAG, MCSWAP };
struct Prim {
  P k = P::NONE;
  reg_t q;
  std::vector<cd> m;
};

const std::unordered_map<std::string, std::string> &sv_gateset() {
  static const std::unordered_map<std::string, std::string> g = {
      {"delay", "id"}, {"id", "id"}, {"x", "mcx"}, {"y", "mcy"}, {"z", "mcz"}, {"s", "s"}, {"sdg", "sdg"},
      {"h", "h"}, {"t", "t"}, {"tdg", "tdg"}, {"p", "mcp"}, {"sx", "mcsx"}, {"sxdg", "mcsxdg"}, {"r", "mcr"},
      {"rx", "mcrx"}, {"ry", "mcry"}, {"rz", "mcrz"}, {"u1", "mcp"}, {"u2", "mcu2"}, {"u3", "mcu3"},
      {"u", "mcu3"}, {"U", "mcu3"}, {"CX", "mcx"}, {"cx", "mcx"}, {"cy", "mcy"}, {"cz", "mcz"}, {"cp", "mcp"},
      {"cu1", "mcp"}, {"cu2", "mcu2"}, {"cu3", "mcu3"}, {"cu", "mcu"}, {"swap", "mcswap"}, {"rxx", "rxx"},
      {"ryy", "ryy"}, {"rzz", "rzz"}, {"rzx", "rzx"}, {"csx", "mcsx"}, {"csxdg", "mcsxdg"}, {"ecr", "ecr"},
      {"crx", "mcrx"}, {"cry", "mcry"}, {"crz", "mcrz"}, {"ccx", "mcx"}, {"ccz", "mcz"}, {"cswap", "mcswap"},
      {"mcx", "mcx"}, {"mcy", "mcy"}, {"mcz", "mcz"}, {"mcr", "mcr"}, {"mcrx", "mcrx"}, {"mcry", "mcry"},
      {"mcrz", "mcrz"}, {"mcphase", "mcp"}, {"mcp", "mcp"}, {"mcu1", "mcp"}, {"mcu2", "mcu2"}, {"mcu3", "mcu3"},
      {"mcu", "mcu"}, {"mcswap", "mcswap"}, {"mcsx", "mcsx"}, {"mcsxdg", "mcsxdg"}, {"mcx_gray", "mcx"}};
  return g;
}

// Gates of QubitUnitary::StateOpSet (unitary_state.hpp:35-54): the gates
// UnitaryFusion may absorb.
const std::unordered_set<std::string> &unitary_gates() {
  static const std::unordered_set<std::string> g = {
      "u1", "u2", "u3", "u", "U", "CX", "cx", "cz", "cy", "cp", "cu1", "cu2", "cu3", "swap", "id", "p",
      "x", "y", "z", "h", "s", "sdg", "t", "tdg", "r", "rx", "ry", "rz", "rxx", "ryy", "rzz", "rzx",
      "ccx", "ccz", "cswap", "mcx", "mcy", "mcz", "mcu1", "mcu2", "mcu3", "mcswap", "mcr", "mcrx", "mcry", "mcrz",
      "sx", "sxdg", "csx", "mcsx", "csxdg", "mcsxdg", "delay", "pauli", "cu", "mcu", "mcp", "ecr", "mcphase",
      "crx", "cry", "crz"};
  return g;
}

// Gates of QubitSuperoperator::StateOpSet (superoperator_state.hpp:35-50).
const std::unordered_set<std::string> &superop_gates() {
  static const std::unordered_set<std::string> g = {
      "U", "CX", "u1", "u2", "u3", "u", "cx", "cy", "cz", "swap", "id", "x", "y", "z", "h", "s", "sdg",
      "t", "tdg", "ccx", "r", "rx", "ry", "rz", "rxx", "ryy", "rzz", "rzx", "p", "cp", "cu1", "sx", "sxdg",
      "x90", "delay", "pauli", "ecr"};
  return g;
}

double par(const Op &op, size_t i) {
  REQUIRE(op.params.size() > i, GBQV_ERR_ARG, "gate '" + op.name + "' is missing parameters");
  return op.params[i];
}

Prim sv_prim(const Op &op) {
  auto it = sv_gateset().find(op.name);
  REQUIRE(it != sv_gateset().end(), GBQV_ERR_ARG, "QubitVectorState::invalid gate instruction '" + op.name + "'.");
  const std::string &g = it->second;
  const double pi = M_PI;
  Prim p;
  p.q = op.qubits;
  if (g == "mcx") p.k = P::MCX;
  else if (g == "mcy") p.k = P::MCY;
  else if (g == "mcz") { p.k = P::MCPHASE; p.m = {-1.0}; }
  else if (g == "mcr") { p.k = P::MCU; p.m = gates::r(par(op, 0), par(op, 1)); }
  else if (g == "mcrx") { p.k = P::MCU; p.m = gates::rx(par(op, 0)); }
  else if (g == "mcry") { p.k = P::MCU; p.m = gates::ry(par(op, 0)); }
  else if (g == "mcrz") { p.k = P::MCU; p.m = gates::rz(par(op, 0)); }
  else if (g == "rxx") { p.k = P::MATRIX; p.m = gates::rxx(par(op, 0)); }
  else if (g == "ryy") { p.k = P::MATRIX; p.m = gates::ryy(par(op, 0)); }
  else if (g == "rzz") { p.k = P::DIAG; p.m = gates::rzz_diag(par(op, 0)); }
  else if (g == "rzx") { p.k = P::MATRIX; p.m = gates::rzx(par(op, 0)); }
  else if (g == "ecr") { p.k = P::MATRIX; p.m = gates::ECR(); }
  else if (g == "id") p.k = P::NONE;
  else if (g == "h") { p.k = P::MCU; p.m = gates::u4(pi / 2., 0., pi, 0.); }
  else if (g == "s") { p.k = P::DIAG; p.q = {op.qubits[0]}; p.m = {1.0, cd(0., 1.)}; }
  else if (g == "sdg") { p.k = P::DIAG; p.q = {op.qubits[0]}; p.m = {1.0, cd(0., -1.)}; }
  else if (g == "t") { const double s = 1. / std::sqrt(2); p.k = P::DIAG; p.q = {op.qubits[0]}; p.m = {1.0, cd(s, s)}; }
  else if (g == "tdg") { const double s = 1. / std::sqrt(2); p.k = P::DIAG; p.q = {op.qubits[0]}; p.m = {1.0, cd(s, -s)}; }
  else if (g == "mcswap") p.k = P::MCSWAP;
  else if (g == "mcu3") { p.k = P::MCU; p.m = gates::u4(par(op, 0), par(op, 1), par(op, 2), 0.); }
  else if (g == "mcu") { p.k = P::MCU; p.m = gates::u4(par(op, 0), par(op, 1), par(op, 2), par(op, 3)); }
  else if (g == "mcu2") { p.k = P::MCU; p.m = gates::u4(pi / 2., par(op, 0), par(op, 1), 0.); }
  else if (g == "mcp") { p.k = P::MCPHASE; p.m = {std::exp(cd(0, 1) * par(op, 0))}; }
  else if (g == "mcsx") { p.k = P::MCU; p.m = gates::SX(); }
  else if (g == "mcsxdg") { p.k = P::MCU; p.m = gates::SXDG(); }
  else throw Error(GBQV_ERR_ARG, "QubitVector::State::invalid gate instruction '" + op.name + "'.");
  return p;
}

// ------------------------------------------------------------------------
// Host qreg for fused-matrix construction (tiny sizes; the role the
// reference's CPU UnitaryMatrix / Superoperator play in fusion.hpp:159-222)
// ------------------------------------------------------------------------
struct HostVec {
  int nb;
  std::vector<cd> v;

  static uint64_t ins0(uint64_t i, const reg_t &sorted) {
    for (uint64_t q : sorted) {
      const uint64_t m = (1ULL << q) - 1;
      i = ((i & ~m) << 1) | (i & m);
    }
    return i;
  }
  void groups(const reg_t &q, std::vector<uint64_t> &offs, reg_t &sorted) const {
    sorted = q;
    std::sort(sorted.begin(), sorted.end());
    offs.assign(1ULL << q.size(), 0);
    for (size_t j = 0; j < q.size(); ++j) {
      const uint64_t n = 1ULL << j, bit = 1ULL << q[j];
      for (uint64_t m = 0; m < n; ++m) offs[n + m] = offs[m] | bit;
    }
  }
  void matrix(const reg_t &q, const cd *mat) {
    std::vector<uint64_t> offs;
    reg_t s;
    groups(q, offs, s);
    const uint64_t D = offs.size(), G = (1ULL << nb) >> q.size();
    std::vector<cd> cache(D);
    for (uint64_t g = 0; g < G; ++g) {
      const uint64_t b = ins0(g, s);
      for (uint64_t a = 0; a < D; ++a) { cache[a] = v[b + offs[a]]; v[b + offs[a]] = 0.0; }
      for (uint64_t a = 0; a < D; ++a)
        for (uint64_t c = 0; c < D; ++c) v[b + offs[a]] += mat[a + D * c] * cache[c];
    }
  }
  void diag(const reg_t &q, const cd *d) {
    for (uint64_t i = 0; i < v.size(); ++i) {
      uint64_t iv = 0;
      for (size_t j = 0; j < q.size(); ++j)
        if (i & (1ULL << q[j])) iv |= 1ULL << j;
      if (d[iv] != 1.0) v[i] *= d[iv];
    }
  }
  // multi-controlled 2x2 on the last qubit, controls all set
  void mc2(const reg_t &q, const cd *m2) {
    uint64_t ctrl = 0;
    for (size_t j = 0; j + 1 < q.size(); ++j) ctrl |= 1ULL << q[j];
    const uint64_t t = 1ULL << q.back();
    for (uint64_t i = 0; i < v.size(); ++i) {
      if ((i & ctrl) != ctrl || (i & t)) continue;
      const cd a0 = v[i], a1 = v[i | t];
      v[i] = m2[0] * a0 + m2[2] * a1;
      v[i | t] = m2[1] * a0 + m2[3] * a1;
    }
  }
  void mcswap(const reg_t &q) {
    uint64_t ctrl = 0;
    for (size_t j = 0; j + 2 < q.size(); ++j) ctrl |= 1ULL << q[j];
    const uint64_t a = 1ULL << q[q.size() - 2], b = 1ULL << q.back();
    for (uint64_t i = 0; i < v.size(); ++i)
      if ((i & ctrl) == ctrl && (i & a) && !(i & b)) std::swap(v[i], v[(i ^ a) | b]);
  }
  void prim(const Prim &p) {
    switch (p.k) {
      case P::NONE: return;
      case P::MCX: { const cd x[4] = {0., 1., 1., 0.}; mc2(p.q, x); return; }
      case P::MCY: { const cd y[4] = {0., cd(0, 1), cd(0, -1), 0.}; mc2(p.q, y); return; }
      case P::MCPHASE: { const cd ph[4] = {1., 0., 0., p.m[0]}; mc2(p.q, ph); return; }
      case P::MCU: mc2(p.q, p.m.data()); return;
      case P::MATRIX: matrix(p.q, p.m.data()); return;
      case P::DIAG: diag(p.q, p.m.data()); return;
      case P::MCSWAP: mcswap(p.q); return;
    }
  }
};

// Unitary of one op on its own qubits (local 0..k-1), column-major.
std::vector<cd> op_unitary(const Op &op) {
  const int k = (int)op.qubits.size();
  const size_t D = 1ULL << k;
  if (op.type == GBQV_OP_MATRIX) return op.mat;
  if (op.type == GBQV_OP_DIAGONAL) {
    std::vector<cd> m(D * D);
    for (size_t i = 0; i < D; ++i) m[i + D * i] = op.mat[i];
    return m;
  }
  HostVec h{2 * k, gates::identity(D)};
  Op local = op;
  for (int i = 0; i < k; ++i) local.qubits[i] = i;
  h.prim(sv_prim(local));
  return h.v;
}

bool is_diagonal_mat(const std::vector<cd> &m, size_t D) {
  for (size_t c = 0; c < D; ++c)
    for (size_t r = 0; r < D; ++r)
      if (r != c && m[r + D * c] != 0.0) return false;
  return true;
}

// ------------------------------------------------------------------------
// Fusion (src/transpile/fusion.hpp) restated
// ------------------------------------------------------------------------
enum class FMethod { UNITARY, SUPEROP, KRAUS };

struct Fusion {
  gbqv_fusion_config cfg;
  FMethod method = FMethod::UNITARY;

  // FusionMethod::can_ignore (fusion.hpp:120-129)
  bool can_ignore(const Op &op) const {
    if (op.type == GBQV_OP_BARRIER) return true;
    if (op.type == GBQV_OP_GATE) return op.name == "id" || op.name == "u0";
    return false;
  }
  // UnitaryFusion::can_apply (fusion.hpp:176-193) / SuperOpFusion::can_apply (:225-242)
  bool unitary_can_apply(const Op &op, uint64_t maxq) const {
    switch (op.type) {
      case GBQV_OP_MATRIX: return op.qubits.size() <= maxq;
      case GBQV_OP_DIAGONAL: return op.qubits.size() <= maxq;
      case GBQV_OP_GATE: return op.qubits.size() <= maxq && unitary_gates().count(op.name);
      default: return false;
    }
  }
  bool can_apply(const Op &op, uint64_t maxq) const {
    // gates with bound parameters stay unfused: they run as per-binding
    // members of cache-blocked runs (execute_bound)
    if (!op.bparams.empty()) return false;
    if (method == FMethod::UNITARY) return unitary_can_apply(op, maxq);
    switch (op.type) {
      case GBQV_OP_KRAUS:
      case GBQV_OP_RESET:
      case GBQV_OP_SUPEROP: return op.qubits.size() <= maxq;
      case GBQV_OP_GATE: return op.qubits.size() <= maxq && superop_gates().count(op.name);
      default: return unitary_can_apply(op, maxq);
    }
  }
  bool support_diagonal() const { return method == FMethod::UNITARY; }

  static bool non_unitary(const std::vector<Op> &ops) {
    for (auto &op : ops)
      if (op.type == GBQV_OP_KRAUS || op.type == GBQV_OP_SUPEROP || op.type == GBQV_OP_RESET) return true;
    return false;
  }

  // FusionMethod::generate_operation (fusion.hpp:38-110): remap onto the
  // sorted union of qubits, simulate, map back.
  Op generate(std::vector<Op> ops, bool diagonal) const {
    std::set<uint64_t> qs;
    for (auto &op : ops) qs.insert(op.qubits.begin(), op.qubits.end());
    reg_t remapped2orig(qs.begin(), qs.end());
    std::map<uint64_t, uint64_t> orig2remapped;
    for (size_t i = 0; i < remapped2orig.size(); ++i) orig2remapped[remapped2orig[i]] = i;
    for (auto &op : ops)
      for (auto &q : op.qubits) q = orig2remapped[q];
    const int k = (int)remapped2orig.size();
    const size_t D = 1ULL << k;
    Op out;
    out.qubits = remapped2orig;
    if (method != FMethod::UNITARY && non_unitary(ops)) {
      out.type = GBQV_OP_SUPEROP;
      out.name = "superop";
      out.mat = superop_sim(ops, k);
      return out;
    }
    // QubitUnitary::State simulation (UnitaryFusion::generate_operation_internal)
    HostVec u{2 * k, gates::identity(D)};
    for (auto &op : ops) {
      switch (op.type) {
        case GBQV_OP_GATE: u.prim(sv_prim(op)); break;
        case GBQV_OP_MATRIX: u.matrix(op.qubits, op.mat.data()); break;
        case GBQV_OP_DIAGONAL: u.diag(op.qubits, op.mat.data()); break;
        default: break;
      }
    }
    if (diagonal) {
      out.type = GBQV_OP_DIAGONAL;
      out.name = "fusion";
      out.mat.resize(D);
      for (size_t i = 0; i < D; ++i) out.mat[i] = u.v[i + D * i];
    } else {
      out.type = GBQV_OP_MATRIX;
      out.name = "fusion";
      out.mat = std::move(u.v);
    }
    return out;
  }

  // QubitSuperoperator::State simulation (SuperOpFusion, fusion.hpp:202-222):
  // the superoperator is a 4k-qubit vector, ops act on (q, q+k).
  std::vector<cd> superop_sim(const std::vector<Op> &ops, int k) const {
    const size_t D = 1ULL << k;
    HostVec s{4 * k, gates::identity(D * D)};
    auto sq = [&](const reg_t &q) {
      reg_t r = q;
      for (uint64_t x : q) r.push_back(x + k);
      return r;
    };
    for (auto &op : ops) {
      const size_t d = 1ULL << op.qubits.size();
      switch (op.type) {
        case GBQV_OP_SUPEROP: s.matrix(sq(op.qubits), op.mat.data()); break;
        case GBQV_OP_KRAUS: {
          std::vector<cd> sup(d * d * d * d, 0.0);
          for (auto &K : op.kraus) {
            auto t = gates::vmat2vsuperop(K.data(), d);
            for (size_t i = 0; i < sup.size(); ++i) sup[i] += t[i];
          }
          s.matrix(sq(op.qubits), sup.data());
          break;
        }
        case GBQV_OP_RESET: s.matrix(sq(op.qubits), gates::reset_superop((int)op.qubits.size()).data()); break;
        case GBQV_OP_DIAGONAL: {
          std::vector<cd> dd(d * d);
          for (size_t i = 0; i < d; ++i)
            for (size_t j = 0; j < d; ++j) dd[i * d + j] = std::conj(op.mat[i]) * op.mat[j];
          s.diag(sq(op.qubits), dd.data());
          break;
        }
        default: {  // gate / matrix: unitary superoperator conj(U) (x) U
          auto U = op_unitary(op);
          s.matrix(sq(op.qubits), gates::vmat2vsuperop(U.data(), d).data());
          break;
        }
      }
    }
    return s.v;
  }

  void allocate_new_operation(std::vector<Op> &ops, uint64_t idx, const std::vector<uint64_t> &idxs,
                              bool diagonal) const {
    std::vector<Op> fusing;
    for (uint64_t i : idxs) fusing.push_back(ops[i]);
    ops[idx] = generate(fusing, diagonal);
    for (uint64_t i : idxs)
      if (i != idx) ops[i].type = OP_NOP;
  }

  // ---- NQubitFusion<N> (fusion.hpp:382-494) ----
  static bool exclude_escaped(reg_t &fusing_qubits, const Op &tgt) {
    bool included = true;
    for (auto q : tgt.qubits) included &= std::find(fusing_qubits.begin(), fusing_qubits.end(), q) != fusing_qubits.end();
    if (included) return false;
    for (auto q : tgt.qubits) {
      auto f = std::find(fusing_qubits.begin(), fusing_qubits.end(), q);
      if (f != fusing_qubits.end()) fusing_qubits.erase(f);
    }
    return true;
  }

  bool nqubit(std::vector<Op> &ops, int N, int start, int end, uint64_t maxq) const {
    bool fused = false;
    for (int op_idx = start; op_idx < end; ++op_idx) {
      if (!can_apply(ops[op_idx], maxq) || ops[op_idx].type == OP_NOP) continue;
      if ((int)ops[op_idx].qubits.size() != N) continue;
      std::vector<uint64_t> idxs = {(uint64_t)op_idx};
      reg_t fq = ops[op_idx].qubits;
      for (int f = op_idx - 1; f >= start; --f) {
        auto &t = ops[f];
        if (t.type == OP_NOP) continue;
        if (!can_apply(t, maxq)) break;
        if (!exclude_escaped(fq, t)) idxs.push_back(f);
        else if (fq.empty()) break;
      }
      std::reverse(idxs.begin(), idxs.end());
      fq = ops[op_idx].qubits;
      for (int f = op_idx + 1; f < end; ++f) {
        auto &t = ops[f];
        if (t.type == OP_NOP) continue;
        if (!can_apply(t, maxq)) break;
        if (!exclude_escaped(fq, t)) idxs.push_back(f);
        else if (fq.empty()) break;
      }
      if (idxs.size() <= 1) continue;
      allocate_new_operation(ops, op_idx, idxs, false);
      fused = true;
    }
    return fused;
  }

  // ---- DiagonalFusion (fusion.hpp:496-680) ----
  static bool is_diagonal_op(const Op &op) {
    if (op.type == GBQV_OP_DIAGONAL) return true;
    if (op.type == GBQV_OP_GATE) {
      if (op.name == "p" || op.name == "cp" || op.name == "u1" || op.name == "cu1" || op.name == "mcu1" ||
          op.name == "rz" || op.name == "rzz")
        return true;
      if (op.name == "u3") return op.params.size() >= 2 && op.params[0] == 0.0 && op.params[1] == 0.0;
    }
    return false;
  }

  int next_diagonal_end(const std::vector<Op> &ops, int from, int end, std::set<uint64_t> &fq) const {
    if (!ops[from].bparams.empty()) return -1;  // bound gates stay unfused
    if (is_diagonal_op(ops[from])) {
      for (auto q : ops[from].qubits) fq.insert(q);
      return from;
    }
    if (ops[from].type != GBQV_OP_GATE) return -1;
    int pos = from;
    for (; pos < end; ++pos)
      if (ops[from].type != GBQV_OP_GATE || ops[pos].name != "cx") break;
    if (pos == from || pos == end) return -1;
    int cx_end = pos - 1;
    bool found = false;
    for (; pos < end; ++pos) {
      if (is_diagonal_op(ops[pos])) found = true;
      else break;
    }
    if (!found) return -1;
    if (pos == end) return -1;
    const int u1_end = pos;
    for (; pos < end; ++pos) {
      if (ops[pos].type == GBQV_OP_GATE && ops[pos].name == ops[cx_end].name && ops[pos].qubits == ops[cx_end].qubits) {
        if (cx_end == from) break;
        --cx_end;
      } else {
        return -1;
      }
    }
    if (pos == end) return -1;
    for (int i = from; i < u1_end; ++i)
      for (auto q : ops[i].qubits) fq.insert(q);
    return pos;
  }

  bool diagonal_fusion(std::vector<Op> &ops, int start, int end, uint64_t maxq) const {
    if (!support_diagonal()) return false;
    const uint64_t min_qubit = 3;
    for (int op_idx = start; op_idx < end; ++op_idx) {
      std::set<uint64_t> checking;
      const int nde0 = next_diagonal_end(ops, op_idx, end, checking);
      if (nde0 < 0) continue;
      if (checking.size() > maxq) continue;
      int next_start = nde0 + 1;
      while (true) {
        // the reference reads ops[next_start] past the window end (an op that
        // exists in the circuit); stop only at the end of the op list
        if (next_start >= (int)ops.size()) break;
        const int nde = next_diagonal_end(ops, next_start, end, checking);
        if (nde < 0 || checking.size() > maxq) break;
        next_start = nde + 1;
      }
      if (checking.size() < min_qubit) continue;
      std::vector<uint64_t> idxs;
      while (op_idx < next_start) idxs.push_back(op_idx++);
      --op_idx;
      allocate_new_operation(ops, op_idx, idxs, true);
    }
    return true;
  }

  // ---- CostBasedFusion (fusion.hpp:996-1150) ----
  static void add_fusion_qubits(reg_t &fq, const Op &op) {
    for (auto q : op.qubits)
      if (std::find(fq.begin(), fq.end(), q) == fq.end()) fq.push_back(q);
  }

  static bool cost_is_diagonal(const std::vector<Op> &ops, uint64_t from, uint64_t until) {
    for (uint64_t i = from; i <= until; ++i) {
      if ((i + 2) <= until && ops[i].name == "cx" && ops[i + 1].name == "u1" && ops[i + 2].name == "cx" &&
          ops[i].qubits.size() > 1 && ops[i + 2].qubits.size() > 1 && !ops[i + 1].qubits.empty() &&
          ops[i].qubits[1] == ops[i + 1].qubits[0] && ops[i + 1].qubits[0] == ops[i + 2].qubits[1] &&
          ops[i].qubits[0] == ops[i + 2].qubits[0]) {
        i += 2;
        continue;
      }
      if (ops[i].name == "u1" || ops[i].name == "cu1" || ops[i].name == "cp") continue;
      return false;
    }
    return true;
  }

  double estimate_cost(const std::vector<Op> &ops, uint64_t from, uint64_t until) const {
    if (cost_is_diagonal(ops, from, until)) return 1.0;
    reg_t fq;
    for (uint64_t i = from; i <= until; ++i) add_fusion_qubits(fq, ops[i]);
    const size_t n = fq.size();
    if (cfg.avx2_costs) {
      switch (n) {
        case 1:
        case 2: return 1.0;
        case 3: return 1.1;
        case 4: return 3;
        default: return std::pow(cfg.cost_factor, (double)std::max<size_t>(n - 2, 1));
      }
    }
    return std::pow(cfg.cost_factor, (double)std::max<size_t>(n - 1, 1));
  }

  bool cost_based(std::vector<Op> &ops, int start, int end, uint64_t maxq) const {
    std::vector<double> costs;
    std::vector<int> fusion_to;
    fusion_to.push_back(start);
    costs.push_back(can_ignore(ops[start]) ? .0 : cfg.cost_factor);
    bool applied = false;
    for (int i = start + 1; i < end; ++i) {
      fusion_to.push_back(i);
      costs.push_back(costs[i - start - 1] + (can_ignore(ops[i]) ? .0 : cfg.cost_factor));
      for (int num_fusion = 2; num_fusion <= (int)maxq; ++num_fusion) {
        reg_t fq;
        add_fusion_qubits(fq, ops[i]);
        for (int j = i - 1; j >= start; --j) {
          add_fusion_qubits(fq, ops[j]);
          if ((int)fq.size() > num_fusion) break;
          const double est = estimate_cost(ops, (uint64_t)j, i) + (j <= start ? 0.0 : costs[j - 1 - start]);
          if (est <= costs[i - start]) {
            costs[i - start] = est;
            fusion_to[i - start] = j;
            applied = true;
          }
        }
      }
    }
    if (!applied) return false;
    for (int i = end - 1; i >= start;) {
      const int to = fusion_to[i - start];
      if (to != i) {
        std::vector<uint64_t> idxs;
        for (int j = to; j <= i; ++j) idxs.push_back(j);
        if (!idxs.empty()) allocate_new_operation(ops, i, idxs, false);
      }
      i = to - 1;
    }
    return true;
  }

  // Fusion::optimize_circuit over a range (fusion.hpp:850-866)
  template <typename Fn>
  void windows(std::vector<Op> &ops, uint64_t maxq, Fn &&fuser) const {
    int fusion_start = 0;
    const int ops_end = (int)ops.size();
    for (int op_idx = 0; op_idx < ops_end; ++op_idx) {
      if (can_ignore(ops[op_idx])) continue;
      if (!can_apply(ops[op_idx], maxq) || op_idx == ops_end - 1) {
        fuser(ops, fusion_start, op_idx, maxq);
        fusion_start = op_idx + 1;
      }
    }
  }

  static bool compact(std::vector<Op> &ops) {
    size_t idx = 0;
    for (size_t i = 0; i < ops.size(); ++i)
      if (ops[i].type != OP_NOP) {
        if (i != idx) ops[idx] = std::move(ops[i]);
        ++idx;
      }
    const bool removed = idx != ops.size();
    ops.resize(idx);
    return removed;
  }
};

}  // namespace

// ============================== C ABI: circuits ==============================

extern "C" int gbqv_circuit_create(int num_qubits, gbqv_circuit_t *out) {
  return guard([&] {
    REQUIRE(out && num_qubits >= 1 && num_qubits <= kMaxQubits, GBQV_ERR_ARG, "bad circuit size");
    auto *c = new gbqv_circuit;
    c->num_qubits = num_qubits;
    *out = c;
  });
}

extern "C" int gbqv_circuit_destroy(gbqv_circuit_t c) {
  delete c;
  return GBQV_OK;
}

extern "C" int gbqv_circuit_gate(gbqv_circuit_t c, const char *name, const uint64_t *qubits, int nq,
                                 const double *params, int nparams) {
  return guard([&] {
    Op op;
    op.type = GBQV_OP_GATE;
    REQUIRE(name, GBQV_ERR_ARG, "null gate name");
    op.name = name;
    op.qubits = check_q(c, qubits, nq);
    op.params.assign(params, params + std::max(nparams, 0));
    // validate the name and arity now, as Circuit::set_params would
    Prim p = sv_prim(op);
    (void)p;
    c->ops.push_back(std::move(op));
    ++c->version;
  });
}

extern "C" int gbqv_circuit_unitary(gbqv_circuit_t c, const uint64_t *qubits, int k, const gbqv_c128 *mat) {
  return guard([&] {
    Op op;
    op.type = GBQV_OP_MATRIX;
    op.name = "unitary";
    op.qubits = check_q(c, qubits, k);
    REQUIRE(mat && k <= kMaxDenseK, GBQV_ERR_ARG, "bad unitary");
    const cd *m = reinterpret_cast<const cd *>(mat);
    op.mat.assign(m, m + (1ULL << (2 * k)));
    c->ops.push_back(std::move(op));
    ++c->version;
  });
}

extern "C" int gbqv_circuit_diagonal(gbqv_circuit_t c, const uint64_t *qubits, int k, const gbqv_c128 *diag) {
  return guard([&] {
    Op op;
    op.type = GBQV_OP_DIAGONAL;
    op.name = "diagonal";
    op.qubits = check_q(c, qubits, k);
    REQUIRE(diag && k <= kMaxDiagK, GBQV_ERR_ARG, "bad diagonal");
    const cd *m = reinterpret_cast<const cd *>(diag);
    op.mat.assign(m, m + (1ULL << k));
    c->ops.push_back(std::move(op));
    ++c->version;
  });
}

extern "C" int gbqv_circuit_superop(gbqv_circuit_t c, const uint64_t *qubits, int k, const gbqv_c128 *mat) {
  return guard([&] {
    Op op;
    op.type = GBQV_OP_SUPEROP;
    op.name = "superop";
    op.qubits = check_q(c, qubits, k);
    REQUIRE(mat && 2 * k <= 10, GBQV_ERR_ARG, "bad superoperator");
    const cd *m = reinterpret_cast<const cd *>(mat);
    op.mat.assign(m, m + (1ULL << (4 * k)));
    c->ops.push_back(std::move(op));
    ++c->version;
  });
}

extern "C" int gbqv_circuit_kraus(gbqv_circuit_t c, const uint64_t *qubits, int k, int nk, const gbqv_c128 *mats) {
  return guard([&] {
    Op op;
    op.type = GBQV_OP_KRAUS;
    op.name = "kraus";
    op.qubits = check_q(c, qubits, k);
    REQUIRE(mats && nk >= 1 && 2 * k <= 10, GBQV_ERR_ARG, "bad Kraus set");
    const cd *m = reinterpret_cast<const cd *>(mats);
    const size_t sz = 1ULL << (2 * k);
    for (int i = 0; i < nk; ++i) op.kraus.emplace_back(m + i * sz, m + (i + 1) * sz);
    c->ops.push_back(std::move(op));
    ++c->version;
  });
}

extern "C" int gbqv_circuit_reset(gbqv_circuit_t c, const uint64_t *qubits, int k) {
  return guard([&] {
    Op op;
    op.type = GBQV_OP_RESET;
    op.name = "reset";
    op.qubits = check_q(c, qubits, k);
    c->ops.push_back(std::move(op));
    ++c->version;
  });
}

extern "C" int gbqv_circuit_barrier(gbqv_circuit_t c, const uint64_t *qubits, int k) {
  return guard([&] {
    Op op;
    op.type = GBQV_OP_BARRIER;
    op.name = "barrier";
    op.qubits = check_q(c, qubits, k, 0);
    c->ops.push_back(std::move(op));
    ++c->version;
  });
}

extern "C" int gbqv_circuit_num_ops(gbqv_circuit_t c, int *out) {
  return guard([&] {
    REQUIRE(c && out, GBQV_ERR_ARG, "null argument");
    *out = (int)c->ops.size();
  });
}

extern "C" int gbqv_circuit_op_info(gbqv_circuit_t c, int i, int *type, int *nq, uint64_t *qubits, int max_qubits,
                                    char *name_buf, int name_len) {
  return guard([&] {
    REQUIRE(c && i >= 0 && i < (int)c->ops.size(), GBQV_ERR_ARG, "op index out of range");
    const Op &op = c->ops[i];
    if (type) *type = op.type;
    if (nq) *nq = (int)op.qubits.size();
    if (qubits)
      for (int j = 0; j < std::min<int>(max_qubits, (int)op.qubits.size()); ++j) qubits[j] = op.qubits[j];
    if (name_buf && name_len > 0) {
      std::strncpy(name_buf, op.name.c_str(), name_len - 1);
      name_buf[name_len - 1] = 0;
    }
  });
}

extern "C" int gbqv_circuit_op_matrix(gbqv_circuit_t c, int i, gbqv_c128 *out, uint64_t len) {
  return guard([&] {
    REQUIRE(c && i >= 0 && i < (int)c->ops.size(), GBQV_ERR_ARG, "op index out of range");
    const Op &op = c->ops[i];
    std::vector<cd> m = op.type == GBQV_OP_GATE ? op_unitary(op) : op.mat;
    REQUIRE(len == m.size(), GBQV_ERR_ARG, "matrix length mismatch: op holds " + std::to_string(m.size()));
    std::memcpy(out, m.data(), sizeof(cd) * m.size());
  });
}

extern "C" int gbqv_circuit_bind_param(gbqv_circuit_t c, int op_index, int param_pos, int nbind,
                                       const double *values) {
  return guard([&] {
    REQUIRE(c && values, GBQV_ERR_ARG, "null argument");
    REQUIRE(nbind >= 1, GBQV_ERR_ARG, "Invalid parameterization: no parameter values");
    REQUIRE(c->nbind == 0 || c->nbind == nbind, GBQV_ERR_ARG,
            "Invalid parameterization: every parameter needs the same number of values (" +
                std::to_string(c->nbind) + ")");
    REQUIRE(op_index >= 0 && op_index < (int)c->ops.size(), GBQV_ERR_ARG,
            "Invalid parameterized qobj: instruction position out of range");
    Op &op = c->ops[op_index];
    REQUIRE(op.type == GBQV_OP_GATE, GBQV_ERR_ARG, "Invalid parameterized qobj: only gate parameters can be bound");
    REQUIRE(param_pos >= 0 && param_pos < (int)op.params.size(), GBQV_ERR_ARG,
            "Invalid parameterized qobj: instruction param position out of range");
    const size_t stride = op.params.size();
    if (op.bparams.empty()) {
      op.bparams.resize(stride * nbind);
      for (int j = 0; j < nbind; ++j) std::copy(op.params.begin(), op.params.end(), op.bparams.begin() + j * stride);
    }
    for (int j = 0; j < nbind; ++j) op.bparams[param_pos + stride * j] = values[j];
    op.params[param_pos] = values[0];
    c->nbind = nbind;
    ++c->version;
  });
}

extern "C" int gbqv_circuit_num_bindings(gbqv_circuit_t c, int *out) {
  return guard([&] {
    REQUIRE(c && out, GBQV_ERR_ARG, "null argument");
    *out = c->nbind;
  });
}

extern "C" int gbqv_fusion_default_config(int method, gbqv_fusion_config *cfg) {
  return guard([&] {
    REQUIRE(cfg && (method == 0 || method == 1), GBQV_ERR_ARG, "bad fusion method");
    cfg->method = method;
    cfg->enable = 1;
    cfg->max_qubit = 5;
    cfg->threshold = 14;
    cfg->cost_factor = 1.8;
    cfg->avx2_costs = 1;
    cfg->allow_superop = 0;
    cfg->allow_kraus = 0;
    if (method == 1) {  // Executor::transpile_fusion halves both for density_matrix
      cfg->threshold /= 2;
      cfg->max_qubit /= 2;
    }
  });
}

// Fusion::optimize_circuit (fusion.hpp:750-846)
extern "C" int gbqv_circuit_fuse(gbqv_circuit_t c, const gbqv_fusion_config *cfg, int *applied, char *method_name,
                                 int method_len) {
  return guard([&] {
    REQUIRE(c && cfg, GBQV_ERR_ARG, "null argument");
    Fusion f;
    f.cfg = *cfg;
    if (applied) *applied = 0;
    auto name_out = [&](const char *s) {
      if (method_name && method_len > 0) {
        std::strncpy(method_name, s, method_len - 1);
        method_name[method_len - 1] = 0;
      }
    };
    name_out("");
    if (!cfg->enable) return;
    if (c->num_qubits <= cfg->threshold || c->ops.size() < 2) return;
    // FusionMethod::find_method (fusion.hpp:279-295): the statevector state
    // allows kraus, the density-matrix state allows superop and kraus.
    bool has_kraus = false, has_superop = false, has_reset = false;
    for (auto &op : c->ops) {
      has_kraus |= op.type == GBQV_OP_KRAUS;
      has_superop |= op.type == GBQV_OP_SUPEROP;
      has_reset |= op.type == GBQV_OP_RESET;
    }
    const bool state_allows_superop = cfg->method == 1;
    if (cfg->allow_superop && state_allows_superop && (has_kraus || has_superop || has_reset))
      f.method = FMethod::SUPEROP;
    else if (cfg->allow_kraus && (has_kraus || has_superop))
      f.method = FMethod::KRAUS;
    else
      f.method = FMethod::UNITARY;
    name_out(f.method == FMethod::UNITARY ? "unitary" : f.method == FMethod::SUPEROP ? "superop" : "kraus");
    if (f.method == FMethod::KRAUS)
      throw Error(GBQV_ERR_ARG, "Kraus-method fusion (sampled Kraus noise on a statevector) is not supported");
    const uint64_t maxq = cfg->max_qubit;
    bool any = false;
    // fusers in order: Diagonal, 1-qubit, 2-qubit, cost-based (fusion.hpp:816-821)
    f.windows(c->ops, maxq, [&](std::vector<Op> &ops, int s, int e, uint64_t m) { f.diagonal_fusion(ops, s, e, m); });
    any |= Fusion::compact(c->ops);
    f.windows(c->ops, maxq, [&](std::vector<Op> &ops, int s, int e, uint64_t m) { f.nqubit(ops, 1, s, e, m); });
    any |= Fusion::compact(c->ops);
    f.windows(c->ops, maxq, [&](std::vector<Op> &ops, int s, int e, uint64_t m) { f.nqubit(ops, 2, s, e, m); });
    any |= Fusion::compact(c->ops);
    f.windows(c->ops, maxq, [&](std::vector<Op> &ops, int s, int e, uint64_t m) {
      if (s < e) f.cost_based(ops, s, e, m);
    });
    any |= Fusion::compact(c->ops);
    ++c->version;
    if (applied) *applied = any ? 1 : 0;
  });
}

// ============================== execution ==============================

namespace {

void exec_prim(Device &d, const Prim &p) {
  switch (p.k) {
    case P::NONE: return;
    case P::MCX: launch_mc(d, p.q, 0, nullptr); return;
    case P::MCY: launch_mc(d, p.q, 1, nullptr); return;
    case P::MCPHASE: launch_mc(d, p.q, 2, p.m.data()); return;
    case P::MCU: apply_mcu_impl(d, p.q, p.m.data()); return;
    case P::MATRIX: apply_matrix_impl(d, p.q, p.m.data()); return;
    case P::DIAG: apply_diag_impl(d, p.q, p.m.data()); return;
    case P::MCSWAP: launch_mc(d, p.q, 5, nullptr); return;
  }
}

// DensityMatrix::State::apply_gate (densitymatrix_state.hpp:641-760)
void exec_dm_gate(Device &d, const Op &op) {
  const std::string &g = op.name;
  const double pi = M_PI;
  const reg_t &q = op.qubits;
  auto unitary = [&](const std::vector<cd> &m) { dm_unitary(d, q, m.data()); };
  auto phase = [&](cd ph) {
    cd dd[4] = {1.0, ph, std::conj(ph), 1.0};
    apply_diag_impl(d, {q[0], q[0] + d.nq}, dd);
  };
  auto cphase = [&](cd ph) {
    std::vector<cd> dd(16, 1.0);
    dd[3] = dd[7] = dd[11] = ph;
    dd[12] = dd[13] = dd[14] = std::conj(ph);
    apply_diag_impl(d, superop_qubits(d, {q[0], q[1]}), dd.data());
  };
  auto perm = [&](const std::vector<std::pair<uint32_t, uint32_t>> &pairs) { launch_swaps(d, superop_qubits(d, q), pairs); };
  if (g == "u3" || g == "u" || g == "U") unitary(gates::u3(par(op, 0), par(op, 1), par(op, 2)));
  else if (g == "u2") unitary(gates::u3(pi / 2., par(op, 0), par(op, 1)));
  else if (g == "u1" || g == "p") phase(std::exp(cd(0., 1.) * par(op, 0)));
  else if (g == "cx" || g == "CX") perm({{1, 3}, {4, 12}, {5, 15}, {6, 14}, {7, 13}, {9, 11}});
  else if (g == "cy") {
    std::vector<cd> cy(16, 0.0);
    cy[0 + 4 * 0] = 1.0; cy[2 + 4 * 2] = 1.0; cy[3 + 4 * 1] = cd(0, 1); cy[1 + 4 * 3] = cd(0, -1);
    unitary(cy);
  }
  else if (g == "cz") cphase(-1.0);
  else if (g == "cp" || g == "cu1") cphase(std::exp(cd(0., 1.) * par(op, 0)));
  else if (g == "id" || g == "delay") return;
  else if (g == "x") perm({{0, 3}, {1, 2}});
  else if (g == "y") launch_dm_y(d, q[0]);
  else if (g == "z") phase(-1.0);
  else if (g == "h") unitary(gates::u3(pi / 2., 0., pi));
  else if (g == "s") phase(cd(0., 1.));
  else if (g == "sdg") phase(cd(0., -1.));
  else if (g == "sx" || g == "x90") unitary(gates::SX());
  else if (g == "sxdg") unitary(gates::SXDG());
  else if (g == "t") { const double s = 1. / std::sqrt(2); phase(cd(s, s)); }
  else if (g == "tdg") { const double s = 1. / std::sqrt(2); phase(cd(s, -s)); }
  else if (g == "swap") perm({{1, 2}, {4, 8}, {5, 10}, {6, 9}, {7, 11}, {13, 14}});
  else if (g == "ecr") unitary(gates::ECR());
  else if (g == "ccx")
    perm({{3, 7}, {11, 15}, {19, 23}, {24, 56}, {25, 57}, {26, 58}, {27, 63}, {28, 60}, {29, 61}, {30, 62},
          {31, 59}, {35, 39}, {43, 47}, {51, 55}});
  else if (g == "r") unitary(gates::r(par(op, 0), par(op, 1)));
  else if (g == "rx") unitary(gates::rx(par(op, 0)));
  else if (g == "ry") unitary(gates::ry(par(op, 0)));
  else if (g == "rz") dm_diag_unitary(d, q, gates::rz_diag(par(op, 0)).data());
  else if (g == "rxx") unitary(gates::rxx(par(op, 0)));
  else if (g == "ryy") unitary(gates::ryy(par(op, 0)));
  else if (g == "rzz") dm_diag_unitary(d, q, gates::rzz_diag(par(op, 0)).data());
  else if (g == "rzx") unitary(gates::rzx(par(op, 0)));
  else throw Error(GBQV_ERR_ARG, "DensityMatrixState::invalid gate instruction '" + g + "'.");
}

void exec_op(Device &d, const Op &op) {
  if (!d.density) {
    switch (op.type) {
      case GBQV_OP_GATE: exec_prim(d, sv_prim(op)); return;
      case GBQV_OP_MATRIX: {
        // Statevector::State::apply_matrix(op): diagonal check first (statevector_state.hpp:879-888)
        const size_t D = 1ULL << op.qubits.size();
        if (is_diagonal_mat(op.mat, D)) {
          std::vector<cd> dg(D);
          for (size_t i = 0; i < D; ++i) dg[i] = op.mat[i + D * i];
          apply_diag_impl(d, op.qubits, dg.data());
        } else {
          apply_matrix_impl(d, op.qubits, op.mat.data());
        }
        return;
      }
      case GBQV_OP_DIAGONAL: apply_diag_impl(d, op.qubits, op.mat.data()); return;
      case GBQV_OP_BARRIER: return;
      default:
        throw Error(GBQV_ERR_KIND, "op '" + op.name + "' needs shot sampling on a statevector; use a density matrix");
    }
  }
  switch (op.type) {
    case GBQV_OP_GATE: exec_dm_gate(d, op); return;
    case GBQV_OP_MATRIX: dm_unitary(d, op.qubits, op.mat.data()); return;
    case GBQV_OP_DIAGONAL: dm_diag_unitary(d, op.qubits, op.mat.data()); return;
    case GBQV_OP_SUPEROP: apply_matrix_impl(d, superop_qubits(d, op.qubits), op.mat.data()); return;
    case GBQV_OP_KRAUS: {
      const size_t dd = 1ULL << op.qubits.size();
      std::vector<cd> sup(dd * dd * dd * dd, 0.0);
      for (auto &K : op.kraus) {
        auto t = gates::vmat2vsuperop(K.data(), dd);
        for (size_t i = 0; i < sup.size(); ++i) sup[i] += t[i];
      }
      apply_matrix_impl(d, superop_qubits(d, op.qubits), sup.data());
      return;
    }
    case GBQV_OP_RESET:
      apply_matrix_impl(d, superop_qubits(d, op.qubits), gates::reset_superop((int)op.qubits.size()).data());
      return;
    case GBQV_OP_BARRIER: return;
  }
}

}  // namespace

namespace {

// The op as a run member (dense or diagonal matrix on vector qubits), when it
// has one on at most 5 vector qubits.  Same arithmetic as exec_op's kernels.
bool as_run_op(const Device &d, const Op &op, RunOp &out) {
  out.qubits.clear();
  out.mat.clear();
  if (!d.density) {
    if (op.type == GBQV_OP_MATRIX) {
      const size_t D = 1ULL << op.qubits.size();
      if (op.qubits.size() > 5) return false;
      out.qubits = op.qubits;
      if (is_diagonal_mat(op.mat, D)) {
        out.kind = 1;
        for (size_t i = 0; i < D; ++i) out.mat.push_back(op.mat[i + D * i]);
      } else {
        out.kind = 0;
        out.mat = op.mat;
      }
      return true;
    }
    if (op.type == GBQV_OP_DIAGONAL) {
      if (op.qubits.size() > 5) return false;
      out.kind = 1;
      out.qubits = op.qubits;
      out.mat = op.mat;
      return true;
    }
    if (op.type == GBQV_OP_GATE) {
      Prim p = sv_prim(op);
      if (p.k == P::NONE || p.q.size() > 5) return false;
      if (p.k == P::DIAG) {
        out.kind = 1;
        out.qubits = p.q;
        out.mat = p.m;
        return true;
      }
      if (p.k == P::MATRIX) {
        out.kind = 0;
        out.qubits = p.q;
        out.mat = p.m;
        return true;
      }
      if (p.k == P::MCPHASE) {
        out.kind = 1;
        out.qubits = p.q;
        out.mat.assign(1ULL << p.q.size(), 1.0);
        out.mat.back() = p.m[0];
        return true;
      }
      if (p.k == P::MCX) {  // exact swaps inside the tile
        out.kind = 2;
        out.qubits = p.q;
        return true;
      }
      return false;
    }
    return false;
  }
  // density matrix: superoperators on (q, q+n), k <= 2
  if (op.qubits.size() > 2) return false;
  const size_t dd = 1ULL << op.qubits.size();
  out.qubits = superop_qubits(d, op.qubits);
  if (op.type == GBQV_OP_SUPEROP) {
    out.kind = 0;
    out.mat = op.mat;
    return true;
  }
  if (op.type == GBQV_OP_MATRIX) {
    out.kind = 0;
    out.mat = gates::vmat2vsuperop(op.mat.data(), dd);
    return true;
  }
  if (op.type == GBQV_OP_DIAGONAL) {
    out.kind = 1;
    out.mat.resize(dd * dd);
    for (size_t i = 0; i < dd; ++i)
      for (size_t j = 0; j < dd; ++j) out.mat[i * dd + j] = std::conj(op.mat[i]) * op.mat[j];
    return true;
  }
  return false;
}

// Ops worth batching into a run: memory-bound ones.  A dense k >= 3 op does
// 4*2^k FMAs per amplitude and is already compute-bound in one pass, so it
// keeps its own streaming kernel; 1-2 qubit dense ops and diagonals are
// bandwidth-bound and share passes.
// Diagonals and 1-2 qubit matrices share a cache-blocked pass; complex128
// dense matrices that the tensor path takes (padded to 4 qubits) go there.
bool worth_batching(const Device &d, const RunOp &r) {
  return r.kind == 1 || r.kind == 2 || (r.qubits.size() <= 2 && !tensor_dense_available(d, (int)r.qubits.size()));
}

// Greedy cache-blocking schedule: starting from the first pending op, take
// every later op that (a) touches no qubit of an op left behind (so moving
// it earlier commutes) and (b) keeps the union of qubits within one tile.
// conv/runnable: each op's run form and whether it joins runs.  With `bound`
// the state is a stack of bound states: tiles stay below bound->state_bits,
// ops with per-binding matrices fill the per-binding pool, and ops outside
// runs (exec_op) act on every state of the stack alike.
void schedule_runs(Device &d, const std::vector<Op> &ops, const std::vector<RunOp> &conv,
                   const std::vector<char> &runnable, const RunBound *bound) {
  const int m = bound ? std::min(run_tile_qubits(d), bound->state_bits) : run_tile_qubits(d);
  const int c = std::min(run_low_qubits(d), m);
  const size_t pool_cap = run_pool_bytes(d) / 16, bound_cap = run_bound_pool_bytes(d) / 16;
  std::vector<char> done(ops.size(), 0);
  const size_t lookahead = 96;
  size_t first = 0;
  while (first < ops.size()) {
    while (first < ops.size() && done[first]) ++first;
    if (first >= ops.size()) break;
    if (!runnable[first]) {
      exec_op(d, ops[first]);
      done[first] = 1;
      continue;
    }
    std::vector<char> inT(d.n, 0), blocked(d.n, 0);
    int tcount = 0;
    for (int q = 0; q < c; ++q) inT[q] = 1, ++tcount;
    std::vector<const RunOp *> run;
    std::vector<size_t> members;
    size_t pool = 0, bpool = 0;
    size_t scanned = 0;
    for (size_t i = first; i < ops.size() && scanned < lookahead; ++i) {
      if (done[i]) continue;
      ++scanned;
      const reg_t &q = runnable[i] ? conv[i].qubits : ops[i].qubits;
      bool clash = false;
      for (auto x : q) clash |= blocked[x] != 0;
      bool take = false;
      const bool per_binding = !conv[i].bmat.empty();
      const size_t msz = conv[i].mat.size();
      if (runnable[i] && !clash && (int)run.size() < run_max_ops() &&
          (per_binding ? bpool + msz <= bound_cap : pool + msz <= pool_cap)) {
        int extra = 0;
        for (auto x : q) extra += !inT[x];
        if (tcount + extra <= m) take = true;
      }
      if (take) {
        for (auto x : q)
          if (!inT[x]) inT[x] = 1, ++tcount;
        run.push_back(&conv[i]);
        members.push_back(i);
        (per_binding ? bpool : pool) += msz;
      } else {
        // a barrier-like op (no qubit list) blocks everything
        if (q.empty() && ops[i].type != GBQV_OP_BARRIER) break;
        for (auto x : q) blocked[x] = 1;
      }
    }
    if (run.size() == 1 && conv[members[0]].qubits.size() <= 1 && conv[members[0]].bmat.empty()) {
      exec_op(d, ops[members[0]]);  // a lone 1-qubit op: the streaming kernel is enough
    } else {
      launch_run(d, run, bound);
    }
    for (auto i : members) done[i] = 1;
  }
}

void execute_blocked(Device &d, const std::vector<Op> &ops) {
  std::vector<RunOp> conv(ops.size());
  std::vector<char> runnable(ops.size());
  for (size_t i = 0; i < ops.size(); ++i) runnable[i] = as_run_op(d, ops[i], conv[i]) && worth_batching(d, conv[i]);
  schedule_runs(d, ops, conv, runnable, nullptr);
}

// ---- runtime parameter binding: many bindings, one stack of states ----

// A gate's prim as a run member: dense / diagonal matrix on its qubits, or a
// multi-controlled X.  dense_only: a controlled 2x2 becomes a dense matrix
// even when it is diagonal.  False when it has no run form.
bool prim_run_form(const Prim &p, bool dense_only, RunOp &out) {
  out.qubits = p.q;
  out.mat.clear();
  const size_t k = p.q.size();
  if (k == 0 || k > 5) return false;
  const size_t D = 1ULL << k;
  auto controlled = [&](const cd *u) {  // identity except the block where every control is set
    const size_t i0 = (D >> 1) - 1, i1 = D - 1;
    if (!dense_only && u[1] == 0.0 && u[2] == 0.0) {
      out.kind = 1;
      out.mat.assign(D, 1.0);
      out.mat[i0] = u[0];
      out.mat[i1] = u[3];
    } else {
      out.kind = 0;
      out.mat = gates::identity(D);
      out.mat[i0 + D * i0] = u[0];
      out.mat[i1 + D * i0] = u[1];
      out.mat[i0 + D * i1] = u[2];
      out.mat[i1 + D * i1] = u[3];
    }
  };
  switch (p.k) {
    case P::MCX: out.kind = 2; return true;
    case P::DIAG: out.kind = 1; out.mat = p.m; return true;
    case P::MATRIX: out.kind = 0; out.mat = p.m; return true;
    case P::MCPHASE:
      out.kind = 1;
      out.mat.assign(D, 1.0);
      out.mat[D - 1] = p.m[0];
      return true;
    case P::MCU: controlled(p.m.data()); return true;
    case P::MCY: {
      const cd y[4] = {0.0, cd(0., 1.), cd(0., -1.), 0.0};
      controlled(y);
      return true;
    }
    case P::MCSWAP: {
      if (k < 2) return false;
      out.kind = 0;
      out.mat.assign(D * D, 0.0);
      const size_t a = D >> 2, b = D >> 1, ctrl = a - 1;  // last two qubits at bits k-2, k-1
      for (size_t i = 0; i < D; ++i) {
        size_t j = i;
        if ((i & ctrl) == ctrl && (((i & a) != 0) != ((i & b) != 0))) j = i ^ (a | b);
        out.mat[j + D * i] = 1.0;
      }
      return true;
    }
    default: return false;
  }
}

// Parameterised gate families whose per-binding matrices are computed
// directly (the values sv_prim + prim_run_form give, without the name
// dispatch per binding).
enum class BF { NONE, MCRX, MCRY, MCRZ, MCP, MCU3, MCU, MCU2, MCR, RXX, RYY, RZZ, RZX };

BF bound_family(const std::string &name) {
  auto it = sv_gateset().find(name);
  if (it == sv_gateset().end()) return BF::NONE;
  static const std::unordered_map<std::string, BF> fam = {
      {"mcrx", BF::MCRX}, {"mcry", BF::MCRY}, {"mcrz", BF::MCRZ}, {"mcp", BF::MCP}, {"mcu3", BF::MCU3},
      {"mcu", BF::MCU},   {"mcu2", BF::MCU2}, {"mcr", BF::MCR},   {"rxx", BF::RXX}, {"ryy", BF::RYY},
      {"rzz", BF::RZZ},   {"rzx", BF::RZX}};
  auto f = fam.find(it->second);
  return f == fam.end() ? BF::NONE : f->second;
}

bool fast_bound_form(const Op &op, int nbind, RunOp &out) {
  const BF f = bound_family(op.name);
  if (f == BF::NONE) return false;
  const size_t k = op.qubits.size(), D = 1ULL << k, stride = op.params.size();
  if (k == 0 || k > 5) return false;
  const bool two = f == BF::RXX || f == BF::RYY || f == BF::RZZ || f == BF::RZX;
  if (two && k != 2) return false;
  const size_t need = f == BF::MCR || f == BF::MCU2 ? 2 : f == BF::MCU3 ? 3 : f == BF::MCU ? 4 : 1;
  if (stride < need) return false;
  const bool diag = f == BF::MCRZ || f == BF::MCP || f == BF::RZZ;
  out.kind = diag ? 1 : 0;
  out.qubits = op.qubits;
  const size_t msz = diag ? D : D * D;
  std::vector<cd> tmpl = diag ? std::vector<cd>(D, 1.0) : gates::identity(D);
  out.bmat.resize(msz * nbind);
  const size_t i0 = (D >> 1) - 1, i1 = D - 1;  // controlled block: every control set
  for (int j = 0; j < nbind; ++j) {
    const double *p = op.bparams.data() + (size_t)j * stride;
    cd *dst = out.bmat.data() + (size_t)j * msz;
    std::copy(tmpl.begin(), tmpl.end(), dst);
    gates::mat_t u;
    switch (f) {
      case BF::MCRX: u = gates::rx(p[0]); break;
      case BF::MCRY: u = gates::ry(p[0]); break;
      case BF::MCRZ: u = gates::rz(p[0]); break;
      case BF::MCU3: u = gates::u4(p[0], p[1], p[2], 0.); break;
      case BF::MCU: u = gates::u4(p[0], p[1], p[2], p[3]); break;
      case BF::MCU2: u = gates::u4(M_PI / 2., p[0], p[1], 0.); break;
      case BF::MCR: u = gates::r(p[0], p[1]); break;
      case BF::MCP: dst[D - 1] = std::exp(cd(0, 1) * p[0]); continue;
      case BF::RXX: u = gates::rxx(p[0]); std::copy(u.begin(), u.end(), dst); continue;
      case BF::RYY: u = gates::ryy(p[0]); std::copy(u.begin(), u.end(), dst); continue;
      case BF::RZX: u = gates::rzx(p[0]); std::copy(u.begin(), u.end(), dst); continue;
      case BF::RZZ: u = gates::rzz_diag(p[0]); std::copy(u.begin(), u.end(), dst); continue;
      default: return false;
    }
    if (diag) {  // controlled rz: diagonal 2x2
      dst[i0] = u[0];
      dst[i1] = u[3];
    } else {
      dst[i0 + D * i0] = u[0];
      dst[i1 + D * i0] = u[1];
      dst[i0 + D * i1] = u[2];
      dst[i1 + D * i1] = u[3];
    }
  }
  out.mat.assign(out.bmat.begin(), out.bmat.begin() + msz);
  return true;
}

// The op's run form over `nbind` bindings: per-binding matrices (bmat) for a
// gate with bound parameters.  False when it has none (then it must not be
// bound, and runs on the whole stack through exec_op).
bool bound_run_op(const Op &op, int nbind, RunOp &out) {
  out = RunOp{};
  if (op.type == GBQV_OP_MATRIX || op.type == GBQV_OP_DIAGONAL) {
    Device dummy;
    dummy.density = false;
    return as_run_op(dummy, op, out);
  }
  if (op.type != GBQV_OP_GATE) return false;
  if (op.bparams.empty()) return prim_run_form(sv_prim(op), false, out);
  if (fast_bound_form(op, nbind, out)) return true;
  out = RunOp{};
  const size_t stride = op.params.size();
  Op b = op;
  b.bparams.clear();
  for (int pass = 0; pass < 2; ++pass) {
    const bool dense_only = pass == 1;
    bool same = true;
    for (int j = 0; j < nbind && same; ++j) {
      b.params.assign(op.bparams.begin() + j * stride, op.bparams.begin() + (j + 1) * stride);
      RunOp r;
      if (!prim_run_form(sv_prim(b), dense_only, r) || r.kind == 2)
        throw Error(GBQV_ERR_KIND, "gate '" + op.name + "' with bound parameters has no per-binding form");
      if (j == 0) {
        out.kind = r.kind;
        out.qubits = r.qubits;
        out.mat = r.mat;
        out.bmat.clear();
        out.bmat.reserve(r.mat.size() * nbind);
      } else if (r.kind != out.kind || r.mat.size() != out.mat.size()) {
        same = false;  // a controlled 2x2 diagonal for some bindings only: all dense
        break;
      }
      out.bmat.insert(out.bmat.end(), r.mat.begin(), r.mat.end());
    }
    if (same) return true;
  }
  throw Error(GBQV_ERR_KIND, "gate '" + op.name + "' with bound parameters has no per-binding form");
}

// Consecutive 1-qubit dense / diagonal ops on the same qubit (no op on that
// qubit between them) become one op per binding, their 2x2 product; the
// kind of fusion Aer's Fusion applies per binding (fusion.hpp:59-101), kept
// to 1-qubit products so that no binding pays for a wider matrix.
void merge_one_qubit_runs(int nbind, std::vector<Op> &ops, std::vector<RunOp> &conv, std::vector<char> &runnable) {
  const size_t nops = ops.size();
  std::vector<char> gone(nops, 0);
  std::map<uint64_t, size_t> last;  // qubit -> index of the pending 1-qubit op on it
  auto is1q = [&](size_t i) { return runnable[i] && conv[i].qubits.size() == 1 && conv[i].kind != 2; };
  // 2x2 column-major of a 1-qubit run op, binding j
  auto mat2 = [&](const RunOp &r, int j, cd *m) {
    const bool b = !r.bmat.empty();
    const cd *src = b ? r.bmat.data() + (size_t)j * r.mat.size() : r.mat.data();
    if (r.kind == 1) {
      m[0] = src[0]; m[1] = 0.0; m[2] = 0.0; m[3] = src[1];
    } else {
      std::copy(src, src + 4, m);
    }
  };
  for (size_t k = 0; k < nops; ++k) {
    if (is1q(k)) {
      const uint64_t q = conv[k].qubits[0];
      auto it = last.find(q);
      if (it != last.end()) {
        const size_t i = it->second;
        RunOp &A = conv[i], &Bop = conv[k];
        const bool both_diag = A.kind == 1 && Bop.kind == 1;
        const bool bound = !A.bmat.empty() || !Bop.bmat.empty();
        const int nb = bound ? nbind : 1;
        RunOp C;
        C.kind = both_diag ? 1 : 0;
        C.qubits = Bop.qubits;
        const size_t msz = both_diag ? 2 : 4;
        std::vector<cd> out((size_t)nb * msz);
        for (int j = 0; j < nb; ++j) {
          cd a[4], b[4];
          mat2(A, j, a);
          mat2(Bop, j, b);
          cd *o = out.data() + (size_t)j * msz;
          if (both_diag) {
            o[0] = b[0] * a[0];
            o[1] = b[3] * a[3];
          } else {
            for (int r = 0; r < 2; ++r)
              for (int cc = 0; cc < 2; ++cc) o[r + 2 * cc] = b[r] * a[2 * cc] + b[r + 2] * a[1 + 2 * cc];
          }
        }
        C.mat.assign(out.begin(), out.begin() + msz);
        if (bound) C.bmat = std::move(out);
        conv[k] = std::move(C);
        gone[i] = 1;
      }
      last[q] = k;
      continue;
    }
    const reg_t &qs = runnable[k] ? conv[k].qubits : ops[k].qubits;
    for (auto x : qs) last.erase(x);
    if (qs.empty()) last.clear();
  }
  size_t w = 0;
  for (size_t i = 0; i < nops; ++i)
    if (!gone[i]) {
      if (w != i) {
        ops[w] = std::move(ops[i]);
        conv[w] = std::move(conv[i]);
        runnable[w] = runnable[i];
      }
      ++w;
    }
  ops.resize(w);
  conv.resize(w);
  runnable.resize(w);
}

void execute_bound(Device &d, gbqv_circuit &c, uint64_t first, uint64_t count) {
  const int sb = c.num_qubits;
  REQUIRE(!d.density, GBQV_ERR_KIND, "parameter binding runs statevectors only");
  const int nb = std::max(c.nbind, 1);
  REQUIRE(count >= 1 && first + count <= (uint64_t)nb, GBQV_ERR_ARG,
          "binding range [" + std::to_string(first) + ", " + std::to_string(first + count) + ") out of " +
              std::to_string(nb));
  REQUIRE(d.n >= sb && (d.n - sb) < 63 && (1ULL << (d.n - sb)) >= count, GBQV_ERR_ARG,
          "the state must stack 2^b states of " + std::to_string(sb) + " qubits, 2^b >= " + std::to_string(count) +
              " (state has " + std::to_string(d.n) + " qubits)");
  if (c.bound_version != c.version) {  // run forms of every op, once per circuit version
    std::vector<Op> ops;
    for (const Op &op : c.ops) {
      if (op.type == GBQV_OP_BARRIER) continue;
      REQUIRE(op.type == GBQV_OP_GATE || op.type == GBQV_OP_MATRIX || op.type == GBQV_OP_DIAGONAL, GBQV_ERR_KIND,
              "op '" + op.name + "' is not unitary: bound execution runs unitary circuits");
      if (op.type == GBQV_OP_GATE && op.bparams.empty() && sv_prim(op).k == P::NONE) continue;
      ops.push_back(op);
    }
    std::vector<RunOp> conv(ops.size());
    std::vector<char> runnable(ops.size());
    for (size_t i = 0; i < ops.size(); ++i) {
      runnable[i] = bound_run_op(ops[i], nb, conv[i]);
      REQUIRE(runnable[i] || ops[i].bparams.empty(), GBQV_ERR_KIND,
              "gate '" + ops[i].name + "' with bound parameters acts on more than 5 qubits");
    }
    merge_one_qubit_runs(nb, ops, conv, runnable);
    c.bound_ops = std::move(ops);
    c.bound_conv = std::move(conv);
    c.bound_runnable = std::move(runnable);
    c.bound_version = c.version;
  }
  RunBound rb{sb, first, count};
  launch_set_basis_segments(d, sb, count);
  schedule_runs(d, c.bound_ops, c.bound_conv, c.bound_runnable, &rb);
}

}  // namespace

extern "C" int gbqv_execute_bound(gbqv_handle h, gbqv_circuit_t c, uint64_t first, uint64_t count) {
  return guard(
      [&] {
        REQUIRE(h && c, GBQV_ERR_ARG, "null argument");
        execute_bound(device_of(h), *c, first, count);
      },
      h);
}

extern "C" int gbqv_execute(gbqv_handle h, gbqv_circuit_t c) {
  return guard(
      [&] {
        REQUIRE(h && c, GBQV_ERR_ARG, "null argument");
        REQUIRE(c->nbind == 0, GBQV_ERR_ARG, "the circuit has parameter bindings: run it with gbqv_execute_bound");
        Device &d = device_of(h);
        REQUIRE(c->num_qubits == d.nq, GBQV_ERR_ARG,
                "circuit has " + std::to_string(c->num_qubits) + " qubits, state has " + std::to_string(d.nq));
        if (d.blocking)
          execute_blocked(d, c->ops);
        else
          for (const Op &op : c->ops) exec_op(d, op);
      },
      h);
}

extern "C" int gbqv_execute_segments(gbqv_handle h, gbqv_circuit_t c) {
  return guard(
      [&] {
        REQUIRE(h && c, GBQV_ERR_ARG, "null argument");
        REQUIRE(c->nbind == 0, GBQV_ERR_ARG, "the circuit has parameter bindings: run it with gbqv_execute_bound");
        Device &d = device_of(h);
        REQUIRE(!d.density && !d.unitary, GBQV_ERR_KIND, "execute_segments: statevector stacks only");
        REQUIRE(c->num_qubits <= d.n, GBQV_ERR_ARG,
                "circuit has " + std::to_string(c->num_qubits) + " qubits, the stacked states have " +
                    std::to_string(d.n));
        for (const Op &op : c->ops)
          REQUIRE(op.type != GBQV_OP_RESET && op.type != GBQV_OP_KRAUS && op.type != GBQV_OP_SUPEROP, GBQV_ERR_KIND,
                  "op '" + op.name + "' acts on the whole vector: execute_segments runs unitary ops");
        if (d.blocking)
          execute_blocked(d, c->ops);
        else
          for (const Op &op : c->ops) exec_op(d, op);
      },
      h);
}

// ============================== adjoint gradients ==============================
// No reference counterpart (Aer has no gradient code).  E(theta) =
// <psi|H|psi> with psi = U_L...U_1|0>; for a gate U = exp(-i theta P / 2)
// with Pauli generator P, dE/dtheta = Im <lam_i| P |psi_i>, where psi_i is
// the state right after the gate and lam_i = U_{i+1}^dag ... U_L^dag H psi.
// The reverse sweep uncomputes psi and lam gate by gate (two state buffers,
// no stored intermediate states).
namespace {

Prim inverse_prim(Prim p) {
  switch (p.k) {
    case P::NONE:
    case P::MCX:
    case P::MCY:
    case P::MCSWAP: return p;  // self-inverse
    case P::MCPHASE: p.m[0] = std::conj(p.m[0]); return p;
    case P::DIAG: for (auto &z : p.m) z = std::conj(z); return p;
    case P::MCU:
    case P::MATRIX: {
      const size_t D = p.k == P::MCU ? 2 : (1ULL << p.q.size());
      std::vector<cd> t(D * D);
      for (size_t r = 0; r < D; ++r)
        for (size_t c = 0; c < D; ++c) t[c + D * r] = std::conj(p.m[r + D * c]);
      p.m = t;
      return p;
    }
  }
  return p;
}

Prim op_prim(const Op &op) {
  if (op.type == GBQV_OP_GATE) return sv_prim(op);
  Prim p;
  p.q = op.qubits;
  if (op.type == GBQV_OP_MATRIX) { p.k = P::MATRIX; p.m = op.mat; return p; }
  if (op.type == GBQV_OP_DIAGONAL) { p.k = P::DIAG; p.m = op.mat; return p; }
  if (op.type == GBQV_OP_BARRIER) return p;
  throw Error(GBQV_ERR_ARG, "adjoint gradients need unitary ops (got '" + op.name + "')");
}

// A 1-qubit prim as a column-major 2x2 matrix (false for anything else).
bool prim_2x2(const Prim &p, uint64_t &q, cd m[4]) {
  if (p.q.size() != 1) return false;
  q = p.q[0];
  switch (p.k) {
    case P::MCU:
    case P::MATRIX:
      if (p.m.size() != 4) return false;
      for (int j = 0; j < 4; ++j) m[j] = p.m[j];
      return true;
    case P::DIAG:
      if (p.m.size() != 2) return false;
      m[0] = p.m[0], m[1] = 0.0, m[2] = 0.0, m[3] = p.m[1];
      return true;
    case P::MCPHASE:
      m[0] = 1.0, m[1] = 0.0, m[2] = 0.0, m[3] = p.m[0];
      return true;
    case P::MCX:
      m[0] = 0.0, m[1] = 1.0, m[2] = 1.0, m[3] = 0.0;
      return true;
    default: return false;
  }
}

// Pauli generator of a parameterised gate, label read right to left.
bool generator(const Op &op, PauliMasks &m, cd &phase) {
  static const std::unordered_map<std::string, std::string> gens = {
      {"rx", "X"}, {"ry", "Y"}, {"rz", "Z"}, {"rxx", "XX"}, {"ryy", "YY"}, {"rzz", "ZZ"}, {"rzx", "XZ"}};
  auto it = gens.find(op.name);
  if (it == gens.end() || it->second.size() != op.qubits.size()) return false;
  m = pauli_masks(op.qubits, it->second.c_str());
  phase = add_y_phase(m.num_y, cd(1.0, 0.0));
  return true;
}

}  // namespace

extern "C" int gbqv_adjoint_expval_grad(gbqv_handle h, gbqv_circuit_t c, const int *param_of_op, const double *params,
                                        int nparams, int nterms, const uint64_t *qubits, const int *offsets,
                                        const char *const *labels, const double *coeffs, double *energy, double *grad) {
  return guard(
      [&] {
        REQUIRE(h && c, GBQV_ERR_ARG, "null argument");
        Device &d = device_of(h);
        REQUIRE(!d.density, GBQV_ERR_KIND, "adjoint gradients need a statevector");
        REQUIRE(c->num_qubits == d.nq, GBQV_ERR_ARG, "circuit and state sizes differ");
        REQUIRE(nparams >= 0 && (params || nparams == 0) && param_of_op, GBQV_ERR_ARG, "bad parameter arrays");
        REQUIRE(nterms >= 1 && offsets && labels, GBQV_ERR_ARG, "bad Hamiltonian arrays");
        // bind parameters
        std::vector<Op> ops = c->ops;
        std::vector<int> slot(ops.size(), -1);
        int nslots = 0;
        for (size_t i = 0; i < ops.size(); ++i) {
          const int pi = param_of_op[i];
          if (pi < 0) continue;
          REQUIRE(pi < nparams, GBQV_ERR_ARG, "parameter index out of range");
          PauliMasks gm;
          cd gph;
          REQUIRE(ops[i].type == GBQV_OP_GATE && generator(ops[i], gm, gph), GBQV_ERR_ARG,
                  "gate '" + ops[i].name + "' has no Pauli-rotation generator");
          ops[i].params.resize(std::max<size_t>(ops[i].params.size(), 1));
          ops[i].params[0] = params[pi];
          slot[i] = nslots++;
        }
        // Hamiltonian terms: coeff * (-i)^{num_y}
        std::vector<HamTerm> ham;
        for (int t = 0; t < nterms; ++t) {
          const int k = offsets[t + 1] - offsets[t];
          reg_t q(qubits + offsets[t], qubits + offsets[t] + k);
          for (auto x : q) REQUIRE(x < (uint64_t)d.n, GBQV_ERR_QUBIT, "Hamiltonian qubit out of range");
          REQUIRE(labels[t] && (int)std::strlen(labels[t]) == k, GBQV_ERR_ARG, "Pauli label length must equal qubit count");
          PauliMasks m = pauli_masks(q, labels[t]);
          const cd ph = add_y_phase(m.num_y, cd(coeffs ? coeffs[t] : 1.0, 0.0));
          ham.push_back(HamTerm{m.x_mask, m.z_mask, ph.real(), ph.imag()});
        }
        // forward: only psi is needed, so the bound ops go through Aer's
        // Fusion pass (statevector defaults) and the cache-blocked runs, as a
        // gbqv_execute of the fused circuit would
        launch_set_basis(d, 0, cd(1.0, 0.0));
        {
          gbqv_circuit fwd;
          fwd.num_qubits = c->num_qubits;
          fwd.ops = ops;
          gbqv_fusion_config cfg;
          REQUIRE(gbqv_fusion_default_config(0, &cfg) == GBQV_OK, GBQV_ERR_ARG, "fusion configuration");
          REQUIRE(gbqv_circuit_fuse(&fwd, &cfg, nullptr, nullptr, 0) == GBQV_OK, GBQV_ERR_ARG,
                  "fusion of the forward pass failed");
          if (d.blocking)
            execute_blocked(d, fwd.ops);
          else
            for (auto &op : fwd.ops) exec_op(d, op);
        }
        // complex128: the sweep runs on float pairs (FP32 pipe) when every op
        // is a 1-qubit gate whose generator (if any) sits on its qubit, or a
        // pure permutation (X-type, swaps), the forms that need no FP64
        struct Step {
          int form = -1;  // -1: permutation / other; 0..2 fused 1-qubit step
          uint64_t q = 0;
          cd m[4];
          PauliMasks gm;
          cd gph;
        };
        std::vector<Step> steps(ops.size());
        bool pairs = d.dbl && d.tensor_c128 != 0;
        for (size_t i = 0; i < ops.size(); ++i) {
          Step &st = steps[i];
          if (slot[i] >= 0) generator(ops[i], st.gm, st.gph);
          const Prim inv = inverse_prim(op_prim(ops[i]));
          if (prim_2x2(inv, st.q, st.m) && (slot[i] < 0 || ((st.gm.x_mask | st.gm.z_mask) & ~(1ULL << st.q)) == 0)) {
            bool real = true;
            for (auto &z : st.m) real &= z.imag() == 0.0;
            st.form = st.m[1] == 0.0 && st.m[2] == 0.0 ? 2 : real ? 1 : 0;
          } else if (slot[i] >= 0 || !(inv.k == P::MCX || inv.k == P::MCSWAP || inv.k == P::NONE)) {
            pairs = false;
          }
        }
        // lam = H psi and <psi|H psi>
        const size_t bytes = d.amps() * d.amp_bytes();
        grow(d.aux, d.aux_cap, bytes);
        void *lam = d.aux;
        grow(reinterpret_cast<void *&>(d.results), d.results_cap, sizeof(double) * 2 * (nslots + 1));
        if (pairs) {
          adjoint_to_pairs(d, d.state);
          ham_apply_pairs(d, d.state, lam, ham);
          const cd one[4] = {1.0, 0.0, 0.0, 1.0};
          adjoint_step_pairs(d, lam, d.state, 0, one, 2, false, false, cd(1.0, 0.0), nslots, false);
        } else {
          ham_apply(d, d.state, lam, ham);
          reduce_pauli_inner(d, d.state, lam, 0, 0, cd(1.0, 0.0), nslots);  // <psi|H psi>
        }
        // reverse sweep.  Consecutive 1-qubit steps on distinct qubits (up to
        // 3) share one pass over psi and lam; permutations and, off the
        // float-pair path, any other op keep their own kernels
        auto host_step = [&](int i) {
          const Step &st = steps[i];
          AdjStepHost h;
          h.q = (int)st.q;
          h.form = st.form;
          h.gx = st.gm.x_mask != 0;
          h.gz = st.gm.z_mask != 0;
          for (int e = 0; e < 4; ++e) h.m[e] = st.m[e];
          h.phase = st.gph;
          h.slot = slot[i];
          return h;
        };
        // CX (one control), X and SWAP without a generator: a run of three or
        // more of them is uncomputed in one gather per state (their product
        // is a linear map of the index bits plus a constant), through the
        // third state buffer
        auto linear_op = [&](int i) {
          if (slot[i] >= 0) return false;
          const Prim inv = inverse_prim(op_prim(ops[i]));
          return (inv.k == P::MCX && inv.q.size() <= 2) || (inv.k == P::MCSWAP && inv.q.size() == 2);
        };
        for (int i = (int)ops.size() - 1; i >= 0;) {
          const Step &st = steps[i];
          if (i > 0 && linear_op(i)) {
            int j = i;
            while (j > 0 && linear_op(j)) --j;  // ops j + 1 .. i (op 0 is never uncomputed)
            if (i - j >= 3) {
              // src(y) = M y ^ c, M's columns composed in application order
              // (i first): CX(a -> b) adds column b to column a, X(q) adds
              // column q to c, SWAP exchanges two columns
              std::vector<uint64_t> col(d.n);
              for (int q = 0; q < d.n; ++q) col[q] = 1ULL << q;
              uint64_t cst = 0;
              for (int k = i; k > j; --k) {
                const Prim inv = inverse_prim(op_prim(ops[k]));
                if (inv.k == P::MCX && inv.q.size() == 1)
                  cst ^= col[inv.q[0]];
                else if (inv.k == P::MCX)
                  col[inv.q[0]] ^= col[inv.q[1]];
                else
                  std::swap(col[inv.q[0]], col[inv.q[1]]);
              }
              LinearGatherHost g;
              g.c = cst;
              for (int q = 0; q < d.n; ++q)
                if (col[q] != (1ULL << q)) {
                  g.q.push_back(q);
                  g.d.push_back(col[q] ^ (1ULL << q));
                }
              grow(d.aux2, d.aux2_cap, bytes);
              gather_linear(d, d.state, d.aux2, g);
              std::swap(d.state, d.aux2);  // the state buffer (exactly `bytes`) becomes the scratch
              d.aux2_cap = bytes;
              gather_linear(d, d.aux, d.aux2, g);
              std::swap(d.aux, d.aux2);
              std::swap(d.aux_cap, d.aux2_cap);
              lam = d.aux;
              i = j;
              continue;
            }
          }
          if (st.form >= 0 && i > 0) {
            std::vector<AdjStepHost> grp;
            std::vector<uint64_t> used;
            int j = i;
            while (j > 0 && grp.size() < 3 && steps[j].form >= 0 &&
                   std::find(used.begin(), used.end(), steps[j].q) == used.end()) {
              grp.push_back(host_step(j));
              used.push_back(steps[j].q);
              --j;
            }
            adjoint_steps(d, d.state, lam, grp, pairs);
            i = j;
            continue;
          }
          if (slot[i] >= 0) {  // the inner product without a step after it
            if (pairs) {
              adjoint_step_pairs(d, d.state, lam, (int)st.q, st.m, st.form, st.gm.x_mask != 0, st.gm.z_mask != 0,
                                 st.gph, slot[i], false);
            } else {
              reduce_pauli_inner(d, lam, d.state, st.gm.x_mask, st.gm.z_mask, st.gph, slot[i]);
            }
          }
          if (i > 0) {
            const Prim inv = inverse_prim(op_prim(ops[i]));
            exec_prim(d, inv);
            std::swap(d.state, d.aux);
            exec_prim(d, inv);
            std::swap(d.state, d.aux);
            lam = d.aux;
          }
          --i;
        }
        if (pairs) adjoint_from_pairs(d, d.state);  // the handle's state back in complex128
        std::vector<double> res(2 * (nslots + 1));
        cuda_check(cudaMemcpyAsync(res.data(), d.results, sizeof(double) * res.size(), cudaMemcpyDeviceToHost, d.stream),
                   "gradient copy");
        cuda_check(cudaStreamSynchronize(d.stream), "stream synchronize");
        if (energy) *energy = res[2 * nslots];
        if (grad) {
          for (int p = 0; p < nparams; ++p) grad[p] = 0.0;
          for (size_t i = 0; i < ops.size(); ++i)
            if (slot[i] >= 0) grad[param_of_op[i]] += res[2 * slot[i] + 1];
        }
      },
      h);
}
