// aer_prelude.hpp — project-written stand-ins that let the reference's
// QubitVector / DensityMatrix / UnitaryMatrix headers compile without
// nlohmann/json and the Op data model (neither is needed by the hot-path
// members this shim calls).  Included before any reference header.
#pragma once
#define _aer_framework_json_hpp_
#define _aer_framework_operations_hpp_
#include <complex>
#include <cstdint>
#include <string>
#include <vector>
struct gbqv_fake_json {
  gbqv_fake_json() = default;
  template <typename... A> gbqv_fake_json(A &&...) {}
  template <typename T> gbqv_fake_json &operator=(const T &) { return *this; }
  gbqv_fake_json &operator[](size_t) { return *this; }
};
using json_t = gbqv_fake_json;
#include "framework/types.hpp"
#include "framework/linalg/matrix_utils/smatrix_defs.hpp"
namespace AER {
namespace Operations {
struct Op {};
}  // namespace Operations
}  // namespace AER
