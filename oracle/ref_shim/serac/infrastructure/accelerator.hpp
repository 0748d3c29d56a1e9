// Stand-in for serac's accelerator header: host-only macros, execution-space
// aliases and SLIC error macros that throw.
#pragma once
#include <cstring>
#include <functional>
#include <iostream>
#include <stdexcept>
#include <string>
#include "axom/core.hpp"

#define SERAC_HOST_DEVICE
#define SERAC_HOST
#define SERAC_DEVICE
#define SERAC_SUPPRESS_NVCC_HOSTDEVICE_WARNING
#define SLIC_ERROR_ROOT_IF(cond, msg) \
  do {                                \
    if (cond) throw std::runtime_error(std::string(msg)); \
  } while (0)
#define SLIC_ERROR_ROOT(msg) throw std::runtime_error(std::string(msg))
#define SLIC_ERROR_IF(cond, msg) SLIC_ERROR_ROOT_IF(cond, msg)
#define SLIC_ERROR(msg) SLIC_ERROR_ROOT(msg)
#define SLIC_WARNING(msg) \
  do {                    \
  } while (0)
#define SLIC_WARNING_ROOT(msg) SLIC_WARNING(msg)

namespace serac {
enum class ExecutionSpace { CPU, GPU, Dynamic };
constexpr ExecutionSpace default_execution_space = ExecutionSpace::CPU;
template <typename T, int dim, ExecutionSpace space = ExecutionSpace::CPU>
using ExecArray = axom::Array<T, dim, axom::MemorySpace::Dynamic>;
template <typename T, int dim, ExecutionSpace space = ExecutionSpace::CPU>
using ExecArrayView = axom::ArrayView<T, dim, axom::MemorySpace::Dynamic>;
template <typename T, int dim>
using CPUArrayView = ExecArrayView<T, dim, ExecutionSpace::CPU>;
namespace detail {
template <typename T, int dim, axom::MemorySpace space>
void zero_out(axom::Array<T, dim, space>& arr) {
  std::memset(arr.data(), 0, static_cast<std::size_t>(arr.size()) * sizeof(T));
}
}  // namespace detail
}  // namespace serac
