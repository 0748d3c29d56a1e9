// Stand-in for serac's Functional header as seen by the material headers:
// pulls in only the tensor / dual-number / element headers they use.
#pragma once
#include "serac/numerics/functional/tensor.hpp"
#include "serac/numerics/functional/tuple.hpp"
#include "serac/numerics/functional/dual.hpp"
#include "serac/numerics/functional/tuple_tensor_dual_functions.hpp"
#include "serac/numerics/functional/finite_element.hpp"
#include "serac/numerics/functional/quadrature_data.hpp"
