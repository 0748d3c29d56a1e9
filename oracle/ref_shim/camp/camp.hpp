// Stand-in for camp's integer-sequence helpers.
#pragma once
#include <utility>
namespace camp {
template <typename T, T... v>
using int_seq = std::integer_sequence<T, v...>;
template <typename T, T N>
using make_int_seq = std::make_integer_sequence<T, N>;
}  // namespace camp
