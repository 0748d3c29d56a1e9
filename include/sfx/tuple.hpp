// sfx — a small aggregate tuple usable in device code, with class template
// argument deduction (`tuple{a, b}`), `get<i>` and structured bindings, as the
// q-function interface of serac::Functional expects (numerics/functional/tuple.hpp).
#pragma once

#include <tuple>
#include <type_traits>
#include <utility>
#include "sfx/tensor.hpp"

namespace sfx {

template <typename... T>
struct tuple;

template <>
struct tuple<> {};

template <typename T0>
struct tuple<T0> {
  T0 v0;
};
template <typename T0, typename T1>
struct tuple<T0, T1> {
  T0 v0;
  T1 v1;
};
template <typename T0, typename T1, typename T2>
struct tuple<T0, T1, T2> {
  T0 v0;
  T1 v1;
  T2 v2;
};
template <typename T0, typename T1, typename T2, typename T3>
struct tuple<T0, T1, T2, T3> {
  T0 v0;
  T1 v1;
  T2 v2;
  T3 v3;
};
template <typename T0, typename T1, typename T2, typename T3, typename T4>
struct tuple<T0, T1, T2, T3, T4> {
  T0 v0;
  T1 v1;
  T2 v2;
  T3 v3;
  T4 v4;
};

template <typename... T>
tuple(T...) -> tuple<T...>;

template <std::size_t i, typename... T>
SFX_HDI constexpr auto& get(tuple<T...>& t) {
  static_assert(i < sizeof...(T), "tuple index");
  if constexpr (i == 0) return t.v0;
  else if constexpr (i == 1) return t.v1;
  else if constexpr (i == 2) return t.v2;
  else if constexpr (i == 3) return t.v3;
  else return t.v4;
}
template <std::size_t i, typename... T>
SFX_HDI constexpr const auto& get(const tuple<T...>& t) {
  static_assert(i < sizeof...(T), "tuple index");
  if constexpr (i == 0) return t.v0;
  else if constexpr (i == 1) return t.v1;
  else if constexpr (i == 2) return t.v2;
  else if constexpr (i == 3) return t.v3;
  else return t.v4;
}

template <typename... T>
SFX_HDI constexpr auto make_tuple(T... args) {
  return tuple<T...>{args...};
}

// elementwise ops on 2-tuples (source, flux) pairs
template <typename A0, typename A1, typename B0, typename B1>
SFX_HDI constexpr auto operator+(const tuple<A0, A1>& a, const tuple<B0, B1>& b) {
  return tuple{a.v0 + b.v0, a.v1 + b.v1};
}
template <typename A0, typename A1, typename S>
SFX_HDI constexpr auto operator*(const tuple<A0, A1>& a, const S& s) {
  return tuple{a.v0 * s, a.v1 * s};
}

}  // namespace sfx

namespace std {
template <typename... T>
struct tuple_size<sfx::tuple<T...>> : std::integral_constant<std::size_t, sizeof...(T)> {};
template <std::size_t i, typename... T>
struct tuple_element<i, sfx::tuple<T...>> {
  using type = typename std::tuple_element<i, std::tuple<T...>>::type;
};
}  // namespace std
