// sfx — forward-mode dual numbers for q-function linearisation.
//
// dual<V, G>: value of scalar type V (double or float) and gradient G, where G
// is V itself (one directional derivative, used by the Jacobian-vector
// product) or tensor<V, k> (k seeded directions, used for element stiffness).
// The derivative rules are those of serac's dual.hpp (numerics/functional/
// dual.hpp:28-200); mixed arithmetic with plain arithmetic scalars keeps the
// dual's own precision V.
#pragma once

#include <cmath>
#include "sfx/tensor.hpp"

namespace sfx {

template <typename V, typename G = V>
struct dual {
  V value;
  G gradient;
  SFX_HDI constexpr dual() : value{}, gradient{} {}
  SFX_HDI constexpr dual(V v, G g) : value(v), gradient(g) {}
  template <typename A, typename = std::enable_if_t<std::is_arithmetic<A>::value>>
  SFX_HDI constexpr dual(A v) : value(V(v)), gradient{} {}
  template <typename A, typename = std::enable_if_t<std::is_arithmetic<A>::value>>
  SFX_HDI constexpr dual& operator=(A v) {
    value = V(v);
    gradient = G{};
    return *this;
  }
};

template <typename T>
struct is_dual : std::false_type {};
template <typename V, typename G>
struct is_dual<dual<V, G>> : std::true_type {};

template <typename V, typename G>
struct scalar_of<dual<V, G>> {
  using type = dual<V, G>;
};

SFX_HDI constexpr double get_value(double a) { return a; }
SFX_HDI constexpr float get_value(float a) { return a; }
template <typename V, typename G>
SFX_HDI constexpr V get_value(const dual<V, G>& a) { return a.value; }
template <typename T, int... n>
SFX_HDI constexpr auto get_value(const tensor<T, n...>& a) {
  using R = decltype(get_value(T{}));
  tensor<R, n...> out{};
  const T* src = reinterpret_cast<const T*>(&a);
  R* dst = reinterpret_cast<R*>(&out);
  constexpr int count = sizeof(tensor<T, n...>) / sizeof(T);
  for (int i = 0; i < count; i++) dst[i] = get_value(src[i]);
  return out;
}
SFX_HDI constexpr zero get_value(zero) { return {}; }

// gradient of the directional (scalar-gradient) dual
SFX_HDI constexpr zero get_gradient(double) { return {}; }
SFX_HDI constexpr zero get_gradient(float) { return {}; }
SFX_HDI constexpr zero get_gradient(zero) { return {}; }
template <typename V, typename G>
SFX_HDI constexpr G get_gradient(const dual<V, G>& a) { return a.gradient; }

// --------------------------------------------------------------- arithmetic
template <typename V, typename G>
SFX_HDI constexpr dual<V, G> operator-(const dual<V, G>& a) {
  return {-a.value, -a.gradient};
}
template <typename V, typename G>
SFX_HDI constexpr dual<V, G> operator+(const dual<V, G>& a, const dual<V, G>& b) {
  return {a.value + b.value, a.gradient + b.gradient};
}
template <typename V, typename G>
SFX_HDI constexpr dual<V, G> operator-(const dual<V, G>& a, const dual<V, G>& b) {
  return {a.value - b.value, a.gradient - b.gradient};
}
template <typename V, typename G>
SFX_HDI constexpr dual<V, G> operator*(const dual<V, G>& a, const dual<V, G>& b) {
  return {a.value * b.value, b.value * a.gradient + a.value * b.gradient};
}
template <typename V, typename G>
SFX_HDI constexpr dual<V, G> operator/(const dual<V, G>& a, const dual<V, G>& b) {
  V ib = V(1) / b.value;
  V q = a.value * ib;
  return {q, (a.gradient - q * b.gradient) * ib};
}

#define SFX_DUAL_SCALAR_OPS(A)                                                                      \
  template <typename V, typename G>                                                                 \
  SFX_HDI constexpr dual<V, G> operator+(const dual<V, G>& a, A b) {                                \
    return {a.value + V(b), a.gradient};                                                            \
  }                                                                                                 \
  template <typename V, typename G>                                                                 \
  SFX_HDI constexpr dual<V, G> operator+(A b, const dual<V, G>& a) {                                \
    return {V(b) + a.value, a.gradient};                                                            \
  }                                                                                                 \
  template <typename V, typename G>                                                                 \
  SFX_HDI constexpr dual<V, G> operator-(const dual<V, G>& a, A b) {                                \
    return {a.value - V(b), a.gradient};                                                            \
  }                                                                                                 \
  template <typename V, typename G>                                                                 \
  SFX_HDI constexpr dual<V, G> operator-(A b, const dual<V, G>& a) {                                \
    return {V(b) - a.value, -a.gradient};                                                           \
  }                                                                                                 \
  template <typename V, typename G>                                                                 \
  SFX_HDI constexpr dual<V, G> operator*(const dual<V, G>& a, A b) {                                \
    return {a.value * V(b), V(b) * a.gradient};                                                     \
  }                                                                                                 \
  template <typename V, typename G>                                                                 \
  SFX_HDI constexpr dual<V, G> operator*(A b, const dual<V, G>& a) {                                \
    return {V(b) * a.value, V(b) * a.gradient};                                                     \
  }                                                                                                 \
  template <typename V, typename G>                                                                 \
  SFX_HDI constexpr dual<V, G> operator/(const dual<V, G>& a, A b) {                                \
    V ib = V(1) / V(b);                                                                             \
    return {a.value * ib, a.gradient * ib};                                                         \
  }                                                                                                 \
  template <typename V, typename G>                                                                 \
  SFX_HDI constexpr dual<V, G> operator/(A b, const dual<V, G>& a) {                                \
    V ia = V(1) / a.value;                                                                          \
    V q = V(b) * ia;                                                                                \
    return {q, (-q * ia) * a.gradient};                                                             \
  }

SFX_DUAL_SCALAR_OPS(double)
SFX_DUAL_SCALAR_OPS(float)
SFX_DUAL_SCALAR_OPS(int)
#undef SFX_DUAL_SCALAR_OPS

template <typename V, typename G, typename T>
SFX_HDI constexpr dual<V, G>& operator+=(dual<V, G>& a, const T& b) {
  a = a + b;
  return a;
}
template <typename V, typename G, typename T>
SFX_HDI constexpr dual<V, G>& operator-=(dual<V, G>& a, const T& b) {
  a = a - b;
  return a;
}
template <typename V, typename G, typename T>
SFX_HDI constexpr dual<V, G>& operator*=(dual<V, G>& a, const T& b) {
  a = a * b;
  return a;
}
template <typename V, typename G, typename T>
SFX_HDI constexpr dual<V, G>& operator/=(dual<V, G>& a, const T& b) {
  a = a / b;
  return a;
}

template <typename V, typename G>
SFX_HDI constexpr bool operator<(const dual<V, G>& a, const dual<V, G>& b) { return a.value < b.value; }
template <typename V, typename G>
SFX_HDI constexpr bool operator>(const dual<V, G>& a, const dual<V, G>& b) { return a.value > b.value; }
template <typename V, typename G>
SFX_HDI constexpr bool operator<(const dual<V, G>& a, double b) { return a.value < b; }
template <typename V, typename G>
SFX_HDI constexpr bool operator>(const dual<V, G>& a, double b) { return a.value > b; }
template <typename V, typename G>
SFX_HDI constexpr bool operator<(double b, const dual<V, G>& a) { return b < a.value; }
template <typename V, typename G>
SFX_HDI constexpr bool operator>(double b, const dual<V, G>& a) { return b > a.value; }

// ------------------------------------------------------------ elementary fns
template <typename V, typename G>
SFX_HDI dual<V, G> sqrt(const dual<V, G>& a) {
  using std::sqrt;
  V r = sqrt(a.value);
  return {r, (V(0.5) / r) * a.gradient};
}
template <typename V, typename G>
SFX_HDI dual<V, G> log(const dual<V, G>& a) {
  using std::log;
  return {log(a.value), (V(1) / a.value) * a.gradient};
}
template <typename V, typename G>
SFX_HDI dual<V, G> log1p(const dual<V, G>& a) {
  using std::log1p;
  return {log1p(a.value), (V(1) / (V(1) + a.value)) * a.gradient};
}
template <typename V, typename G>
SFX_HDI dual<V, G> exp(const dual<V, G>& a) {
  using std::exp;
  V e = exp(a.value);
  return {e, e * a.gradient};
}
template <typename V, typename G>
SFX_HDI dual<V, G> sin(const dual<V, G>& a) {
  using std::cos;
  using std::sin;
  return {sin(a.value), cos(a.value) * a.gradient};
}
template <typename V, typename G>
SFX_HDI dual<V, G> cos(const dual<V, G>& a) {
  using std::cos;
  using std::sin;
  return {cos(a.value), -sin(a.value) * a.gradient};
}
template <typename V, typename G>
SFX_HDI dual<V, G> abs(const dual<V, G>& a) {
  return (a.value < V(0)) ? -a : a;
}
template <typename V, typename G>
SFX_HDI dual<V, G> pow(const dual<V, G>& a, double b) {
  using std::pow;
  V pb = pow(a.value, V(b - 1.0));
  return {pb * a.value, (V(b) * pb) * a.gradient};
}
template <typename V, typename G>
SFX_HDI dual<V, G> pow(const dual<V, G>& a, const dual<V, G>& b) {
  using std::log;
  using std::pow;
  V v = pow(a.value, b.value);
  return {v, (b.value * pow(a.value, b.value - V(1))) * a.gradient + (v * log(a.value)) * b.gradient};
}

// arithmetic between dual and tensor<scalar> handled in tensor.hpp; dual x dual
// with tensor gradients uses the tensor operators above.

}  // namespace sfx
