// sfx — fixed-size tensors for q-functions on device and host.
//
// Semantics follow serac's tensor library (numerics/functional/tensor.hpp):
// row-major nested arrays, `dot` contracts the last index of the left operand
// with the first of the right, `double_dot` contracts two indices, `zero` is a
// compile-time zero that prunes terms.  Mixed arithmetic between a plain
// arithmetic scalar and a tensor / dual keeps the precision of the tensor /
// dual operand (so FP32 q-functions stay FP32 when they multiply by double
// literals or parameters).
#pragma once

#include <cmath>
#include <type_traits>
#include <utility>

#if defined(__CUDACC__)
#define SFX_HD __host__ __device__
#else
#define SFX_HD
#endif
#define SFX_HDI SFX_HD inline

namespace sfx {

// ------------------------------------------------------------------ zero
struct zero {
  SFX_HD constexpr operator double() const { return 0.0; }
  template <typename... T>
  SFX_HD constexpr zero operator()(T...) const { return {}; }
};
template <typename T>
struct is_zero : std::false_type {};
template <>
struct is_zero<zero> : std::true_type {};

SFX_HDI constexpr zero operator+(zero, zero) { return {}; }
template <typename T>
SFX_HDI constexpr T operator+(zero, const T& a) { return a; }
template <typename T>
SFX_HDI constexpr T operator+(const T& a, zero) { return a; }
SFX_HDI constexpr zero operator-(zero) { return {}; }
SFX_HDI constexpr zero operator-(zero, zero) { return {}; }
template <typename T>
SFX_HDI constexpr T operator-(const T& a, zero) { return a; }
template <typename T>
SFX_HDI constexpr auto operator-(zero, const T& a) { return -a; }
template <typename T>
SFX_HDI constexpr zero operator*(zero, const T&) { return {}; }
template <typename T>
SFX_HDI constexpr zero operator*(const T&, zero) { return {}; }
SFX_HDI constexpr zero operator*(zero, zero) { return {}; }
template <typename T>
SFX_HDI constexpr zero operator/(zero, const T&) { return {}; }

// --------------------------------------------------------------- tensor
template <typename T, int... n>
struct tensor;

template <typename T, int m>
struct tensor<T, m> {
  using type = T;
  static constexpr int ndim = 1;
  static constexpr int first_dim = m;
  T data[m];
  SFX_HDI constexpr T& operator[](int i) { return data[i]; }
  SFX_HDI constexpr const T& operator[](int i) const { return data[i]; }
  SFX_HDI constexpr T& operator()(int i) { return data[i]; }
  SFX_HDI constexpr const T& operator()(int i) const { return data[i]; }
};

template <typename T, int m, int... n>
struct tensor<T, m, n...> {
  using type = T;
  static constexpr int ndim = 1 + sizeof...(n);
  static constexpr int first_dim = m;
  tensor<T, n...> data[m];
  SFX_HDI constexpr tensor<T, n...>& operator[](int i) { return data[i]; }
  SFX_HDI constexpr const tensor<T, n...>& operator[](int i) const { return data[i]; }
  SFX_HDI constexpr tensor<T, n...>& operator()(int i) { return data[i]; }
  SFX_HDI constexpr const tensor<T, n...>& operator()(int i) const { return data[i]; }
  template <typename... I>
  SFX_HDI constexpr auto& operator()(int i, I... rest) { return data[i](rest...); }
  template <typename... I>
  SFX_HDI constexpr const auto& operator()(int i, I... rest) const { return data[i](rest...); }
};

template <typename T, int m>
tensor(const T (&)[m]) -> tensor<T, m>;

template <typename T>
struct is_tensor : std::false_type {};
template <typename T, int... n>
struct is_tensor<tensor<T, n...>> : std::true_type {};

// scalar type of a number-like object (double, float, dual<...>)
template <typename T, typename = void>
struct scalar_of {
  using type = T;
};
template <typename T, int... n>
struct scalar_of<tensor<T, n...>> {
  using type = typename scalar_of<T>::type;
};

// ----------------------------------------------------------- generic maps
template <typename F, typename T, int... n>
SFX_HDI constexpr auto tmap(F&& f, const tensor<T, n...>& a) {
  using R = decltype(f(a.data[0]));
  constexpr int m = tensor<T, n...>::first_dim;
  tensor<typename std::conditional<tensor<T, n...>::ndim == 1, R, typename R::type>::type, n...> out{};
  for (int i = 0; i < m; i++) out.data[i] = f(a.data[i]);
  return out;
}

template <typename T, int... n>
SFX_HDI constexpr tensor<T, n...> operator-(const tensor<T, n...>& a) {
  tensor<T, n...> out{};
  for (int i = 0; i < tensor<T, n...>::first_dim; i++) out.data[i] = -a.data[i];
  return out;
}

template <typename S, typename T, int... n>
SFX_HDI constexpr auto operator+(const tensor<S, n...>& a, const tensor<T, n...>& b) {
  tensor<decltype(S{} + T{}), n...> out{};
  for (int i = 0; i < tensor<T, n...>::first_dim; i++) out.data[i] = a.data[i] + b.data[i];
  return out;
}
template <typename S, typename T, int... n>
SFX_HDI constexpr auto operator-(const tensor<S, n...>& a, const tensor<T, n...>& b) {
  tensor<decltype(S{} - T{}), n...> out{};
  for (int i = 0; i < tensor<T, n...>::first_dim; i++) out.data[i] = a.data[i] - b.data[i];
  return out;
}
template <typename S, typename T, int... n>
SFX_HDI constexpr tensor<S, n...>& operator+=(tensor<S, n...>& a, const tensor<T, n...>& b) {
  for (int i = 0; i < tensor<T, n...>::first_dim; i++) a.data[i] += b.data[i];
  return a;
}
template <typename S, typename T, int... n>
SFX_HDI constexpr tensor<S, n...>& operator-=(tensor<S, n...>& a, const tensor<T, n...>& b) {
  for (int i = 0; i < tensor<T, n...>::first_dim; i++) a.data[i] -= b.data[i];
  return a;
}
template <typename S, int... n>
SFX_HDI constexpr tensor<S, n...>& operator+=(tensor<S, n...>& a, zero) { return a; }

// scalar (arithmetic) x tensor: keeps the tensor's element precision
template <typename A, typename T, int... n, typename = std::enable_if_t<std::is_arithmetic<A>::value>>
SFX_HDI constexpr tensor<T, n...> operator*(A s, const tensor<T, n...>& a) {
  tensor<T, n...> out{};
  for (int i = 0; i < tensor<T, n...>::first_dim; i++) out.data[i] = s * a.data[i];
  return out;
}
template <typename A, typename T, int... n, typename = std::enable_if_t<std::is_arithmetic<A>::value>>
SFX_HDI constexpr tensor<T, n...> operator*(const tensor<T, n...>& a, A s) {
  return s * a;
}
template <typename A, typename T, int... n, typename = std::enable_if_t<std::is_arithmetic<A>::value>>
SFX_HDI constexpr tensor<T, n...> operator/(const tensor<T, n...>& a, A s) {
  tensor<T, n...> out{};
  for (int i = 0; i < tensor<T, n...>::first_dim; i++) out.data[i] = a.data[i] / s;
  return out;
}
template <typename A, typename T, int... n, typename = std::enable_if_t<std::is_arithmetic<A>::value>>
SFX_HDI constexpr tensor<T, n...>& operator*=(tensor<T, n...>& a, A s) {
  for (int i = 0; i < tensor<T, n...>::first_dim; i++) a.data[i] *= s;
  return a;
}

// non-arithmetic scalar (dual) x tensor
template <typename S, typename T, int... n,
          typename = std::enable_if_t<!std::is_arithmetic<S>::value && !is_tensor<S>::value && !is_zero<S>::value>>
SFX_HDI constexpr auto operator*(const S& s, const tensor<T, n...>& a) {
  using R = decltype(s * a.data[0]);
  tensor<typename std::conditional<tensor<T, n...>::ndim == 1, R, typename scalar_of<R>::type>::type, n...> out{};
  for (int i = 0; i < tensor<T, n...>::first_dim; i++) out.data[i] = s * a.data[i];
  return out;
}
template <typename S, typename T, int... n,
          typename = std::enable_if_t<!std::is_arithmetic<S>::value && !is_tensor<S>::value && !is_zero<S>::value>>
SFX_HDI constexpr auto operator*(const tensor<T, n...>& a, const S& s) {
  return s * a;
}
template <typename S, typename T, int... n,
          typename = std::enable_if_t<!std::is_arithmetic<S>::value && !is_tensor<S>::value && !is_zero<S>::value>>
SFX_HDI constexpr auto operator/(const tensor<T, n...>& a, const S& s) {
  using R = decltype(a.data[0] / s);
  tensor<typename std::conditional<tensor<T, n...>::ndim == 1, R, typename scalar_of<R>::type>::type, n...> out{};
  for (int i = 0; i < tensor<T, n...>::first_dim; i++) out.data[i] = a.data[i] / s;
  return out;
}

// --------------------------------------------------------------- builders
template <int n, typename T = double>
SFX_HDI constexpr tensor<T, n, n> Identity() {
  tensor<T, n, n> I{};
  for (int i = 0; i < n; i++) I[i][i] = T(1);
  return I;
}

template <int m, typename F>
SFX_HDI constexpr auto make_tensor(F&& f) {
  using R = decltype(f(0));
  tensor<R, m> out{};
  for (int i = 0; i < m; i++) out[i] = f(i);
  return out;
}
template <int m, int n, typename F>
SFX_HDI constexpr auto make_tensor(F&& f) {
  using R = decltype(f(0, 0));
  tensor<R, m, n> out{};
  for (int i = 0; i < m; i++)
    for (int j = 0; j < n; j++) out[i][j] = f(i, j);
  return out;
}
template <int m, int n, int p, typename F>
SFX_HDI constexpr auto make_tensor(F&& f) {
  using R = decltype(f(0, 0, 0));
  tensor<R, m, n, p> out{};
  for (int i = 0; i < m; i++)
    for (int j = 0; j < n; j++)
      for (int k = 0; k < p; k++) out[i][j][k] = f(i, j, k);
  return out;
}
template <int m, int n, int p, int q, typename F>
SFX_HDI constexpr auto make_tensor(F&& f) {
  using R = decltype(f(0, 0, 0, 0));
  tensor<R, m, n, p, q> out{};
  for (int i = 0; i < m; i++)
    for (int j = 0; j < n; j++)
      for (int k = 0; k < p; k++)
        for (int l = 0; l < q; l++) out[i][j][k][l] = f(i, j, k, l);
  return out;
}

// ---------------------------------------------------------- contractions
// vector . vector
template <typename S, typename T, int n>
SFX_HDI constexpr auto dot(const tensor<S, n>& a, const tensor<T, n>& b) {
  auto s = a[0] * b[0];
  for (int i = 1; i < n; i++) s = s + a[i] * b[i];
  return s;
}
// vector . matrix
template <typename S, typename T, int m, int n>
SFX_HDI constexpr auto dot(const tensor<S, m>& a, const tensor<T, m, n>& B) {
  tensor<decltype(S{} * T{}), n> out{};
  for (int j = 0; j < n; j++) {
    auto s = a[0] * B[0][j];
    for (int i = 1; i < m; i++) s = s + a[i] * B[i][j];
    out[j] = s;
  }
  return out;
}
// matrix . vector
template <typename S, typename T, int m, int n>
SFX_HDI constexpr auto dot(const tensor<S, m, n>& A, const tensor<T, n>& b) {
  tensor<decltype(S{} * T{}), m> out{};
  for (int i = 0; i < m; i++) out[i] = dot(A[i], b);
  return out;
}
// matrix . matrix
template <typename S, typename T, int m, int n, int p>
SFX_HDI constexpr auto dot(const tensor<S, m, n>& A, const tensor<T, n, p>& B) {
  tensor<decltype(S{} * T{}), m, p> out{};
  for (int i = 0; i < m; i++)
    for (int j = 0; j < p; j++) {
      auto s = A[i][0] * B[0][j];
      for (int k = 1; k < n; k++) s = s + A[i][k] * B[k][j];
      out[i][j] = s;
    }
  return out;
}
// rank-3 . vector / matrix (last index)
template <typename S, typename T, int m, int n, int p>
SFX_HDI constexpr auto dot(const tensor<S, m, n, p>& A, const tensor<T, p>& b) {
  tensor<decltype(S{} * T{}), m, n> out{};
  for (int i = 0; i < m; i++) out[i] = dot(A[i], b);
  return out;
}
template <typename T, int... n>
SFX_HDI constexpr zero dot(const tensor<T, n...>&, zero) { return {}; }
template <typename T, int... n>
SFX_HDI constexpr zero dot(zero, const tensor<T, n...>&) { return {}; }

template <typename S, typename T, int m, int n>
SFX_HDI constexpr auto operator*(const tensor<S, m, n>& A, const tensor<T, n>& b) { return dot(A, b); }
template <typename S, typename T, int m, int n, int p>
SFX_HDI constexpr auto operator*(const tensor<S, m, n>& A, const tensor<T, n, p>& B) { return dot(A, B); }

// double contractions
template <typename S, typename T, int m, int n>
SFX_HDI constexpr auto double_dot(const tensor<S, m, n>& A, const tensor<T, m, n>& B) {
  auto s = A[0][0] * B[0][0];
  for (int i = 0; i < m; i++)
    for (int j = 0; j < n; j++)
      if (i || j) s = s + A[i][j] * B[i][j];
  return s;
}
template <typename S, typename T, int m, int n, int p>
SFX_HDI constexpr auto double_dot(const tensor<S, m, n, p>& A, const tensor<T, n, p>& B) {
  tensor<decltype(S{} * T{}), m> out{};
  for (int i = 0; i < m; i++) out[i] = double_dot(A[i], B);
  return out;
}
template <typename S, typename T, int m, int n, int p, int q>
SFX_HDI constexpr auto double_dot(const tensor<S, m, n, p, q>& A, const tensor<T, p, q>& B) {
  tensor<decltype(S{} * T{}), m, n> out{};
  for (int i = 0; i < m; i++)
    for (int j = 0; j < n; j++) out[i][j] = double_dot(A[i][j], B);
  return out;
}

template <typename S, typename T, int m, int n>
SFX_HDI constexpr auto outer(const tensor<S, m>& a, const tensor<T, n>& b) {
  tensor<decltype(S{} * T{}), m, n> out{};
  for (int i = 0; i < m; i++)
    for (int j = 0; j < n; j++) out[i][j] = a[i] * b[j];
  return out;
}

// ---------------------------------------------------------- matrix algebra
template <typename T, int m, int n>
SFX_HDI constexpr tensor<T, n, m> transpose(const tensor<T, m, n>& A) {
  tensor<T, n, m> out{};
  for (int i = 0; i < m; i++)
    for (int j = 0; j < n; j++) out[j][i] = A[i][j];
  return out;
}
template <typename T, int n>
SFX_HDI constexpr T tr(const tensor<T, n, n>& A) {
  T s = A[0][0];
  for (int i = 1; i < n; i++) s = s + A[i][i];
  return s;
}
template <typename T, int n>
SFX_HDI constexpr tensor<T, n, n> sym(const tensor<T, n, n>& A) {
  tensor<T, n, n> out{};
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) out[i][j] = 0.5 * (A[i][j] + A[j][i]);
  return out;
}
template <typename T, int n>
SFX_HDI constexpr tensor<T, n, n> dev(const tensor<T, n, n>& A) {
  tensor<T, n, n> out = A;
  T t = tr(A) / double(n);
  for (int i = 0; i < n; i++) out[i][i] = out[i][i] - t;
  return out;
}
template <typename T>
SFX_HDI constexpr T det(const tensor<T, 2, 2>& A) {
  return A[0][0] * A[1][1] - A[0][1] * A[1][0];
}
template <typename T>
SFX_HDI constexpr T det(const tensor<T, 3, 3>& A) {
  return A[0][0] * A[1][1] * A[2][2] + A[0][1] * A[1][2] * A[2][0] + A[0][2] * A[1][0] * A[2][1] -
         A[0][0] * A[1][2] * A[2][1] - A[0][1] * A[1][0] * A[2][2] - A[0][2] * A[1][1] * A[2][0];
}
// det(I + A) - 1, accurate for small A: tr A + (tr(A)^2 - tr(A^2)) / 2 + det A
template <typename T>
SFX_HDI constexpr T detApIm1(const tensor<T, 3, 3>& A) {
  T trA = tr(A);
  T trA2 = A[0][0] * A[0][0];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      if (i || j) trA2 = trA2 + A[i][j] * A[j][i];
  return trA + 0.5 * (trA * trA - trA2) + det(A);
}
template <typename T>
SFX_HDI constexpr tensor<T, 3, 3> inv(const tensor<T, 3, 3>& A) {
  T d = det(A);
  T id = T(1.0) / d;
  tensor<T, 3, 3> r{};
  r[0][0] = (A[1][1] * A[2][2] - A[1][2] * A[2][1]) * id;
  r[0][1] = (A[0][2] * A[2][1] - A[0][1] * A[2][2]) * id;
  r[0][2] = (A[0][1] * A[1][2] - A[0][2] * A[1][1]) * id;
  r[1][0] = (A[1][2] * A[2][0] - A[1][0] * A[2][2]) * id;
  r[1][1] = (A[0][0] * A[2][2] - A[0][2] * A[2][0]) * id;
  r[1][2] = (A[0][2] * A[1][0] - A[0][0] * A[1][2]) * id;
  r[2][0] = (A[1][0] * A[2][1] - A[1][1] * A[2][0]) * id;
  r[2][1] = (A[0][1] * A[2][0] - A[0][0] * A[2][1]) * id;
  r[2][2] = (A[0][0] * A[1][1] - A[0][1] * A[1][0]) * id;
  return r;
}
template <typename T>
SFX_HDI constexpr tensor<T, 2, 2> inv(const tensor<T, 2, 2>& A) {
  T id = T(1.0) / det(A);
  return {{{A[1][1] * id, -A[0][1] * id}, {-A[1][0] * id, A[0][0] * id}}};
}

template <typename T, int... n>
SFX_HDI constexpr auto squared_norm(const tensor<T, n...>& A) {
  auto s = squared_norm(A.data[0]);
  for (int i = 1; i < tensor<T, n...>::first_dim; i++) s = s + squared_norm(A.data[i]);
  return s;
}
template <typename T, int m>
SFX_HDI constexpr T squared_norm(const tensor<T, m>& a) {
  T s = a[0] * a[0];
  for (int i = 1; i < m; i++) s = s + a[i] * a[i];
  return s;
}
template <typename T, int... n>
SFX_HDI auto norm(const tensor<T, n...>& A) {
  using std::sqrt;
  return sqrt(squared_norm(A));
}
template <typename T, int... n>
SFX_HDI auto normalize(const tensor<T, n...>& A) {
  return A / norm(A);
}

template <typename T>
SFX_HDI constexpr tensor<T, 3> cross(const tensor<T, 3>& a, const tensor<T, 3>& b) {
  return {{a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]}};
}
// normal of a surface parametrisation: columns of the 3x2 Jacobian
template <typename T>
SFX_HDI constexpr tensor<T, 3> cross(const tensor<T, 3, 2>& J) {
  return {{J[1][0] * J[2][1] - J[2][0] * J[1][1], J[2][0] * J[0][1] - J[0][0] * J[2][1],
           J[0][0] * J[1][1] - J[1][0] * J[0][1]}};
}

}  // namespace sfx
