// Stand-in for the few mfem declarations that serac's header-only element
// math names (geometry enum, a vector type, dense-matrix stubs). Used only to
// compile the reference element kernels into the oracle's checker library.
#pragma once
#include <cmath>
#include <cstddef>
#include <iostream>
#include <map>
#include <memory>
#include <stdexcept>
#include <vector>

namespace mfem {
struct Geometry {
  enum Type { INVALID = -1, POINT = 0, SEGMENT, TRIANGLE, SQUARE, TETRAHEDRON, CUBE, PRISM, PYRAMID, NUM_GEOMETRIES };
};
class Vector {
 public:
  Vector() = default;
  explicit Vector(int n) : d_(std::size_t(n)) {}
  double* ReadWrite() { return d_.data(); }
  const double* Read() const { return d_.data(); }
  double* GetData() { return d_.data(); }
  int Size() const { return int(d_.size()); }
  double& operator[](int i) { return d_[std::size_t(i)]; }
 private:
  std::vector<double> d_;
};
struct FaceInformation {
  bool IsInterior() const { return true; }
};
// Mesh is never instantiated by the checker; these members only let the
// element-counting helpers in geometry.hpp compile.
class Mesh {
 public:
  int GetNE() const { return 0; }
  Geometry::Type GetElementGeometry(int) const { return Geometry::CUBE; }
  int GetNumFaces() const { return 0; }
  FaceInformation GetFaceInformation(int) const { return {}; }
  Geometry::Type GetFaceGeometry(int) const { return Geometry::SQUARE; }
};
class IntegrationRule;
class DenseMatrix {
 public:
  DenseMatrix(int m, int n) : m_(m), d_(std::size_t(m * n)) {}
  double& operator()(int i, int j) { return d_[std::size_t(i + m_ * j)]; }
 private:
  int m_;
  std::vector<double> d_;
};
class DenseMatrixEigensystem {
 public:
  explicit DenseMatrixEigensystem(DenseMatrix&) { throw std::runtime_error("eigensystem not available in shim"); }
  void Eval() {}
  double Eigenvalue(int) { return 0.0; }
  Vector& Eigenvector(int) { static Vector v; return v; }
};
}  // namespace mfem
