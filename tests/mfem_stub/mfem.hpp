// Minimal stand-in for the parts of mfem.hpp that include/hcurl_mfem.hpp uses,
// so that the shim can be type-checked where MFEM is not installed.
#pragma once
#include <cstdlib>
#include <iostream>
#include <vector>

#define MFEM_ABORT(msg)                  \
  do {                                   \
    std::cerr << msg << std::endl;       \
    std::abort();                        \
  } while (0)

namespace mfem {
class Vector {
public:
  explicit Vector(int n = 0) : d_(n, 0.0) {}
  int Size() const { return (int)d_.size(); }
  const double* HostRead() const { return d_.data(); }
  double* HostWrite() { return d_.data(); }
  double* HostReadWrite() { return d_.data(); }
  Vector& operator=(double v) {
    for (auto& x : d_) x = v;
    return *this;
  }
  double& operator()(int i) { return d_[i]; }

private:
  std::vector<double> d_;
};
class DenseMatrix {  // column-major, like MFEM's
public:
  DenseMatrix(int h = 0, int w = 0) : h_(h), w_(w), d_((size_t)h * w, 0.0) {}
  int Height() const { return h_; }
  int Width() const { return w_; }
  double& operator()(int i, int j) { return d_[(size_t)j * h_ + i]; }
  const double& operator()(int i, int j) const { return d_[(size_t)j * h_ + i]; }

private:
  int h_, w_;
  std::vector<double> d_;
};
template <typename T>
class Array {
public:
  int Size() const { return (int)d_.size(); }
  void SetSize(int n) { d_.resize(n); }
  T& operator[](int i) { return d_[i]; }
  const T& operator[](int i) const { return d_[i]; }

private:
  std::vector<T> d_;
};
struct Geometry {
  enum Type { TETRAHEDRON = 4 };
  template <int G>
  struct Constants;
};
template <>
struct Geometry::Constants<Geometry::TETRAHEDRON> {
  static constexpr int Edges[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
};
class FiniteElement {
public:
  virtual ~FiniteElement() = default;
};
class VectorTensorFiniteElement : public FiniteElement {
public:
  const Array<int>& GetDofMap() const { return dof_map_; }

private:
  Array<int> dof_map_;
};
class FiniteElementSpace {
public:
  int GetNE() const { return 0; }
  void GetElementDofs(int, Array<int>& dofs) const { dofs.SetSize(0); }
  const FiniteElement* GetFE(int) const { return nullptr; }
};
class Mesh {
public:
  void GetElementVertices(int, Array<int>& v) const { v.SetSize(4); }
};
class Operator {
public:
  virtual ~Operator() = default;
  int Height() const { return height; }
  int Width() const { return width; }
  virtual void Mult(const Vector& x, Vector& y) const = 0;
  virtual Operator& GetGradient(const Vector&) const { std::abort(); }
  virtual void AssembleDiagonal(Vector&) const {}

protected:
  int height = 0, width = 0;
};
class Solver : public Operator {
public:
  bool iterative_mode = false;
  virtual void SetOperator(const Operator& op) = 0;
};
}  // namespace mfem
