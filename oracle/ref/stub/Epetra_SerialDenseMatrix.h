// Minimal dense matrix with the Epetra_SerialDenseMatrix members the
// reference's stateMatrix derives from and calls, so that its headers compile
// without Trilinos.  The element computations of the oracle pin do not use
// stateMatrix.  Test infrastructure (oracle/ref/Makefile).
#pragma once
#include <vector>
#include "Epetra_SerialDenseVector.h"
class Epetra_SerialDenseMatrix {
 public:
  Epetra_SerialDenseMatrix() {}
  Epetra_SerialDenseMatrix(int r, int c) : r_(r), c_(c), v_((size_t)r * c, 0.0) {}
  int M() const { return r_; }
  int N() const { return c_; }
  int RowDim() const { return r_; }
  int ColDim() const { return c_; }
  int Shape(int r, int c) { r_ = r; c_ = c; v_.assign((size_t)r * c, 0.0); return 0; }
  int Reshape(int r, int c) { return Shape(r, c); }
  double& operator()(int i, int j) { return v_[(size_t)j * r_ + i]; }
  const double& operator()(int i, int j) const { return v_[(size_t)j * r_ + i]; }
  double* A() { return v_.data(); }
  const double* A() const { return v_.data(); }
 private:
  int r_ = 0, c_ = 0;
  std::vector<double> v_;
};
