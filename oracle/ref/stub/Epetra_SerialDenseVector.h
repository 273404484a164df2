// Minimal dense vector with the Epetra_SerialDenseVector members the
// reference's stateVector derives from and calls, so that its headers compile
// without Trilinos.  The element computations of the oracle pin do not use
// stateVector.  Test infrastructure (oracle/ref/Makefile).
#pragma once
#include <vector>
enum Epetra_DataAccess { Copy, View };
class Epetra_SerialDenseVector {
 public:
  Epetra_SerialDenseVector() {}
  explicit Epetra_SerialDenseVector(int n) : v_(n, 0.0) {}
  Epetra_SerialDenseVector(Epetra_DataAccess, double* p, int n) : v_(p, p + n) {}
  int Length() const { return (int)v_.size(); }
  int RowDim() const { return (int)v_.size(); }
  int ColDim() const { return 1; }
  int Size(int n) { v_.assign(n, 0.0); return 0; }
  int Resize(int n) { v_.resize(n, 0.0); return 0; }
  double& operator()(int i) { return v_[i]; }
  const double& operator()(int i) const { return v_[i]; }
  double& operator[](int i) { return v_[i]; }
  const double& operator[](int i) const { return v_[i]; }
  double* Values() { return v_.data(); }
  const double* Values() const { return v_.data(); }
 private:
  std::vector<double> v_;
};
