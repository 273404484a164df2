// Test double of the Epetra_MultiVector surface the adapter uses (not Trilinos).
#pragma once
#include <vector>
#include "Epetra_Map.h"
class Epetra_MultiVector {
 public:
  Epetra_MultiVector(const Epetra_Map& map, int numVectors)
      : len_(map.NumMyElements()), data_((size_t)numVectors * map.NumMyElements(), 0.0), ptr_(numVectors)
  {
    for (int v = 0; v < numVectors; ++v) ptr_[v] = data_.data() + (size_t)v * len_;
  }
  int NumVectors() const { return (int)ptr_.size(); }
  int MyLength() const { return len_; }
  double*& operator[](int i) { return ptr_[i]; }
  double* const& operator[](int i) const { return ptr_[i]; }
 private:
  int len_;
  std::vector<double> data_;
  std::vector<double*> ptr_;
};
