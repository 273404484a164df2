// Test double of the Epetra_FECrsMatrix surface the adapter uses (not
// Trilinos): records the inserted rows so a test can compare them.
#pragma once
#include <map>
#include <utility>
#include <vector>
#include "Epetra_Map.h"
enum Epetra_DataAccess { Copy, View };
class Epetra_FECrsMatrix {
 public:
  Epetra_FECrsMatrix(Epetra_DataAccess, const Epetra_Map& rowMap, int* numEntriesPerRow)
      : map_(rowMap), alloc_(numEntriesPerRow, numEntriesPerRow + rowMap.NumMyElements())
  {
  }
  int InsertGlobalValues(int globalRow, int numEntries, double* values, int* indices)
  {
    if (filled_ || globalRow < 0 || globalRow >= map_.NumGlobalElements()) return -1;
    if (numEntries > alloc_[globalRow]) return 1;  // Epetra returns a positive code when it had to grow
    auto& row = rows_[globalRow];
    for (int k = 0; k < numEntries; ++k) row.emplace_back(indices[k], values[k]);
    return 0;
  }
  int GlobalAssemble(bool callFillComplete = true)
  {
    filled_ = callFillComplete;
    domain_ = range_ = map_.NumGlobalElements();
    return 0;
  }
  int GlobalAssemble(const Epetra_Map& domainMap, const Epetra_Map& rangeMap, bool callFillComplete = true)
  {
    filled_ = callFillComplete;
    domain_ = domainMap.NumGlobalElements();
    range_ = rangeMap.NumGlobalElements();
    return 0;
  }
  int NumGlobalDomain() const { return domain_; }
  int NumGlobalRange() const { return range_; }
  bool Filled() const { return filled_; }
  const std::map<int, std::vector<std::pair<int, double>>>& Rows() const { return rows_; }
 private:
  const Epetra_Map& map_;
  std::vector<int> alloc_;
  std::map<int, std::vector<std::pair<int, double>>> rows_;
  bool filled_ = false;
  int domain_ = 0, range_ = 0;
};
