// Test double of the Epetra_Map surface the adapter uses (not Trilinos): a
// contiguous one-process map.
#pragma once
#include "Epetra_Comm.h"
class Epetra_Map {
 public:
  Epetra_Map(int numGlobal, int indexBase, const Epetra_Comm& comm) : n_(numGlobal), base_(indexBase), comm_(comm) {}
  int NumGlobalElements() const { return n_; }
  int NumMyElements() const { return n_; }
  int IndexBase() const { return base_; }
  const Epetra_Comm& Comm() const { return comm_; }
 private:
  int n_, base_;
  const Epetra_Comm& comm_;
};
