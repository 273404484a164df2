// Test double of the Epetra_Operator interface (not Trilinos): the pure
// virtual functions an operator implements.
#pragma once
#include "Epetra_Comm.h"
#include "Epetra_Map.h"
#include "Epetra_MultiVector.h"
class Epetra_Operator {
 public:
  virtual ~Epetra_Operator() {}
  virtual int SetUseTranspose(bool UseTranspose) = 0;
  virtual int Apply(const Epetra_MultiVector& X, Epetra_MultiVector& Y) const = 0;
  virtual int ApplyInverse(const Epetra_MultiVector& X, Epetra_MultiVector& Y) const = 0;
  virtual double NormInf() const = 0;
  virtual const char* Label() const = 0;
  virtual bool UseTranspose() const = 0;
  virtual bool HasNormInf() const = 0;
  virtual const Epetra_Comm& Comm() const = 0;
  virtual const Epetra_Map& OperatorDomainMap() const = 0;
  virtual const Epetra_Map& OperatorRangeMap() const = 0;
};
