// Test double of the Epetra_Comm surface the adapter uses (not Trilinos).
#pragma once
class Epetra_Comm {
 public:
  virtual ~Epetra_Comm() {}
  virtual int NumProc() const = 0;
  virtual int MyPID() const = 0;
};
class Epetra_SerialComm : public Epetra_Comm {
 public:
  int NumProc() const override { return 1; }
  int MyPID() const override { return 0; }
};
