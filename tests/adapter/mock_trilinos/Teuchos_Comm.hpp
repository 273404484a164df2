// Test double of Teuchos::Comm (not Trilinos): one process.
#pragma once
namespace Teuchos {
template <typename Ordinal> class Comm {
 public:
  virtual ~Comm() {}
  virtual int getRank() const { return 0; }
  virtual int getSize() const { return 1; }
};
}  // namespace Teuchos
