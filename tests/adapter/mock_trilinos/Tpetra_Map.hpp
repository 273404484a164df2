// Test double of the Tpetra::Map surface the adapter uses (not Trilinos): a
// contiguous one-process map with the default ordinal types.
#pragma once
#include <cstddef>
#include "Teuchos_Comm.hpp"
#include "Teuchos_RCP.hpp"
namespace Tpetra {
typedef size_t global_size_t;
template <class LO = int, class GO = long long, class Node = void> class Map {
 public:
  typedef LO local_ordinal_type;
  typedef GO global_ordinal_type;
  Map(global_size_t numGlobal, GO indexBase, const Teuchos::RCP<const Teuchos::Comm<int>>& comm)
      : n_(numGlobal), base_(indexBase), comm_(comm) {}
  global_size_t getGlobalNumElements() const { return n_; }
  GO getIndexBase() const { return base_; }
 private:
  global_size_t n_;
  GO base_;
  Teuchos::RCP<const Teuchos::Comm<int>> comm_;
};
}  // namespace Tpetra
