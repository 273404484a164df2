// Test double of the Tpetra::CrsMatrix surface the adapter uses (not
// Trilinos): records the inserted rows so a test can compare them.
#pragma once
#include <map>
#include <stdexcept>
#include <utility>
#include <vector>
#include "Teuchos_ArrayView.hpp"
#include "Teuchos_RCP.hpp"
#include "Tpetra_Map.hpp"
namespace Tpetra {
template <class Scalar = double, class LO = int, class GO = long long, class Node = void> class CrsMatrix {
 public:
  typedef Scalar scalar_type;
  typedef LO local_ordinal_type;
  typedef GO global_ordinal_type;
  typedef Map<LO, GO, Node> map_type;
  CrsMatrix(const Teuchos::RCP<const map_type>& rowMap, const Teuchos::ArrayView<const size_t>& numEntPerRow)
      : map_(rowMap), alloc_(numEntPerRow.size())
  {
    for (size_t i = 0; i < numEntPerRow.size(); ++i) alloc_[i] = numEntPerRow[i];
  }
  void insertGlobalValues(const GO globalRow, const LO numEnt, const Scalar vals[], const GO inds[])
  {
    if (filled_ || globalRow < 0 || (size_t)globalRow >= alloc_.size() || (size_t)numEnt > alloc_[globalRow])
      throw std::runtime_error("insertGlobalValues: bad row or more entries than allocated");
    auto& row = rows_[globalRow];
    for (LO k = 0; k < numEnt; ++k) row.emplace_back(inds[k], vals[k]);
  }
  void fillComplete()
  {
    filled_ = true;
    domain_ = range_ = map_->getGlobalNumElements();
  }
  void fillComplete(const Teuchos::RCP<const map_type>& domainMap, const Teuchos::RCP<const map_type>& rangeMap)
  {
    filled_ = true;
    domain_ = domainMap->getGlobalNumElements();
    range_ = rangeMap->getGlobalNumElements();
  }
  size_t DomainSize() const { return domain_; }
  size_t RangeSize() const { return range_; }
  bool isFillComplete() const { return filled_; }
  const std::map<GO, std::vector<std::pair<GO, Scalar>>>& Rows() const { return rows_; }
 private:
  Teuchos::RCP<const map_type> map_;
  std::vector<size_t> alloc_;
  std::map<GO, std::vector<std::pair<GO, Scalar>>> rows_;
  bool filled_ = false;
  size_t domain_ = 0, range_ = 0;
};
}  // namespace Tpetra
