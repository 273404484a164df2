// Test double of Teuchos::ArrayView (not Trilinos): a pointer and a size.
#pragma once
#include <cstddef>
namespace Teuchos {
template <typename T> class ArrayView {
 public:
  ArrayView(T* p, size_t n) : p_(p), n_(n) {}
  size_t size() const { return n_; }
  T& operator[](size_t i) const { return p_[i]; }
 private:
  T* p_;
  size_t n_;
};
}  // namespace Teuchos
