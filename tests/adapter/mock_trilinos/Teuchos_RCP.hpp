// Test double of the Teuchos::RCP surface the adapter uses (not Trilinos).
#pragma once
#include <memory>
namespace Teuchos {
template <typename T> using RCP = std::shared_ptr<T>;
template <typename T> RCP<T> rcp(T* p) { return RCP<T>(p); }
}  // namespace Teuchos
