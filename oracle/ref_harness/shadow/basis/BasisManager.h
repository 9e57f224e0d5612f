// Minimal stand-in for the reference's basis/BasisManager.h: only the type
// alias that FECellWiseDataOperations needs.  Test-infrastructure only.
#pragma once
#include <utils/TypeConfig.h>
#include <utils/MemoryStorage.h>
namespace dftefe {
namespace basis {
template <typename ValueType, utils::MemorySpace memorySpace>
struct BasisManager {
  using SizeTypeVector = utils::MemoryStorage<size_type, memorySpace>;
};
}  // namespace basis
}  // namespace dftefe
