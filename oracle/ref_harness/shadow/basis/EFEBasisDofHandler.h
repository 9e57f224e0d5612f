#pragma once
#include <utils/TypeConfig.h>
#include <utils/MemorySpaceType.h>
namespace dftefe {
namespace basis {
template <typename A, typename B, utils::MemorySpace m, size_type d>
class EFEBasisDofHandler;
}
}  // namespace dftefe
