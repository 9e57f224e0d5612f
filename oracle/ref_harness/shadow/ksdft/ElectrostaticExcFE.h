#pragma once
#include <ksdft/Hamiltonian.h>
namespace dftefe {
namespace ksdft {
template <typename A, typename B, typename C, typename D, utils::MemorySpace m, size_type dim>
struct ElectrostaticExcFE : Hamiltonian<B, m> {
  std::shared_ptr<const Hamiltonian<B, m>> getElectrostaticFE() const { return nullptr; }
};
}  // namespace ksdft
}  // namespace dftefe
