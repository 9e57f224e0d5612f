// Stand-in for ksdft/ElectrostaticONCVNonLocFE.h: a Hamiltonian component
// whose local part is a given set of cell matrices and whose nonlocal part is
// an AtomCenterNonLocalOpContextFE (or none).  Test-infrastructure only: the
// original builds both from UPF data and deal.II quadrature.
#pragma once
#include <ksdft/Hamiltonian.h>
#include <basis/AtomCenterNonLocalOpContextFE.h>
#include <memory>
#include <vector>
namespace dftefe {
namespace ksdft {
template <typename A, typename B, typename C, typename D, utils::MemorySpace m, size_type dim>
struct ElectrostaticONCVNonLocFE : Hamiltonian<A, m> {
  using NonLocalOp = basis::AtomCenterNonLocalOpContextFE<C, D, m, dim>;
  std::vector<A> localMats;
  std::shared_ptr<const NonLocalOp> nonLocal;

  void getLocal(utils::MemoryStorage<A, m> &s) const override {
    s.resize(localMats.size());
    s.copyFrom(localMats);
  }
  void applyNonLocal(linearAlgebra::MultiVector<A, m> &X, linearAlgebra::MultiVector<A, m> &Y, bool gx,
                     bool gy) const override {
    nonLocal->apply(X, Y, gx, gy);
  }
  bool hasLocalComponent() const override { return true; }
  bool hasNonLocalComponent() const override { return nonLocal != nullptr; }
  std::shared_ptr<const NonLocalOp> getAtomCenterNonLocalOpContextFE() const { return nonLocal; }
};
}  // namespace ksdft
}  // namespace dftefe
