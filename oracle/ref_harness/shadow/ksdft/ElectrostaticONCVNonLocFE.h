// Stand-in: no nonlocal pseudopotential part (the configurations use a local
// potential only).  Test-infrastructure only.
#pragma once
#include <ksdft/Hamiltonian.h>
namespace dftefe {
namespace ksdft {
struct NoNonLocalOp {
  void reinitCX(size_type) const {}
  void setCXToZero() const {}
  template <class P, class X>
  void applyCconjtransOnX(P, X) const {}
  void applyAllReduceOnCconjtransX() const {}
  void applyVOnCconjtransX() const {}
  template <class P, class X>
  void applyCOnVCconjtransX(P, X) const {}
};
template <typename A, typename B, typename C, typename D, utils::MemorySpace m, size_type dim>
struct ElectrostaticONCVNonLocFE : Hamiltonian<A, m> {
  bool hasNonLocalComponent() const override { return false; }
  std::shared_ptr<const NoNonLocalOp> getAtomCenterNonLocalOpContextFE() const { return nullptr; }
};
}  // namespace ksdft
}  // namespace dftefe
