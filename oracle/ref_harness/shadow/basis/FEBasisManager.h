// Stand-in for basis/FEBasisManager.h holding exactly what the operator
// contexts read: the cell -> dof map, the MPI pattern (serial) and the
// constraints.  Test-infrastructure only; the deal.II-backed original cannot
// be built here.
#pragma once
#include <basis/BasisManager.h>
#include <basis/ConstraintsLocal.h>
#include <utils/MPIPatternP2P.h>
#include <memory>
#include <vector>
namespace dftefe {
namespace basis {
struct BasisDofHandler {
  virtual ~BasisDofHandler() = default;
};
template <typename ValueTypeBasisCoeff, typename ValueTypeBasisData, utils::MemorySpace memorySpace, size_type dim>
struct FEBasisManager {
  size_type nCells = 0;
  std::vector<size_type> cellDofs;
  utils::MemoryStorage<size_type, memorySpace> cellIds;
  std::shared_ptr<const utils::mpi::MPIPatternP2P<memorySpace>> pattern;
  const ConstraintsLocal<ValueTypeBasisCoeff, memorySpace> *constraints = nullptr;
  // locally owned (classical, enrichment) id ranges, as an EFE basis reports them
  std::vector<std::pair<global_size_type, global_size_type>> ownedRanges;
  size_type nLocallyOwnedCells() const { return nCells; }
  size_type nLocallyOwnedCellDofs(size_type c) const { return cellDofs[c]; }
  const size_type *locallyOwnedCellLocalDofIdsBegin() const { return cellIds.data(); }
  std::shared_ptr<const utils::mpi::MPIPatternP2P<memorySpace>> getMPIPatternP2P() const { return pattern; }
  const ConstraintsLocal<ValueTypeBasisCoeff, memorySpace> &getConstraints() const { return *constraints; }
  std::vector<std::pair<global_size_type, global_size_type>> getLocallyOwnedRanges() const { return ownedRanges; }
  const BasisDofHandler &getBasisDofHandler() const;
};
}  // namespace basis
}  // namespace dftefe
