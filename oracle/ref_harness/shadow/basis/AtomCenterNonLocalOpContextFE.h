// Stand-in declaration of basis::AtomCenterNonLocalOpContextFE for the
// reference harness.  TEST INFRASTRUCTURE ONLY.
//
// The reference's constructor (AtomCenterNonLocalOpContextFE.t.cpp:267-634)
// builds its arrays from UPF atom data, deal.II quadrature and the enrichment
// id partition, none of which build here.  This declaration keeps the data
// members the reference's apply-side member functions read, under the names
// they use, and takes those arrays from the caller instead.  The member
// function bodies themselves (apply, reinitCX, setCXToZero,
// applyCconjtransOnX, applyAllReduceOnCconjtransX, applyVOnCconjtransX,
// applyCOnVCconjtransX) and the AtomCenterNonLocalOpContextFEInternal helpers
// are the reference's own, cut from its .t.cpp into oracle/_ref/patched/ by
// oracle/build_ref.sh and included below when present.
#pragma once
#include <basis/FEBasisManager.h>
#include <linearAlgebra/OperatorContext.h>
#include <linearAlgebra/MultiVector.h>
#include <linearAlgebra/LinAlgOpContext.h>
#include <linearAlgebra/BlasLapack.h>
#include <utils/MemoryStorage.h>
#include <utils/MPIPatternP2P.h>
#include <memory>
#include <utility>
#include <vector>

namespace dftefe {
namespace basis {
template <typename ValueTypeOperator, typename ValueTypeOperand, utils::MemorySpace memorySpace, size_type dim>
class AtomCenterNonLocalOpContextFE
    : public linearAlgebra::OperatorContext<ValueTypeOperator, ValueTypeOperand, memorySpace> {
 public:
  using ValueType = linearAlgebra::blasLapack::scalar_type<ValueTypeOperator, ValueTypeOperand>;

  // nProj projectors; per cell the number of projectors, the projector id of
  // each (cell, projector) slot, the np x nd column-major blocks C_c and the
  // diagonal coupling per projector.
  AtomCenterNonLocalOpContextFE(const FEBasisManager<ValueTypeOperand, ValueTypeOperator, memorySpace, dim> &fe,
                                size_type nProj, const std::vector<size_type> &projPerCell,
                                const std::vector<size_type> &projIds, const std::vector<ValueTypeOperator> &cellC,
                                const std::vector<ValueTypeOperator> &coupling, size_type maxCellBlock,
                                size_type maxFieldBlock,
                                std::shared_ptr<linearAlgebra::LinAlgOpContext<memorySpace>> ctx)
      : d_feBasisManager(&fe), d_maxCellBlock(maxCellBlock), d_maxWaveFnBatch(maxFieldBlock),
        d_linAlgOpContext(ctx) {
    d_numLocallyOwnedCells = fe.nLocallyOwnedCells();
    d_numProjsInCells = projPerCell;
    d_numCellDofs.resize(d_numLocallyOwnedCells);
    size_type maxProj = 1;
    for (size_type c = 0; c < d_numLocallyOwnedCells; ++c) {
      d_numCellDofs[c] = fe.nLocallyOwnedCellDofs(c);
      if (projPerCell[c] > maxProj) maxProj = projPerCell[c];
    }
    d_cellWiseC.resize(cellC.size());
    if (!cellC.empty()) d_cellWiseC.copyFrom(cellC);
    d_locallyOwnedCellLocalProjectorIds.resize(projIds.size());
    if (!projIds.empty()) d_locallyOwnedCellLocalProjectorIds.copyFrom(projIds);
    d_V.resize(coupling.size());
    if (!coupling.empty()) d_V.copyFrom(coupling);
    d_mpiPatternP2PProj = std::make_shared<const utils::mpi::MPIPatternP2P<memorySpace>>(nProj);
    d_CX = std::make_shared<linearAlgebra::MultiVector<ValueType, memorySpace>>(d_mpiPatternP2PProj, ctx,
                                                                                maxFieldBlock);
    d_CXCellValues.resize(maxCellBlock * maxFieldBlock * maxProj, ValueType());
  }

  void apply(linearAlgebra::MultiVector<ValueTypeOperand, memorySpace> &X,
             linearAlgebra::MultiVector<ValueType, memorySpace> &Y, bool updateGhostX = false,
             bool updateGhostY = false) const override;
  void reinitCX(size_type waveFuncBlockSize) const;
  void setCXToZero() const;
  void applyCconjtransOnX(std::pair<size_type, size_type> cellRange, const ValueTypeOperand *xCellValuesBegin) const;
  void applyAllReduceOnCconjtransX() const;
  void applyVOnCconjtransX() const;
  void applyCOnVCconjtransX(std::pair<size_type, size_type> cellRange, ValueTypeOperand *yCellValuesBegin) const;

 private:
  const FEBasisManager<ValueTypeOperand, ValueTypeOperator, memorySpace, dim> *d_feBasisManager;
  const size_type d_maxCellBlock;
  const size_type d_maxWaveFnBatch;
  std::shared_ptr<linearAlgebra::LinAlgOpContext<memorySpace>> d_linAlgOpContext;
  size_type d_numLocallyOwnedCells = 0;
  std::vector<size_type> d_numCellDofs;
  std::vector<size_type> d_numProjsInCells;
  utils::MemoryStorage<ValueTypeOperator, memorySpace> d_cellWiseC;
  utils::MemoryStorage<size_type, memorySpace> d_locallyOwnedCellLocalProjectorIds;
  utils::MemoryStorage<ValueTypeOperator, memorySpace> d_V;
  std::shared_ptr<const utils::mpi::MPIPatternP2P<memorySpace>> d_mpiPatternP2PProj;
  mutable std::shared_ptr<linearAlgebra::MultiVector<ValueType, memorySpace>> d_CX;
  mutable utils::MemoryStorage<ValueType, memorySpace> d_CXCellValues;
};
}  // namespace basis
}  // namespace dftefe

#if __has_include(<AtomCenterNonLocalOpContextFE.members.t.cpp>)
#include <AtomCenterNonLocalOpContextFE.members.t.cpp>
#define GBFE_REF_HAS_NONLOCAL 1
#endif
