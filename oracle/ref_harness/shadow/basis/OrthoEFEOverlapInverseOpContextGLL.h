// Stand-in declaration of basis::OrthoEFEOverlapInverseOpContextGLL for the
// reference harness.  TEST INFRASTRUCTURE ONLY.
//
// The reference's constructors (OrthoEFEOverlapInverseOpContextGLL.t.cpp:
// 845-1170) build the GLL diagonal and the enrichment overlap block from
// deal.II basis data, which does not build here.  This declaration keeps the
// data members the reference's apply() reads, under the names it uses, and
// takes the diagonal and the block from the caller.  The apply() body itself
// (.t.cpp:1173-1305) is the reference's own, cut into oracle/_ref/patched/ by
// oracle/build_ref.sh and included below when present; the harness always
// builds the operator with the direct (non-CG) branch.
#pragma once
#include <basis/FEBasisManager.h>
#include <linearAlgebra/OperatorContext.h>
#include <linearAlgebra/MultiVector.h>
#include <linearAlgebra/Vector.h>
#include <linearAlgebra/LinAlgOpContext.h>
#include <linearAlgebra/BlasLapack.h>
#include <linearAlgebra/LinearSolverFunction.h>
#include <linearAlgebra/LinearSolverImpl.h>
#include <utils/MemoryStorage.h>
#include <utils/MPIWrapper.h>
#include <memory>
#include <utility>
#include <vector>

namespace dftefe {
namespace basis {
// the global (classical, enrichment) id ranges the apply reads from the EFE
// dof handler
struct EFEGlobalRanges {
  std::vector<std::pair<global_size_type, global_size_type>> ranges;
  std::vector<std::pair<global_size_type, global_size_type>> getGlobalRanges() const { return ranges; }
};

namespace OrthoEFEOverlapInverseOpContextGLLInternal {
// the CG branch's solver function: declared so that apply() compiles; the
// harness never takes that branch
template <typename ValueTypeOperator, typename ValueTypeOperand, utils::MemorySpace memorySpace, size_type dim>
class OverlapMatrixInverseLinearSolverFunctionFE
    : public linearAlgebra::LinearSolverFunction<ValueTypeOperator, ValueTypeOperand, memorySpace> {
 public:
  void reinit(linearAlgebra::MultiVector<ValueTypeOperand, memorySpace> &) {}
};
}  // namespace OrthoEFEOverlapInverseOpContextGLLInternal

template <typename ValueTypeOperator, typename ValueTypeOperand, utils::MemorySpace memorySpace, size_type dim>
class OrthoEFEOverlapInverseOpContextGLL
    : public linearAlgebra::OperatorContext<ValueTypeOperator, ValueTypeOperand, memorySpace> {
 public:
  using ValueType = linearAlgebra::blasLapack::scalar_type<ValueTypeOperator, ValueTypeOperand>;

  // diagonalInv: the inverse GLL-lumped overlap on every dof; block: the
  // nEnr x nEnr inverse enrichment overlap block, column-major (the
  // enrichment ids are the last nEnr ids)
  OrthoEFEOverlapInverseOpContextGLL(const FEBasisManager<ValueTypeOperand, ValueTypeOperator, memorySpace, dim> &fe,
                                     const EFEGlobalRanges &efeRanges, const std::vector<ValueTypeOperator> &diagonalInv,
                                     size_type nEnr, const std::vector<ValueTypeOperator> &block,
                                     std::shared_ptr<linearAlgebra::LinAlgOpContext<memorySpace>> ctx)
      : d_feBasisManager(&fe), d_efebasisDofHandler(&efeRanges), d_diagonalInv(fe.getMPIPatternP2P(), ctx),
        d_nglobalEnrichmentIds(nEnr), d_linAlgOpContext(ctx), d_isCGSolved(false) {
    std::copy(diagonalInv.begin(), diagonalInv.end(), d_diagonalInv.data());
    d_basisOverlapEnrichmentBlock = std::make_shared<utils::MemoryStorage<ValueTypeOperator, memorySpace>>(block.size());
    d_basisOverlapEnrichmentBlock->copyFrom(block);
  }

  void apply(linearAlgebra::MultiVector<ValueTypeOperand, memorySpace> &X,
             linearAlgebra::MultiVector<ValueType, memorySpace> &Y, bool updateGhostX = false,
             bool updateGhostY = false) const override;

 private:
  const FEBasisManager<ValueTypeOperand, ValueTypeOperator, memorySpace, dim> *d_feBasisManager;
  const EFEGlobalRanges *d_efebasisDofHandler;
  linearAlgebra::Vector<ValueTypeOperator, memorySpace> d_diagonalInv;
  std::shared_ptr<utils::MemoryStorage<ValueTypeOperator, memorySpace>> d_basisOverlapEnrichmentBlock;
  size_type d_nglobalEnrichmentIds;
  std::shared_ptr<linearAlgebra::LinAlgOpContext<memorySpace>> d_linAlgOpContext;
  bool d_isCGSolved;
  std::shared_ptr<linearAlgebra::LinearSolverFunction<ValueTypeOperator, ValueTypeOperand, memorySpace>>
      d_overlapInvPoisson;
  std::shared_ptr<linearAlgebra::LinearSolverImpl<ValueTypeOperator, ValueTypeOperand, memorySpace>> d_CGSolve;
};
}  // namespace basis
}  // namespace dftefe

#if __has_include(<OrthoEFEOverlapInverseOpContextGLL.apply.t.cpp>)
#include <OrthoEFEOverlapInverseOpContextGLL.apply.t.cpp>
#define GBFE_REF_HAS_ORTHO_EFE_INVERSE 1
#endif
