// gbfe_operator_context.hpp -- drop-in dft-efe OperatorContext backed by
// libgbfe (include/gbfe.h).
//
// A maintainer adds this header to a dft-efe build and constructs
// GpuCellOperatorContext in place of KohnShamOperatorContextFE
// (ksdft/KohnShamOperatorContextFE.h:102-112), CFEOverlapOperatorContext or
// LaplaceOperatorContextFE, and GpuDiagonalOperatorContext in place of
// CFEOverlapInverseOpContextGLL's diagonal branch.  The solvers
// (ChebyshevFilteredEigenSolver, KohnShamEigenSolver, CGLinearSolver,
// LanczosExtremeEigenSolver) take them as `const OperatorContext &` unchanged
// (linearAlgebra/OperatorContext.h:47-109).
//
//  * MemorySpace::DEVICE MultiVectors are wrapped in place (gbfe_mv_wrap):
//    no copy, the reference's [dof][vector] layout is the library's layout.
//  * MemorySpace::HOST MultiVectors are staged through device buffers owned by
//    the context (X is copied back because apply() modifies it through the
//    constraints, as OperatorContext.h:79-83 documents).
//  * Errors surface as utils::throwException, like the reference's own
//    contract checks.
#pragma once

#include "gbfe.h"

#include <linearAlgebra/MultiVector.h>
#include <linearAlgebra/OperatorContext.h>
#include <utils/Exceptions.h>

#include <memory>
#include <string>
#include <type_traits>
#include <vector>

namespace dftefe {
namespace gb300 {

inline void gbfeCheck(gbfe_ctx *ctx, int rc, const char *what) {
  if (rc != GBFE_OK) {
    char buf[512] = {0};
    if (ctx) gbfe_last_error(ctx, buf, sizeof buf);
    utils::throwException(false, std::string("libgbfe ") + what + ": " + buf);
  }
}

// One GPU context with the cell -> dof map and constraints of a basis manager.
// cellDofIds / numCellDofs are what FEBasisManager::locallyOwnedCellLocalDofIdsBegin
// and nLocallyOwnedCellDofs return; the constraint arrays are the CSR arrays of
// ConstraintsInternal (basis/ConstraintsInternal.h).
class GpuFEContext {
 public:
  GpuFEContext(int device, const std::vector<uint32_t> &numCellDofs, const std::vector<uint32_t> &cellDofIds,
               uint64_t nDofs, const std::vector<uint32_t> &rowIds, const std::vector<uint32_t> &rowSizes,
               const std::vector<uint32_t> &colIds, const std::vector<uint32_t> &rowAcc,
               const std::vector<double> &colValues, const std::vector<double> &inhomogeneities) {
    gbfeCheck(nullptr, gbfe_ctx_create(device, &ctx), "ctx_create");
    gbfeCheck(ctx, gbfe_mesh_upload(ctx, (uint32_t)numCellDofs.size(), numCellDofs.data(), cellDofIds.data(), nDofs,
                                    &mesh),
              "mesh_upload");
    gbfeCheck(ctx, gbfe_constraints_upload(mesh, (uint32_t)rowIds.size(), rowIds.data(), rowSizes.data(),
                                           colIds.data(), rowAcc.data(), colValues.data(), inhomogeneities.data(),
                                           &cons),
              "constraints_upload");
  }
  ~GpuFEContext() {
    gbfe_constraints_destroy(cons);
    gbfe_mesh_destroy(mesh);
    gbfe_ctx_destroy(ctx);
  }
  GpuFEContext(const GpuFEContext &) = delete;
  GpuFEContext &operator=(const GpuFEContext &) = delete;

  gbfe_ctx *ctx = nullptr;
  gbfe_mesh *mesh = nullptr;
  gbfe_cons *cons = nullptr;
};

template <typename ValueTypeOperator, typename ValueTypeOperand, utils::MemorySpace memorySpace>
class GpuOperatorContextBase
    : public linearAlgebra::OperatorContext<ValueTypeOperator, ValueTypeOperand, memorySpace> {
  static_assert(std::is_same<ValueTypeOperand, double>::value || std::is_same<ValueTypeOperand, float>::value,
                "libgbfe block vectors are double (FP64 path) or float (mixed path)");

 public:
  using ValueType = linearAlgebra::blasLapack::scalar_type<ValueTypeOperator, ValueTypeOperand>;

  void apply(linearAlgebra::MultiVector<ValueTypeOperand, memorySpace> &X,
             linearAlgebra::MultiVector<ValueType, memorySpace> &Y, bool /*updateGhostX*/ = false,
             bool /*updateGhostY*/ = false) const override {
    const uint32_t m = (uint32_t)X.getNumberComponents();
    const int dt = std::is_same<ValueTypeOperand, double>::value ? GBFE_F64 : GBFE_F32;
    gbfe_mv *x = nullptr, *y = nullptr;
    if (memorySpace == utils::MemorySpace::DEVICE) {
      gbfeCheck(d_fe->ctx, gbfe_mv_wrap(d_fe->mesh, m, dt, (void *)X.data(), &x), "mv_wrap");
      gbfeCheck(d_fe->ctx, gbfe_mv_wrap(d_fe->mesh, m, dt, (void *)Y.data(), &y), "mv_wrap");
      const int rc = gbfe_apply(d_op, x, y);
      gbfe_mv_destroy(x);
      gbfe_mv_destroy(y);
      gbfeCheck(d_fe->ctx, rc, "apply");
    } else {
      gbfeCheck(d_fe->ctx, gbfe_mv_create(d_fe->mesh, m, dt, &x), "mv_create");
      gbfeCheck(d_fe->ctx, gbfe_mv_create(d_fe->mesh, m, dt, &y), "mv_create");
      int rc = gbfe_mv_copy_in(x, X.data());
      if (rc == GBFE_OK) rc = gbfe_apply(d_op, x, y);
      if (rc == GBFE_OK) rc = gbfe_mv_copy_out(y, Y.data());
      if (rc == GBFE_OK) rc = gbfe_mv_copy_out(x, X.data());  // constraints modified X
      gbfe_mv_destroy(x);
      gbfe_mv_destroy(y);
      gbfeCheck(d_fe->ctx, rc, "apply");
    }
  }

  ~GpuOperatorContextBase() { gbfe_op_destroy(d_op); }

 protected:
  std::shared_ptr<GpuFEContext> d_fe;
  gbfe_op *d_op = nullptr;
};

// Cell-matrix operator (H, consistent M, or K): cellMatrices is the reference's
// d_hamiltonianInAllCells layout (column-major nd_c x nd_c, cells concatenated).
template <typename ValueTypeOperator, typename ValueTypeOperand, utils::MemorySpace memorySpace>
class GpuCellOperatorContext : public GpuOperatorContextBase<ValueTypeOperator, ValueTypeOperand, memorySpace> {
 public:
  GpuCellOperatorContext(std::shared_ptr<GpuFEContext> fe, const std::vector<double> &cellMatrices,
                         bool mixedPrecision = false) {
    this->d_fe = fe;
    gbfeCheck(fe->ctx,
              gbfe_cellmat_upload(fe->mesh, fe->cons, cellMatrices.data(),
                                  GBFE_PREC_FP64 | (mixedPrecision ? GBFE_PREC_MIXED : 0), &this->d_op),
              "cellmat_upload");
  }
};

// Diagonal operator with constraints (GLL-lumped M^-1: pass the inverted diagonal).
template <typename ValueTypeOperator, typename ValueTypeOperand, utils::MemorySpace memorySpace>
class GpuDiagonalOperatorContext : public GpuOperatorContextBase<ValueTypeOperator, ValueTypeOperand, memorySpace> {
 public:
  GpuDiagonalOperatorContext(std::shared_ptr<GpuFEContext> fe, const std::vector<double> &diagonal) {
    this->d_fe = fe;
    gbfeCheck(fe->ctx, gbfe_diag_upload(fe->mesh, fe->cons, diagonal.data(), &this->d_op), "diag_upload");
  }
};

}  // namespace gb300
}  // namespace dftefe
