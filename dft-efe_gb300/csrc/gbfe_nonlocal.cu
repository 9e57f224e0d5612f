// gbfe_nonlocal.cu -- the separable nonlocal pseudopotential part
//   Y = P_c^T (sum_c G_c^T C_c^T) V (sum_c C_c G_c) P_c X
// of basis/AtomCenterNonLocalOpContextFE.t.cpp:715-849 (standalone apply) and
// its fused form inside the Kohn-Sham apply
// (ksdft/KohnShamOperatorContextFE.t.cpp:1022-1080 and :1177-1180).
//
// C_c is the reference's d_cellWiseC block of cell c: np_c x nd_c,
// column-major (projector index fastest), C_c(b, i) = int p_b N_i
// (AtomCenterNonLocalOpContextFE.t.cpp:438-499).  Three kernels:
//   k_nl_project: CXc[s][v] = sum_i C_c(b, i) X[ids_c[i]][v]   (s = slot of (c, b));
//                 the reference's cellWiseGEMM with transB = 'C' (:43-152)
//   k_nl_reduce : W[p][v] = V[p] * sum_{s in slots(p)} CXc[s][v], slots in
//                 cell order -- the serial scatter of addCellWiseDataToFieldData
//                 into d_CX followed by the diagonal scale applyVOnCconjtransX
//                 (:957-988); fixed order, no atomics
//   k_nl_add    : Yc[off_c + i][v] += sum_b C_c(b, i) W[pid(c, b)][v]: the
//                 beta = 1 cellWiseGEMM of applyCOnVCconjtransX (:990-1045) that
//                 adds the nonlocal block into the cell-wise result before the
//                 dof-owned assembly.
// Only cells with projectors launch work.  The FP32 copies serve the
// mixed-precision apply (FP32 cell buffer).
#include "gbfe_internal.cuh"

#include <algorithm>
#include <vector>

using namespace gbfe;

namespace {

constexpr uint32_t NL_THREADS = 128;
constexpr size_t NL_SMEM = 96 * 1024;

template <class T>
__global__ void __launch_bounds__(NL_THREADS)
    k_nl_project(const T *__restrict__ X, uint32_t m, const uint32_t *__restrict__ ids,
                 const uint32_t *__restrict__ cell_off, const uint32_t *__restrict__ cells,
                 const uint32_t *__restrict__ slot_off, const uint64_t *__restrict__ c_off,
                 const T *__restrict__ cmat, uint32_t mt, T *__restrict__ CX) {
  extern __shared__ unsigned char nl_smem[];
  T *Xs = reinterpret_cast<T *>(nl_smem);
  const uint32_t b = blockIdx.x;
  const uint32_t c = cells[b];
  const uint32_t off = cell_off[c], nd = cell_off[c + 1] - off;
  const uint32_t s0 = slot_off[b], np = slot_off[b + 1] - s0;
  const uint32_t v0 = blockIdx.y * mt;
  const uint32_t mv = min(mt, m - v0);
  for (uint32_t idx = threadIdx.x; idx < nd * mv; idx += blockDim.x) {
    const uint32_t a = idx / mv, v = idx - a * mv;
    Xs[a * mt + v] = X[(uint64_t)ids[off + a] * m + v0 + v];
  }
  __syncthreads();
  const T *Cc = cmat + c_off[b];
  for (uint32_t t = threadIdx.x; t < np * mv; t += blockDim.x) {
    const uint32_t beta = t / mv, v = t - beta * mv;
    T acc = T(0);
    for (uint32_t i = 0; i < nd; ++i) acc = fma(Cc[beta + (uint64_t)np * i], Xs[i * mt + v], acc);
    CX[(uint64_t)(s0 + beta) * m + v0 + v] = acc;
  }
}

template <class T>
__global__ void k_nl_reduce(const T *__restrict__ CX, uint32_t m, uint32_t n_proj,
                            const uint32_t *__restrict__ pslot_ptr, const uint32_t *__restrict__ pslot,
                            const T *__restrict__ V, T *__restrict__ W) {
  const uint64_t total = (uint64_t)n_proj * m;
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
       t += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t p = (uint32_t)(t / m), v = (uint32_t)(t - (uint64_t)p * m);
    T acc = T(0);
    for (uint32_t q = pslot_ptr[p], e = pslot_ptr[p + 1]; q < e; ++q) acc = acc + CX[(uint64_t)pslot[q] * m + v];
    W[t] = V[p] * acc;
  }
}

template <class T>
__global__ void __launch_bounds__(NL_THREADS)
    k_nl_add(T *__restrict__ Yc, uint32_t m, const uint32_t *__restrict__ cell_off,
             const uint32_t *__restrict__ cells, const uint32_t *__restrict__ slot_off,
             const uint32_t *__restrict__ pids, const uint64_t *__restrict__ c_off, const T *__restrict__ cmat,
             const T *__restrict__ W, uint32_t mt) {
  extern __shared__ unsigned char nl_smem[];
  T *Ws = reinterpret_cast<T *>(nl_smem);
  const uint32_t b = blockIdx.x;
  const uint32_t c = cells[b];
  const uint32_t off = cell_off[c], nd = cell_off[c + 1] - off;
  const uint32_t s0 = slot_off[b], np = slot_off[b + 1] - s0;
  const uint32_t v0 = blockIdx.y * mt;
  const uint32_t mv = min(mt, m - v0);
  for (uint32_t idx = threadIdx.x; idx < np * mv; idx += blockDim.x) {
    const uint32_t beta = idx / mv, v = idx - beta * mv;
    Ws[beta * mt + v] = W[(uint64_t)pids[s0 + beta] * m + v0 + v];
  }
  __syncthreads();
  const T *Cc = cmat + c_off[b];
  for (uint32_t t = threadIdx.x; t < nd * mv; t += blockDim.x) {
    const uint32_t i = t / mv, v = t - i * mv;
    T acc = T(0);
    for (uint32_t beta = 0; beta < np; ++beta) acc = fma(Cc[beta + (uint64_t)np * i], Ws[beta * mt + v], acc);
    T *y = Yc + (uint64_t)(off + i) * m + v0 + v;
    *y = *y + acc;
  }
}

template <class T>
void set_smem_attr_once(int device) {
  static PerDeviceOnce once;
  once.run(device, [] {
    GBFE_CUDA(cudaFuncSetAttribute(k_nl_project<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)NL_SMEM));
    GBFE_CUDA(cudaFuncSetAttribute(k_nl_add<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)NL_SMEM));
  });
}

// vectors per CTA: the gathered tile (nd x mt or np x mt) must fit NL_SMEM
uint32_t nl_tile(const gbfe_nl *nl, uint32_t m, size_t elem) {
  const uint32_t rows = std::max(nl->mesh->nd_max, nl->np_max);
  uint32_t mt = (uint32_t)std::min<size_t>(std::min<uint32_t>(m, 64), NL_SMEM / (elem * rows));
  GBFE_REQUIRE(mt > 0, "nonlocal: cell too large for one shared-memory tile");
  const uint32_t vt = (m + mt - 1) / mt;
  return (m + vt - 1) / vt;
}

template <class T>
void project_t(const gbfe_nl *nl, const T *X, uint32_t m, T *CX, T *W, const T *cm, const T *V) {
  gbfe_mesh *me = nl->mesh;
  gbfe_ctx *ctx = me->ctx;
  set_smem_attr_once<T>(ctx->device);
  const uint32_t mt = nl_tile(nl, m, sizeof(T));
  const dim3 grid(nl->n_cells_nl, (m + mt - 1) / mt);
  {
    ProfScope prof(ctx, "nonlocal_project", 2.0 * m * (double)nl->cmat.n, (double)sizeof(T) * nl->cmat.n);
    k_nl_project<T><<<grid, NL_THREADS, sizeof(T) * (size_t)me->nd_max * mt, ctx->stream>>>(
        X, m, me->ids.p, me->cell_off.p, nl->cells.p, nl->slot_off.p, nl->c_off.p, cm, mt, CX);
    check_launch(ctx, "nonlocal_project");
  }
  const uint64_t n = (uint64_t)nl->n_proj * m;
  k_nl_reduce<T><<<grid_for(n, 256), 256, 0, ctx->stream>>>(CX, m, nl->n_proj, nl->pslot_ptr.p, nl->pslot.p, V, W);
  check_launch(ctx, "nonlocal_reduce");
}

template <class T>
void add_t(const gbfe_nl *nl, uint32_t m, T *Yc, const T *cm, const T *W) {
  gbfe_mesh *me = nl->mesh;
  gbfe_ctx *ctx = me->ctx;
  set_smem_attr_once<T>(ctx->device);
  const uint32_t mt = nl_tile(nl, m, sizeof(T));
  const dim3 grid(nl->n_cells_nl, (m + mt - 1) / mt);
  ProfScope prof(ctx, "nonlocal_add", 2.0 * m * (double)nl->cmat.n, (double)sizeof(T) * nl->cmat.n);
  k_nl_add<T><<<grid, NL_THREADS, sizeof(T) * (size_t)nl->np_max * mt, ctx->stream>>>(
      Yc, m, me->cell_off.p, nl->cells.p, nl->slot_off.p, nl->pids.p, nl->c_off.p, cm, W, mt);
  check_launch(ctx, "nonlocal_add");
}

}  // namespace

namespace gbfe {

void nonlocal_project(const gbfe_nl *nl, const gbfe_mv *X) {
  if (!nl->n_cells_nl || !X->m) return;
  const uint32_t m = X->m;
  if (X->dtype == GBFE_F64) {
    nl->cx.ensure((size_t)nl->n_slots * m);
    nl->w.ensure((size_t)nl->n_proj * m);
    project_t<double>(nl, X->d.p, m, nl->cx.p, nl->w.p, nl->cmat.p, nl->v.p);
  } else {
    nl->cx_f32.ensure((size_t)nl->n_slots * m);
    nl->w_f32.ensure((size_t)nl->n_proj * m);
    project_t<float>(nl, X->f.p, m, nl->cx_f32.p, nl->w_f32.p, nl->cmat_f32.p, nl->v_f32.p);
  }
}

// W must come from nonlocal_project of the same X (same precision and m)
void nonlocal_add(const gbfe_nl *nl, uint32_t m, int dtype, void *Yc) {
  if (!nl->n_cells_nl || !m) return;
  const size_t need = (size_t)nl->n_proj * m;
  if (dtype == GBFE_F64) {
    GBFE_REQUIRE(nl->w.p && nl->w.n >= need, "nonlocal: add without a projection of this block");
    add_t<double>(nl, m, static_cast<double *>(Yc), nl->cmat.p, nl->w.p);
  } else {
    GBFE_REQUIRE(nl->w_f32.p && nl->w_f32.n >= need, "nonlocal: add without a projection of this block");
    add_t<float>(nl, m, static_cast<float *>(Yc), nl->cmat_f32.p, nl->w_f32.p);
  }
}

}  // namespace gbfe

namespace {
__global__ void k_d2f(const double *__restrict__ s, float *__restrict__ d, uint64_t n) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x)
    d[t] = (float)s[t];
}
}  // namespace

extern "C" {

int gbfe_nonlocal_upload(gbfe_mesh *mesh, uint32_t n_proj, const uint32_t *proj_per_cell, const uint32_t *proj_ids,
                         const double *cell_c, const double *coupling, gbfe_nl **out) {
  if (!mesh || !proj_per_cell || !out || (n_proj && !coupling)) return GBFE_ERR_ARG;
  gbfe_ctx *ctx = mesh->ctx;
  *out = nullptr;
  return gbfe_guard(ctx, [&] {
    auto nl = std::make_unique<gbfe_nl>();
    nl->mesh = mesh;
    nl->n_proj = n_proj;
    const uint32_t C = mesh->n_cells;
    std::vector<uint32_t> cells, slot_off{0}, pids;
    std::vector<uint64_t> c_off;
    std::vector<double> cm;
    std::vector<uint32_t> count(n_proj + 1, 0);
    uint64_t src_c = 0, src_s = 0;
    for (uint32_t c = 0; c < C; ++c) {
      const uint32_t np = proj_per_cell[c], nd = mesh->h_nd[c];
      if (np) {
        GBFE_REQUIRE(proj_ids && cell_c, "nonlocal_upload: projector ids and cell matrices are required");
        cells.push_back(c);
        c_off.push_back(cm.size());
        cm.insert(cm.end(), cell_c + src_c, cell_c + src_c + (uint64_t)np * nd);
        for (uint32_t b = 0; b < np; ++b) {
          const uint32_t p = proj_ids[src_s + b];
          GBFE_REQUIRE(p < n_proj, "nonlocal_upload: projector id out of range");
          pids.push_back(p);
          ++count[p + 1];
        }
        slot_off.push_back((uint32_t)pids.size());
        nl->np_max = std::max(nl->np_max, np);
      }
      src_c += (uint64_t)np * nd;
      src_s += np;
    }
    nl->n_cells_nl = (uint32_t)cells.size();
    nl->n_slots = (uint32_t)pids.size();
    // projector -> slots, ascending slot (= cell) order
    for (uint32_t p = 0; p < n_proj; ++p) count[p + 1] += count[p];
    std::vector<uint32_t> pslot(pids.size()), fill(count.begin(), count.end() - 1);
    for (uint32_t s = 0; s < pids.size(); ++s) pslot[fill[pids[s]]++] = s;
    std::vector<float> vf(coupling ? coupling : (const double *)nullptr,
                          coupling ? coupling + n_proj : (const double *)nullptr);
    cudaStream_t st = ctx->stream;
    if (nl->n_cells_nl) {
      nl->cells.upload(cells.data(), cells.size(), st);
      nl->slot_off.upload(slot_off.data(), slot_off.size(), st);
      nl->c_off.upload(c_off.data(), c_off.size(), st);
      nl->pids.upload(pids.data(), pids.size(), st);
      nl->pslot.upload(pslot.data(), pslot.size(), st);
      nl->cmat.upload(cm.data(), cm.size(), st);
      nl->cmat_f32.alloc(cm.size());
      k_d2f<<<grid_for(cm.size(), 256), 256, 0, st>>>(nl->cmat.p, nl->cmat_f32.p, cm.size());
      check_launch(ctx, "nonlocal_f32");
    }
    if (n_proj) {
      nl->pslot_ptr.upload(count.data(), count.size(), st);
      nl->v.upload(coupling, n_proj, st);
      nl->v_f32.upload(vf.data(), vf.size(), st);
    }
    GBFE_CUDA(cudaStreamSynchronize(st));
    *out = nl.release();
  });
}

int gbfe_nonlocal_destroy(gbfe_nl *nl) {
  if (!nl) return GBFE_OK;
  cudaStreamSynchronize(nl->mesh->ctx->stream);  // no launch of the context still reads its arrays
  delete nl;
  return GBFE_OK;
}

int gbfe_op_attach_nonlocal(gbfe_op *op, const gbfe_nl *nl) {
  if (!op) return GBFE_ERR_ARG;
  return gbfe_guard(op->mesh->ctx, [&] {
    GBFE_REQUIRE(op->kind == OP_CELL, "attach_nonlocal: needs a cell-matrix operator");
    GBFE_REQUIRE(!nl || nl->mesh == op->mesh, "attach_nonlocal: projectors belong to a different mesh");
    op->nl = nl;
  });
}

int gbfe_nonlocal_apply(const gbfe_nl *nl, const gbfe_cons *cons, gbfe_mv *X, gbfe_mv *Y) {
  if (!nl || !X || !Y) return GBFE_ERR_ARG;
  gbfe_mesh *me = nl->mesh;
  gbfe_ctx *ctx = me->ctx;
  return gbfe_guard(ctx, [&] {
    GBFE_REQUIRE(X->mesh == me && Y->mesh == me, "nonlocal_apply: vectors belong to a different mesh");
    GBFE_REQUIRE(X->m == Y->m && X->dtype == Y->dtype && X != Y, "nonlocal_apply: X and Y do not match");
    GBFE_REQUIRE(!cons || cons->mesh == me, "nonlocal_apply: constraints belong to a different mesh");
    const uint32_t m = X->m;
    if (!m) return;
    constraints_p2c(ctx, cons, X);
    nonlocal_project(nl, X);
    // cell-wise result: zero, plus the nonlocal block of the cells with projectors
    void *Yc;
    const size_t nc = (size_t)me->total_cell_dofs * m;
    if (X->dtype == GBFE_F64) {
      nl->ycell.ensure(nc);
      Yc = nl->ycell.p;
      GBFE_CUDA(cudaMemsetAsync(Yc, 0, nc * sizeof(double), ctx->stream));
    } else {
      nl->ycell_f32.ensure(nc);
      Yc = nl->ycell_f32.p;
      GBFE_CUDA(cudaMemsetAsync(Yc, 0, nc * sizeof(float), ctx->stream));
    }
    nonlocal_add(nl, m, X->dtype, Yc);
    assemble_cells(me, cons, X->dtype, Yc, Y);
  });
}

}  // extern "C"
