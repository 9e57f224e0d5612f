// gbfe_core.cu -- handles, uploads and the FP64 cellwise operator apply.
//
// The apply Y = P^T (sum_c G_c^T A_c G_c) P X of
// ksdft/KohnShamOperatorContextFE.t.cpp:1326-1443 runs as three kernels on
// the context's stream:
//   1. k_p2c            X[r] = inh_r + sum_j w_rj X[c_j]        (constraint rows)
//   2. k_cell_apply_f64 per cell: gather X[ids] into shared memory, then
//                       Yc = A_c^T Xc (the reference's column-major
//                       C(m x nd) = Xc(m x nd) * A_c(nd x nd)), written to a
//                       cell-wise scratch buffer
//   3. k_assemble       per dof: sum of its cell slots in ascending cell order,
//                       plus w * (row sum) for every constraint row that names
//                       it as a parent (distributeChildToParent), rows -> 0.
// No float atomics anywhere: every output element has exactly one writer and a
// fixed summation order, so results are bitwise reproducible run to run.
#include "gbfe_internal.cuh"
#include "gbfe_tc_ptx.cuh"

#include <algorithm>
#include <cstring>
#include <numeric>
#include <cstdlib>

using namespace gbfe;

namespace {

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
// Check of the bounded-wait path of the tensor-core kernels: one thread waits
// on an mbarrier that nothing arrives on, with the same wait routine and a
// caller-chosen time limit.  The wait gives up, writes GBFE_ERR_TIMEOUT into
// the status word, and the kernel returns; no copy or MMA is in flight, so
// the context stays usable.
__global__ void k_wait_unset_barrier(int *status, uint64_t max_ns) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) tc::mbar_init(&bar, 1);
  __syncthreads();
  if (threadIdx.x == 0) tc::mbar_wait_limited(&bar, 0, status, GBFE_ERR_TIMEOUT, tc::WAIT_LIMIT, max_ns);
}

template <class T>
__global__ void k_p2c(T *__restrict__ x, uint32_t m, uint32_t n_rows, const uint32_t *__restrict__ row_ids,
                      const uint32_t *__restrict__ row_sizes, const uint32_t *__restrict__ col_ids,
                      const uint32_t *__restrict__ row_acc, const double *__restrict__ col_vals,
                      const double *__restrict__ inh) {
  const uint64_t total = (uint64_t)n_rows * m;
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
       t += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t i = (uint32_t)(t / m), v = (uint32_t)(t - (uint64_t)i * m);
    T val = (T)inh[i];
    const uint32_t a = row_acc[i], s = row_sizes[i];
    for (uint32_t j = 0; j < s; ++j) val += (T)col_vals[a + j] * x[(uint64_t)col_ids[a + j] * m + v];
    x[(uint64_t)row_ids[i] * m + v] = val;
  }
}

// Constraint rows are zeroed and parents collect w * x[row] in row order.
template <class T>
__global__ void k_c2p_inplace(T *__restrict__ x, uint32_t m, uint64_t n_dofs, const uint32_t *__restrict__ par_ptr,
                              const uint32_t *__restrict__ par_row, const double *__restrict__ par_w) {
  const uint64_t total = n_dofs * m;
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
       t += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = t / m;
    const uint32_t v = (uint32_t)(t - i * m);
    const uint32_t b = par_ptr[i], e = par_ptr[i + 1];
    if (b == e) continue;
    T acc = x[t];
    for (uint32_t q = b; q < e; ++q) acc += (T)par_w[q] * x[(uint64_t)par_row[q] * m + v];
    x[t] = acc;
  }
}

template <class T>
__global__ void k_zero_rows(T *__restrict__ x, uint32_t m, uint32_t n_rows, const uint32_t *__restrict__ row_ids) {
  const uint64_t total = (uint64_t)n_rows * m;
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
       t += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t i = (uint32_t)(t / m), v = (uint32_t)(t - (uint64_t)i * m);
    x[(uint64_t)row_ids[i] * m + v] = (T)0;
  }
}

// FP64 cell product.  grid = (cells, vector tiles, row splits); block = 256.
// Shared memory: Xs[nd][mtc] for this cell's vector tile.
__global__ void __launch_bounds__(256) k_cell_apply_f64(
    const double *__restrict__ X, uint32_t m, const uint32_t *__restrict__ ids,
    const uint32_t *__restrict__ cell_off, const uint64_t *__restrict__ mat_off,
    const double *__restrict__ mats, double *__restrict__ Yc, uint32_t mt, uint32_t jsplit) {
  extern __shared__ double Xs[];
  const uint32_t c = blockIdx.x;
  const uint32_t v0 = blockIdx.y * mt;
  const uint32_t mtc = min(mt, m - v0);
  const uint32_t off = cell_off[c];
  const uint32_t nd = cell_off[c + 1] - off;
  const double *__restrict__ A = mats + mat_off[c];
  const uint32_t nin = nd * mtc;
  for (uint32_t idx = threadIdx.x; idx < nin; idx += blockDim.x) {
    const uint32_t k = idx / mtc, v = idx - k * mtc;
    Xs[idx] = X[(uint64_t)ids[off + k] * m + v0 + v];
  }
  __syncthreads();
  const uint32_t jper = (nd + jsplit - 1) / jsplit;
  const uint32_t j0 = blockIdx.z * jper;
  const uint32_t j1 = min(nd, j0 + jper);
  if (j0 >= j1) return;
  const uint32_t nout = (j1 - j0) * mtc;
  for (uint32_t o = threadIdx.x; o < nout; o += blockDim.x) {
    const uint32_t jj = o / mtc, v = o - jj * mtc;
    const uint32_t j = j0 + jj;
    const double *__restrict__ Aj = A + (uint64_t)nd * j;  // column j of A_c
    double acc0 = 0.0, acc1 = 0.0;
    uint32_t k = 0;
    for (; k + 1 < nd; k += 2) {
      acc0 = fma(__ldg(Aj + k), Xs[k * mtc + v], acc0);
      acc1 = fma(__ldg(Aj + k + 1), Xs[(k + 1) * mtc + v], acc1);
    }
    if (k < nd) acc0 = fma(__ldg(Aj + k), Xs[k * mtc + v], acc0);
    Yc[(uint64_t)(off + j) * m + v0 + v] = acc0 + acc1;
  }
}

// Assembly with the constraint epilogue fused in.  One thread per (dof, vec).
template <class TC, class TY>
__global__ void k_assemble(const TC *__restrict__ Yc, uint32_t m, uint64_t n_dofs,
                           const uint32_t *__restrict__ slot_ptr, const uint32_t *__restrict__ slot,
                           const uint8_t *__restrict__ is_row, const uint32_t *__restrict__ par_ptr,
                           const uint32_t *__restrict__ par_row, const double *__restrict__ par_w,
                           TY *__restrict__ Y, const FastDiv fm) {
  const uint64_t total = n_dofs * m;
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
       t += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t i;
    uint32_t v;
    fm.divmod(t, i, v);
    if (is_row && is_row[i]) {
      Y[t] = (TY)0;
      continue;
    }
    TY acc = (TY)0;
    for (uint32_t p = slot_ptr[i], e = slot_ptr[i + 1]; p < e; ++p) acc = acc + (TY)Yc[(uint64_t)slot[p] * m + v];
    if (par_ptr) {
      for (uint32_t q = par_ptr[i], qe = par_ptr[i + 1]; q < qe; ++q) {
        const uint32_t r = par_row[q];
        TY sr = (TY)0;
        for (uint32_t p = slot_ptr[r], e = slot_ptr[r + 1]; p < e; ++p) sr = sr + (TY)Yc[(uint64_t)slot[p] * m + v];
        acc += (TY)par_w[q] * sr;
      }
    }
    Y[t] = acc;
  }
}

// per-dof factor of B^-1 for folding into A (fused filter): d[i], 0 on
// homogeneous Dirichlet rows, 1 on the rows of the dense block (those rows
// are computed separately and substituted in the gather)
__global__ void k_fold_scale(const double *__restrict__ d, const uint8_t *__restrict__ is_row, uint64_t n,
                             uint64_t blk_begin, uint64_t blk_n, double *__restrict__ out) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = (is_row && is_row[i]) ? 0.0 : ((i - blk_begin) < blk_n ? 1.0 : d[i]);
}

// Assembly of a FP32 cell-wise result with one Chebyshev recurrence step fused
// in (homogeneous Dirichlet rows only): with S the assembled A B^-1 RN,
//   R = alpha1 S + (-c alpha1) RN + alpha2 R + (alpha1 eF2[j]) Y
// in the operation order of the separate step kernel.  The constrained rows of
// RN read as zero and are zeroed in place: the parent-to-child step that the
// separate B^-1 apply runs on its input (the cell product never sees those
// rows: their factor in the folded tiles is zero).
template <bool SH>
__global__ void k_assemble_cheb(const float *__restrict__ Yc, uint32_t m, uint64_t n_dofs,
                                const uint32_t *__restrict__ slot_ptr, const uint32_t *__restrict__ slot,
                                const uint8_t *__restrict__ is_row, const double *__restrict__ coef,
                                float *__restrict__ RN, float *__restrict__ R, const double *__restrict__ eF2,
                                const float *__restrict__ Y, const FastDiv fm) {
  extern __shared__ __align__(16) unsigned char col_sh[];
  float *g = reinterpret_cast<float *>(col_sh);
  const double alpha1 = coef[0], c = coef[1], alpha2 = coef[2];
  if (SH) {
    load_col_factors(g, m, alpha1, eF2);
    __syncthreads();
  }
  const float a1 = (float)alpha1, b1 = (float)(-c * alpha1), a2 = (float)alpha2;
  const uint64_t total = n_dofs * m;
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
       t += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t i;
    uint32_t v;
    fm.divmod(t, i, v);
    float acc = 0.f;
    const bool crow = is_row && is_row[i];
    if (!crow)
      for (uint32_t p = slot_ptr[i], e = slot_ptr[i + 1]; p < e; ++p) acc = acc + Yc[(uint64_t)slot[p] * m + v];
    const float s1 = a1 * acc + b1 * (crow ? 0.f : RN[t]);
    const float r = s1 + a2 * R[t];
    R[t] = r + (SH ? g[v] : (float)(alpha1 * eF2[v])) * Y[t];
    if (crow) RN[t] = 0.f;
  }
}

// k_assemble without hanging-node terms on 16-byte groups of W vectors
// (W = 4 floats or 2 doubles; m % W == 0): same sums in the same order
template <class T, int W>
__global__ void k_assemble_vec(const T *__restrict__ Yc, uint32_t m, uint64_t n_dofs,
                               const uint32_t *__restrict__ slot_ptr, const uint32_t *__restrict__ slot,
                               const uint8_t *__restrict__ is_row, T *__restrict__ Y, const FastDiv fq) {
  struct alignas(16) V {
    T x[W];
  };
  const uint32_t mw = m / W;
  const uint64_t total = n_dofs * mw;
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
       t += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t i;
    uint32_t q;
    fq.divmod(t, i, q);
    const uint32_t v = W * q;
    V acc;
#pragma unroll
    for (int w = 0; w < W; ++w) acc.x[w] = (T)0;
    const uint32_t p0 = slot_ptr[i], e = slot_ptr[i + 1];
    if (!(is_row && is_row[i]) && p0 < e) {
      // the first slot starts the sum (no add to zero: for FP64 blocks the
      // adds run on GB300's narrow FP64 pipe); slots in batches of four: the
      // indices, then the rows (four loads in flight), then the adds in slot order
      bool first = true;
      for (uint32_t p = p0; p < e; p += 4) {
        uint32_t sl[4];
        V y[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) sl[u] = p + u < e ? slot[p + u] : 0u;
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (p + u < e) y[u] = *reinterpret_cast<const V *>(Yc + (uint64_t)sl[u] * m + v);
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (p + u < e) {
            if (first) {
              acc = y[u];
              first = false;
            } else {
#pragma unroll
              for (int w = 0; w < W; ++w) acc.x[w] = acc.x[w] + y[u].x[w];
            }
          }
      }
    }
    *reinterpret_cast<V *>(Y + i * m + v) = acc;
  }
}

// k_assemble_cheb on float4 groups of vectors (m % 4 == 0): the same
// per-component arithmetic in the same order, a quarter of the load
// instructions and 16-byte transactions
template <bool SH>
__global__ void k_assemble_cheb4(const float *__restrict__ Yc, uint32_t m, uint64_t n_dofs,
                                 const uint32_t *__restrict__ slot_ptr, const uint32_t *__restrict__ slot,
                                 const uint8_t *__restrict__ is_row, const double *__restrict__ coef,
                                 float *__restrict__ RN, float *__restrict__ R, const double *__restrict__ eF2,
                                 const float *__restrict__ Y, const FastDiv fq) {
  extern __shared__ __align__(16) unsigned char col_sh[];
  float *g = reinterpret_cast<float *>(col_sh);
  const double alpha1 = coef[0], c = coef[1], alpha2 = coef[2];
  if (SH) {
    load_col_factors(g, m, alpha1, eF2);
    __syncthreads();
  }
  const float a1 = (float)alpha1, b1 = (float)(-c * alpha1), a2 = (float)alpha2;
  const uint32_t m4 = m / 4;
  const uint64_t total = n_dofs * m4;
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
       t += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t i;
    uint32_t q;
    fq.divmod(t, i, q);
    const uint32_t v = 4 * q;
    const uint64_t o = i * m + v;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    const bool crow = is_row && is_row[i];
    if (!crow)
      for (uint32_t p = slot_ptr[i], e = slot_ptr[i + 1]; p < e; ++p) {
        const float4 y = __ldg(reinterpret_cast<const float4 *>(Yc + (uint64_t)slot[p] * m + v));
        acc.x = acc.x + y.x;
        acc.y = acc.y + y.y;
        acc.z = acc.z + y.z;
        acc.w = acc.w + y.w;
      }
    const float4 rn = crow ? make_float4(0.f, 0.f, 0.f, 0.f) : *reinterpret_cast<const float4 *>(RN + o);
    const float4 r0 = *reinterpret_cast<const float4 *>(R + o);
    const float4 yy = *reinterpret_cast<const float4 *>(Y + o);
    const float4 gg = SH ? *reinterpret_cast<const float4 *>(g + v)
                         : make_float4((float)(alpha1 * eF2[v]), (float)(alpha1 * eF2[v + 1]),
                                       (float)(alpha1 * eF2[v + 2]), (float)(alpha1 * eF2[v + 3]));
    float4 out;
    out.x = (a1 * acc.x + b1 * rn.x + a2 * r0.x) + gg.x * yy.x;
    out.y = (a1 * acc.y + b1 * rn.y + a2 * r0.y) + gg.y * yy.y;
    out.z = (a1 * acc.z + b1 * rn.z + a2 * r0.z) + gg.z * yy.z;
    out.w = (a1 * acc.w + b1 * rn.w + a2 * r0.w) + gg.w * yy.w;
    *reinterpret_cast<float4 *>(R + o) = out;
    if (crow) *reinterpret_cast<float4 *>(RN + o) = make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

// Rows of a dense block times rows of X: out[r][v] = sum_j blk(r, j) X[bb + j][v]
// for r < nb (blk column-major nb x nb; out rows m apart), the j-sum in order
// with fused multiply-adds.  One launch for the small enrichment blocks
// (OrthoEFEOverlapInverseOpContextGLL's dense part) instead of a library GEMM
// that splits the K dimension over two launches.
constexpr uint32_t BLOCK_ROWS_MAX = 512;
template <class T>
__global__ void k_block_rows(const T *__restrict__ X, uint32_t m, uint64_t bb, uint32_t nb,
                             const T *__restrict__ blk, T *__restrict__ out) {
  const uint32_t r = blockIdx.x, v = blockIdx.y * blockDim.x + threadIdx.x;
  if (r >= nb || v >= m) return;
  T acc = (T)0;
  for (uint32_t j = 0; j < nb; ++j) acc = fma(blk[r + (uint64_t)j * nb], X[(bb + j) * m + v], acc);
  out[(uint64_t)r * m + v] = acc;
}

template <class T>
void block_rows(gbfe_ctx *ctx, const T *X, uint32_t m, uint64_t bb, uint32_t nb, const T *blk, T *out) {
  if (nb <= BLOCK_ROWS_MAX) {
    k_block_rows<T><<<dim3(nb, (m + 127) / 128), 128, 0, ctx->stream>>>(X, m, bb, nb, blk, out);
    check_launch(ctx, "block_rows");
    return;
  }
  const T one = (T)1, zero = (T)0;
  if constexpr (sizeof(T) == 8)
    GBFE_CUBLAS(cublasDgemm(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_T, (int)m, (int)nb, (int)nb, &one, X + bb * m, (int)m,
                            blk, (int)nb, &zero, out, (int)m));
  else
    GBFE_CUBLAS(cublasSgemm(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_T, (int)m, (int)nb, (int)nb, &one, X + bb * m, (int)m,
                            blk, (int)nb, &zero, out, (int)m));
  count_launch(ctx);
}

// Diagonal operator with the constraint epilogue fused in.
// (d in the vectors' precision: the FP32 path reads a float copy of the
// diagonal, no FP64 conversion per element)
template <class T>
__global__ void k_diag_apply(const T *__restrict__ X, uint32_t m, uint64_t n_dofs, const T *__restrict__ d,
                             const uint8_t *__restrict__ is_row, const uint32_t *__restrict__ par_ptr,
                             const uint32_t *__restrict__ par_row, const double *__restrict__ par_w,
                             T *__restrict__ Y, const FastDiv fm) {
  const uint64_t total = n_dofs * m;
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
       t += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t i;
    uint32_t v;
    fm.divmod(t, i, v);
    if (is_row && is_row[i]) {
      Y[t] = (T)0;
      continue;
    }
    T acc = d[i] * X[t];
    if (par_ptr) {
      for (uint32_t q = par_ptr[i], qe = par_ptr[i + 1]; q < qe; ++q) {
        const uint32_t r = par_row[q];
        acc += (T)par_w[q] * (d[r] * X[(uint64_t)r * m + v]);
      }
    }
    Y[t] = acc;
  }
}

template <class TS, class TD>
__global__ void k_convert(const TS *__restrict__ s, TD *__restrict__ d, uint64_t n) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x)
    d[t] = (TD)s[t];
}

template <class T>
__global__ void k_fill(T *__restrict__ d, uint64_t n, T v) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x)
    d[t] = v;
}

// FP64 FMA throughput probe: 8 independent dependency chains per thread
__global__ void k_dfma_probe(double *out, int iters, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

unsigned stride_grid(gbfe_ctx *ctx, uint64_t n, unsigned block = 256) {
  uint64_t g = (n + block - 1) / block;
  const uint64_t cap = (uint64_t)ctx->sm_count * 16;
  if (g > cap) g = cap;
  return (unsigned)(g ? g : 1);
}

}  // namespace

// ---------------------------------------------------------------------------
// internal API
// ---------------------------------------------------------------------------
namespace gbfe {

void constraints_p2c(gbfe_ctx *ctx, const gbfe_cons *c, gbfe_mv *x) {
  if (!c || c->n_rows == 0 || x->m == 0) return;
  ProfScope prof_k(ctx, "k:p2c", 0.0, 0.0);
  const uint64_t n = (uint64_t)c->n_rows * x->m;
  if (c->pure_dirichlet) {
    if (x->dtype == GBFE_F64)
      k_zero_rows<double><<<stride_grid(ctx, n), 256, 0, ctx->stream>>>(x->d.p, x->m, c->n_rows, c->row_ids.p);
    else
      k_zero_rows<float><<<stride_grid(ctx, n), 256, 0, ctx->stream>>>(x->f.p, x->m, c->n_rows, c->row_ids.p);
  } else {
    if (x->dtype == GBFE_F64)
      k_p2c<double><<<stride_grid(ctx, n), 256, 0, ctx->stream>>>(x->d.p, x->m, c->n_rows, c->row_ids.p,
                                                                   c->row_sizes.p, c->col_ids.p, c->row_acc.p,
                                                                   c->col_vals.p, c->inh.p);
    else
      k_p2c<float><<<stride_grid(ctx, n), 256, 0, ctx->stream>>>(x->f.p, x->m, c->n_rows, c->row_ids.p,
                                                                  c->row_sizes.p, c->col_ids.p, c->row_acc.p,
                                                                  c->col_vals.p, c->inh.p);
  }
  check_launch(ctx, "p2c");
}

static void constraints_c2p(gbfe_ctx *ctx, const gbfe_cons *c, gbfe_mv *x) {
  if (!c || c->n_rows == 0 || x->m == 0) return;
  const uint64_t n = x->count();
  if (!c->pure_dirichlet) {
    if (x->dtype == GBFE_F64)
      k_c2p_inplace<double><<<stride_grid(ctx, n), 256, 0, ctx->stream>>>(x->d.p, x->m, x->mesh->n_dofs,
                                                                           c->par_ptr.p, c->par_row.p, c->par_w.p);
    else
      k_c2p_inplace<float><<<stride_grid(ctx, n), 256, 0, ctx->stream>>>(x->f.p, x->m, x->mesh->n_dofs,
                                                                          c->par_ptr.p, c->par_row.p, c->par_w.p);
    check_launch(ctx, "c2p");
  }
  const uint64_t nr = (uint64_t)c->n_rows * x->m;
  if (x->dtype == GBFE_F64)
    k_zero_rows<double><<<stride_grid(ctx, nr), 256, 0, ctx->stream>>>(x->d.p, x->m, c->n_rows, c->row_ids.p);
  else
    k_zero_rows<float><<<stride_grid(ctx, nr), 256, 0, ctx->stream>>>(x->f.p, x->m, c->n_rows, c->row_ids.p);
  check_launch(ctx, "zero_rows");
}

static void cell_apply_f64(const gbfe_op *op, gbfe_mv *X, double *Yc) {
  gbfe_mesh *me = op->mesh;
  gbfe_ctx *ctx = me->ctx;
  const uint32_t m = X->m;
  const size_t smem_cap = 96 * 1024;
  uint32_t mt = (uint32_t)std::min<size_t>(m, smem_cap / (sizeof(double) * me->nd_max));
  if (mt == 0) throw Error(GBFE_ERR_ARG, "cell too large for the FP64 apply");
  const uint32_t vt = (m + mt - 1) / mt;
  mt = (m + vt - 1) / vt;  // balance vector tiles
  uint64_t base = (uint64_t)me->n_cells * vt;
  uint32_t jsplit = 1;
  const uint64_t target = (uint64_t)ctx->sm_count * 12;
  while (base * jsplit < target && jsplit * 8 < me->nd_min) jsplit *= 2;
  const size_t smem = sizeof(double) * (size_t)me->nd_max * mt;
  static PerDeviceOnce attr_once;
  attr_once.run(ctx->device, [&] {
    GBFE_CUDA(cudaFuncSetAttribute(k_cell_apply_f64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_cap));
  });
  dim3 grid(me->n_cells, vt, jsplit);
  ProfScope prof(ctx, "cell_apply_f64", 2.0 * m * (double)me->total_mat,
                 8.0 * (2.0 * (double)me->n_dofs * m + (double)me->total_mat));
  k_cell_apply_f64<<<grid, 256, smem, ctx->stream>>>(X->d.p, m, me->ids.p, me->cell_off.p, op_mat_off(op),
                                                     op->mats.p, Yc, mt, jsplit);
  check_launch(ctx, "cell_apply_f64");
}

// the FP64 cell product alone (no constraints, no assembly): the sliced
// tensor-core product when the operator carries the slices and the FP64 mode
// selects it, else the FP64 FMA kernel
void cell_product_f64(const gbfe_op *op, gbfe_mv *X, double *Yc) {
  GBFE_REQUIRE(X->mesh == op->mesh && X->dtype == GBFE_F64, "cell product: X must be FP64 on the operator's mesh");
  if (op->mesh->ctx->fp64_tc && op->oz_aoff.p)
    cell_apply_oz(op, X, Yc);
  else
    cell_apply_f64(op, X, Yc);
}

void apply_op(const gbfe_op *op, gbfe_mv *X, gbfe_mv *Y) {
  gbfe_mesh *me = op->mesh;
  gbfe_ctx *ctx = me->ctx;
  GBFE_REQUIRE(X->mesh == me && Y->mesh == me, "apply: vectors belong to a different mesh");
  GBFE_REQUIRE(X->m == Y->m, "apply: X and Y have different numbers of vectors");
  GBFE_REQUIRE(X->dtype == Y->dtype, "apply: X and Y have different precisions");
  GBFE_REQUIRE(X != Y, "apply: X and Y must be distinct");
  const uint32_t m = X->m;
  if (m == 0) return;
  const gbfe_cons *c = op->cons;
  const bool has_par = c && !c->pure_dirichlet;
  const uint64_t n = (uint64_t)me->n_dofs * m;

  if (op->kind == OP_JACOBI) {
    if (X->dtype == GBFE_F64)
      k_diag_apply<double><<<stride_grid(ctx, n), 256, 0, ctx->stream>>>(X->d.p, m, me->n_dofs, op->diag.p, nullptr,
                                                                         nullptr, nullptr, nullptr, Y->d.p, FastDiv(m));
    else
      k_diag_apply<float><<<stride_grid(ctx, n), 256, 0, ctx->stream>>>(X->f.p, m, me->n_dofs, op->diag_f32.p, nullptr,
                                                                        nullptr, nullptr, nullptr, Y->f.p, FastDiv(m));
    check_launch(ctx, "jacobi_apply");
    return;
  }
  constraints_p2c(ctx, c, X);
  if (op->kind == OP_DIAG_BLOCK) {
    // OrthoEFEOverlapInverseOpContextGLL.t.cpp:1182-1270: diagonal on every
    // dof, the enrichment rows replaced by block * X_enr, then child-to-parent
    if (X->dtype == GBFE_F64)
      k_diag_apply<double><<<stride_grid(ctx, n), 256, 0, ctx->stream>>>(X->d.p, m, me->n_dofs, op->diag.p, nullptr,
                                                                         nullptr, nullptr, nullptr, Y->d.p, FastDiv(m));
    else
      k_diag_apply<float><<<stride_grid(ctx, n), 256, 0, ctx->stream>>>(X->f.p, m, me->n_dofs, op->diag_f32.p, nullptr,
                                                                        nullptr, nullptr, nullptr, Y->f.p, FastDiv(m));
    check_launch(ctx, "diag_apply");
    if (X->dtype == GBFE_F64)
      block_rows<double>(ctx, X->d.p, m, op->blk_begin, (uint32_t)op->blk_n, op->blk.p, Y->d.p + op->blk_begin * m);
    else
      block_rows<float>(ctx, X->f.p, m, op->blk_begin, (uint32_t)op->blk_n, op->blk_f32.p,
                        Y->f.p + op->blk_begin * m);
    constraints_c2p(ctx, c, Y);
    return;
  }
  if (op->kind == OP_DIAG) {
    ProfScope prof_k(ctx, "k:diag_apply", 0.0, 0.0);
    const uint8_t *isr = c ? c->is_row.p : nullptr;
    if (X->dtype == GBFE_F64)
      k_diag_apply<double><<<stride_grid(ctx, n), 256, 0, ctx->stream>>>(
          X->d.p, m, me->n_dofs, op->diag.p, isr, has_par ? c->par_ptr.p : nullptr, has_par ? c->par_row.p : nullptr,
          has_par ? c->par_w.p : nullptr, Y->d.p, FastDiv(m));
    else
      k_diag_apply<float><<<stride_grid(ctx, n), 256, 0, ctx->stream>>>(
          X->f.p, m, me->n_dofs, op->diag_f32.p, isr, has_par ? c->par_ptr.p : nullptr, has_par ? c->par_row.p : nullptr,
          has_par ? c->par_w.p : nullptr, Y->f.p, FastDiv(m));
    check_launch(ctx, "diag_apply");
    return;
  }
  // cell operator; the nonlocal projection (if any) reads X after p2c and
  // is added into the cell-wise result before the assembly
  if (op->nl) nonlocal_project(op->nl, X);
  if (X->dtype == GBFE_F32) {
    apply_cell_mixed(op, X, Y);
    return;
  }
  op->cellbuf.ensure((size_t)me->total_cell_dofs * m);
  if (ctx->fp64_tc && op->oz_aoff.p)
    cell_apply_oz(op, X, op->cellbuf.p);
  else
    cell_apply_f64(op, X, op->cellbuf.p);
  if (op->nl) nonlocal_add(op->nl, m, GBFE_F64, op->cellbuf.p);
  assemble_cells(me, c, GBFE_F64, op->cellbuf.p, Y);
}

void apply_pair_f64(const gbfe_op *A, const gbfe_op *B, gbfe_mv *X, gbfe_mv *AX, gbfe_mv *BX) {
  gbfe_ctx *ctx = A->mesh->ctx;
  const bool pair = X->dtype == GBFE_F64 && A->kind == OP_CELL && B->kind == OP_CELL && A->mesh == B->mesh &&
                    X->mesh == A->mesh && A->cons == B->cons && !A->nl && !B->nl && ctx->fp64_tc &&
                    A->oz_aoff.p && B->oz_aoff.p && ctx->split_groups && !ctx->profiling && X->m > 0 &&
                    AX != BX && AX != X && BX != X && AX->m == X->m && BX->m == X->m &&
                    AX->dtype == GBFE_F64 && BX->dtype == GBFE_F64;
  if (!pair) {
    apply_op(B, X, BX);
    apply_op(A, X, AX);
    return;
  }
  gbfe_mesh *me = A->mesh;
  const uint32_t m = X->m;
  constraints_p2c(ctx, A->cons, X);  // once: both applies read the same constrained X
  const int *xexp = oz_column_exponents(A, X);
  ensure_side_stream(ctx);
  GBFE_CUDA(cudaEventRecord(ctx->fork_ev, ctx->stream));
  GBFE_CUDA(cudaStreamWaitEvent(ctx->side_stream, ctx->fork_ev, 0));
  B->cellbuf.ensure((size_t)me->total_cell_dofs * m);
  A->cellbuf.ensure((size_t)me->total_cell_dofs * m);
  cell_apply_oz(B, X, B->cellbuf.p, xexp, ctx->side_stream);
  assemble_cells(me, B->cons, GBFE_F64, B->cellbuf.p, BX, ctx->side_stream);
  cell_apply_oz(A, X, A->cellbuf.p, xexp, ctx->stream);
  assemble_cells(me, A->cons, GBFE_F64, A->cellbuf.p, AX, ctx->stream);
  GBFE_CUDA(cudaEventRecord(ctx->join_ev, ctx->side_stream));
  GBFE_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->join_ev, 0));
}

void h2d_staged(gbfe_ctx *ctx, PinnedSlot &slot, void *dst, const void *src, size_t n) {
  if (!n) return;
  if (slot.done) GBFE_CUDA(cudaEventSynchronize(slot.done));  // the previous staged copy has left
  if (slot.cap < n) {
    if (slot.h) GBFE_CUDA(cudaFreeHost(slot.h));
    slot.h = nullptr;
    GBFE_CUDA(cudaMallocHost(&slot.h, n));
    slot.cap = n;
  }
  if (!slot.done) GBFE_CUDA(cudaEventCreateWithFlags(&slot.done, cudaEventDisableTiming));
  std::memcpy(slot.h, src, n);
  GBFE_CUDA(cudaMemcpyAsync(dst, slot.h, n, cudaMemcpyHostToDevice, ctx->stream));
  GBFE_CUDA(cudaEventRecord(slot.done, ctx->stream));
}

void assemble_cells(gbfe_mesh *me, const gbfe_cons *c, int dtype, const void *Yc, gbfe_mv *Y, cudaStream_t stream) {
  gbfe_ctx *ctx = me->ctx;
  if (!stream) stream = ctx->stream;
  const bool has_par = c && !c->pure_dirichlet;
  const uint64_t n = (uint64_t)me->n_dofs * Y->m;
  const uint8_t *isr = c ? c->is_row.p : nullptr;
  if (!has_par && Y->m % (dtype == GBFE_F64 ? 2 : 4) == 0) {
    ProfScope prof_k(ctx, dtype == GBFE_F64 ? "k:assemble_f64" : "k:assemble_f32", 0.0, 0.0);
    if (dtype == GBFE_F64)
      k_assemble_vec<double, 2><<<stride_grid(ctx, n / 2), 256, 0, stream>>>(
          static_cast<const double *>(Yc), Y->m, me->n_dofs, me->slot_ptr.p, me->slot.p, isr, Y->d.p,
          FastDiv(Y->m / 2));
    else
      k_assemble_vec<float, 4><<<stride_grid(ctx, n / 4), 256, 0, stream>>>(
          static_cast<const float *>(Yc), Y->m, me->n_dofs, me->slot_ptr.p, me->slot.p, isr, Y->f.p,
          FastDiv(Y->m / 4));
    check_launch(ctx, "assemble_vec");
    return;
  }
  if (dtype == GBFE_F64) {
    {
      ProfScope prof_k(ctx, "k:assemble_f64", 0.0, 0.0);
      k_assemble<double, double><<<stride_grid(ctx, n), 256, 0, stream>>>(
          static_cast<const double *>(Yc), Y->m, me->n_dofs, me->slot_ptr.p, me->slot.p, isr,
          has_par ? c->par_ptr.p : nullptr, has_par ? c->par_row.p : nullptr, has_par ? c->par_w.p : nullptr, Y->d.p,
          FastDiv(Y->m));
      check_launch(ctx, "assemble_f64");
    }
  } else {
    {
      ProfScope prof_k(ctx, "k:assemble_f32", 0.0, 0.0);
      k_assemble<float, float><<<stride_grid(ctx, n), 256, 0, stream>>>(
          static_cast<const float *>(Yc), Y->m, me->n_dofs, me->slot_ptr.p, me->slot.p, isr,
          has_par ? c->par_ptr.p : nullptr, has_par ? c->par_row.p : nullptr, has_par ? c->par_w.p : nullptr, Y->f.p,
          FastDiv(Y->m));
      check_launch(ctx, "assemble_f32");
    }
  }
}

// assembly entry used by the mixed path (FP32 cell buffer -> FP32 Y), with
// the fused nonlocal block added first
void assemble_f32(const gbfe_op *op, float *Yc, gbfe_mv *Y) {
  if (op->nl) nonlocal_add(op->nl, Y->m, GBFE_F32, Yc);
  assemble_cells(op->mesh, op->cons, GBFE_F32, Yc, Y);
}

bool filter_step_fused(const gbfe_op *A, const gbfe_op *BInv, gbfe_mv *RN, gbfe_mv *R, const double *coef,
                       const double *eF2, const gbfe_mv *Y) {
  gbfe_mesh *me = A->mesh;
  gbfe_ctx *ctx = me->ctx;
  const gbfe_cons *c = BInv->cons;
  if (RN->dtype != GBFE_F32 || A->kind != OP_CELL || !(A->prec & GBFE_PREC_MIXED) || A->nl || !ctx->use_tc ||
      ctx->tc_version != 2 || !A->tc_aoff.p || (BInv->kind != OP_DIAG && BInv->kind != OP_DIAG_BLOCK) ||
      BInv->mesh != me || A->cons != c || (c && !c->pure_dirichlet) || RN->m == 0)
    return false;
  const uint32_t m = RN->m;
  if (!BInv->fold_scale.p) return false;  // built at upload for diagonal operators
  // BInv's parent-to-child on RN (zero rows) happens in the assembly kernel
  // below; before it only the dense block reads rows of RN, so it runs here
  // only when a constrained row lies inside the block
  if (BInv->blk_cons) constraints_p2c(ctx, c, RN);
  // fork point of the size groups that do not read the substituted rows
  // (they need not wait for the block rows below)
  const bool fork = ctx->split_groups && !ctx->profiling && ctx->side_stream;
  if (fork) GBFE_CUDA(cudaEventRecord(ctx->fork_ev, ctx->stream));
  const float *xsub = nullptr;
  if (BInv->kind == OP_DIAG_BLOCK) {
    // the enrichment rows of B^-1 RN: the dense block times those rows of RN,
    // the same product as the separate B^-1 apply
    BInv->blk_out_f32.ensure((size_t)BInv->blk_n * m);
    block_rows<float>(ctx, RN->f.p, m, BInv->blk_begin, (uint32_t)BInv->blk_n, BInv->blk_f32.p,
                      BInv->blk_out_f32.p);
    xsub = BInv->blk_out_f32.p;
  }
  if (A->folded_for != BInv->serial) {
    // A diag(B^-1 factor) in split tiles, built on the first fused step
    build_tc_mats_folded(A, BInv->fold_scale.p, A->mats_hi_folded);
    A->folded_for = BInv->serial;
  }
  A->cellbuf_f32.ensure((size_t)me->total_cell_dofs * m);
  cell_apply_tc(A, RN, A->cellbuf_f32.p, A->mats_hi_folded.p, xsub, (uint32_t)BInv->blk_begin,
                xsub ? (uint32_t)BInv->blk_n : 0u, fork);
  const uint64_t n = (uint64_t)me->n_dofs * m;
  {
    ProfScope prof_k(ctx, "k:assemble_cheb", 0.0, 0.0);
    const size_t sh = col_factor_smem<float>(m);
    const uint8_t *isr = c ? c->is_row.p : nullptr;
    if (m % 4 == 0)
      (sh ? k_assemble_cheb4<true> : k_assemble_cheb4<false>)<<<stride_grid(ctx, n / 4), 256, sh, ctx->stream>>>(
          A->cellbuf_f32.p, m, me->n_dofs, me->slot_ptr.p, me->slot.p, isr, coef, RN->f.p, R->f.p, eF2, Y->f.p,
          FastDiv(m / 4));
    else
      (sh ? k_assemble_cheb<true> : k_assemble_cheb<false>)<<<stride_grid(ctx, n), 256, sh, ctx->stream>>>(
          A->cellbuf_f32.p, m, me->n_dofs, me->slot_ptr.p, me->slot.p, isr, coef, RN->f.p, R->f.p, eF2, Y->f.p,
          FastDiv(m));
    check_launch(ctx, "assemble_cheb");
  }
  return true;
}

void convert_mv(gbfe_ctx *ctx, const gbfe_mv *src, gbfe_mv *dst) {
  const uint64_t n = src->count();
  if (src->dtype == dst->dtype) {
    GBFE_CUDA(cudaMemcpyAsync(dst->ptr(), src->ptr(), n * (src->dtype == GBFE_F64 ? 8 : 4),
                              cudaMemcpyDeviceToDevice, ctx->stream));
    return;
  }
  if (src->dtype == GBFE_F64)
    k_convert<double, float><<<stride_grid(ctx, n), 256, 0, ctx->stream>>>(src->d.p, dst->f.p, n);
  else
    k_convert<float, double><<<stride_grid(ctx, n), 256, 0, ctx->stream>>>(src->f.p, dst->d.p, n);
  check_launch(ctx, "convert");
}

void fill_mv(gbfe_ctx *ctx, gbfe_mv *x, double v) {
  const uint64_t n = x->count();
  if (!n) return;
  if (x->dtype == GBFE_F64)
    k_fill<double><<<stride_grid(ctx, n), 256, 0, ctx->stream>>>(x->d.p, n, v);
  else
    k_fill<float><<<stride_grid(ctx, n), 256, 0, ctx->stream>>>(x->f.p, n, (float)v);
  check_launch(ctx, "fill");
}

}  // namespace gbfe

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

int gbfe_ctx_create(int device, gbfe_ctx **out) {
  if (!out) return GBFE_ERR_ARG;
  *out = nullptr;
  gbfe_ctx *ctx = nullptr;
  try {
    ctx = new gbfe_ctx();
  } catch (...) {
    return GBFE_ERR_ALLOC;
  }
  int rc = gbfe_guard(ctx, [&] {
    int n = 0;
    GBFE_CUDA(cudaGetDeviceCount(&n));
    GBFE_REQUIRE(device >= 0 && device < n, "no such CUDA device");
    GBFE_CUDA(cudaSetDevice(device));
    int major = 0, minor = 0;
    GBFE_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device));
    GBFE_CUDA(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device));
    GBFE_REQUIRE(major == 10 && minor == 3, "libgbfe is built for sm_103a (GB300) only");
    ctx->device = device;
    ctx->cc_major = major;
    GBFE_CUDA(cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device));
    GBFE_CUDA(cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking));
    ctx->stream = ctx->own_stream;
    GBFE_CUBLAS(cublasCreate(&ctx->cublas));
    GBFE_CUBLAS(cublasSetStream(ctx->cublas, ctx->stream));
    GBFE_CUBLAS(cublasSetPointerMode(ctx->cublas, CUBLAS_POINTER_MODE_HOST));
    GBFE_CUSOLVER(cusolverDnCreate(&ctx->cusolver));
    GBFE_CUSOLVER(cusolverDnSetStream(ctx->cusolver, ctx->stream));
    ctx->status.alloc(4);
    GBFE_CUDA(cudaMemsetAsync(ctx->status.p, 0, 4 * sizeof(int), ctx->stream));
    if (const char *cache = getenv("GBFE_AUTOTUNE_CACHE")) {
      ctx->tune_cache = cache;
      FILE *f = fopen(cache, "r");
      if (f) {
        // "tc2 nd_max mtiles m N stages occupancy ms [tmem buffers [prefetch [swapped]]]"
        // (lines of other shapes are skipped)
        char line[256], kind[16];
        unsigned nd, mt, mm, N, st, occ, nbuf = 0, pf = 0, sw = 0;
        float ms;
        while (fgets(line, sizeof line, f)) {
          nbuf = 0;
          pf = 0;
          sw = 0;
          const int got = sscanf(line, "%15s %u %u %u %u %u %u %f %u %u %u", kind, &nd, &mt, &mm, &N, &st, &occ, &ms,
                                 &nbuf, &pf, &sw);
          if (got >= 8 && std::string(kind) == "tc2")
            ctx->tc_tune[std::make_tuple(nd, mt, mm)] = TcTune{
                N, st, ms, occ, got >= 9 ? nbuf : 0u, got >= 10 ? std::min(pf, 3u) : 0u, got >= 11 && sw ? 1u : 0u};
        }
        fclose(f);
      }
    }
    const char *tc = getenv("GBFE_TENSOR_CORES");
    if (tc && tc[0] == '0') ctx->use_tc = 0;
    if (tc && tc[0] == '1') ctx->tc_version = 1;
  });
  if (rc != GBFE_OK) {
    std::string msg = ctx->last_error;
    gbfe_ctx_destroy(ctx);
    fprintf(stderr, "gbfe_ctx_create: %s\n", msg.c_str());
    return rc;
  }
  *out = ctx;
  return GBFE_OK;
}

int gbfe_ctx_destroy(gbfe_ctx *ctx) {
  if (!ctx) return GBFE_OK;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  ctx->red.reset();
  ctx->small.reset();
  ctx->info.reset();
  ctx->lwork.reset();
  for (auto &kv : ctx->kstats)
    for (auto &pr : kv.second.pending) {
      cudaEventDestroy(pr.first);
      cudaEventDestroy(pr.second);
    }
  for (cudaEvent_t e : ctx->event_free) cudaEventDestroy(e);
  if (ctx->side_stream) {
    cudaStreamSynchronize(ctx->side_stream);
    cudaStreamDestroy(ctx->side_stream);
  }
  if (ctx->fork_ev) cudaEventDestroy(ctx->fork_ev);
  if (ctx->join_ev) cudaEventDestroy(ctx->join_ev);
  if (ctx->host_ev) cudaEventDestroy(ctx->host_ev);
  for (cudaGraphExec_t g : ctx->fw_exec_pool) cudaGraphExecDestroy(g);
  if (ctx->cusolver) cusolverDnDestroy(ctx->cusolver);
  if (ctx->cublas) cublasDestroy(ctx->cublas);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
  return GBFE_OK;
}

int gbfe_last_error(const gbfe_ctx *ctx, char *buf, size_t len) {
  if (!ctx || !buf || !len) return GBFE_ERR_ARG;
  snprintf(buf, len, "%s", ctx->last_error.c_str());
  return GBFE_OK;
}

int gbfe_ctx_set_stream(gbfe_ctx *ctx, void *stream) {
  if (!ctx) return GBFE_ERR_ARG;
  return gbfe_guard(ctx, [&] {
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
    GBFE_CUBLAS(cublasSetStream(ctx->cublas, ctx->stream));
    GBFE_CUSOLVER(cusolverDnSetStream(ctx->cusolver, ctx->stream));
  });
}

int gbfe_ctx_synchronize(gbfe_ctx *ctx) {
  if (!ctx) return GBFE_ERR_ARG;
  return gbfe_guard(ctx, [&] { GBFE_CUDA(cudaStreamSynchronize(ctx->stream)); });
}

int gbfe_ctx_check_status(gbfe_ctx *ctx) {
  if (!ctx) return GBFE_ERR_ARG;
  int st = 0;
  int rc = gbfe_guard(ctx, [&] {
    GBFE_CUDA(cudaMemcpyAsync(&st, ctx->status.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    GBFE_CUDA(cudaStreamSynchronize(ctx->stream));
    if (st != 0) {
      GBFE_CUDA(cudaMemsetAsync(ctx->status.p, 0, sizeof(int), ctx->stream));
      ctx->last_error = "a bounded device wait gave up (code " + std::to_string(st) + ")";
    }
  });
  if (rc != GBFE_OK) return rc;
  return st ? GBFE_ERR_TIMEOUT : GBFE_OK;
}

int gbfe_ctx_check_wait_timeout(gbfe_ctx *ctx, double limit_s) {
  if (!ctx || !(limit_s >= 0.0 && limit_s <= 1.0)) return GBFE_ERR_ARG;
  return gbfe_guard(ctx, [&] {
    k_wait_unset_barrier<<<1, 32, 0, ctx->stream>>>(ctx->status.p, (uint64_t)(limit_s * 1e9));
    check_launch(ctx, "wait_unset_barrier");
    GBFE_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

int gbfe_ctx_set_sm_budget(gbfe_ctx *ctx, int sms) {
  if (!ctx || sms < 0) return GBFE_ERR_ARG;
  return gbfe_guard(ctx, [&] {
    int dev_sms = 0;
    GBFE_CUDA(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, ctx->device));
    ctx->sm_count = (sms == 0 || sms > dev_sms) ? dev_sms : sms;
  });
}

int gbfe_ctx_set_split_groups(gbfe_ctx *ctx, int on) {
  if (!ctx) return GBFE_ERR_ARG;
  ctx->split_groups = on ? 1 : 0;
  return GBFE_OK;
}

int gbfe_ctx_set_tensor_cores(gbfe_ctx *ctx, int mode) {
  if (!ctx || mode < 0 || mode > 3) return GBFE_ERR_ARG;
  ctx->use_tc = mode ? 1 : 0;
  if (mode) ctx->tc_version = mode == 3 ? 2 : mode;
  ctx->tc_gather4 = mode == 3 ? 0 : 1;
  return GBFE_OK;
}

int gbfe_autotune(const gbfe_op *op, uint32_t m, char *report, size_t report_len) {
  if (!op) return GBFE_ERR_ARG;
  gbfe_ctx *ctx = op->mesh->ctx;
  return gbfe_guard(ctx, [&] {
    std::vector<std::string> log, fresh;
    autotune_tc(op, m, log, fresh);
    std::string all, add;
    for (auto &l : log) all += l + "\n";
    for (auto &l : fresh) add += l + "\n";
    if (report && report_len) snprintf(report, report_len, "%s", all.c_str());
    if (!ctx->tune_cache.empty() && !add.empty()) {
      FILE *f = fopen(ctx->tune_cache.c_str(), "a");
      if (f) {
        fputs(add.c_str(), f);
        fclose(f);
      }
    }
  });
}

int gbfe_ctx_set_graphs(gbfe_ctx *ctx, int on) {
  if (!ctx) return GBFE_ERR_ARG;
  ctx->use_graphs = on ? 1 : 0;
  return GBFE_OK;
}

int gbfe_ctx_set_profile_filter(gbfe_ctx *ctx, const char *names) {
  if (!ctx) return GBFE_ERR_ARG;
  ctx->prof_only.clear();
  if (names) {
    std::string all(names), cur;
    for (char ch : all) {
      if (ch == ',') {
        if (!cur.empty()) ctx->prof_only.push_back(cur);
        cur.clear();
      } else {
        cur += ch;
      }
    }
    if (!cur.empty()) ctx->prof_only.push_back(cur);
  }
  return GBFE_OK;
}

int gbfe_ctx_set_fused_filter(gbfe_ctx *ctx, int on) {
  if (!ctx || on < 0 || on > 1) return GBFE_ERR_ARG;
  ctx->fuse_filter = on;
  return GBFE_OK;
}

int gbfe_ctx_set_small_eig(gbfe_ctx *ctx, int mode) {
  if (!ctx || mode < 0 || mode > 1) return GBFE_ERR_ARG;
  ctx->small_eig_host = mode;
  return GBFE_OK;
}

int gbfe_ctx_set_fp64_apply(gbfe_ctx *ctx, int mode) {
  if (!ctx || mode < 0 || mode > 2) return GBFE_ERR_ARG;
  ctx->fp64_tc = mode ? 1 : 0;
  ctx->fp64_tc_dense = mode == 1 ? 1 : 0;
  return GBFE_OK;
}

int gbfe_ctx_kernel_launches(const gbfe_ctx *ctx, uint64_t *count) {
  if (!ctx || !count) return GBFE_ERR_ARG;
  *count = ctx->launches;
  return GBFE_OK;
}

int gbfe_ctx_set_profiling(gbfe_ctx *ctx, int on) {
  if (!ctx) return GBFE_ERR_ARG;
  ctx->profiling = on ? 1 : 0;
  return GBFE_OK;
}

int gbfe_ctx_kernel_stats(gbfe_ctx *ctx, const char *name, uint64_t *launches, double *total_ms, double *flops,
                          double *bytes) {
  if (!ctx || !name) return GBFE_ERR_ARG;
  return gbfe_guard(ctx, [&] {
    GBFE_CUDA(cudaStreamSynchronize(ctx->stream));
    auto it = ctx->kstats.find(name);
    KernelStat empty;
    KernelStat &st = it == ctx->kstats.end() ? empty : it->second;
    for (auto &pr : st.pending) {
      float ms = 0.f;
      GBFE_CUDA(cudaEventElapsedTime(&ms, pr.first, pr.second));
      st.ms += ms;
      ctx->event_free.push_back(pr.first);
      ctx->event_free.push_back(pr.second);
    }
    st.pending.clear();
    if (launches) *launches = st.launches;
    if (total_ms) *total_ms = st.ms;
    if (flops) *flops = st.flops;
    if (bytes) *bytes = st.bytes;
  });
}

int gbfe_ctx_reset_kernel_stats(gbfe_ctx *ctx) {
  if (!ctx) return GBFE_ERR_ARG;
  return gbfe_guard(ctx, [&] {
    GBFE_CUDA(cudaStreamSynchronize(ctx->stream));
    for (auto &kv : ctx->kstats)
      for (auto &pr : kv.second.pending) {
        ctx->event_free.push_back(pr.first);
        ctx->event_free.push_back(pr.second);
      }
    ctx->kstats.clear();
  });
}

int gbfe_probe_fp64_peak(gbfe_ctx *ctx, double *gflops) {
  if (!ctx || !gflops) return GBFE_ERR_ARG;
  return gbfe_guard(ctx, [&] {
    const int blocks = ctx->sm_count * 8, threads = 256, iters = 4096;
    DBuf<double> out;
    out.alloc((size_t)blocks * threads);
    cudaEvent_t e0, e1;
    GBFE_CUDA(cudaEventCreate(&e0));
    GBFE_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
      GBFE_CUDA(cudaEventRecord(e0, ctx->stream));
      k_dfma_probe<<<blocks, threads, 0, ctx->stream>>>(out.p, iters, 0.999, 1e-3);
      GBFE_CUDA(cudaEventRecord(e1, ctx->stream));
      GBFE_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      GBFE_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      best = std::min(best, ms);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *gflops = 2.0 * 8 * iters * (double)blocks * threads / (best * 1e6);
  });
}

int gbfe_mesh_upload(gbfe_ctx *ctx, uint32_t n_cells, const uint32_t *nd_per_cell, const uint32_t *cell_dof_ids,
                     uint64_t n_dofs, gbfe_mesh **out) {
  if (!ctx || !out) return GBFE_ERR_ARG;
  *out = nullptr;
  gbfe_mesh *me = nullptr;
  int rc = gbfe_guard(ctx, [&] {
    GBFE_REQUIRE(n_cells > 0 && nd_per_cell && cell_dof_ids && n_dofs > 0, "mesh_upload: empty mesh");
    GBFE_REQUIRE(n_dofs < 0xffffffffULL, "mesh_upload: n_dofs must fit in uint32 (size_type)");
    me = new gbfe_mesh();
    me->ctx = ctx;
    me->n_dofs = n_dofs;
    me->n_cells = n_cells;
    me->h_nd.assign(nd_per_cell, nd_per_cell + n_cells);
    me->h_cell_off.resize(n_cells + 1);
    me->h_mat_off.resize(n_cells + 1);
    me->h_cell_off[0] = 0;
    me->h_mat_off[0] = 0;
    uint64_t tot = 0, totm = 0;
    me->nd_max = 0;
    me->nd_min = 0xffffffffu;
    for (uint32_t c = 0; c < n_cells; ++c) {
      const uint32_t nd = nd_per_cell[c];
      GBFE_REQUIRE(nd > 0, "mesh_upload: cell with zero dofs");
      tot += nd;
      totm += (uint64_t)nd * nd;
      GBFE_REQUIRE(tot < 0xffffffffULL, "mesh_upload: too many cell dofs for uint32 offsets");
      me->h_cell_off[c + 1] = (uint32_t)tot;
      me->h_mat_off[c + 1] = totm;
      me->nd_max = std::max(me->nd_max, nd);
      me->nd_min = std::min(me->nd_min, nd);
    }
    me->total_cell_dofs = tot;
    me->total_mat = totm;
    // dof -> slots transpose (counting sort keeps ascending slot order)
    std::vector<uint32_t> cnt(n_dofs + 1, 0);
    for (uint64_t p = 0; p < tot; ++p) {
      const uint32_t g = cell_dof_ids[p];
      GBFE_REQUIRE(g < n_dofs, "mesh_upload: dof id out of range");
      cnt[g + 1]++;
    }
    for (uint64_t i = 0; i < n_dofs; ++i) cnt[i + 1] += cnt[i];
    std::vector<uint32_t> slot(tot), pos(cnt.begin(), cnt.end() - 1);
    for (uint64_t p = 0; p < tot; ++p) slot[pos[cell_dof_ids[p]]++] = (uint32_t)p;
    // size bins (distinct nd values), cells grouped by bin in ascending cell order
    std::vector<uint32_t> nds(me->h_nd);
    std::sort(nds.begin(), nds.end());
    nds.erase(std::unique(nds.begin(), nds.end()), nds.end());
    me->bin_nd = nds;
    std::vector<uint32_t> bcells;
    bcells.reserve(n_cells);
    for (uint32_t b = 0; b < nds.size(); ++b) {
      me->bin_begin.push_back((uint32_t)bcells.size());
      uint32_t mx = 0;
      for (uint32_t c = 0; c < n_cells; ++c)
        if (me->h_nd[c] == nds[b]) {
          bcells.push_back(c);
          for (uint32_t a = me->h_cell_off[c]; a < me->h_cell_off[c + 1]; ++a) mx = std::max(mx, cell_dof_ids[a]);
        }
      me->bin_max_id.push_back(mx);
    }
    me->bin_begin.push_back((uint32_t)bcells.size());
    cudaStream_t s = ctx->stream;
    me->ids.upload(cell_dof_ids, tot, s);
    me->nd.upload(nd_per_cell, n_cells, s);
    me->cell_off.upload(me->h_cell_off.data(), n_cells + 1, s);
    me->mat_off.upload(me->h_mat_off.data(), n_cells + 1, s);
    me->slot_ptr.upload(cnt.data(), n_dofs + 1, s);
    me->slot.upload(slot.data(), tot, s);
    me->bin_cells.upload(bcells.data(), bcells.size(), s);
    GBFE_CUDA(cudaStreamSynchronize(s));
  });
  if (rc != GBFE_OK) {
    delete me;
    return rc;
  }
  *out = me;
  return GBFE_OK;
}

int gbfe_mesh_destroy(gbfe_mesh *mesh) {
  if (!mesh) return GBFE_OK;
  cudaStreamSynchronize(mesh->ctx->stream);
  delete mesh;
  return GBFE_OK;
}

int gbfe_constraints_upload(gbfe_mesh *mesh, uint32_t n_rows, const uint32_t *row_ids, const uint32_t *row_sizes,
                            const uint32_t *col_ids, const uint32_t *row_acc, const double *col_values,
                            const double *inhomogeneities, gbfe_cons **out) {
  if (!mesh || !out) return GBFE_ERR_ARG;
  *out = nullptr;
  gbfe_ctx *ctx = mesh->ctx;
  gbfe_cons *c = nullptr;
  int rc = gbfe_guard(ctx, [&] {
    GBFE_REQUIRE(n_rows == 0 || (row_ids && row_sizes && row_acc && inhomogeneities),
                 "constraints_upload: null array");
    c = new gbfe_cons();
    c->mesh = mesh;
    c->n_rows = n_rows;
    const uint64_t N = mesh->n_dofs;
    std::vector<uint8_t> is_row(N, 0);
    uint64_t nnz = 0;
    for (uint32_t i = 0; i < n_rows; ++i) {
      GBFE_REQUIRE(row_ids[i] < N, "constraints_upload: row id out of range");
      GBFE_REQUIRE(!is_row[row_ids[i]], "constraints_upload: duplicate constraint row");
      is_row[row_ids[i]] = 1;
      nnz = std::max<uint64_t>(nnz, (uint64_t)row_acc[i] + row_sizes[i]);
      if (row_sizes[i] != 0 || inhomogeneities[i] != 0.0) c->pure_dirichlet = false;
    }
    GBFE_REQUIRE(nnz == 0 || (col_ids && col_values), "constraints_upload: null column arrays");
    c->nnz = nnz;
    // transpose: parent column -> (row dof, weight) in ascending constraint-row order
    std::vector<uint32_t> cnt(N + 1, 0);
    for (uint32_t i = 0; i < n_rows; ++i)
      for (uint32_t j = 0; j < row_sizes[i]; ++j) {
        const uint32_t col = col_ids[row_acc[i] + j];
        GBFE_REQUIRE(col < N, "constraints_upload: column id out of range");
        GBFE_REQUIRE(!is_row[col], "constraints_upload: constraints are not closed (a column is a constrained row)");
        cnt[col + 1]++;
      }
    for (uint64_t i = 0; i < N; ++i) cnt[i + 1] += cnt[i];
    const uint64_t tnnz = cnt[N];
    std::vector<uint32_t> prow(tnnz), pos(cnt.begin(), cnt.end() - 1);
    std::vector<double> pw(tnnz);
    for (uint32_t i = 0; i < n_rows; ++i)
      for (uint32_t j = 0; j < row_sizes[i]; ++j) {
        const uint32_t col = col_ids[row_acc[i] + j];
        const uint32_t q = pos[col]++;
        prow[q] = row_ids[i];
        pw[q] = col_values[row_acc[i] + j];
      }
    cudaStream_t s = ctx->stream;
    if (n_rows) {
      c->row_ids.upload(row_ids, n_rows, s);
      c->row_sizes.upload(row_sizes, n_rows, s);
      c->row_acc.upload(row_acc, n_rows, s);
      c->inh.upload(inhomogeneities, n_rows, s);
    }
    if (nnz) {
      c->col_ids.upload(col_ids, nnz, s);
      c->col_vals.upload(col_values, nnz, s);
    }
    c->is_row.upload(is_row.data(), N, s);
    if (!c->pure_dirichlet) {
      c->par_ptr.upload(cnt.data(), N + 1, s);
      if (tnnz) {
        c->par_row.upload(prow.data(), tnnz, s);
        c->par_w.upload(pw.data(), tnnz, s);
      } else {
        c->par_row.alloc(1);
        c->par_w.alloc(1);
      }
    }
    GBFE_CUDA(cudaStreamSynchronize(s));
  });
  if (rc != GBFE_OK) {
    delete c;
    return rc;
  }
  *out = c;
  return GBFE_OK;
}

int gbfe_constraints_destroy(gbfe_cons *cons) {
  if (!cons) return GBFE_OK;
  cudaStreamSynchronize(cons->mesh->ctx->stream);
  delete cons;
  return GBFE_OK;
}

int gbfe_constraints_distribute_parent_to_child(const gbfe_cons *cons, gbfe_mv *x) {
  if (!cons || !x) return GBFE_ERR_ARG;
  gbfe_ctx *ctx = cons->mesh->ctx;
  return gbfe_guard(ctx, [&] {
    GBFE_REQUIRE(x->mesh == cons->mesh, "p2c: vector on another mesh");
    constraints_p2c(ctx, cons, x);
  });
}

int gbfe_constraints_distribute_child_to_parent(const gbfe_cons *cons, gbfe_mv *x) {
  if (!cons || !x) return GBFE_ERR_ARG;
  gbfe_ctx *ctx = cons->mesh->ctx;
  return gbfe_guard(ctx, [&] {
    GBFE_REQUIRE(x->mesh == cons->mesh, "c2p: vector on another mesh");
    constraints_c2p(ctx, cons, x);
  });
}

int gbfe_cellmat_upload(gbfe_mesh *mesh, const gbfe_cons *cons, const double *mats, int prec_flags, gbfe_op **out) {
  if (!mesh || !out) return GBFE_ERR_ARG;
  *out = nullptr;
  gbfe_op *op = nullptr;
  int rc = gbfe_guard(mesh->ctx, [&] {
    GBFE_REQUIRE(mats, "cellmat_upload: null matrices");
    GBFE_REQUIRE(!cons || cons->mesh == mesh, "cellmat_upload: constraints on another mesh");
    op = new gbfe_op();
    op->mesh = mesh;
    op->cons = cons;
    op->kind = OP_CELL;
    op->prec = prec_flags | GBFE_PREC_FP64;
    op->mats_count = mesh->total_mat;
    op->mats.upload(mats, mesh->total_mat, mesh->ctx->stream);
    if (prec_flags & GBFE_PREC_MIXED) build_mixed_mats(op);
    if ((prec_flags & GBFE_PREC_FP64_TENSOR) && oz_supported(mesh)) build_oz_mats(op);
    GBFE_CUDA(cudaStreamSynchronize(mesh->ctx->stream));
  });
  if (rc != GBFE_OK) {
    delete op;
    return rc;
  }
  *out = op;
  return GBFE_OK;
}

int gbfe_cellmat_upload_indexed(gbfe_mesh *mesh, const gbfe_cons *cons, uint32_t n_mats, const double *mats,
                                const uint32_t *cell_to_mat, int prec_flags, gbfe_op **out) {
  if (!mesh || !out) return GBFE_ERR_ARG;
  *out = nullptr;
  gbfe_op *op = nullptr;
  int rc = gbfe_guard(mesh->ctx, [&] {
    GBFE_REQUIRE(mats && cell_to_mat && n_mats > 0, "cellmat_upload_indexed: null arrays");
    GBFE_REQUIRE(!cons || cons->mesh == mesh, "cellmat_upload_indexed: constraints on another mesh");
    // every cell that names matrix u must have the same nd; u's size is that nd^2
    std::vector<uint32_t> nd_of(n_mats, 0);
    for (uint32_t c = 0; c < mesh->n_cells; ++c) {
      const uint32_t u = cell_to_mat[c];
      GBFE_REQUIRE(u < n_mats, "cellmat_upload_indexed: matrix index out of range");
      GBFE_REQUIRE(nd_of[u] == 0 || nd_of[u] == mesh->h_nd[c],
                   "cellmat_upload_indexed: cells sharing a matrix have different sizes");
      nd_of[u] = mesh->h_nd[c];
    }
    std::vector<uint64_t> uoff(n_mats + 1, 0);
    for (uint32_t u = 0; u < n_mats; ++u) uoff[u + 1] = uoff[u] + (uint64_t)nd_of[u] * nd_of[u];
    std::vector<uint64_t> coff(mesh->n_cells + 1, 0);
    for (uint32_t c = 0; c < mesh->n_cells; ++c) coff[c] = uoff[cell_to_mat[c]];
    op = new gbfe_op();
    op->mesh = mesh;
    op->cons = cons;
    op->kind = OP_CELL;
    op->prec = prec_flags | GBFE_PREC_FP64;
    op->mats_count = uoff[n_mats];
    op->mats.upload(mats, uoff[n_mats], mesh->ctx->stream);
    op->mat_off_own.upload(coff.data(), coff.size(), mesh->ctx->stream);
    if (prec_flags & GBFE_PREC_MIXED) build_mixed_mats(op);
    if ((prec_flags & GBFE_PREC_FP64_TENSOR) && oz_supported(mesh)) build_oz_mats(op);
    GBFE_CUDA(cudaStreamSynchronize(mesh->ctx->stream));
  });
  if (rc != GBFE_OK) {
    delete op;
    return rc;
  }
  *out = op;
  return GBFE_OK;
}

static int diag_upload_impl(gbfe_mesh *mesh, const gbfe_cons *cons, const double *diag, int kind, gbfe_op **out) {
  if (!mesh || !out) return GBFE_ERR_ARG;
  *out = nullptr;
  gbfe_op *op = nullptr;
  int rc = gbfe_guard(mesh->ctx, [&] {
    GBFE_REQUIRE(diag, "diag_upload: null diagonal");
    GBFE_REQUIRE(!cons || cons->mesh == mesh, "diag_upload: constraints on another mesh");
    op = new gbfe_op();
    op->mesh = mesh;
    op->cons = cons;
    op->kind = kind;
    std::vector<double> dv(diag, diag + mesh->n_dofs);
    if (kind == OP_JACOBI)
      for (double &x : dv) x = 1.0 / x;
    std::vector<float> df(dv.begin(), dv.end());
    op->diag_f32.upload(df.data(), mesh->n_dofs, mesh->ctx->stream);
    if (kind == OP_JACOBI) {
      op->diag.upload(dv.data(), mesh->n_dofs, mesh->ctx->stream);
      GBFE_CUDA(cudaStreamSynchronize(mesh->ctx->stream));
    } else {
      op->diag.upload(diag, mesh->n_dofs, mesh->ctx->stream);
      if ((kind == OP_DIAG || kind == OP_DIAG_BLOCK) && (!cons || cons->pure_dirichlet)) {
        // gather factor of the fused mixed filter step
        // the B^-1 factor folded into a Hamiltonian's tiles by the fused filter
        // (block rows, if any, are set by gbfe_diag_block_upload)
        op->fold_scale.alloc(mesh->n_dofs);
        k_fold_scale<<<grid_for(mesh->n_dofs, 256), 256, 0, mesh->ctx->stream>>>(
            op->diag.p, cons ? cons->is_row.p : nullptr, mesh->n_dofs, 0, 0, op->fold_scale.p);
        check_launch(mesh->ctx, "fold_scale");
      }
      GBFE_CUDA(cudaStreamSynchronize(mesh->ctx->stream));
    }
  });
  if (rc != GBFE_OK) {
    delete op;
    return rc;
  }
  *out = op;
  return GBFE_OK;
}

int gbfe_diag_upload(gbfe_mesh *mesh, const gbfe_cons *cons, const double *diag, gbfe_op **out) {
  return diag_upload_impl(mesh, cons, diag, OP_DIAG, out);
}

int gbfe_diag_block_upload(gbfe_mesh *mesh, const gbfe_cons *cons, const double *diag, uint64_t blk_begin,
                           uint64_t blk_n, const double *blk, gbfe_op **out) {
  if (!mesh || !out) return GBFE_ERR_ARG;
  int rc = diag_upload_impl(mesh, cons, diag, OP_DIAG_BLOCK, out);
  if (rc != GBFE_OK) return rc;
  gbfe_op *op = *out;
  rc = gbfe_guard(mesh->ctx, [&] {
    GBFE_REQUIRE(blk && blk_n > 0 && blk_begin + blk_n <= mesh->n_dofs, "diag_block_upload: block out of range");
    op->blk_begin = blk_begin;
    op->blk_n = blk_n;
    op->blk.upload(blk, blk_n * blk_n, mesh->ctx->stream);
    if (cons && cons->n_rows) {
      std::vector<uint32_t> rows(cons->n_rows);
      GBFE_CUDA(cudaMemcpyAsync(rows.data(), cons->row_ids.p, rows.size() * 4, cudaMemcpyDeviceToHost,
                                mesh->ctx->stream));
      GBFE_CUDA(cudaStreamSynchronize(mesh->ctx->stream));
      for (uint32_t r : rows) op->blk_cons = op->blk_cons || (r >= blk_begin && r - blk_begin < blk_n);
    }
    if (op->fold_scale.p) {
      k_fold_scale<<<grid_for(mesh->n_dofs, 256), 256, 0, mesh->ctx->stream>>>(
          op->diag.p, cons ? cons->is_row.p : nullptr, mesh->n_dofs, blk_begin, blk_n, op->fold_scale.p);
      check_launch(mesh->ctx, "fold_scale");
    }
    std::vector<float> f(blk, blk + blk_n * blk_n);
    op->blk_f32.upload(f.data(), f.size(), mesh->ctx->stream);
    GBFE_CUDA(cudaStreamSynchronize(mesh->ctx->stream));
  });
  if (rc != GBFE_OK) {
    delete op;
    *out = nullptr;
  }
  return rc;
}

int gbfe_jacobi_upload(gbfe_mesh *mesh, const double *diagonal, gbfe_op **out) {
  return diag_upload_impl(mesh, nullptr, diagonal, OP_JACOBI, out);
}

int gbfe_op_destroy(gbfe_op *op) {
  if (!op) return GBFE_OK;
  cudaStreamSynchronize(op->mesh->ctx->stream);
  delete op;
  return GBFE_OK;
}

int gbfe_mv_create(gbfe_mesh *mesh, uint32_t m, int dtype, gbfe_mv **out) {
  if (!mesh || !out) return GBFE_ERR_ARG;
  *out = nullptr;
  gbfe_mv *mv = nullptr;
  int rc = gbfe_guard(mesh->ctx, [&] {
    GBFE_REQUIRE(dtype == GBFE_F64 || dtype == GBFE_F32, "mv_create: dtype must be GBFE_F64 or GBFE_F32");
    mv = new gbfe_mv();
    mv->mesh = mesh;
    mv->m = m;
    mv->dtype = dtype;
    const size_t n = mv->count();
    if (dtype == GBFE_F64) {
      mv->d.alloc(n);
      if (n) GBFE_CUDA(cudaMemsetAsync(mv->d.p, 0, n * 8, mesh->ctx->stream));
    } else {
      mv->f.alloc(n);
      if (n) GBFE_CUDA(cudaMemsetAsync(mv->f.p, 0, n * 4, mesh->ctx->stream));
    }
  });
  if (rc != GBFE_OK) {
    delete mv;
    return rc;
  }
  *out = mv;
  return GBFE_OK;
}

int gbfe_mv_wrap(gbfe_mesh *mesh, uint32_t m, int dtype, void *device_ptr, gbfe_mv **out) {
  if (!mesh || !out || !device_ptr) return GBFE_ERR_ARG;
  *out = nullptr;
  gbfe_mv *mv = nullptr;
  int rc = gbfe_guard(mesh->ctx, [&] {
    GBFE_REQUIRE(dtype == GBFE_F64 || dtype == GBFE_F32, "mv_wrap: dtype must be GBFE_F64 or GBFE_F32");
    cudaPointerAttributes attr;
    GBFE_CUDA(cudaPointerGetAttributes(&attr, device_ptr));
    GBFE_REQUIRE(attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged,
                 "mv_wrap: pointer is not device memory");
    GBFE_REQUIRE(((uintptr_t)device_ptr % (dtype == GBFE_F64 ? 8 : 4)) == 0, "mv_wrap: misaligned pointer");
    mv = new gbfe_mv();
    mv->mesh = mesh;
    mv->m = m;
    mv->dtype = dtype;
    if (dtype == GBFE_F64)
      mv->d.wrap((double *)device_ptr, mv->count());
    else
      mv->f.wrap((float *)device_ptr, mv->count());
  });
  if (rc != GBFE_OK) {
    delete mv;
    return rc;
  }
  *out = mv;
  return GBFE_OK;
}

int gbfe_mv_destroy(gbfe_mv *mv) {
  if (!mv) return GBFE_OK;
  cudaStreamSynchronize(mv->mesh->ctx->stream);
  delete mv;
  return GBFE_OK;
}

int gbfe_mv_copy_in(gbfe_mv *mv, const void *host) {
  if (!mv || !host) return GBFE_ERR_ARG;
  gbfe_ctx *ctx = mv->mesh->ctx;
  return gbfe_guard(ctx, [&] {
    const size_t bytes = mv->count() * (mv->dtype == GBFE_F64 ? 8 : 4);
    if (bytes) GBFE_CUDA(cudaMemcpyAsync(mv->ptr(), host, bytes, cudaMemcpyHostToDevice, ctx->stream));
    GBFE_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

int gbfe_mv_copy_out(const gbfe_mv *mv, void *host) {
  if (!mv || !host) return GBFE_ERR_ARG;
  gbfe_ctx *ctx = mv->mesh->ctx;
  return gbfe_guard(ctx, [&] {
    const size_t bytes = mv->count() * (mv->dtype == GBFE_F64 ? 8 : 4);
    if (bytes) GBFE_CUDA(cudaMemcpyAsync(host, mv->ptr(), bytes, cudaMemcpyDeviceToHost, ctx->stream));
    GBFE_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

int gbfe_mv_copy(const gbfe_mv *src, gbfe_mv *dst) {
  if (!src || !dst) return GBFE_ERR_ARG;
  gbfe_ctx *ctx = src->mesh->ctx;
  return gbfe_guard(ctx, [&] {
    GBFE_REQUIRE(src->mesh == dst->mesh && src->m == dst->m, "mv_copy: shape mismatch");
    convert_mv(ctx, src, dst);
  });
}

int gbfe_mv_set_value(gbfe_mv *mv, double value) {
  if (!mv) return GBFE_ERR_ARG;
  gbfe_ctx *ctx = mv->mesh->ctx;
  return gbfe_guard(ctx, [&] { fill_mv(ctx, mv, value); });
}

int gbfe_mv_device_ptr(const gbfe_mv *mv, void **ptr) {
  if (!mv || !ptr) return GBFE_ERR_ARG;
  *ptr = mv->ptr();
  return GBFE_OK;
}

int gbfe_apply(const gbfe_op *op, gbfe_mv *X, gbfe_mv *Y) {
  if (!op || !X || !Y) return GBFE_ERR_ARG;
  gbfe_ctx *ctx = op->mesh->ctx;
  return gbfe_guard(ctx, [&] { apply_op(op, X, Y); });
}

}  // extern "C"

// ---------------------------------------------------------------------------
// FP64 apply with a fixed, library-owned scratch buffer (no allocation)
// ---------------------------------------------------------------------------
// Some callers cannot call cudaMalloc when they apply an operator: code that
// runs while another component owns all device memory through its own pool
// (a framework allocator that has reserved the GPU), and code that must not
// take the implicit device-wide synchronisation a cudaMalloc can cause (for
// example inside a latency-critical step loop).  gbfe_apply_f64_noalloc gives
// them the FP64 cell apply with its cell-wise scratch in the file-scope array
// below instead of the grow-on-demand buffer gbfe_apply keeps per operator.
namespace {
constexpr uint64_t kNoAllocScratchDoubles = 8ull << 20;  // 64 MiB per GPU, held until exit
static __device__ __align__(256) double g_noalloc_cell_scratch[kNoAllocScratchDoubles];
// device address of the array per device, looked up on the first call there;
// atomic because server slot threads may make their first calls concurrently
// (every thread that looks it up stores the same address)
std::atomic<double *> g_noalloc_ptr[kMaxDevices];
}  // namespace

extern "C" int gbfe_apply_f64_noalloc(const gbfe_op *op, double *X_dev, double *Y_dev, uint32_t m) {
  if (!op || !X_dev || !Y_dev) return GBFE_ERR_ARG;
  gbfe_mesh *me = op->mesh;
  gbfe_ctx *ctx = me->ctx;
  return gbfe_guard(ctx, [&] {
    GBFE_REQUIRE(op->kind == OP_CELL, "apply_f64_noalloc: needs a cell-matrix operator");
    GBFE_REQUIRE(X_dev != Y_dev, "apply_f64_noalloc: X and Y must be distinct");
    if (m == 0) return;
    const uint64_t need = me->total_cell_dofs * (uint64_t)m;
    if (need > kNoAllocScratchDoubles)
      throw Error(GBFE_ERR_ARG, "apply_f64_noalloc: sum over cells of nd_c times m = " + std::to_string(need) +
                                    " exceeds the fixed scratch of " + std::to_string(kNoAllocScratchDoubles) +
                                    " doubles; use gbfe_apply");
    int dev = -1;
    GBFE_CUDA(cudaGetDevice(&dev));
    GBFE_REQUIRE(dev == ctx->device, "apply_f64_noalloc: the context's device must be current");
    GBFE_REQUIRE(dev >= 0 && dev < kMaxDevices, "apply_f64_noalloc: device index out of range");
    double *Yc = g_noalloc_ptr[dev].load(std::memory_order_acquire);
    if (!Yc) {
      // once per device, with that device current: the symbol's host-side name
      // is not a device address, so fetch the real one
      void *p = nullptr;
      GBFE_CUDA(cudaGetSymbolAddress(&p, g_noalloc_cell_scratch));
      Yc = (double *)p;
      g_noalloc_ptr[dev].store(Yc, std::memory_order_release);
    }
    GBFE_REQUIRE(!op->nl, "apply_f64_noalloc: operators with a nonlocal part need gbfe_apply");
    const uint32_t Nn = (uint32_t)me->n_dofs;
    (void)Nn;
    // constraints on X (the same kernels gbfe_apply launches)
    const gbfe_cons *c = op->cons;
    if (c && c->n_rows) {
      const uint64_t nr = (uint64_t)c->n_rows * m;
      if (c->pure_dirichlet)
        k_zero_rows<double><<<stride_grid(ctx, nr), 256, 0, ctx->stream>>>(X_dev, m, c->n_rows, c->row_ids.p);
      else
        k_p2c<double><<<stride_grid(ctx, nr), 256, 0, ctx->stream>>>(X_dev, m, c->n_rows, c->row_ids.p,
                                                                     c->row_sizes.p, c->col_ids.p, c->row_acc.p,
                                                                     c->col_vals.p, c->inh.p);
      check_launch(ctx, "p2c");
    }
    // cell products into the fixed scratch (every element is written, so
    // nothing needs clearing between calls)
    const size_t smem_cap = 96 * 1024;
    uint32_t mt = (uint32_t)std::min<size_t>(m, smem_cap / (sizeof(double) * me->nd_max));
    GBFE_REQUIRE(mt > 0, "cell too large for the FP64 apply");
    const uint32_t vt = (m + mt - 1) / mt;
    mt = (m + vt - 1) / vt;
    uint32_t jsplit = 1;
    const uint64_t target = (uint64_t)ctx->sm_count * 12;
    while ((uint64_t)me->n_cells * vt * jsplit < target && jsplit * 8 < me->nd_min) jsplit *= 2;
    GBFE_CUDA(cudaFuncSetAttribute(k_cell_apply_f64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_cap));
    k_cell_apply_f64<<<dim3(me->n_cells, vt, jsplit), 256, sizeof(double) * (size_t)me->nd_max * mt, ctx->stream>>>(
        X_dev, m, me->ids.p, me->cell_off.p, op_mat_off(op), op->mats.p, Yc, mt, jsplit);
    check_launch(ctx, "cell_apply_f64_noalloc");
    const bool has_par = c && !c->pure_dirichlet;
    const uint64_t n = me->n_dofs * (uint64_t)m;
    k_assemble<double, double><<<stride_grid(ctx, n), 256, 0, ctx->stream>>>(
        Yc, m, me->n_dofs, me->slot_ptr.p, me->slot.p, c ? c->is_row.p : nullptr, has_par ? c->par_ptr.p : nullptr,
        has_par ? c->par_row.p : nullptr, has_par ? c->par_w.p : nullptr, Y_dev, FastDiv(m));
    check_launch(ctx, "assemble_f64_noalloc");
  });
}
