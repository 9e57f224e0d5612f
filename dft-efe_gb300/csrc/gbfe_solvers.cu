// gbfe_solvers.cu -- Chebyshev filters, FP64 dense stages, ChFSI pass loop,
// Lanczos spectrum bounds and CG, all device-resident on the context stream.
//
// Reductions (column dots and norms) are two-stage with a fixed grid and a
// fixed summation order, so they are bitwise reproducible run to run.
// Dense m x m work (potrf, triangular solve, syevd) and the tall-skinny Gram /
// rotation GEMMs are plain library calls (cuSOLVER / cuBLAS), in FP64.
#include "gbfe_internal.cuh"

#include <algorithm>
#include <cmath>
#include <memory>
#include <random>

using namespace gbfe;

namespace gbfe {
void assemble_f32(const gbfe_op *op, float *Yc, gbfe_mv *Y);
void convert_mv(gbfe_ctx *ctx, const gbfe_mv *src, gbfe_mv *dst);
void fill_mv(gbfe_ctx *ctx, gbfe_mv *x, double v);
}  // namespace gbfe

namespace {

constexpr unsigned kRedBlocks = 304;  // fixed reduction grid (2 x 152 SMs)

template <class T>
__global__ void k_axpby(uint64_t n, double a, const T *__restrict__ x, double b, const T *__restrict__ y,
                        T *__restrict__ z) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x)
    z[t] = (T)a * x[t] + (T)b * y[t];
}

// z[i][j] = a1*alpha[j]*x[i][j] + b1*beta[j]*y[i][j] (blasLapack::axpbyBlocked)
template <class T, bool SH>
__global__ void k_axpby_blocked(uint64_t rows, uint32_t m, double a1, const double *__restrict__ alpha,
                                const T *__restrict__ x, double b1, const double *__restrict__ beta,
                                const T *__restrict__ y, T *__restrict__ z, const FastDiv fm) {
  extern __shared__ __align__(16) unsigned char col_sh[];
  T *fa = reinterpret_cast<T *>(col_sh), *fb = fa + m;
  if (SH) {
    load_col_factors(fa, m, a1, alpha);
    load_col_factors(fb, m, b1, beta);
    __syncthreads();
  }
  const uint64_t n = rows * m;
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t i;
    uint32_t j;
    fm.divmod(t, i, j);
    z[t] = (SH ? fa[j] : (T)(a1 * alpha[j])) * x[t] + (SH ? fb[j] : (T)(b1 * beta[j])) * y[t];
  }
}

// R = alpha1*AS + (-c*alpha1)*RN + alpha2*R + alpha1*eF2[j]*Y, one sweep
// (the axpby, axpby and axpbyBlocked of ChebyshevFilter.t.cpp:375-409 fused)
template <class T, bool SH>
__global__ void k_cheb_step(uint64_t n, uint32_t m, double alpha1, double c, double alpha2,
                            const T *__restrict__ AS, const T *__restrict__ RN, T *__restrict__ R,
                            const double *__restrict__ eF2, const T *__restrict__ Y, const FastDiv fm) {
  extern __shared__ __align__(16) unsigned char col_sh[];
  T *g = reinterpret_cast<T *>(col_sh);
  if (SH) {
    load_col_factors(g, m, alpha1, eF2);
    __syncthreads();
  }
  const T a1 = (T)alpha1, b1 = (T)(-c * alpha1), a2 = (T)alpha2;
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t i;
    uint32_t j;
    fm.divmod(t, i, j);
    T s1 = a1 * AS[t] + b1 * RN[t];
    T r = s1 + a2 * R[t];
    R[t] = r + (SH ? g[j] : (T)(alpha1 * eF2[j])) * Y[t];
  }
}

// the same step with its scalars read from a device table {alpha1, c, alpha2},
// so one captured graph serves every pass
template <class T, bool SH>
__global__ void k_cheb_step_dev(uint64_t n, uint32_t m, const double *__restrict__ coef, const T *__restrict__ AS,
                                const T *__restrict__ RN, T *__restrict__ R, const double *__restrict__ eF2,
                                const T *__restrict__ Y, const FastDiv fm) {
  extern __shared__ __align__(16) unsigned char col_sh[];
  T *g = reinterpret_cast<T *>(col_sh);
  const double alpha1 = coef[0], c = coef[1], alpha2 = coef[2];
  if (SH) {
    load_col_factors(g, m, alpha1, eF2);
    __syncthreads();
  }
  const T a1 = (T)alpha1, b1 = (T)(-c * alpha1), a2 = (T)alpha2;
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t i;
    uint32_t j;
    fm.divmod(t, i, j);
    T s1 = a1 * AS[t] + b1 * RN[t];
    T r = s1 + a2 * R[t];
    R[t] = r + (SH ? g[j] : (T)(alpha1 * eF2[j])) * Y[t];
  }
}

// Start of the mixed filter from a residual R0 held in FP64, in one sweep:
// Yf = float(R0), RN = alpha1 Yf (the same expression as k_axpby<float> with
// b = 0), R = 0 -- what a copy, a conversion, an axpby and a fill would leave
__global__ void k_filter_start_mixed(uint64_t n, double a, const double *__restrict__ R0, float *__restrict__ Yf,
                                     float *__restrict__ RN, float *__restrict__ R) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x) {
    const float y = (float)R0[t];
    Yf[t] = y;
    RN[t] = (float)a * y + (float)0.0 * y;
    R[t] = 0.f;
  }
}

// Y = R + eF2[j] * X, with R in FP32 and X, Y in FP64 (mixed filter epilogue)
__global__ void k_cheb_final_mixed(uint64_t n, uint32_t m, const float *__restrict__ R, const double *__restrict__ eF2,
                                   const double *__restrict__ X, double *__restrict__ Y, const FastDiv fm) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t i;
    uint32_t j;
    fm.divmod(t, i, j);
    Y[t] = (double)R[t] + eF2[j] * X[t];
  }
}

// stage 1 of a column reduction: partial[b][j] = sum over this block's rows
template <class T>
__global__ void k_coldot_partial(const T *__restrict__ x, const T *__restrict__ y, uint64_t rows, uint32_t m,
                                 double *__restrict__ partial) {
  extern __shared__ double sh[];
  const uint32_t tcols = min(m, 256u);
  const uint32_t rpb = 256u / tcols;
  const uint32_t r = threadIdx.x / tcols, jj = threadIdx.x % tcols;
  const uint64_t per = (rows + gridDim.x - 1) / gridDim.x;
  const uint64_t r0 = blockIdx.x * per, r1 = min(rows, r0 + per);
  for (uint32_t jb = 0; jb < m; jb += tcols) {
    const uint32_t j = jb + jj;
    double acc = 0.0;
    if (r < rpb && j < m)
      for (uint64_t i = r0 + r; i < r1; i += rpb) acc += (double)x[i * m + j] * (double)y[i * m + j];
    sh[threadIdx.x] = acc;
    __syncthreads();
    if (r == 0 && j < m) {
      double s = 0.0;
      for (uint32_t q = 0; q < rpb; ++q) s += sh[q * tcols + jj];
      partial[(uint64_t)blockIdx.x * m + j] = s;
    }
    __syncthreads();
  }
}

// stage 2: a block takes 32 columns with eight warps, warp g summing the
// partials of blocks g, g + 8, ... in ascending order; the eight sums are
// then added in warp order (a fixed order: deterministic)
__global__ void __launch_bounds__(256) k_coldot_final(const double *__restrict__ partial, uint32_t nb, uint32_t m,
                                                      double *__restrict__ out, int take_sqrt) {
  __shared__ double red[8][32];
  const uint32_t lane = threadIdx.x % 32, g = threadIdx.x / 32;
  for (uint32_t j0 = blockIdx.x * 32; j0 < m; j0 += gridDim.x * 32) {
    const uint32_t j = j0 + lane;
    double s = 0.0;
    if (j < m)
#pragma unroll 4
      for (uint32_t b = g; b < nb; b += 8) s += partial[(uint64_t)b * m + j];
    red[g][lane] = s;
    __syncthreads();
    if (g == 0 && j < m) {
      double v = red[0][lane];
#pragma unroll
      for (int k = 1; k < 8; ++k) v += red[k][lane];
      out[j] = take_sqrt ? sqrt(v) : v;
    }
    __syncthreads();
  }
}

__global__ void k_zero_upper(double *__restrict__ S, uint32_t m) {
  const uint64_t n = (uint64_t)m * m;
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t col = (uint32_t)(t / m), row = (uint32_t)(t % m);
    if (row < col) S[t] = 0.0;
  }
}

unsigned sgrid(gbfe_ctx *ctx, uint64_t n) {
  uint64_t g = (n + 255) / 256, cap = (uint64_t)ctx->sm_count * 16;
  return (unsigned)std::max<uint64_t>(1, std::min(g, cap));
}

// temporary device block vector with the shape of `like`
std::unique_ptr<gbfe_mv> make_like(const gbfe_mv *like, int dtype) {
  std::unique_ptr<gbfe_mv> v(new gbfe_mv());
  v->mesh = like->mesh;
  v->m = like->m;
  v->dtype = dtype;
  if (dtype == GBFE_F64) {
    v->d.alloc(v->count());
    GBFE_CUDA(cudaMemsetAsync(v->d.p, 0, v->count() * 8, like->mesh->ctx->stream));
  } else {
    v->f.alloc(v->count());
    GBFE_CUDA(cudaMemsetAsync(v->f.p, 0, v->count() * 4, like->mesh->ctx->stream));
  }
  return v;
}

std::unique_ptr<gbfe_mv> make_mv(gbfe_mesh *me, uint32_t m, int dtype) {
  gbfe_mv tmp;
  tmp.mesh = me;
  tmp.m = m;
  tmp.dtype = dtype;
  return make_like(&tmp, dtype);
}

void d_axpby(gbfe_ctx *ctx, double a, const gbfe_mv *x, double b, const gbfe_mv *y, gbfe_mv *z) {
  const uint64_t n = z->count();
  if (z->dtype == GBFE_F64)
    k_axpby<double><<<sgrid(ctx, n), 256, 0, ctx->stream>>>(n, a, x->d.p, b, y->d.p, z->d.p);
  else
    k_axpby<float><<<sgrid(ctx, n), 256, 0, ctx->stream>>>(n, a, x->f.p, b, y->f.p, z->f.p);
  check_launch(ctx, "axpby");
}

void d_axpby_blocked(gbfe_ctx *ctx, double a1, const double *alpha_d, const gbfe_mv *x, double b1,
                     const double *beta_d, const gbfe_mv *y, gbfe_mv *z) {
  const uint64_t n = z->count();
  if (z->dtype == GBFE_F64) {
    const size_t sh = col_factor_smem<double>(z->m, 2);
    (sh ? k_axpby_blocked<double, true> : k_axpby_blocked<double, false>)<<<sgrid(ctx, n), 256, sh, ctx->stream>>>(
        z->mesh->n_dofs, z->m, a1, alpha_d, x->d.p, b1, beta_d, y->d.p, z->d.p, FastDiv(z->m));
  } else {
    const size_t sh = col_factor_smem<float>(z->m, 2);
    (sh ? k_axpby_blocked<float, true> : k_axpby_blocked<float, false>)<<<sgrid(ctx, n), 256, sh, ctx->stream>>>(
        z->mesh->n_dofs, z->m, a1, alpha_d, x->f.p, b1, beta_d, y->f.p, z->f.p, FastDiv(z->m));
  }
  check_launch(ctx, "axpby_blocked");
}

// per-column x.y (or sqrt of x.x) into a device array of length m
void d_coldots(gbfe_ctx *ctx, const gbfe_mv *x, const gbfe_mv *y, double *out_d, bool take_sqrt) {
  const uint32_t m = x->m;
  const uint64_t rows = x->mesh->n_dofs;
  const unsigned nb = (unsigned)std::min<uint64_t>(kRedBlocks, std::max<uint64_t>(1, rows));
  ctx->red.ensure((size_t)nb * m);
  if (x->dtype == GBFE_F64)
    k_coldot_partial<double><<<nb, 256, 256 * sizeof(double), ctx->stream>>>(x->d.p, y->d.p, rows, m, ctx->red.p);
  else
    k_coldot_partial<float><<<nb, 256, 256 * sizeof(double), ctx->stream>>>(x->f.p, y->f.p, rows, m, ctx->red.p);
  check_launch(ctx, "coldot_partial");
  k_coldot_final<<<(m + 31) / 32, 256, 0, ctx->stream>>>(ctx->red.p, nb, m, out_d, take_sqrt ? 1 : 0);
  check_launch(ctx, "coldot_final");
}

// Short-lived device vector of doubles (length m scalars of a pass), taken
// from a per-context stack of buffers: no cudaMalloc / cudaFree (and their
// implicit device synchronisation) in the pass loop.  Scoped use only (LIFO).
struct DevVec {
  gbfe_ctx *ctx;
  double *p;
  size_t idx;
  DevVec(gbfe_ctx *c, size_t n) : ctx(c) {
    idx = ctx->vec_top++;
    if (ctx->vec_pool.size() <= idx) {
      ctx->vec_pool.emplace_back(new DBuf<double>());
      ctx->vec_pin.emplace_back(new PinnedSlot());
    }
    ctx->vec_pool[idx]->ensure(std::max<size_t>(n, 1));
    p = ctx->vec_pool[idx]->p;
  }
  ~DevVec() { --ctx->vec_top; }
  DevVec(const DevVec &) = delete;
  DevVec &operator=(const DevVec &) = delete;
  void set(gbfe_ctx *, const double *h, size_t n) { h2d_staged(ctx, *ctx->vec_pin[idx], p, h, n * 8); }
  void get(gbfe_ctx *, double *h, size_t n) const {
    GBFE_CUDA(cudaMemcpyAsync(h, p, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    GBFE_CUDA(cudaStreamSynchronize(ctx->stream));
  }
};

void host_coldots(gbfe_ctx *ctx, const gbfe_mv *x, const gbfe_mv *y, double *h, bool take_sqrt) {
  DevVec o(ctx, x->m);
  d_coldots(ctx, x, y, o.p, take_sqrt);
  o.get(ctx, h, x->m);
}

// S (m x m, col-major, lower triangle valid) = X^T * Y  over the rows
void gram(gbfe_ctx *ctx, const gbfe_mv *X, const gbfe_mv *Y, double *S) {
  const int m = (int)X->m;
  const int N = (int)X->mesh->n_dofs;
  const double one = 1.0, zero = 0.0;
  // row-major [N][m] == col-major m x N with ld m
  GBFE_CUBLAS(cublasDgemm(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_T, m, m, N, &one, X->d.p, m, Y->d.p, m, &zero, S, m));
  count_launch(ctx);
}

// ------------------------------------------------------------ dense stages
int cholesky_gs_impl(const gbfe_op *B, gbfe_mv *X, gbfe_mv *Xo, std::string &msg) {
  gbfe_ctx *ctx = X->mesh->ctx;
  const uint32_t m = X->m;
  if (X->mesh->n_dofs < m) {
    msg = "NON_ORTHONORMALIZABLE_MULTIVECTOR: global size smaller than the number of vectors";
    return GBFE_ERR_NOT_ORTHONORMALIZABLE;
  }
  auto BX = make_like(X, GBFE_F64);
  apply_op(B, X, BX.get());
  ctx->small.ensure((size_t)m * m);
  double *S = ctx->small.p;
  gram(ctx, X, BX.get(), S);
  int lwork = 0;
  GBFE_CUSOLVER(cusolverDnDpotrf_bufferSize(ctx->cusolver, CUBLAS_FILL_MODE_LOWER, (int)m, S, (int)m, &lwork));
  ctx->lwork.ensure(std::max(lwork, 1));
  ctx->info.ensure(1);
  GBFE_CUSOLVER(cusolverDnDpotrf(ctx->cusolver, CUBLAS_FILL_MODE_LOWER, (int)m, S, (int)m, ctx->lwork.p, lwork,
                                 ctx->info.p));
  count_launch(ctx);
  int info = 0;
  GBFE_CUDA(cudaMemcpyAsync(&info, ctx->info.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  std::vector<double> hS((size_t)m * m);
  GBFE_CUDA(cudaMemcpyAsync(hS.data(), S, hS.size() * 8, cudaMemcpyDeviceToHost, ctx->stream));
  GBFE_CUDA(cudaStreamSynchronize(ctx->stream));
  if (info != 0) {
    msg = "LAPACK_ERROR: FAILED_CHOLESKY_FACTORIZATION (potrf info " + std::to_string(info) + ")";
    return GBFE_ERR_LAPACK;
  }
  for (uint32_t i = 0; i < m; ++i)
    if (std::fabs(hS[(size_t)i * m + i]) < 1e-14) {
      msg = "Chol GS cannot orthogonalize the given multivector (near-zero diagonal of L)";
      return GBFE_ERR_NOT_ORTHONORMALIZABLE;
    }
  // X_o (col-major m x N) = L^{-1} X  (potrf('L') + trtri('L') + gemm of the
  // reference, done here as one triangular solve)
  GBFE_CUDA(cudaMemcpyAsync(Xo->d.p, X->d.p, X->count() * 8, cudaMemcpyDeviceToDevice, ctx->stream));
  const double one = 1.0;
  GBFE_CUBLAS(cublasDtrsm(ctx->cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT,
                          (int)m, (int)X->mesh->n_dofs, &one, S, (int)m, Xo->d.p, (int)m));
  count_launch(ctx);
  return GBFE_OK;
}

// Eigen-decomposition of the m x m symmetric device matrix dA (lower triangle
// read), the syevd('V','L') of RayleighRitzEigenSolver.t.cpp:233-301: on
// return dA holds the eigenvectors (columns) and eig_h the eigenvalues,
// ascending.  For m <= SMALL_EIG_HOST_MAX and ctx->small_eig_host the
// decomposition runs on the host (gbfe_host_eig.cpp: one copy down, one up),
// else in cuSOLVER's syevd (a chain of small launches for small m).
constexpr int SMALL_EIG_HOST_MAX = 128;

int small_syevd(gbfe_ctx *ctx, int m, double *dA, double *eig_h, std::string &msg) {
  if (ctx->small_eig_host && m <= SMALL_EIG_HOST_MAX) {
    std::vector<double> h((size_t)m * m);
    GBFE_CUDA(cudaMemcpyAsync(h.data(), dA, h.size() * 8, cudaMemcpyDeviceToHost, ctx->stream));
    GBFE_CUDA(cudaStreamSynchronize(ctx->stream));
    if (host_sym_eig(m, h.data(), eig_h) != 0) {
      msg = "LAPACK_ERROR: FAILED_STANDARD_EIGENPROBLEM (QR iteration did not converge)";
      return GBFE_ERR_LAPACK;
    }
    h2d_staged(ctx, ctx->pin_small, dA, h.data(), h.size() * 8);
    return GBFE_OK;
  }
  DevVec W(ctx, m);
  int lwork = 0;
  GBFE_CUSOLVER(cusolverDnDsyevd_bufferSize(ctx->cusolver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, m, dA, m,
                                            W.p, &lwork));
  ctx->lwork.ensure(std::max(lwork, 1));
  ctx->info.ensure(1);
  GBFE_CUSOLVER(cusolverDnDsyevd(ctx->cusolver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, m, dA, m, W.p,
                                 ctx->lwork.p, lwork, ctx->info.p));
  count_launch(ctx);
  int info = 0;
  GBFE_CUDA(cudaMemcpyAsync(&info, ctx->info.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  W.get(ctx, eig_h, m);
  if (info != 0) {
    msg = "LAPACK_ERROR: FAILED_STANDARD_EIGENPROBLEM (syevd info " + std::to_string(info) + ")";
    return GBFE_ERR_LAPACK;
  }
  return GBFE_OK;
}

int rayleigh_ritz_impl(const gbfe_op *A, gbfe_mv *X, double *eig_h, gbfe_mv *Xout, std::string &msg,
                       gbfe_mv *AX_keep = nullptr) {
  gbfe_ctx *ctx = X->mesh->ctx;
  const uint32_t m = X->m;
  std::unique_ptr<gbfe_mv> AXo;
  gbfe_mv *AX = AX_keep;
  if (!AX) {
    AXo = make_like(X, GBFE_F64);
    AX = AXo.get();
  }
  apply_op(A, X, AX);
  ctx->small.ensure((size_t)m * m);
  double *S = ctx->small.p;
  gram(ctx, X, AX, S);
  const int rc = small_syevd(ctx, (int)m, S, eig_h, msg);
  if (rc != GBFE_OK) return rc;
  // Psi (col-major m x N) = Q^T X   (gemm('T','N') of the reference)
  const double one = 1.0, zero = 0.0;
  GBFE_CUBLAS(cublasDgemm(ctx->cublas, CUBLAS_OP_T, CUBLAS_OP_N, (int)m, (int)X->mesh->n_dofs, (int)m, &one, S,
                          (int)m, X->d.p, (int)m, &zero, Xout->d.p, (int)m));
  count_launch(ctx);
  return GBFE_OK;
}

// ------------------------------------------------------------ filters
// Host-side schedule of ResidualChebyshevFilterGEP: the per-degree scalars and
// the per-column filtered eigenvalue recurrences (eigenValuesFiltered1/2 of
// ChebyshevFilter.t.cpp:297-420) depend only on host data, so the whole table
// is computed up front and uploaded once.
struct ChebSchedule {
  double e, c, alpha1_init;
  std::vector<double> alpha1, alpha2;  // per degree 2..d (index deg-2)
  std::vector<double> eF2;             // [(d-1)+1][m]: row k is eF2 used at step k; last row final
};

ChebSchedule cheb_schedule(const double *eig, uint32_t m, uint32_t degree, double wl, double wu, double uu) {
  ChebSchedule s;
  s.e = 0.5 * (uu - wu);
  s.c = 0.5 * (uu + wu);
  double sigma = s.e / (wl - s.c);
  const double sigma1 = sigma, gamma = 2.0 / sigma1;
  std::vector<double> eF(eig, eig + m), eF1(m, 1.0), eF2(m);
  double alpha1 = sigma1 / s.e, alpha2 = -s.c;
  s.alpha1_init = alpha1;
  for (uint32_t j = 0; j < m; ++j) eF2[j] = alpha1 * alpha2;
  for (uint32_t j = 0; j < m; ++j) eF2[j] = 1.0 * 1.0 * eF2[j] + alpha1 * eF[j] * eF1[j];
  for (uint32_t deg = 2; deg <= degree; ++deg) {
    const double sigma2 = 1.0 / (gamma - sigma);
    alpha1 = 2.0 * sigma2 / s.e;
    alpha2 = -(sigma * sigma2);
    s.alpha1.push_back(alpha1);
    s.alpha2.push_back(alpha2);
    s.eF2.insert(s.eF2.end(), eF2.begin(), eF2.end());
    for (uint32_t j = 0; j < m; ++j) eF1[j] = (-s.c * alpha1) * eF2[j] + alpha2 * eF1[j];
    for (uint32_t j = 0; j < m; ++j) eF1[j] = 1.0 * 1.0 * eF1[j] + alpha1 * eF[j] * eF2[j];
    std::swap(eF1, eF2);
    sigma = sigma2;
  }
  s.eF2.insert(s.eF2.end(), eF2.begin(), eF2.end());  // final row
  return s;
}

template <class T>
void launch_cheb_step(gbfe_ctx *ctx, uint64_t n, uint32_t m, double alpha1, double c, double alpha2,
                      const gbfe_mv *AS, const gbfe_mv *RN, gbfe_mv *R, const double *eF2, const gbfe_mv *Y);
template <>
void launch_cheb_step<double>(gbfe_ctx *ctx, uint64_t n, uint32_t m, double alpha1, double c, double alpha2,
                              const gbfe_mv *AS, const gbfe_mv *RN, gbfe_mv *R, const double *eF2, const gbfe_mv *Y) {
  const size_t sh = col_factor_smem<double>(m);
  (sh ? k_cheb_step<double, true> : k_cheb_step<double, false>)<<<sgrid(ctx, n), 256, sh, ctx->stream>>>(
      n, m, alpha1, c, alpha2, AS->d.p, RN->d.p, R->d.p, eF2, Y->d.p, FastDiv(m));
  check_launch(ctx, "cheb_step");
}
template <>
void launch_cheb_step<float>(gbfe_ctx *ctx, uint64_t n, uint32_t m, double alpha1, double c, double alpha2,
                             const gbfe_mv *AS, const gbfe_mv *RN, gbfe_mv *R, const double *eF2, const gbfe_mv *Y) {
  const size_t sh = col_factor_smem<float>(m);
  (sh ? k_cheb_step<float, true> : k_cheb_step<float, false>)<<<sgrid(ctx, n), 256, sh, ctx->stream>>>(
      n, m, alpha1, c, alpha2, AS->f.p, RN->f.p, R->f.p, eF2, Y->f.p, FastDiv(m));
  check_launch(ctx, "cheb_step_f32");
}

// Persistent buffers of the filter across passes, and the captured graph of its
// recurrence (valid for one operator pair, degree, width and precision).
struct FilterWork {
  std::unique_ptr<gbfe_mv> s1, s2, R, RN, Yf;
  DBuf<double> tab, coef;
  cudaGraphExec_t exec = nullptr;
  gbfe_ctx *owner = nullptr;  // the context whose pool takes exec back
  std::vector<GraphProf> prof;
  gbfe_ctx *prof_ctx = nullptr;  // replay whose event timings are not read yet
  uint64_t per_replay = 0;
  const gbfe_op *A = nullptr, *BInv = nullptr;
  uint32_t degree = 0, m = 0;
  int prec = -1, uses = 0, graph_failed = 0;
  // kernel timings of the last replay (event-record nodes inside the graph);
  // read lazily, before the next replay or when the graph goes away, so the
  // profiled run does not wait for each replay
  void flush_prof() {
    if (!prof_ctx) return;
    gbfe_ctx *ctx = prof_ctx;
    prof_ctx = nullptr;
    if (prof.empty() || cudaEventSynchronize(prof.back().e1) != cudaSuccess) return;
    for (auto &g : prof) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, g.e0, g.e1) != cudaSuccess) continue;
      KernelStat &st = ctx->kstats[g.name];
      st.ms += ms;
      st.launches++;
      st.flops += g.flops;
      st.bytes += g.bytes;
    }
  }
  void drop_graph() {
    flush_prof();
    // back to the context's pool once no replay of it is in flight (every
    // replay is on the context stream); the pool keeps a few
    if (exec) {
      if (owner && owner->fw_exec_pool.size() < 4 && cudaStreamSynchronize(owner->stream) == cudaSuccess)
        owner->fw_exec_pool.push_back(exec);
      else
        cudaGraphExecDestroy(exec);
    }
    exec = nullptr;
    for (auto &g : prof) {
      cudaEventDestroy(g.e0);
      cudaEventDestroy(g.e1);
    }
    prof.clear();
  }
  ~FilterWork() { drop_graph(); }
};

// precision GBFE_F64: the recurrence in FP64.  GBFE_F32: the initial residual
// (A X - Lambda B X) and the final Y = B^-1 R + Lambda~ X stay FP64; the d-1
// recurrence steps run on FP32 block vectors with split-BF16 tensor-core cell
// products (the operator must carry GBFE_PREC_MIXED matrices).
void residual_filter(const gbfe_op *A, const gbfe_op *B, const gbfe_op *BInv, const double *eig_h, gbfe_mv *X,
                     uint32_t degree, double wl, double wu, double uu, gbfe_mv *Y, int prec,
                     const gbfe_mv *R0 = nullptr, FilterWork *fw = nullptr) {
  gbfe_ctx *ctx = X->mesh->ctx;
  const uint32_t m = X->m;
  const bool mixed = prec == GBFE_F32;
  GBFE_REQUIRE(!mixed || (A->prec & GBFE_PREC_MIXED), "mixed filter: operator A was not built with GBFE_PREC_MIXED");
  const int rt = mixed ? GBFE_F32 : GBFE_F64;
  const ChebSchedule s = cheb_schedule(eig_h, m, degree, wl, wu, uu);
  FilterWork local;
  FilterWork &w = fw ? *fw : local;
  if (!w.s1 || w.m != m || w.prec != prec || w.degree != degree || w.A != A || w.BInv != BInv) {
    w.drop_graph();
    w.s1 = make_like(X, rt);
    w.s2 = make_like(X, rt);
    w.R = make_like(X, rt);
    w.RN = make_like(X, rt);
    w.Yf = mixed ? make_like(X, GBFE_F32) : nullptr;
    w.tab.alloc(s.eF2.size());
    w.coef.alloc(3 * std::max<uint32_t>(1, degree));
    w.A = A;
    w.BInv = BInv;
    w.m = m;
    w.prec = prec;
    w.degree = degree;
    w.uses = 0;
  }
  std::vector<double> coef(3 * std::max<uint32_t>(1, degree), 0.0);
  for (uint32_t k = 0; k + 2 <= degree; ++k) {
    coef[3 * k] = s.alpha1[k];
    coef[3 * k + 1] = s.c;
    coef[3 * k + 2] = s.alpha2[k];
  }
  DevVec d_ones(ctx, m), d_eig(ctx, m);
  std::vector<double> ones(m, 1.0);
  d_ones.set(ctx, ones.data(), m);
  d_eig.set(ctx, eig_h, m);
  h2d_staged(ctx, ctx->pin_tab, w.tab.p, s.eF2.data(), s.eF2.size() * 8);
  h2d_staged(ctx, ctx->pin_coef, w.coef.p, coef.data(), coef.size() * 8);
  gbfe_mv *s1 = w.s1.get(), *s2 = w.s2.get();
  std::unique_ptr<gbfe_mv> &R = w.R, &RN = w.RN;
  const gbfe_mv *Yr = Y;
  if (R0 && mixed) {
    // the caller holds A X - Lambda B X in FP64: Y itself is only written by
    // the final step, so the FP32 start reads R0 directly
    const uint64_t n0 = X->count();
    k_filter_start_mixed<<<sgrid(ctx, n0), 256, 0, ctx->stream>>>(n0, s.alpha1_init, R0->d.p, w.Yf->f.p, RN->f.p,
                                                                  R->f.p);
    check_launch(ctx, "filter_start_mixed");
    Yr = w.Yf.get();
  } else if (R0) {
    // the caller already holds A X - Lambda B X (the residual of the previous
    // Rayleigh-Ritz step), so the two initial applies are skipped
    GBFE_CUDA(cudaMemcpyAsync(Y->d.p, R0->d.p, Y->count() * 8, cudaMemcpyDeviceToDevice, ctx->stream));
  } else {
    auto s3 = make_like(X, GBFE_F64);
    apply_pair_f64(A, B, X, s3.get(), Y);
    d_axpby_blocked(ctx, 1.0, d_ones.p, s3.get(), -1.0, d_eig.p, Y, Y);  // Y = AX - lambda BX
  }
  if (!(R0 && mixed)) {
    if (mixed) {
      convert_mv(ctx, Y, w.Yf.get());
      Yr = w.Yf.get();
    }
    d_axpby(ctx, s.alpha1_init, Yr, 0.0, Yr, RN.get());  // ResidualNew = alpha1 * Y
    fill_mv(ctx, R.get(), 0.0);
  }
  const uint64_t n = X->count();
  // the d-1 recurrence steps: pointers and table offsets are fixed for a given
  // degree, the scalars come from device tables -> one graph for every pass
  auto recurrence = [&]() {
    for (uint32_t deg = 2; deg <= degree; ++deg) {
      const uint32_t k = deg - 2;
      gbfe_mv *rn = ((deg - 2) % 2 == 0) ? RN.get() : R.get();
      gbfe_mv *r = ((deg - 2) % 2 == 0) ? R.get() : RN.get();
      if (mixed && ctx->fuse_filter &&
          filter_step_fused(A, BInv, rn, r, w.coef.p + 3 * k, w.tab.p + (size_t)k * m, Yr))
        continue;
      apply_op(BInv, rn, s1);
      apply_op(A, s1, s2);
      if (mixed) {
        const size_t sh = col_factor_smem<float>(m);
        (sh ? k_cheb_step_dev<float, true> : k_cheb_step_dev<float, false>)<<<sgrid(ctx, n), 256, sh, ctx->stream>>>(
            n, m, w.coef.p + 3 * k, s2->f.p, rn->f.p, r->f.p, w.tab.p + (size_t)k * m, Yr->f.p, FastDiv(m));
      } else {
        const size_t sh = col_factor_smem<double>(m);
        (sh ? k_cheb_step_dev<double, true> : k_cheb_step_dev<double, false>)<<<sgrid(ctx, n), 256, sh, ctx->stream>>>(
            n, m, w.coef.p + 3 * k, s2->d.p, rn->d.p, r->d.p, w.tab.p + (size_t)k * m, Yr->d.p, FastDiv(m));
      }
      check_launch(ctx, "cheb_step");
    }
  };
  const bool can_graph = fw && ctx->use_graphs && !w.graph_failed && degree >= 2 && w.uses >= 1;
  if (can_graph && !w.exec) {
    // capture on the second use: every lazily sized buffer exists by then
    const uint64_t l0 = ctx->launches;
    std::vector<GraphProf> prof;
    if (ctx->profiling) ctx->capture_prof = &prof;
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      try {
        recurrence();
      } catch (...) {
        e = cudaErrorStreamCaptureInvalidated;
      }
      const cudaError_t e2 = cudaStreamEndCapture(ctx->stream, &graph);
      if (e == cudaSuccess) e = e2;
    }
    ctx->capture_prof = nullptr;
    if (e == cudaSuccess) {
      // a pooled graph of the same topology takes the new node parameters
      // (every pointer and table of this capture); else a new instantiation
      bool updated = false;
      while (!updated && !ctx->fw_exec_pool.empty()) {
        cudaGraphExec_t cand = ctx->fw_exec_pool.back();
        ctx->fw_exec_pool.pop_back();
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(cand, graph, &info) == cudaSuccess) {
          w.exec = cand;
          updated = true;
        } else {
          (void)cudaGetLastError();
          cudaGraphExecDestroy(cand);
        }
      }
      if (!updated) e = cudaGraphInstantiate(&w.exec, graph, 0);
      w.owner = ctx;
    }
    if (graph) cudaGraphDestroy(graph);
    w.per_replay = ctx->launches - l0;
    ctx->launches = l0;
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      for (auto &g : prof) {
        cudaEventDestroy(g.e0);
        cudaEventDestroy(g.e1);
      }
      w.exec = nullptr;
      w.graph_failed = 1;
    } else {
      w.prof = std::move(prof);
    }
  }
  if (can_graph && w.exec) {
    w.flush_prof();  // the previous replay's events, before this replay re-records them
    GBFE_CUDA(cudaGraphLaunch(w.exec, ctx->stream));
    ctx->launches += w.per_replay;
    if (!w.prof.empty() && ctx->profiling) w.prof_ctx = ctx;
  } else {
    recurrence();
  }
  w.uses++;
  gbfe_mv *last = (degree >= 2 && (degree - 2) % 2 == 0) ? R.get() : RN.get();  // holds the newest iterate
  gbfe_mv *other = last == R.get() ? RN.get() : R.get();
  apply_op(BInv, last, other);
  gbfe_mv *Rfin = other;
  const double *eF2_final = w.tab.p + (size_t)(degree - 1) * m;
  if (mixed) {
    {
      ProfScope prof_k(ctx, "k:cheb_final_mixed", 0.0, 0.0);
      k_cheb_final_mixed<<<sgrid(ctx, n), 256, 0, ctx->stream>>>(n, m, Rfin->f.p, eF2_final, X->d.p, Y->d.p,
                                                                 FastDiv(m));
      check_launch(ctx, "cheb_final_mixed");
    }
  } else {
    d_axpby_blocked(ctx, 1.0, d_ones.p, Rfin, 1.0, eF2_final, X, Y);
  }
  // no host sync: the callers' next operations are ordered on the stream
}

// ------------------------------------------------------------ small host eigensolver
// cyclic Jacobi on a dense symmetric k x k matrix (k <= ~64); eigenvalues ascending
void host_sym_eigvals(std::vector<double> a, int k, std::vector<double> &w) {
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < k; ++p)
      for (int q = p + 1; q < k; ++q) off += a[p * k + q] * a[p * k + q];
    if (off < 1e-30) break;
    for (int p = 0; p < k; ++p)
      for (int q = p + 1; q < k; ++q) {
        const double apq = a[p * k + q];
        if (std::fabs(apq) < 1e-300) continue;
        const double theta = (a[q * k + q] - a[p * k + p]) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double cs = 1.0 / std::sqrt(t * t + 1.0), sn = t * cs;
        for (int r = 0; r < k; ++r) {
          const double arp = a[r * k + p], arq = a[r * k + q];
          a[r * k + p] = cs * arp - sn * arq;
          a[r * k + q] = sn * arp + cs * arq;
        }
        for (int r = 0; r < k; ++r) {
          const double apr = a[p * k + r], aqr = a[q * k + r];
          a[p * k + r] = cs * apr - sn * aqr;
          a[q * k + r] = sn * apr + cs * aqr;
        }
      }
  }
  w.resize(k);
  for (int i = 0; i < k; ++i) w[i] = a[i * k + i];
  std::sort(w.begin(), w.end());
}

// start: the initial vector (n_dofs values, host or device memory), or nullptr
// for a seeded uniform [0, 1) vector (the reference draws std::rand() /
// RAND_MAX per entry, LanczosExtremeEigenSolver.t.cpp:40-52)
void lanczos_impl(const gbfe_op *A, const gbfe_op *B, const gbfe_op *BInv, uint32_t steps, uint64_t seed,
                  double *out3, const double *start = nullptr) {
  gbfe_mesh *me = A->mesh;
  gbfe_ctx *ctx = me->ctx;
  const uint64_t N = me->n_dofs;
  auto x0 = make_mv(me, 1, GBFE_F64), temp = make_mv(me, 1, GBFE_F64), v = make_mv(me, 1, GBFE_F64);
  auto q = make_mv(me, 1, GBFE_F64), qPrev = make_mv(me, 1, GBFE_F64);
  if (start) {
    GBFE_CUDA(cudaMemcpyAsync(x0->d.p, start, N * 8, cudaMemcpyDefault, ctx->stream));
  } else {
    std::vector<double> h(N);
    std::mt19937_64 g(seed);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    for (auto &x : h) x = U(g);
    GBFE_CUDA(cudaMemcpyAsync(x0->d.p, h.data(), N * 8, cudaMemcpyHostToDevice, ctx->stream));
    GBFE_CUDA(cudaStreamSynchronize(ctx->stream));  // h is freed on return
  }
  double alpha = 0.0, beta = 0.0;
  apply_op(B, x0.get(), temp.get());
  host_coldots(ctx, x0.get(), temp.get(), &alpha, false);
  alpha = std::sqrt(alpha);
  d_axpby(ctx, 1.0 / alpha, x0.get(), 0.0, x0.get(), q.get());
  std::vector<double> av, bv;
  for (uint32_t it = 1; it <= steps; ++it) {
    apply_op(A, q.get(), temp.get());
    apply_op(BInv, temp.get(), v.get());
    host_coldots(ctx, q.get(), temp.get(), &alpha, false);
    av.push_back(alpha);
    d_axpby(ctx, 1.0, v.get(), -alpha, q.get(), v.get());
    d_axpby(ctx, 1.0, v.get(), -beta, qPrev.get(), v.get());
    apply_op(B, v.get(), temp.get());
    host_coldots(ctx, v.get(), temp.get(), &beta, false);
    beta = std::sqrt(beta);
    bv.push_back(beta);
    GBFE_CUDA(cudaMemcpyAsync(qPrev->d.p, q->d.p, N * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    if (beta < 1e-14) break;
    d_axpby(ctx, 1.0 / beta, v.get(), 0.0, v.get(), q.get());
  }
  const int k = (int)av.size();
  std::vector<double> T((size_t)k * k, 0.0), w;
  for (int i = 0; i < k; ++i) {
    T[i * k + i] = av[i];
    if (i + 1 < k) T[i * k + i + 1] = T[(i + 1) * k + i] = bv[i];
  }
  host_sym_eigvals(T, k, w);
  out3[0] = w.front();
  out3[1] = w.back();
  out3[2] = bv.back();
}

int residual_norms_impl(const gbfe_op *A, const gbfe_op *B, gbfe_mv *X, const double *eig_h, double *norms_h) {
  gbfe_ctx *ctx = X->mesh->ctx;
  const uint32_t m = X->m;
  auto HX = make_like(X, GBFE_F64), MX = make_like(X, GBFE_F64), Rr = make_like(X, GBFE_F64);
  apply_pair_f64(A, B, X, HX.get(), MX.get());
  std::vector<double> nOnes(m, -1.0);
  DevVec d_no(ctx, m), d_e(ctx, m);
  d_no.set(ctx, nOnes.data(), m);
  d_e.set(ctx, eig_h, m);
  d_axpby_blocked(ctx, 1.0, d_no.p, HX.get(), 1.0, d_e.p, MX.get(), Rr.get());
  host_coldots(ctx, Rr.get(), Rr.get(), norms_h, true);
  return GBFE_OK;
}

int chfsi_pass_impl(const gbfe_op *A, const gbfe_op *B, const gbfe_op *BInv, gbfe_mv *X, double *eig_h,
                    uint32_t degree, double wl, double wu, double uu, int prec, std::string &msg) {
  auto Yf = make_like(X, GBFE_F64), Xo = make_like(X, GBFE_F64);
  residual_filter(A, B, BInv, eig_h, X, degree, wl, wu, uu, Yf.get(), prec);
  int rc = cholesky_gs_impl(B, Yf.get(), Xo.get(), msg);
  if (rc != GBFE_OK) return rc;
  return rayleigh_ritz_impl(A, Xo.get(), eig_h, X, msg);
}


// ------------------------------------------------------------ fused KS pass
// One ChFSI pass with two FP64 operator applies:
//   Y    = filter(residual R, Ritz vectors X)           (d-1 A applies, mixed or FP64)
//   MY   = B Y,  HY = A Y                               (FP64)
//   S_M  = Y^T MY = L L^T,   S_H = Y^T HY
//   Hp   = L^-1 S_H L^-T = V diag(eps) V^T              (syevd, FP64)
//   T    = L^-T V;   X = Y T,  HX = HY T,  MX = MY T
//   R    = HX - MX diag(eps)                            (next pass's filter input)
// (with the sliced products, X and R come from one launch: R = [HY | MY]
// [T; -T diag(eps)], and HX, MX are never stored)
// This is the reference's filter -> Cholesky-GS -> Rayleigh-Ritz -> residual
// sequence (ChebyshevFilteredEigenSolver.t.cpp:194-437,
// KohnShamEigenSolver.t.cpp:574-684) with H X and M X carried through the
// m x m rotations instead of re-applied.
struct FusedState {
  std::unique_ptr<gbfe_mv> Y, MY, HY, HX, MX, R;
  DBuf<double> SM, SH, V;
  FilterWork fw;
};

int fused_pass(const gbfe_op *A, const gbfe_op *B, const gbfe_op *BInv, gbfe_mv *X, double *eig_h,
               uint32_t degree, double wl, double wu, double uu, int prec, FusedState &st, double *res_h,
               std::string &msg) {
  gbfe_ctx *ctx = X->mesh->ctx;
  const int m = (int)X->m;
  const int N = (int)X->mesh->n_dofs;
  ProfScope prof_pass(ctx, "pass_total", 0.0, 0.0);
  {
    ProfScope prof(ctx, "pass_filter", 0.0, 0.0);
    residual_filter(A, B, BInv, eig_h, X, degree, wl, wu, uu, st.Y.get(), prec, st.R.get(), &st.fw);
  }
  {
    ProfScope prof(ctx, "pass_fp64_applies", 0.0, 0.0);
    apply_pair_f64(A, B, st.Y.get(), st.HY.get(), st.MY.get());
  }
  // FP64 Gram matrices and rotations: the sliced tensor-core products when
  // the FP64 applies use them, else DGEMM
  const bool oz_dense = ctx->fp64_tc && ctx->fp64_tc_dense && oz_gemm_supported(ctx, (uint32_t)m);
  // the host pool's workers wake while the device forms the Gram matrices and
  // sleep again after the m x m block
  struct PoolArm {
    bool on;
    explicit PoolArm(bool o) : on(o) {
      if (on) host_pool_arm(true);
    }
    ~PoolArm() {
      if (on) host_pool_arm(false);
    }
  } pool_arm(ctx->small_eig_host && m <= SMALL_EIG_HOST_MAX);
  if (oz_dense) {
    // S = (MY|HY)^T Y: the transposes of Y^T MY and Y^T HY (both symmetric)
    const double *As[2] = {st.MY->d.p, st.HY->d.p};
    double *Ss[2] = {st.SM.p, st.SH.p};
    // the sliced apply of A on Y left Y's column exponents with A
    const int *yexp = (A->oz_aoff.p && A->oz_xexp.p && A->oz_xexp.n >= (size_t)m) ? A->oz_xexp.p : nullptr;
    oz_gram(ctx, As, 2, (uint32_t)m, st.Y->d.p, (uint32_t)m, (uint64_t)N, Ss, yexp);
  } else {
    ProfScope prof(ctx, "gram_f64_dgemm", 4.0 * (double)N * m * m, 24.0 * (double)N * m);
    gram(ctx, st.Y.get(), st.MY.get(), st.SM.p);
    gram(ctx, st.Y.get(), st.HY.get(), st.SH.p);
  }
  const double *rot_in[3] = {st.Y->d.p, st.HY->d.p, st.MY->d.p};
  bool rows_ready = false;
  // X and the residual R straight from Y, HY, MY (the rotated HY, MY are not kept)
  const bool oz_resid = oz_dense && oz_rotate_residual_supported(ctx, (uint32_t)m);
  // the context stream waits for the side stream's work once armed
  struct SideJoin {
    gbfe_ctx *ctx;
    bool armed = false;
    void join() {
      if (armed) cudaStreamWaitEvent(ctx->stream, ctx->join_ev, 0);
      armed = false;
    }
    ~SideJoin() { join(); }
  } side_join{ctx};
  // potrf, L^-1 S_H L^-T, syevd, L^-T V: the m x m stages, timed as one block
  auto eig_prof = std::make_unique<ProfScope>(ctx, "eig_small_f64", 0.0, 0.0);
  const bool host_eig = ctx->small_eig_host && m <= SMALL_EIG_HOST_MAX;
  const char *chol_fail = "Chol GS cannot orthogonalize the given multivector (near-zero diagonal of L)";
  if (host_eig) {
    // the whole block on one host core after one download: the FP64 library
    // kernels for 64 x 64 factors and solves run on one SM's FP64 pipe and
    // take longer than the host (and each adds a launch)
    std::vector<double> hL((size_t)m * m), hS((size_t)m * m);
    GBFE_CUDA(cudaMemcpyAsync(hL.data(), st.SM.p, hL.size() * 8, cudaMemcpyDeviceToHost, ctx->stream));
    GBFE_CUDA(cudaMemcpyAsync(hS.data(), st.SH.p, hS.size() * 8, cudaMemcpyDeviceToHost, ctx->stream));
    if (!ctx->host_ev) GBFE_CUDA(cudaEventCreateWithFlags(&ctx->host_ev, cudaEventDisableTiming));
    GBFE_CUDA(cudaEventRecord(ctx->host_ev, ctx->stream));
    // the row exponents of the rotation inputs run on the device while the
    // host works on the m x m block (the host waits for the download only)
    if (oz_dense) {
      oz_rotate_rows(ctx, rot_in, (uint32_t)m, 3, (uint64_t)N, oz_resid);
      rows_ready = true;
    }
    GBFE_CUDA(cudaEventSynchronize(ctx->host_ev));
    const int info = host_cholesky(m, hL.data());
    if (info != 0) {
      msg = "LAPACK_ERROR: FAILED_CHOLESKY_FACTORIZATION (potrf info " + std::to_string(info) + ")";
      return GBFE_ERR_LAPACK;
    }
    for (int i = 0; i < m; ++i)
      if (std::fabs(hL[(size_t)i * m + i]) < 1e-14) {
        msg = chol_fail;
        return GBFE_ERR_NOT_ORTHONORMALIZABLE;
      }
    host_sandwich(m, hL.data(), hS.data());
    if (host_sym_eig(m, hS.data(), eig_h) != 0) {
      msg = "LAPACK_ERROR: FAILED_STANDARD_EIGENPROBLEM (QR iteration did not converge)";
      return GBFE_ERR_LAPACK;
    }
    host_trsm_lower_t(m, hL.data(), hS.data());  // T = L^-T V
    host_pool_arm(false);
    pool_arm.on = false;
    h2d_staged(ctx, ctx->pin_small, st.SH.p, hS.data(), hS.size() * 8);
  } else {
    // the row digits of the rotation inputs depend on Y, HY, MY only: they are
    // cut on the side stream while cuSOLVER works through the m x m block
    // (short launches that leave most SMs idle); the guard joins the side
    // stream back on every way out of this block
    if (oz_dense && !ctx->profiling) {
      ensure_side_stream(ctx);
      GBFE_CUDA(cudaEventRecord(ctx->fork_ev, ctx->stream));
      GBFE_CUDA(cudaStreamWaitEvent(ctx->side_stream, ctx->fork_ev, 0));
      oz_rotate_rows(ctx, rot_in, (uint32_t)m, 3, (uint64_t)N, oz_resid, ctx->side_stream);
      GBFE_CUDA(cudaEventRecord(ctx->join_ev, ctx->side_stream));
      side_join.armed = true;
      rows_ready = true;
    }
    int lwork = 0;
    GBFE_CUSOLVER(cusolverDnDpotrf_bufferSize(ctx->cusolver, CUBLAS_FILL_MODE_LOWER, m, st.SM.p, m, &lwork));
    ctx->lwork.ensure(std::max(lwork, 1));
    ctx->info.ensure(1);
    GBFE_CUSOLVER(cusolverDnDpotrf(ctx->cusolver, CUBLAS_FILL_MODE_LOWER, m, st.SM.p, m, ctx->lwork.p, lwork,
                                   ctx->info.p));
    count_launch(ctx);
    int info = 0;
    std::vector<double> hL((size_t)m * m);
    GBFE_CUDA(cudaMemcpyAsync(&info, ctx->info.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    GBFE_CUDA(cudaMemcpyAsync(hL.data(), st.SM.p, hL.size() * 8, cudaMemcpyDeviceToHost, ctx->stream));
    GBFE_CUDA(cudaStreamSynchronize(ctx->stream));
    if (info != 0) {
      msg = "LAPACK_ERROR: FAILED_CHOLESKY_FACTORIZATION (potrf info " + std::to_string(info) + ")";
      return GBFE_ERR_LAPACK;
    }
    for (int i = 0; i < m; ++i)
      if (std::fabs(hL[(size_t)i * m + i]) < 1e-14) {
        msg = chol_fail;
        return GBFE_ERR_NOT_ORTHONORMALIZABLE;
      }
    const double one = 1.0;
    // Hp = L^-1 S_H L^-T
    GBFE_CUBLAS(cublasDtrsm(ctx->cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT,
                            m, m, &one, st.SM.p, m, st.SH.p, m));
    GBFE_CUBLAS(cublasDtrsm(ctx->cublas, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T, CUBLAS_DIAG_NON_UNIT,
                            m, m, &one, st.SM.p, m, st.SH.p, m));
    count_launch(ctx, 2);
    const int rc = small_syevd(ctx, m, st.SH.p, eig_h, msg);
    if (rc != GBFE_OK) return rc;
    // T = L^-T V (in place in SH)
    GBFE_CUBLAS(cublasDtrsm(ctx->cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T, CUBLAS_DIAG_NON_UNIT,
                            m, m, &one, st.SM.p, m, st.SH.p, m));
    count_launch(ctx);
  }
  eig_prof.reset();
  side_join.join();
  const double *T = st.SH.p;
  std::vector<double> nOnes(m, -1.0);
  DevVec d_no(ctx, m), d_e(ctx, m);
  d_e.set(ctx, eig_h, m);
  if (oz_resid) {
    oz_rotate_residual(ctx, T, d_e.p, (uint32_t)m, st.Y->d.p, st.HY->d.p, st.MY->d.p, X->d.p, st.R->d.p,
                       (uint64_t)N, rows_ready);
    host_coldots(ctx, st.R.get(), st.R.get(), res_h, true);
    return GBFE_OK;
  }
  if (oz_dense) {
    double *out[3] = {X->d.p, st.HX->d.p, st.MX->d.p};
    oz_rotate(ctx, T, (uint32_t)m, (uint32_t)m, rot_in, out, 3, (uint64_t)N, rows_ready);
  } else {
    ProfScope prof(ctx, "rotate_f64_dgemm", 6.0 * (double)N * m * m, 48.0 * (double)N * m);
    const double one = 1.0, zero = 0.0;
    // rows times T: col-major (m x N) out = T^T * in
    GBFE_CUBLAS(
        cublasDgemm(ctx->cublas, CUBLAS_OP_T, CUBLAS_OP_N, m, N, m, &one, T, m, st.Y->d.p, m, &zero, X->d.p, m));
    GBFE_CUBLAS(cublasDgemm(ctx->cublas, CUBLAS_OP_T, CUBLAS_OP_N, m, N, m, &one, T, m, st.HY->d.p, m, &zero,
                            st.HX->d.p, m));
    GBFE_CUBLAS(cublasDgemm(ctx->cublas, CUBLAS_OP_T, CUBLAS_OP_N, m, N, m, &one, T, m, st.MY->d.p, m, &zero,
                            st.MX->d.p, m));
    count_launch(ctx, 3);
  }
  d_no.set(ctx, nOnes.data(), m);
  // R = HX - MX diag(eps)   (getLinearEigenSolveResidual's axpbyBlocked with the sign flipped)
  d_axpby_blocked(ctx, -1.0, d_no.p, st.HX.get(), -1.0, d_e.p, st.MX.get(), st.R.get());
  host_coldots(ctx, st.R.get(), st.R.get(), res_h, true);
  return GBFE_OK;
}

int ks_solve_fused(const gbfe_op *A, const gbfe_op *B, const gbfe_op *BInv, gbfe_mv *X, const gbfe_ks_params *prm,
                   double wl, double wu, double uu, double *eig_h, double *res_h, uint32_t *passes_out,
                   std::string &msg) {
  gbfe_ctx *ctx = X->mesh->ctx;
  const uint32_t m = X->m;
  FusedState st;
  st.Y = make_like(X, GBFE_F64);
  st.MY = make_like(X, GBFE_F64);
  st.HY = make_like(X, GBFE_F64);
  st.HX = make_like(X, GBFE_F64);
  st.MX = make_like(X, GBFE_F64);
  st.R = make_like(X, GBFE_F64);
  st.SM.alloc((size_t)m * m);
  st.SH.alloc((size_t)m * m);
  // initial residual of the input block: R = A X - Lambda B X
  apply_pair_f64(A, B, X, st.HX.get(), st.MX.get());
  {
    std::vector<double> ones(m, 1.0);
    DevVec d_o(ctx, m), d_e(ctx, m);
    d_o.set(ctx, ones.data(), m);
    d_e.set(ctx, eig_h, m);
    d_axpby_blocked(ctx, 1.0, d_o.p, st.HX.get(), -1.0, d_e.p, st.MX.get(), st.R.get());
    GBFE_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  int status = GBFE_ERR_NOT_CONVERGED;
  uint32_t pass = 0;
  for (; pass < prm->max_passes; ++pass) {
    if (ctx->cancel && ctx->cancel->load()) {
      status = GBFE_ERR_CANCELLED;
      msg = "cancelled";
      break;
    }
    const int r = fused_pass(A, B, BInv, X, eig_h, prm->degree, wl, wu, uu, prm->filter_precision, st, res_h, msg);
    if (r != GBFE_OK) {
      status = r;
      break;
    }
    bool conv = true;
    for (uint32_t i = 0; i < prm->n_wanted; ++i) conv &= res_h[i] <= prm->residual_tol;
    if (conv && !prm->fixed_passes) {
      status = GBFE_OK;
      ++pass;
      break;
    }
    if (prm->fixed_passes && pass + 1 == prm->max_passes) status = conv ? GBFE_OK : GBFE_ERR_NOT_CONVERGED;
    wl = eig_h[0];
    wu = eig_h[m - 1];
  }
  if (passes_out) *passes_out = pass;
  return status;
}
}  // namespace

namespace gbfe {
void axpby(gbfe_ctx *ctx, size_t, double a, const gbfe_mv *x, double b, const gbfe_mv *y, gbfe_mv *z) {
  d_axpby(ctx, a, x, b, y, z);
}
void col_dots(gbfe_ctx *ctx, const gbfe_mv *x, const gbfe_mv *y, double *host_out) {
  host_coldots(ctx, x, y, host_out, false);
}
}  // namespace gbfe

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
#define CTX_OF(obj) ((obj)->mesh->ctx)

extern "C" {

int gbfe_mv_l2_norms(const gbfe_mv *mv, double *norms_host) {
  if (!mv || !norms_host) return GBFE_ERR_ARG;
  return gbfe_guard(CTX_OF(mv), [&] { host_coldots(CTX_OF(mv), mv, mv, norms_host, true); });
}

int gbfe_mv_dots(const gbfe_mv *x, const gbfe_mv *y, double *dots_host) {
  if (!x || !y || !dots_host) return GBFE_ERR_ARG;
  return gbfe_guard(CTX_OF(x), [&] {
    GBFE_REQUIRE(x->mesh == y->mesh && x->m == y->m && x->dtype == y->dtype, "mv_dots: shape mismatch");
    host_coldots(CTX_OF(x), x, y, dots_host, false);
  });
}

int gbfe_residual_chebyshev_filter(const gbfe_op *A, const gbfe_op *B, const gbfe_op *BInv, const double *eigenvalues,
                                   gbfe_mv *X, uint32_t degree, double wl, double wu, double uu, int precision,
                                   gbfe_mv *Y) {
  if (!A || !B || !BInv || !eigenvalues || !X || !Y) return GBFE_ERR_ARG;
  return gbfe_guard(CTX_OF(X), [&] {
    GBFE_REQUIRE(X->dtype == GBFE_F64 && Y->dtype == GBFE_F64, "filter: X and Y must be FP64 block vectors");
    GBFE_REQUIRE(X->m == Y->m && X->mesh == Y->mesh, "filter: shape mismatch");
    GBFE_REQUIRE(degree >= 1, "filter: degree must be >= 1");
    residual_filter(A, B, BInv, eigenvalues, X, degree, wl, wu, uu, Y, precision);
    GBFE_CUDA(cudaStreamSynchronize(CTX_OF(X)->stream));
  });
}

int gbfe_chebyshev_filter(const gbfe_op *A, const gbfe_op *BInv, gbfe_mv *X, uint32_t degree, double wl, double wu,
                          double uu, gbfe_mv *Y) {
  if (!A || !BInv || !X || !Y) return GBFE_ERR_ARG;
  gbfe_ctx *ctx = CTX_OF(X);
  return gbfe_guard(ctx, [&] {
    GBFE_REQUIRE(X->dtype == GBFE_F64 && Y->dtype == GBFE_F64 && X->m == Y->m, "filter: shape mismatch");
    const double e = 0.5 * (uu - wu), c = 0.5 * (uu + wu);
    double sigma = e / (wl - c);
    const double sigma1 = sigma, gamma = 2.0 / sigma1;
    auto s1 = make_like(X, GBFE_F64), s2 = make_like(X, GBFE_F64);
    auto bufA = make_like(X, GBFE_F64), bufB = make_like(X, GBFE_F64);
    GBFE_CUDA(cudaMemcpyAsync(bufA->d.p, X->d.p, X->count() * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    gbfe_mv *guess = bufA.get(), *filt = bufB.get();
    apply_op(A, guess, s1.get());
    apply_op(BInv, s1.get(), s2.get());
    d_axpby(ctx, sigma1 / e, s2.get(), -sigma1 / e * c, guess, filt);
    for (uint32_t deg = 2; deg <= degree; ++deg) {
      const double sigma2 = 1.0 / (gamma - sigma);
      apply_op(A, filt, s1.get());
      apply_op(BInv, s1.get(), s2.get());
      d_axpby(ctx, 2.0 * sigma2 / e, s2.get(), -2.0 * sigma2 / e * c, filt, s1.get());
      d_axpby(ctx, 1.0, s1.get(), -sigma * sigma2, guess, guess);
      std::swap(guess, filt);
      sigma = sigma2;
    }
    // the swap moves storage, so the newest iterate is `filt`; the reference
    // then copies it into eigenSubspaceGuess as well
    GBFE_CUDA(cudaMemcpyAsync(Y->d.p, filt->d.p, X->count() * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    GBFE_CUDA(cudaMemcpyAsync(X->d.p, filt->d.p, X->count() * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    GBFE_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

int gbfe_cholesky_gram_schmidt(const gbfe_op *B, gbfe_mv *X, gbfe_mv *X_ortho) {
  if (!B || !X || !X_ortho) return GBFE_ERR_ARG;
  gbfe_ctx *ctx = CTX_OF(X);
  int status = GBFE_OK;
  int rc = gbfe_guard(ctx, [&] {
    GBFE_REQUIRE(X->dtype == GBFE_F64 && X_ortho->dtype == GBFE_F64 && X->m == X_ortho->m, "ortho: shape mismatch");
    std::string msg;
    status = cholesky_gs_impl(B, X, X_ortho, msg);
    if (status != GBFE_OK) ctx->last_error = msg;
    GBFE_CUDA(cudaStreamSynchronize(ctx->stream));
  });
  return rc != GBFE_OK ? rc : status;
}

int gbfe_rayleigh_ritz(const gbfe_op *A, gbfe_mv *X, double *eigenvalues_host, gbfe_mv *X_out) {
  if (!A || !X || !eigenvalues_host || !X_out) return GBFE_ERR_ARG;
  gbfe_ctx *ctx = CTX_OF(X);
  int status = GBFE_OK;
  int rc = gbfe_guard(ctx, [&] {
    GBFE_REQUIRE(X->dtype == GBFE_F64 && X_out->dtype == GBFE_F64 && X->m == X_out->m, "RR: shape mismatch");
    GBFE_REQUIRE(X != X_out, "RR: X and X_out must be distinct");
    std::string msg;
    status = rayleigh_ritz_impl(A, X, eigenvalues_host, X_out, msg);
    if (status != GBFE_OK) ctx->last_error = msg;
    GBFE_CUDA(cudaStreamSynchronize(ctx->stream));
  });
  return rc != GBFE_OK ? rc : status;
}

int gbfe_mv_gram(const gbfe_mv *X, const gbfe_mv *Y, double *S_host) {
  if (!X || !Y || !S_host) return GBFE_ERR_ARG;
  gbfe_ctx *ctx = CTX_OF(X);
  return gbfe_guard(ctx, [&] {
    GBFE_REQUIRE(X->mesh == Y->mesh && X->dtype == GBFE_F64 && Y->dtype == GBFE_F64,
                 "gram: X and Y must be FP64 blocks of one mesh");
    const uint32_t mx = X->m, my = Y->m;
    ctx->small.ensure((size_t)mx * my);
    if (ctx->fp64_tc && ctx->fp64_tc_dense && oz_gemm_supported(ctx, mx)) {
      const double *As[1] = {X->d.p};
      double *Ss[1] = {ctx->small.p};
      oz_gram(ctx, As, 1, mx, Y->d.p, my, X->mesh->n_dofs, Ss);
    } else {
      const double one = 1.0, zero = 0.0;
      GBFE_CUBLAS(cublasDgemm(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_T, (int)mx, (int)my, (int)X->mesh->n_dofs, &one,
                              X->d.p, (int)mx, Y->d.p, (int)my, &zero, ctx->small.p, (int)mx));
      count_launch(ctx);
    }
    GBFE_CUDA(cudaMemcpyAsync(S_host, ctx->small.p, (size_t)mx * my * 8, cudaMemcpyDeviceToHost, ctx->stream));
    GBFE_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

int gbfe_mv_rotate(const gbfe_mv *X, const double *T_host, gbfe_mv *Y) {
  if (!X || !T_host || !Y) return GBFE_ERR_ARG;
  gbfe_ctx *ctx = CTX_OF(X);
  return gbfe_guard(ctx, [&] {
    GBFE_REQUIRE(X->mesh == Y->mesh && X->dtype == GBFE_F64 && Y->dtype == GBFE_F64 && X != Y,
                 "rotate: X and Y must be distinct FP64 blocks of one mesh");
    const uint32_t m = X->m, mo = Y->m;
    DBuf<double> T;
    T.upload(T_host, (size_t)m * mo, ctx->stream);
    if (ctx->fp64_tc && ctx->fp64_tc_dense && oz_gemm_supported(ctx, m)) {
      const double *in[1] = {X->d.p};
      double *out[1] = {Y->d.p};
      oz_rotate(ctx, T.p, m, mo, in, out, 1, X->mesh->n_dofs);
    } else {
      const double one = 1.0, zero = 0.0;
      GBFE_CUBLAS(cublasDgemm(ctx->cublas, CUBLAS_OP_T, CUBLAS_OP_N, (int)mo, (int)X->mesh->n_dofs, (int)m, &one,
                              T.p, (int)m, X->d.p, (int)m, &zero, Y->d.p, (int)mo));
      count_launch(ctx);
    }
    GBFE_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

int gbfe_eigen_residual_norms(const gbfe_op *A, const gbfe_op *B, gbfe_mv *X, const double *eigenvalues,
                              double *norms_host) {
  if (!A || !B || !X || !eigenvalues || !norms_host) return GBFE_ERR_ARG;
  return gbfe_guard(CTX_OF(X), [&] {
    GBFE_REQUIRE(X->dtype == GBFE_F64, "residual: X must be FP64");
    residual_norms_impl(A, B, X, eigenvalues, norms_host);
  });
}

int gbfe_chfsi_pass(const gbfe_op *A, const gbfe_op *B, const gbfe_op *BInv, gbfe_mv *X, double *eigenvalues,
                    uint32_t degree, double wl, double wu, double uu, int filter_precision) {
  if (!A || !B || !BInv || !X || !eigenvalues) return GBFE_ERR_ARG;
  gbfe_ctx *ctx = CTX_OF(X);
  int status = GBFE_OK;
  int rc = gbfe_guard(ctx, [&] {
    GBFE_REQUIRE(X->dtype == GBFE_F64, "chfsi: X must be FP64");
    std::string msg;
    status = chfsi_pass_impl(A, B, BInv, X, eigenvalues, degree, wl, wu, uu, filter_precision, msg);
    if (status != GBFE_OK) ctx->last_error = msg;
    GBFE_CUDA(cudaStreamSynchronize(ctx->stream));
  });
  return rc != GBFE_OK ? rc : status;
}

int gbfe_lanczos_bounds(const gbfe_op *A, const gbfe_op *B, const gbfe_op *BInv, uint32_t steps, uint64_t seed,
                        double *out3) {
  if (!A || !B || !BInv || !out3) return GBFE_ERR_ARG;
  return gbfe_guard(A->mesh->ctx, [&] {
    GBFE_REQUIRE(steps >= 2, "lanczos: need at least 2 steps");
    lanczos_impl(A, B, BInv, steps, seed, out3);
  });
}

int gbfe_lanczos_bounds_from(const gbfe_op *A, const gbfe_op *B, const gbfe_op *BInv, uint32_t steps,
                             const double *start, double *out3) {
  if (!A || !B || !BInv || !start || !out3) return GBFE_ERR_ARG;
  return gbfe_guard(A->mesh->ctx, [&] {
    GBFE_REQUIRE(steps >= 2, "lanczos: need at least 2 steps");
    lanczos_impl(A, B, BInv, steps, 0, out3, start);
  });
}

int gbfe_ks_eigen_solve(const gbfe_op *A, const gbfe_op *B, const gbfe_op *BInv, gbfe_mv *X,
                        const gbfe_ks_params *prm, double *eigenvalues, double *residuals, uint32_t *passes_out) {
  if (!A || !B || !BInv || !X || !prm || !eigenvalues || !residuals) return GBFE_ERR_ARG;
  gbfe_ctx *ctx = CTX_OF(X);
  int status = GBFE_OK;
  int rc = gbfe_guard(ctx, [&] {
    GBFE_REQUIRE(X->dtype == GBFE_F64, "ks solve: X must be FP64");
    const uint32_t m = X->m;
    GBFE_REQUIRE(prm->n_wanted >= 1 && prm->n_wanted <= m, "ks solve: n_wanted must be in [1, m]");
    double wl = prm->wanted_lower, wu = prm->wanted_upper, uu = prm->unwanted_upper;
    if (prm->use_lanczos) {
      double b3[3];
      lanczos_impl(A, B, BInv, prm->lanczos_steps ? prm->lanczos_steps : 20, prm->lanczos_seed, b3,
                   prm->lanczos_start);
      const double res = b3[2] / 10.0;  // KohnShamEigenSolver.t.cpp:270-273
      wl = b3[0];
      uu = b3[1] + res;
      wu = (b3[1] + res - b3[0]) * ((double)m * 200.0 / (double)X->mesh->n_dofs) + b3[0];
      if (wu >= uu) wu = (uu + b3[0]) * 0.5;
    }
    uint32_t pass = 0;
    std::string msg;
    struct Restore {
      gbfe_ctx *c;
      int tc, dense;
      ~Restore() {
        c->fp64_tc = tc;
        c->fp64_tc_dense = dense;
      }
    } restore{ctx, ctx->fp64_tc, ctx->fp64_tc_dense};
    ctx->fp64_tc = prm->fp64_apply ? 1 : 0;
    ctx->fp64_tc_dense = prm->fp64_apply == 1 ? 1 : 0;
    if (!prm->faithful_passes) {
      status = ks_solve_fused(A, B, BInv, X, prm, wl, wu, uu, eigenvalues, residuals, passes_out, msg);
      if (status != GBFE_OK) ctx->last_error = msg.empty() ? "KS_MAX_PASS_ERROR: residual tolerance not reached" : msg;
      GBFE_CUDA(cudaStreamSynchronize(ctx->stream));
      return;
    }
    status = GBFE_ERR_NOT_CONVERGED;
    for (; pass < prm->max_passes; ++pass) {
      int r = chfsi_pass_impl(A, B, BInv, X, eigenvalues, prm->degree, wl, wu, uu, prm->filter_precision, msg);
      if (r != GBFE_OK) {
        status = r;
        ctx->last_error = msg;
        break;
      }
      residual_norms_impl(A, B, X, eigenvalues, residuals);
      bool conv = true;
      for (uint32_t i = 0; i < prm->n_wanted; ++i) conv &= residuals[i] <= prm->residual_tol;
      if (conv && !prm->fixed_passes) {
        status = GBFE_OK;
        ++pass;
        break;
      }
      if (prm->fixed_passes && pass + 1 == prm->max_passes) status = conv ? GBFE_OK : GBFE_ERR_NOT_CONVERGED;
      wl = eigenvalues[0];
      wu = eigenvalues[m - 1];
    }
    if (status == GBFE_ERR_NOT_CONVERGED) ctx->last_error = "KS_MAX_PASS_ERROR: residual tolerance not reached";
    if (passes_out) *passes_out = pass;
    GBFE_CUDA(cudaStreamSynchronize(ctx->stream));
  });
  return rc != GBFE_OK ? rc : status;
}

int gbfe_cg_solve(const gbfe_op *A, const gbfe_op *PC, const gbfe_mv *b, gbfe_mv *x, uint32_t max_iter,
                  double abs_tol, double rel_tol, double div_tol, uint32_t *iters_out, double *rnorm_host) {
  if (!A || !PC || !b || !x) return GBFE_ERR_ARG;
  gbfe_ctx *ctx = CTX_OF(x);
  int status = GBFE_OK;
  int rc = gbfe_guard(ctx, [&] {
    GBFE_REQUIRE(b->dtype == GBFE_F64 && x->dtype == GBFE_F64 && b->m == x->m && b->mesh == x->mesh,
                 "cg: shape mismatch");
    const uint32_t k = b->m;
    auto xw = make_like(x, GBFE_F64), xc = make_like(x, GBFE_F64), r = make_like(x, GBFE_F64);
    auto w = make_like(x, GBFE_F64), z = make_like(x, GBFE_F64), p = make_like(x, GBFE_F64);
    const size_t bytes = x->count() * 8;
    GBFE_CUDA(cudaMemcpyAsync(xw->d.p, x->d.p, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    GBFE_CUDA(cudaMemcpyAsync(xc->d.p, x->d.p, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    std::vector<double> bn(k), rn(k), zr(k), pw(k), zrn(k), ones(k, 1.0), nones(k, -1.0), coef(k);
    std::vector<char> conv(k, 0);
    host_coldots(ctx, b, b, bn.data(), true);
    DevVec d_ones(ctx, k), d_nones(ctx, k), d_coef(ctx, k);
    d_ones.set(ctx, ones.data(), k);
    d_nones.set(ctx, nones.data(), k);
    bool diverge = false, all = false;
    status = 99;
    uint32_t iter = 0;
    for (; iter <= max_iter; ++iter) {
      if (ctx->cancel && ctx->cancel->load()) {
        status = GBFE_ERR_CANCELLED;
        break;
      }
      if (iter == 0) {
        apply_op(A, xw.get(), w.get());
        d_axpby_blocked(ctx, 1.0, d_ones.p, b, 1.0, d_nones.p, w.get(), r.get());
        apply_op(PC, r.get(), z.get());
        GBFE_CUDA(cudaMemcpyAsync(p->d.p, z->d.p, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
      } else {
        apply_op(A, p.get(), w.get());
        host_coldots(ctx, z.get(), r.get(), zr.data(), false);
        host_coldots(ctx, p.get(), w.get(), pw.data(), false);
        for (uint32_t j = 0; j < k; ++j) coef[j] = zr[j] / pw[j];
        d_coef.set(ctx, coef.data(), k);
        d_axpby_blocked(ctx, 1.0, d_ones.p, xw.get(), 1.0, d_coef.p, p.get(), xw.get());
        GBFE_CUDA(cudaStreamSynchronize(ctx->stream));
        for (uint32_t j = 0; j < k; ++j) coef[j] = -zr[j] / pw[j];
        d_coef.set(ctx, coef.data(), k);
        d_axpby_blocked(ctx, 1.0, d_ones.p, r.get(), 1.0, d_coef.p, w.get(), r.get());
        apply_op(PC, r.get(), z.get());
        host_coldots(ctx, z.get(), r.get(), zrn.data(), false);
        for (uint32_t j = 0; j < k; ++j) coef[j] = zrn[j] / zr[j];
        d_coef.set(ctx, coef.data(), k);
        d_axpby_blocked(ctx, 1.0, d_ones.p, z.get(), 1.0, d_coef.p, p.get(), p.get());
      }
      host_coldots(ctx, r.get(), r.get(), rn.data(), true);
      for (uint32_t j = 0; j < k; ++j) {
        const double tol = std::max(abs_tol, bn[j] * rel_tol);
        if (rn[j] < tol && !conv[j]) {
          status = GBFE_OK;
          conv[j] = 1;
          // copy column j of xw into xc
          GBFE_CUDA(cudaMemcpy2DAsync(xc->d.p + j, (size_t)k * 8, xw->d.p + j, (size_t)k * 8, 8, x->mesh->n_dofs,
                                      cudaMemcpyDeviceToDevice, ctx->stream));
        }
        if (rn[j] > div_tol && !diverge) {
          status = GBFE_ERR_DIVERGED;
          diverge = true;
        }
      }
      all = std::all_of(conv.begin(), conv.end(), [](char c) { return c != 0; });
      if (diverge || all) break;
    }
    if (iter > max_iter && status != GBFE_ERR_CANCELLED) status = GBFE_ERR_NOT_CONVERGED;
    if (status == 99) status = GBFE_ERR_NOT_CONVERGED;
    GBFE_CUDA(cudaMemcpyAsync(x->d.p, xc->d.p, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    GBFE_CUDA(cudaStreamSynchronize(ctx->stream));
    if (iters_out) *iters_out = iter;
    if (rnorm_host) std::copy(rn.begin(), rn.end(), rnorm_host);
    if (status == GBFE_ERR_NOT_CONVERGED) ctx->last_error = "FAILED_TO_CONVERGE";
    if (status == GBFE_ERR_DIVERGED) ctx->last_error = "RESIDUAL_DIVERGENCE";
    if (status == GBFE_ERR_CANCELLED) ctx->last_error = "cancelled";
  });
  return rc != GBFE_OK ? rc : status;
}

}  // extern "C"
