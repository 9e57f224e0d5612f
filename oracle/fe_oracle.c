/*
 * fe_oracle.c -- CPU oracle for the cellwise FE operator apply path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is a plain-C restatement of the
 * reference (dft-efe) algorithms on the ChFSI / Poisson hot path.  It is the
 * checker the parity tests compare the CUDA path against, and the CPU
 * baseline that bench.py times; the product library never links or calls it.
 *
 * What is restated, with the reference location each routine follows:
 *   orc_p2c      basis/ConstraintsInternal.cpp:37-107
 *                (constraintsDistributeParentToChild: x_r = inh_r + sum w x_c)
 *   orc_c2p      basis/ConstraintsInternal.cpp:112-170
 *                (constraintsDistributeChildToParent: x_c += w x_r; x_r = 0)
 *   orc_apply    ksdft/KohnShamOperatorContextFE.t.cpp:1326-1443 with
 *                computeAxCellWiseLocal :766-949, the gather of
 *                basis/FECellWiseDataOperations.t.cpp:31-84, the per-cell
 *                gemm of linearAlgebra/BlasLapack.t.cpp:391-436
 *                (C(m x nd) = Xc(m x nd, ld m) * Hc(nd x nd, ld nd), 'N','N')
 *                and the scatter of FECellWiseDataOperations.t.cpp:87-151;
 *                the same structure is CFEOverlapOperatorContext.t.cpp:587-640
 *                and LaplaceOperatorContextFE.t.cpp:397-467.
 *   orc_apply with a nonlocal part (orc_nl)
 *                the fused Kohn-Sham apply with an ONCV component,
 *                ksdft/KohnShamOperatorContextFE.t.cpp:1022-1080, :1177-1180:
 *                CX = sum_c scatter(Xc * C_c^T) (gemm 'N','C', beta 0), CX *= V,
 *                then per cell Yc = Xc * H_c and Yc += CXc * C_c (gemm
 *                'N','N', beta 1) before the scatter -- the member functions
 *                of basis/AtomCenterNonLocalOpContextFE.t.cpp:883-1045 and
 *                the cellWiseGEMM of :43-152.  Without cell matrices (mats =
 *                NULL) it is the standalone AtomCenterNonLocalOpContextFE::apply
 *                (:715-849).
 *   orc_apply (diagonal kind)
 *                basis/CFEOverlapInverseOpContextGLL.t.cpp:528-559
 *                (p2c, Y = d o X, c2p) and, without constraints,
 *                linearAlgebra/PreconditionerJacobi.t.cpp:56-80.
 *   orc_residual_chebyshev_filter
 *                linearAlgebra/ChebyshevFilter.t.cpp:242-444
 *   orc_chebyshev_filter
 *                linearAlgebra/ChebyshevFilter.t.cpp:39-135
 *   orc_cg       linearAlgebra/CGLinearSolver.t.cpp:68-313
 *   orc_sweep    one column-scaled sweep z = a x + b coef[j] y, the loop form
 *                of the filter's axpby / axpbyBlocked updates above
 *                (linearAlgebra/BlasLapackKernels.cpp:477-502); timed by the
 *                CPU baseline's per-operation sample
 *
 * The per-cell product goes through a caller-supplied Fortran dgemm (the
 * reference calls dgemm_ through blasWrapper::gemm); with none supplied a
 * plain triple loop computes the same product.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef void (*orc_dgemm_fn)(const char *, const char *, const int *, const int *, const int *,
                             const double *, const double *, const int *, const double *,
                             const int *, const double *, double *, const int *);

typedef struct {
  uint64_t n_dofs;
  uint32_t n_cells;
  const uint32_t *nd;       /* [n_cells] dofs per cell */
  const uint32_t *ids;      /* [sum nd] cell-major local->global */
  const uint64_t *cell_off; /* [n_cells+1] prefix sum of nd */
  const uint64_t *mat_off;  /* [n_cells+1] prefix sum of nd^2 */
} orc_mesh;

typedef struct {
  uint32_t nrows;
  const uint32_t *row_ids;
  const uint32_t *row_sizes;
  const uint32_t *col_ids;
  const uint32_t *row_acc;
  const double *col_vals;
  const double *inh;
} orc_cons;

typedef struct {
  uint32_t n_proj;
  const uint32_t *np;     /* [n_cells] projectors per cell */
  const uint32_t *pids;   /* [sum np] projector of each (cell, projector) slot */
  const uint64_t *p_off;  /* [n_cells+1] prefix sum of np */
  const uint64_t *c_off;  /* [n_cells+1] prefix sum of np * nd */
  const double *cmat;     /* per cell np x nd column-major (projector fastest) */
  const double *v;        /* [n_proj] diagonal coupling */
} orc_nl;

typedef struct {
  int kind; /* 0: cell matrices, 1: diagonal with constraints, 2: diagonal without,
               3: diagonal + dense block on [blk_begin, blk_begin + blk_n) with constraints */
  const orc_mesh *mesh;
  const orc_cons *cons;
  const double *mats; /* kind 0: column-major per cell, concatenated */
  const double *diag; /* kind 1/2/3: [n_dofs] */
  uint64_t blk_begin;
  uint64_t blk_n;
  const double *blk; /* kind 3: column-major blk_n x blk_n */
  const orc_nl *nl;  /* kind 0: nonlocal part (NULL: none) */
} orc_op;

static orc_dgemm_fn g_dgemm = 0;

void orc_set_dgemm(void *fn) { g_dgemm = (orc_dgemm_fn)fn; }

/* ConstraintsInternal.cpp:37-107 */
void orc_p2c(const orc_cons *c, double *x, uint32_t m) {
  double *nv = (double *)malloc(sizeof(double) * (m ? m : 1));
  for (uint32_t i = 0; i < c->nrows; ++i) {
    for (uint32_t v = 0; v < m; ++v) nv[v] = c->inh[i];
    const uint64_t rowStart = (uint64_t)c->row_ids[i] * m;
    const uint32_t colIndexStart = c->row_acc[i];
    for (uint32_t j = 0; j < c->row_sizes[i]; ++j) {
      const uint64_t colStart = (uint64_t)c->col_ids[colIndexStart + j] * m;
      const double a = c->col_vals[colIndexStart + j];
      for (uint32_t v = 0; v < m; ++v) nv[v] += a * x[colStart + v];
    }
    memcpy(x + rowStart, nv, sizeof(double) * m);
  }
  free(nv);
}

/* ConstraintsInternal.cpp:112-170 */
void orc_c2p(const orc_cons *c, double *x, uint32_t m) {
  for (uint32_t i = 0; i < c->nrows; ++i) {
    const uint64_t rowStart = (uint64_t)c->row_ids[i] * m;
    const uint32_t colIndexStart = c->row_acc[i];
    for (uint32_t j = 0; j < c->row_sizes[i]; ++j) {
      const uint64_t colStart = (uint64_t)c->col_ids[colIndexStart + j] * m;
      const double a = c->col_vals[colIndexStart + j];
      for (uint32_t v = 0; v < m; ++v) x[colStart + v] += a * x[rowStart + v];
    }
    memset(x + rowStart, 0, sizeof(double) * m);
  }
}

/* Per-cell C(m x nd) = Xc(m x nd, ld m) * Hc(nd x nd, ld nd) */
static void cell_gemm(int m, int nd, const double *Xc, const double *Hc, double *Yc) {
  if (g_dgemm) {
    const double one = 1.0, zero = 0.0;
    g_dgemm("N", "N", &m, &nd, &nd, &one, Xc, &m, Hc, &nd, &zero, Yc, &m);
    return;
  }
  for (int j = 0; j < nd; ++j) {
    double *yj = Yc + (size_t)j * m;
    for (int v = 0; v < m; ++v) yj[v] = 0.0;
    for (int k = 0; k < nd; ++k) {
      const double h = Hc[k + (size_t)nd * j];
      const double *xk = Xc + (size_t)k * m;
      for (int v = 0; v < m; ++v) yj[v] += xk[v] * h;
    }
  }
}

/* C(m x n) = A(m x k, ld m) * op(B) + beta C; op(B) = B (k x n, ld k) or
   B^T with B stored n x k (ld n) -- the two products of the nonlocal part */
static void small_gemm(int transb, int m, int n, int k, const double *A, const double *B, double beta, double *Cm) {
  if (g_dgemm) {
    const double one = 1.0;
    const int ldb = transb ? n : k;
    g_dgemm("N", transb ? "T" : "N", &m, &n, &k, &one, A, &m, B, &ldb, &beta, Cm, &m);
    return;
  }
  for (int j = 0; j < n; ++j) {
    double *cj = Cm + (size_t)j * m;
    for (int v = 0; v < m; ++v) cj[v] = beta == 0.0 ? 0.0 : beta * cj[v];
    for (int q = 0; q < k; ++q) {
      const double b = transb ? B[j + (size_t)n * q] : B[q + (size_t)k * j];
      const double *aq = A + (size_t)q * m;
      for (int v = 0; v < m; ++v) cj[v] += aq[v] * b;
    }
  }
}

static uint32_t max_nd(const orc_mesh *me) {
  uint32_t mx = 0;
  for (uint32_t c = 0; c < me->n_cells; ++c)
    if (me->nd[c] > mx) mx = me->nd[c];
  return mx;
}

/* Y = op(X); X is modified by the constraints exactly as in the reference. */
int orc_apply(const orc_op *op, double *X, double *Y, uint32_t m) {
  const orc_mesh *me = op->mesh;
  const uint64_t N = me->n_dofs;
  if (op->kind == 0) {
    if (op->cons) orc_p2c(op->cons, X, m);
    memset(Y, 0, sizeof(double) * N * m);
    const uint32_t ndm = max_nd(me);
    double *Xc = (double *)malloc(sizeof(double) * (size_t)ndm * m);
    double *Yc = (double *)malloc(sizeof(double) * (size_t)ndm * m);
    if (!Xc || !Yc) { free(Xc); free(Yc); return 3; }
    const orc_nl *nl = op->nl;
    double *CX = 0, *CXc = 0;
    if (nl) {
      uint32_t npm = 1;
      for (uint32_t c = 0; c < me->n_cells; ++c)
        if (nl->np[c] > npm) npm = nl->np[c];
      CX = (double *)calloc((size_t)nl->n_proj * m + 1, sizeof(double));
      CXc = (double *)malloc(sizeof(double) * (size_t)npm * m);
      if (!CX || !CXc) { free(Xc); free(Yc); free(CX); free(CXc); return 3; }
      /* CX = sum over cells of Xc * C_c^T, scattered in cell order */
      for (uint32_t c = 0; c < me->n_cells; ++c) {
        const uint32_t nd = me->nd[c], np = nl->np[c];
        if (!np) continue;
        const uint32_t *ids = me->ids + me->cell_off[c];
        for (uint32_t i = 0; i < nd; ++i) memcpy(Xc + (size_t)i * m, X + (uint64_t)ids[i] * m, sizeof(double) * m);
        small_gemm(1, (int)m, (int)np, (int)nd, Xc, nl->cmat + nl->c_off[c], 0.0, CXc);
        const uint32_t *pid = nl->pids + nl->p_off[c];
        for (uint32_t b = 0; b < np; ++b)
          for (uint32_t v = 0; v < m; ++v) CX[(uint64_t)pid[b] * m + v] += CXc[(size_t)b * m + v];
      }
      for (uint32_t p = 0; p < nl->n_proj; ++p)
        for (uint32_t v = 0; v < m; ++v) CX[(uint64_t)p * m + v] = nl->v[p] * CX[(uint64_t)p * m + v];
    }
    for (uint32_t c = 0; c < me->n_cells; ++c) {
      const uint32_t nd = me->nd[c];
      const uint32_t *ids = me->ids + me->cell_off[c];
      for (uint32_t i = 0; i < nd; ++i) memcpy(Xc + (size_t)i * m, X + (uint64_t)ids[i] * m, sizeof(double) * m);
      if (op->mats)
        cell_gemm((int)m, (int)nd, Xc, op->mats + me->mat_off[c], Yc);
      else
        memset(Yc, 0, sizeof(double) * (size_t)nd * m);
      if (nl && nl->np[c]) {
        const uint32_t np = nl->np[c];
        const uint32_t *pid = nl->pids + nl->p_off[c];
        for (uint32_t b = 0; b < np; ++b) memcpy(CXc + (size_t)b * m, CX + (uint64_t)pid[b] * m, sizeof(double) * m);
        small_gemm(0, (int)m, (int)nd, (int)np, CXc, nl->cmat + nl->c_off[c], 1.0, Yc);
      }
      for (uint32_t i = 0; i < nd; ++i) {
        double *y = Y + (uint64_t)ids[i] * m;
        const double *yc = Yc + (size_t)i * m;
        for (uint32_t v = 0; v < m; ++v) y[v] += yc[v];
      }
    }
    free(Xc);
    free(Yc);
    free(CX);
    free(CXc);
    if (op->cons) orc_c2p(op->cons, Y, m);
    return 0;
  }
  const int with_cons = (op->kind == 1 || op->kind == 3) && op->cons;
  if (with_cons) orc_p2c(op->cons, X, m);
  for (uint64_t i = 0; i < N; ++i)
    for (uint32_t v = 0; v < m; ++v) Y[i * m + v] = op->diag[i] * X[i * m + v];
  if (op->kind == 3) {
    /* OrthoEFEOverlapInverseOpContextGLL.t.cpp:1182-1270: the enrichment rows
       of Y are replaced by the dense block times the enrichment rows of X
       (gemm('N','T') on the column-major [m x nEnr] view) */
    const uint64_t b0 = op->blk_begin, nb = op->blk_n;
    for (uint64_t e = 0; e < nb; ++e)
      for (uint32_t v = 0; v < m; ++v) {
        double acc = 0.0;
        for (uint64_t f = 0; f < nb; ++f) acc += op->blk[e + nb * f] * X[(b0 + f) * m + v];
        Y[(b0 + e) * m + v] = acc;
      }
  }
  if (with_cons) orc_c2p(op->cons, Y, m);
  return 0;
}

/* ChebyshevFilter.t.cpp:242-444 (ResidualChebyshevFilterGEP). */
int orc_residual_chebyshev_filter(const orc_op *A, const orc_op *B, const orc_op *BInv,
                                  const double *eigenvalues, double *X, uint32_t m, uint32_t degree,
                                  double wantedLower, double wantedUpper, double unwantedUpper,
                                  double *Y) {
  const uint64_t n = A->mesh->n_dofs * (uint64_t)m;
  const double e = 0.5 * (unwantedUpper - wantedUpper);
  const double c = 0.5 * (unwantedUpper + wantedUpper);
  double sigma = e / (wantedLower - c);
  const double sigma1 = sigma;
  const double gamma = 2.0 / sigma1;
  double sigma2;
  double *s1 = (double *)calloc(n, sizeof(double));
  double *s2 = (double *)calloc(n, sizeof(double));
  double *s3 = (double *)calloc(n, sizeof(double));
  double *R = (double *)calloc(n, sizeof(double));
  double *RN = (double *)calloc(n, sizeof(double));
  double *eF = (double *)malloc(sizeof(double) * m);
  double *eF1 = (double *)malloc(sizeof(double) * m);
  double *eF2 = (double *)malloc(sizeof(double) * m);
  if (!s1 || !s2 || !s3 || !R || !RN || !eF || !eF1 || !eF2) return 3;
  for (uint32_t j = 0; j < m; ++j) { eF[j] = eigenvalues[j]; eF1[j] = 1.0; eF2[j] = eigenvalues[j]; }
  double alpha1 = sigma1 / e, alpha2 = -c;

  orc_apply(B, X, Y, m);
  orc_apply(A, X, s3, m);
  for (uint64_t i = 0; i < n; ++i) { /* Y = AX - lambda BX */
    const uint32_t j = (uint32_t)(i % m);
    Y[i] = 1.0 * 1.0 * s3[i] + -1.0 * eF[j] * Y[i];
  }
  memcpy(RN, Y, sizeof(double) * n);
  memset(R, 0, sizeof(double) * n);
  for (uint32_t j = 0; j < m; ++j) eF2[j] = alpha1 * alpha2;
  for (uint32_t j = 0; j < m; ++j) eF2[j] = 1.0 * 1.0 * eF2[j] + alpha1 * eF[j] * eF1[j];
  for (uint64_t i = 0; i < n; ++i) RN[i] = alpha1 * RN[i];

  for (uint32_t deg = 2; deg <= degree; ++deg) {
    sigma2 = 1.0 / (gamma - sigma);
    alpha1 = 2.0 * sigma2 / e;
    alpha2 = -(sigma * sigma2);
    orc_apply(BInv, RN, s1, m);
    orc_apply(A, s1, s2, m);
    for (uint64_t i = 0; i < n; ++i) s1[i] = alpha1 * s2[i] + (-c * alpha1) * RN[i];
    for (uint64_t i = 0; i < n; ++i) R[i] = 1.0 * s1[i] + alpha2 * R[i];
    for (uint64_t i = 0; i < n; ++i) {
      const uint32_t j = (uint32_t)(i % m);
      R[i] = 1.0 * 1.0 * R[i] + alpha1 * eF2[j] * Y[i];
    }
    for (uint32_t j = 0; j < m; ++j) eF1[j] = (-c * alpha1) * eF2[j] + alpha2 * eF1[j];
    for (uint32_t j = 0; j < m; ++j) eF1[j] = 1.0 * 1.0 * eF1[j] + alpha1 * eF[j] * eF2[j];
    double *t = RN; RN = R; R = t;
    t = eF1; eF1 = eF2; eF2 = t;
    sigma = sigma2;
  }
  orc_apply(BInv, RN, R, m);
  for (uint64_t i = 0; i < n; ++i) {
    const uint32_t j = (uint32_t)(i % m);
    Y[i] = 1.0 * 1.0 * R[i] + 1.0 * eF2[j] * X[i];
  }
  free(s1); free(s2); free(s3); free(R); free(RN); free(eF); free(eF1); free(eF2);
  return 0;
}

/* ChebyshevFilter.t.cpp:39-135 (standard form; X is scratch, result in Y). */
int orc_chebyshev_filter(const orc_op *A, const orc_op *BInv, double *X, uint32_t m, uint32_t degree,
                         double wantedLower, double wantedUpper, double unwantedUpper, double *Y) {
  const uint64_t n = A->mesh->n_dofs * (uint64_t)m;
  const double e = 0.5 * (unwantedUpper - wantedUpper);
  const double c = 0.5 * (unwantedUpper + wantedUpper);
  double sigma = e / (wantedLower - c);
  const double sigma1 = sigma, gamma = 2.0 / sigma1;
  double sigma2;
  double *s1 = (double *)calloc(n, sizeof(double));
  double *s2 = (double *)calloc(n, sizeof(double));
  if (!s1 || !s2) return 3;
  double *guess = X, *filt = Y;
  orc_apply(A, guess, s1, m);
  orc_apply(BInv, s1, s2, m);
  for (uint64_t i = 0; i < n; ++i) filt[i] = sigma1 / e * s2[i] + -sigma1 / e * c * guess[i];
  for (uint32_t deg = 2; deg <= degree; ++deg) {
    sigma2 = 1.0 / (gamma - sigma);
    orc_apply(A, filt, s1, m);
    orc_apply(BInv, s1, s2, m);
    for (uint64_t i = 0; i < n; ++i) s1[i] = 2.0 * sigma2 / e * s2[i] + -2.0 * sigma2 / e * c * filt[i];
    for (uint64_t i = 0; i < n; ++i) guess[i] = 1.0 * s1[i] + -sigma * sigma2 * guess[i];
    double *t = guess; guess = filt; filt = t;
    sigma = sigma2;
  }
  /* MultiVector swap moves storage between the two objects, so the newest
     iterate is the one `filt` points at; the reference then copies it into
     eigenSubspaceGuess (eigenSubspaceGuess = filteredSubspace). */
  if (filt != Y) memcpy(Y, filt, sizeof(double) * n);
  if (filt != X) memcpy(X, filt, sizeof(double) * n);
  free(s1); free(s2);
  return 0;
}

static void col_dots(const double *a, const double *b, uint64_t N, uint32_t k, double *out) {
  for (uint32_t j = 0; j < k; ++j) out[j] = 0.0;
  for (uint64_t i = 0; i < N; ++i)
    for (uint32_t j = 0; j < k; ++j) out[j] += a[i * k + j] * b[i * k + j];
}

/* CGLinearSolver.t.cpp:68-313.  Returns 0 on success, 6 failed to converge,
   7 residual divergence.  iters_out receives the final iteration index. */
int orc_cg(const orc_op *A, const orc_op *PC, const double *b, double *x_inout, uint32_t k,
           uint32_t maxIter, double absTol, double relTol, double divTol, uint32_t *iters_out,
           double *rnorm_out) {
  const uint64_t N = A->mesh->n_dofs, n = N * (uint64_t)k;
  double *x = (double *)malloc(sizeof(double) * n);
  double *xc = (double *)malloc(sizeof(double) * n);
  double *r = (double *)calloc(n, sizeof(double));
  double *w = (double *)calloc(n, sizeof(double));
  double *z = (double *)calloc(n, sizeof(double));
  double *p = (double *)calloc(n, sizeof(double));
  double *bn = (double *)malloc(sizeof(double) * k);
  double *rn = (double *)malloc(sizeof(double) * k);
  double *zr = (double *)malloc(sizeof(double) * k);
  double *pw = (double *)malloc(sizeof(double) * k);
  double *zrn = (double *)malloc(sizeof(double) * k);
  char *conv = (char *)calloc(k, 1);
  memcpy(x, x_inout, sizeof(double) * n);
  memcpy(xc, x_inout, sizeof(double) * n);
  col_dots(b, b, N, k, bn);
  for (uint32_t j = 0; j < k; ++j) bn[j] = sqrt(bn[j]);
  int err = 99, diverge = 0, all = 0;
  uint32_t iter = 0;
  for (; iter <= maxIter; ++iter) {
    if (iter == 0) {
      orc_apply(A, x, w, k);
      for (uint64_t i = 0; i < n; ++i) r[i] = 1.0 * b[i] + -1.0 * w[i];
      orc_apply(PC, r, z, k);
      memcpy(p, z, sizeof(double) * n);
    } else {
      orc_apply(A, p, w, k);
      col_dots(z, r, N, k, zr);
      col_dots(p, w, N, k, pw);
      for (uint64_t i = 0; i < n; ++i) { const uint32_t j = i % k; x[i] = 1.0 * x[i] + (zr[j] / pw[j]) * p[i]; }
      for (uint64_t i = 0; i < n; ++i) { const uint32_t j = i % k; r[i] = 1.0 * r[i] + (-zr[j] / pw[j]) * w[i]; }
      orc_apply(PC, r, z, k);
      col_dots(z, r, N, k, zrn);
      for (uint64_t i = 0; i < n; ++i) { const uint32_t j = i % k; p[i] = 1.0 * z[i] + (zrn[j] / zr[j]) * p[i]; }
    }
    col_dots(r, r, N, k, rn);
    for (uint32_t j = 0; j < k; ++j) rn[j] = sqrt(rn[j]);
    for (uint32_t j = 0; j < k; ++j) {
      const double tol = absTol > bn[j] * relTol ? absTol : bn[j] * relTol;
      if (rn[j] < tol && !conv[j]) {
        err = 0;
        conv[j] = 1;
        for (uint64_t i = 0; i < N; ++i) xc[i * k + j] = x[i * k + j];
      }
      if (rn[j] > divTol && !diverge) { err = 7; diverge = 1; }
    }
    all = 1;
    for (uint32_t j = 0; j < k; ++j) all &= conv[j];
    if (diverge || all) break;
  }
  if (iter > maxIter) err = 6;
  memcpy(x_inout, xc, sizeof(double) * n);
  if (iters_out) *iters_out = iter;
  if (rnorm_out) memcpy(rnorm_out, rn, sizeof(double) * k);
  free(x); free(xc); free(r); free(w); free(z); free(p); free(bn); free(rn); free(zr); free(pw); free(zrn); free(conv);
  return err;
}

/* z[i][j] = a x[i][j] + b coef[j] y[i][j] over n = N m entries (row-major, m
   columns): the cost of one of the filter's vector updates. */
void orc_sweep(uint64_t n, uint32_t m, double a, const double *x, double b, const double *coef, const double *y,
               double *z) {
  for (uint64_t i = 0; i < n; ++i) {
    const uint32_t j = (uint32_t)(i % m);
    z[i] = a * x[i] + b * coef[j] * y[i];
  }
}
