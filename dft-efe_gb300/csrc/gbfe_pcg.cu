// gbfe_pcg.cu -- batched Jacobi-preconditioned CG over independent Poisson
// instances stored as one block-diagonal system.
//
// Each instance i owns the dof range [off_i, off_{i+1}) of the concatenated
// vectors; the operator is the block-diagonal union of the instances' cell
// operators (one cell launch serves all of them).  Every scalar of
// CGLinearSolver::solve (linearAlgebra/CGLinearSolver.t.cpp:68-313) -- the
// dots z.r and p.w, alpha, beta, the residual norm and the convergence /
// divergence tests -- is kept per instance on the device, so an iteration is
// a fixed sequence of kernels with no host round trip.  That sequence is
// captured once into a CUDA graph and replayed; the host reads the count of
// still-active instances every `chunk` iterations.
//
// A converged (or diverged) instance is frozen: alpha = beta = 0, so its x
// stays the iterate at which it converged -- the xConverged of the reference.
// Reductions are segmented, with a fixed number of blocks per instance and a
// fixed summation order, so results are bitwise reproducible.
#include "gbfe_internal.cuh"

#include <algorithm>
#include <cmath>

using namespace gbfe;

namespace {

constexpr unsigned kSegBlocks = 32;  // reduction blocks per instance
constexpr unsigned kThreads = 256;

// partial[i*kSegBlocks + b] = sum over block b's slice of instance i of x*y
__global__ void k_seg_dot_partial(const double *__restrict__ x, const double *__restrict__ y,
                                  const uint64_t *__restrict__ off, double *__restrict__ partial) {
  __shared__ double sh[kThreads];
  const uint32_t i = blockIdx.y, b = blockIdx.x;
  const uint64_t o0 = off[i], len = off[i + 1] - o0;
  const uint64_t per = (len + kSegBlocks - 1) / kSegBlocks;
  const uint64_t s0 = o0 + b * per, s1 = min(o0 + len, s0 + per);
  double acc = 0.0;
  for (uint64_t t = s0 + threadIdx.x; t < s1; t += kThreads) acc += x[t] * y[t];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (unsigned w = kThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[(uint64_t)i * kSegBlocks + b] = sh[0];
}

__global__ void k_seg_dot_final(const double *__restrict__ partial, uint32_t n, double *__restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (unsigned b = 0; b < kSegBlocks; ++b) s += partial[(uint64_t)i * kSegBlocks + b];
  out[i] = s;
}

struct PcgScalars {
  double *bnorm, *zr, *pw, *zrn, *rr, *alpha, *beta, *rnorm;
  int *active, *status;
  uint32_t *iters, *iter;
};

__global__ void k_alpha(PcgScalars s, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  s.alpha[i] = s.active[i] ? s.zr[i] / s.pw[i] : 0.0;
}

__global__ void k_beta(PcgScalars s, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  s.beta[i] = s.active[i] ? s.zrn[i] / s.zr[i] : 0.0;
  if (s.active[i]) s.zr[i] = s.zrn[i];
}

// x = x + alpha p ;  r = r - alpha w     (add(ones, x, alpha, p, x) etc.)
__global__ void k_update_xr(double *__restrict__ x, double *__restrict__ r, const double *__restrict__ p,
                            const double *__restrict__ w, const double *__restrict__ alpha,
                            const uint32_t *__restrict__ inst, uint64_t N) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < N; t += (uint64_t)gridDim.x * blockDim.x) {
    const double a = alpha[inst[t]];
    if (a == 0.0) continue;
    x[t] = 1.0 * x[t] + a * p[t];
    r[t] = 1.0 * r[t] + (-a) * w[t];
  }
}

// p = z + beta p
__global__ void k_update_p(double *__restrict__ p, const double *__restrict__ z, const double *__restrict__ beta,
                           const int *__restrict__ active, const uint32_t *__restrict__ inst, uint64_t N) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < N; t += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t i = inst[t];
    if (!active[i]) continue;
    p[t] = 1.0 * z[t] + beta[i] * p[t];
  }
}

// r = b - w (iteration 0)
__global__ void k_residual0(double *__restrict__ r, const double *__restrict__ b, const double *__restrict__ w,
                            uint64_t N) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < N; t += (uint64_t)gridDim.x * blockDim.x)
    r[t] = 1.0 * b[t] + (-1.0) * w[t];
}

// convergence / divergence tests of the current iteration, then iter++
__global__ void k_check(PcgScalars s, uint32_t n, double abs_tol, double rel_tol, double div_tol, uint32_t max_iter) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t it = *s.iter;
  if (i < n && s.active[i]) {
    const double rn = sqrt(s.rr[i]);
    s.rnorm[i] = rn;
    const double tol = fmax(abs_tol, s.bnorm[i] * rel_tol);
    if (rn < tol) {
      s.active[i] = 0;
      s.status[i] = GBFE_OK;
      s.iters[i] = it;
    } else if (rn > div_tol) {
      s.active[i] = 0;
      s.status[i] = GBFE_ERR_DIVERGED;
      s.iters[i] = it;
    } else if (it >= max_iter) {
      s.active[i] = 0;
      s.status[i] = GBFE_ERR_NOT_CONVERGED;
      s.iters[i] = it + 1;
    }
  }
}

__global__ void k_next_iter(uint32_t *iter) { *iter = *iter + 1; }

__global__ void k_count_active(const int *__restrict__ active, uint32_t n, int *__restrict__ out) {
  __shared__ int sh[256];
  int c = 0;
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) c += active[i];
  sh[threadIdx.x] = c;
  __syncthreads();
  for (unsigned w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

__global__ void k_sqrt_inplace(double *v, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = sqrt(v[i]);
}

__global__ void k_init_flags(int *active, int *status, uint32_t *iters, uint32_t *iter, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    active[i] = 1;
    status[i] = GBFE_ERR_NOT_CONVERGED;
    iters[i] = 0;
  }
  if (i == 0) *iter = 0;
}

__global__ void k_fill_inst(uint32_t *inst, const uint64_t *off, uint32_t n) {
  const uint32_t i = blockIdx.y;
  for (uint64_t t = off[i] + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < off[i + 1];
       t += (uint64_t)gridDim.x * blockDim.x)
    inst[t] = i;
}

}  // namespace

extern "C" int gbfe_pcg_solve_batched(const gbfe_op *A, const gbfe_op *PC, const gbfe_mv *b, gbfe_mv *x,
                                      uint32_t n_inst, const uint64_t *inst_dof_off, uint32_t max_iter,
                                      double abs_tol, double rel_tol, double div_tol, uint32_t iters_chunk,
                                      uint32_t *iters_out, int *status_out, double *rnorm_out) {
  if (!A || !PC || !b || !x || !inst_dof_off || n_inst == 0) return GBFE_ERR_ARG;
  gbfe_ctx *ctx = x->mesh->ctx;
  return gbfe_guard(ctx, [&] {
    gbfe_mesh *me = x->mesh;
    GBFE_REQUIRE(b->mesh == me && A->mesh == me && PC->mesh == me, "pcg_batched: operands on different meshes");
    GBFE_REQUIRE(b->m == 1 && x->m == 1 && b->dtype == GBFE_F64 && x->dtype == GBFE_F64,
                 "pcg_batched: b and x are FP64 single vectors over all instances");
    GBFE_REQUIRE(inst_dof_off[0] == 0 && inst_dof_off[n_inst] == me->n_dofs,
                 "pcg_batched: instance offsets must cover [0, n_dofs)");
    for (uint32_t i = 0; i < n_inst; ++i)
      GBFE_REQUIRE(inst_dof_off[i + 1] > inst_dof_off[i], "pcg_batched: empty or unsorted instance range");
    const uint64_t N = me->n_dofs;
    const int was_profiling = ctx->profiling;
    ctx->profiling = 0;  // event brackets cannot be captured into the graph
    DBuf<uint64_t> off;
    off.upload(inst_dof_off, n_inst + 1, ctx->stream);
    DBuf<uint32_t> inst;
    inst.alloc(N);
    k_fill_inst<<<dim3(64, n_inst), 256, 0, ctx->stream>>>(inst.p, off.p, n_inst);
    check_launch(ctx, "fill_inst");
    DBuf<double> sc;
    sc.alloc((size_t)8 * n_inst);
    DBuf<int> flags;
    flags.alloc((size_t)2 * n_inst + 1);
    DBuf<uint32_t> cnt;
    cnt.alloc((size_t)n_inst + 1);
    DBuf<double> partial;
    partial.alloc((size_t)n_inst * kSegBlocks);
    PcgScalars s{sc.p, sc.p + n_inst, sc.p + 2 * n_inst, sc.p + 3 * n_inst, sc.p + 4 * n_inst, sc.p + 5 * n_inst,
                 sc.p + 6 * n_inst, sc.p + 7 * n_inst, flags.p, flags.p + n_inst, cnt.p, cnt.p + n_inst};
    int *d_active_count = flags.p + 2 * n_inst;
    gbfe_mv r, z, p, w;
    for (gbfe_mv *v : {&r, &z, &p, &w}) {
      v->mesh = me;
      v->m = 1;
      v->dtype = GBFE_F64;
      v->d.alloc(N);
      GBFE_CUDA(cudaMemsetAsync(v->d.p, 0, N * 8, ctx->stream));
    }
    const unsigned g1 = (n_inst + 255) / 256;
    const unsigned gN = (unsigned)std::min<uint64_t>((N + 255) / 256, (uint64_t)ctx->sm_count * 16);
    auto seg_dot = [&](const gbfe_mv *u, const gbfe_mv *v, double *out) {
      k_seg_dot_partial<<<dim3(kSegBlocks, n_inst), kThreads, 0, ctx->stream>>>(u->d.p, v->d.p, off.p, partial.p);
      k_seg_dot_final<<<g1, 256, 0, ctx->stream>>>(partial.p, n_inst, out);
      count_launch(ctx, 2);
    };
    // iteration 0 (outside the graph; it also sizes the apply's scratch)
    k_init_flags<<<g1, 256, 0, ctx->stream>>>(s.active, s.status, s.iters, s.iter, n_inst);
    seg_dot(b, b, s.bnorm);
    k_sqrt_inplace<<<g1, 256, 0, ctx->stream>>>(s.bnorm, n_inst);
    count_launch(ctx, 2);
    apply_op(A, x, &w);
    k_residual0<<<gN, 256, 0, ctx->stream>>>(r.d.p, b->d.p, w.d.p, N);
    count_launch(ctx);
    apply_op(PC, &r, &z);
    GBFE_CUDA(cudaMemcpyAsync(p.d.p, z.d.p, N * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    seg_dot(&z, &r, s.zr);
    seg_dot(&r, &r, s.rr);
    k_check<<<g1, 256, 0, ctx->stream>>>(s, n_inst, abs_tol, rel_tol, div_tol, max_iter);
    k_next_iter<<<1, 1, 0, ctx->stream>>>(s.iter);
    count_launch(ctx, 2);
    // one CG iteration, captured
    auto iteration = [&]() {
      apply_op(A, &p, &w);
      seg_dot(&p, &w, s.pw);
      k_alpha<<<g1, 256, 0, ctx->stream>>>(s, n_inst);
      k_update_xr<<<gN, 256, 0, ctx->stream>>>(x->d.p, r.d.p, p.d.p, w.d.p, s.alpha, inst.p, N);
      apply_op(PC, &r, &z);
      seg_dot(&z, &r, s.zrn);
      k_beta<<<g1, 256, 0, ctx->stream>>>(s, n_inst);
      k_update_p<<<gN, 256, 0, ctx->stream>>>(p.d.p, z.d.p, s.beta, s.active, inst.p, N);
      seg_dot(&r, &r, s.rr);
      k_check<<<g1, 256, 0, ctx->stream>>>(s, n_inst, abs_tol, rel_tol, div_tol, max_iter);
      k_next_iter<<<1, 1, 0, ctx->stream>>>(s.iter);
      count_launch(ctx, 5);
    };
    const uint32_t chunk = std::max<uint32_t>(1, iters_chunk);
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    const uint64_t launches_before = ctx->launches;
    GBFE_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    for (uint32_t k = 0; k < chunk; ++k) iteration();
    GBFE_CUDA(cudaStreamEndCapture(ctx->stream, &graph));
    const uint64_t per_replay = ctx->launches - launches_before;
    ctx->launches = launches_before;
    GBFE_CUDA(cudaGraphInstantiate(&exec, graph, 0));
    int active = 1;
    uint32_t done_iters = 0;
    while (true) {
      k_count_active<<<1, 256, 0, ctx->stream>>>(s.active, n_inst, d_active_count);
      count_launch(ctx);
      GBFE_CUDA(cudaMemcpyAsync(&active, d_active_count, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
      GBFE_CUDA(cudaStreamSynchronize(ctx->stream));
      if (active == 0 || done_iters > max_iter) break;
      if (ctx->cancel && ctx->cancel->load()) {
        cudaGraphExecDestroy(exec);
        cudaGraphDestroy(graph);
        ctx->profiling = was_profiling;
        throw Error(GBFE_ERR_CANCELLED, "cancelled");
      }
      GBFE_CUDA(cudaGraphLaunch(exec, ctx->stream));
      ctx->launches += per_replay;
      done_iters += chunk;
    }
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    ctx->profiling = was_profiling;
    std::vector<double> rn(n_inst);
    GBFE_CUDA(cudaMemcpyAsync(rn.data(), s.rnorm, n_inst * 8, cudaMemcpyDeviceToHost, ctx->stream));
    if (iters_out) GBFE_CUDA(cudaMemcpyAsync(iters_out, s.iters, n_inst * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (status_out) GBFE_CUDA(cudaMemcpyAsync(status_out, s.status, n_inst * 4, cudaMemcpyDeviceToHost, ctx->stream));
    GBFE_CUDA(cudaStreamSynchronize(ctx->stream));
    if (rnorm_out) std::copy(rn.begin(), rn.end(), rnorm_out);
  });
}
