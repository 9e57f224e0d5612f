// gbfe_serve.cu -- continuous-batching request loop for independent KS
// eigen solves and Poisson solves on one GPU.
//
// A server owns `slots` contexts (each its own CUDA stream, cuBLAS and
// cuSOLVER handles) and one worker thread per slot.  Requests are admitted in
// arrival order as soon as a slot is free and the estimated HBM footprint of
// the request fits the budget next to the requests already resident; a
// request that can never fit is rejected with GBFE_ERR_ALLOC.  An admitted
// request uploads its mesh, constraints, cell matrices and block vectors to
// the device, keeps them resident until it finishes, and runs its solve on its
// slot's stream, so the kernels of different requests overlap on the SMs.
// Finishing a request frees its memory and admits the next waiting ones.
//
// Results do not depend on the mix: each request has private buffers and every
// kernel is deterministic, so a request's output is identical alone and with
// others in flight.
#include "gbfe_internal.cuh"

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>

using namespace gbfe;

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

enum ReqState { RQ_QUEUED = 0, RQ_RUNNING = 1, RQ_DONE = 2 };

struct Request {
  uint64_t id = 0;
  int kind = 0;  // 0 KS, 1 Poisson
  // mesh + constraints
  std::vector<uint32_t> nd, ids, rows, rsz, cols, racc;
  std::vector<double> cvals, inh;
  uint64_t n_dofs = 0;
  // KS
  std::vector<double> H, M, minv, X0, blk, lanczos_start;
  uint64_t blk_begin = 0, blk_n = 0;
  gbfe_ks_params ks{};
  uint32_t m = 0;
  // Poisson
  std::vector<double> K, diag, b;
  std::vector<uint32_t> cell_to_mat;
  uint32_t n_mats = 0, max_iter = 0;
  double abs_tol = 0, rel_tol = 0, div_tol = 0;
  // bookkeeping
  uint64_t footprint = 0;
  int state = RQ_QUEUED;
  int status = GBFE_OK;
  std::string message;
  double t_submit = 0, t_admit = 0, t_done = 0;
  std::atomic<int> cancel{0};
  // results
  std::vector<double> eig, res, x;
  uint32_t passes = 0, iters = 0;
};

struct Slot {
  gbfe_ctx *ctx = nullptr;
  // Poisson requests admitted together (same iteration limit and
  // tolerances) run as one batched solve; empty for a single request
  std::vector<Request *> batch;
  // Poisson requests run on this stream of the highest priority: when a
  // KS solve's kernel ends, the block scheduler starts the short requests'
  // pending blocks first, so they are not queued behind whole KS passes
  cudaStream_t hi = nullptr;
  Request *req = nullptr;
  std::thread th;
};

}  // namespace

struct gbfe_server {
  int device = 0;
  uint64_t budget = 0, used = 0;
  std::vector<Slot> slots;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request *> queue;
  std::map<uint64_t, std::unique_ptr<Request>> reqs;
  uint64_t next_id = 1;
  bool stop = false;
  int inject_alloc_failures = 0;  // host-side fault injection: fail the next N uploads
  uint64_t admitted = 0, completed = 0, rejected = 0;
  uint64_t poisson_batches = 0, poisson_batched = 0;  // batched solves, and the requests they carried
  uint32_t max_poisson_batch = 32;
};

namespace {

uint64_t ks_footprint(const Request &r) {
  uint64_t snd = 0, snd2 = 0;
  for (uint32_t v : r.nd) {
    snd += v;
    snd2 += (uint64_t)v * v;
  }
  const bool mixed = r.ks.filter_precision == GBFE_F32;
  uint64_t b = 2 * snd2 * 8;                          // H, M FP64
  if (mixed) b += 2 * (snd2 * 4 + snd2 * 5);          // FP32 copies + split-BF16 tiles (padded)
  b += 12 * r.n_dofs * (uint64_t)r.m * 8;              // block vectors of the fused pass + filter
  b += snd * (uint64_t)r.m * 12;                       // cell-wise scratch (FP64 + FP32)
  b += snd * 12 + r.n_dofs * 16;                       // ids, slots, constraints
  return b + (16u << 20);
}

uint64_t poisson_footprint(const Request &r) {
  uint64_t snd = 0;
  for (uint32_t v : r.nd) snd += v;
  return r.K.size() * 8 + 8 * r.n_dofs * 8 + snd * 8 + snd * 12 + r.n_dofs * 16 + (16u << 20);
}

// Results are out (on the host, or the failure recorded): the requests are
// done for their callers.  Called before the teardown of the requests'
// device objects, whose frees synchronise the device and would otherwise
// hold each result back until every other slot's queued kernels finished.
// The slot, and the HBM budget the requests hold, stay taken until the
// teardown is over (the worker releases them).
void publish(gbfe_server *sv, const std::vector<Request *> &done) {
  std::lock_guard<std::mutex> lk(sv->mu);
  const double t = now_s();
  for (Request *q : done) {
    q->t_done = t;
    q->state = RQ_DONE;
    ++sv->completed;
  }
  sv->cv_done.notify_all();
}

// runs one request on a slot's context; every device object is freed on exit
void run_request(gbfe_server *sv, gbfe_ctx *ctx, Request *r) {
  gbfe_mesh *me = nullptr;
  gbfe_cons *cons = nullptr;
  gbfe_op *A = nullptr, *B = nullptr, *BI = nullptr;
  gbfe_mv *X = nullptr, *bv = nullptr;
  auto fail = [&](int rc) {
    r->status = rc;
    char buf[512] = {0};
    gbfe_last_error(ctx, buf, sizeof buf);
    r->message = buf;
  };
  int rc = GBFE_OK;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    if (sv->inject_alloc_failures > 0) {
      --sv->inject_alloc_failures;
      rc = GBFE_ERR_ALLOC;
    }
  }
  if (rc != GBFE_OK) {
    r->status = rc;
    r->message = "injected allocation failure";
  } else if (r->cancel.load()) {
    r->status = GBFE_ERR_CANCELLED;
    r->message = "cancelled before start";
  } else {
    do {
      if ((rc = gbfe_mesh_upload(ctx, (uint32_t)r->nd.size(), r->nd.data(), r->ids.data(), r->n_dofs, &me))) break;
      if ((rc = gbfe_constraints_upload(me, (uint32_t)r->rows.size(), r->rows.data(), r->rsz.data(), r->cols.data(),
                                        r->racc.data(), r->cvals.data(), r->inh.data(), &cons)))
        break;
      if (r->kind == 0) {
        const int prec = GBFE_PREC_FP64 | (r->ks.filter_precision == GBFE_F32 ? GBFE_PREC_MIXED : 0);
        if ((rc = gbfe_cellmat_upload(me, cons, r->H.data(), prec, &A))) break;
        if ((rc = gbfe_cellmat_upload(me, cons, r->M.data(), prec, &B))) break;
        if (r->blk_n)
          rc = gbfe_diag_block_upload(me, cons, r->minv.data(), r->blk_begin, r->blk_n, r->blk.data(), &BI);
        else
          rc = gbfe_diag_upload(me, cons, r->minv.data(), &BI);
        if (rc) break;
        if ((rc = gbfe_mv_create(me, r->m, GBFE_F64, &X))) break;
        if ((rc = gbfe_mv_copy_in(X, r->X0.data()))) break;
        r->eig.assign(r->m, 0.0);
        r->res.assign(r->m, 0.0);
        ctx->cancel = &r->cancel;
        rc = gbfe_ks_eigen_solve(A, B, BI, X, &r->ks, r->eig.data(), r->res.data(), &r->passes);
        ctx->cancel = nullptr;
      } else {
        if ((rc = gbfe_cellmat_upload_indexed(me, cons, r->n_mats, r->K.data(), r->cell_to_mat.data(), GBFE_PREC_FP64,
                                              &A)))
          break;
        if ((rc = gbfe_jacobi_upload(me, r->diag.data(), &BI))) break;
        if ((rc = gbfe_mv_create(me, 1, GBFE_F64, &bv))) break;
        if ((rc = gbfe_mv_copy_in(bv, r->b.data()))) break;
        if ((rc = gbfe_mv_create(me, 1, GBFE_F64, &X))) break;
        ctx->cancel = &r->cancel;
        const uint64_t off[2] = {0, r->n_dofs};
        int st = GBFE_OK;
        double rn = 0.0;
        rc = gbfe_pcg_solve_batched(A, BI, bv, X, 1, off, r->max_iter, r->abs_tol, r->rel_tol, r->div_tol, 16,
                                    &r->iters, &st, &rn);
        ctx->cancel = nullptr;
        if (rc == GBFE_OK) rc = st;
        if (rc == GBFE_OK || rc == GBFE_ERR_NOT_CONVERGED || rc == GBFE_ERR_DIVERGED) {
          r->x.resize(r->n_dofs);
          const int rc2 = gbfe_mv_copy_out(X, r->x.data());
          if (rc2) rc = rc2;
        }
      }
    } while (false);
    if (rc != GBFE_OK) fail(rc);
  }
  publish(sv, std::vector<Request *>{r});
  gbfe_mv_destroy(X);
  gbfe_mv_destroy(bv);
  gbfe_op_destroy(A);
  gbfe_op_destroy(B);
  gbfe_op_destroy(BI);
  gbfe_constraints_destroy(cons);
  gbfe_mesh_destroy(me);
}

// Poisson requests of one batch as a single block-diagonal solve: the meshes,
// constraints, indexed Laplace matrices, Jacobi diagonals and right-hand
// sides are concatenated (dof, constraint-column and matrix indices shifted),
// and gbfe_pcg_solve_batched advances every instance in the same kernels.
// Its per-instance scalars and fixed per-instance reductions make each
// instance's arithmetic the same as in a solve of its own, so results do not
// depend on the batch.  A batch is not cancellable once it runs.
void run_poisson_batch(gbfe_server *sv, gbfe_ctx *ctx, const std::vector<Request *> &batch) {
  int rc = GBFE_OK;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    if (sv->inject_alloc_failures > 0) {
      --sv->inject_alloc_failures;
      rc = GBFE_ERR_ALLOC;
    }
  }
  if (rc != GBFE_OK) {
    for (Request *r : batch) {
      r->status = rc;
      r->message = "injected allocation failure";
    }
    publish(sv, batch);
    return;
  }
  std::vector<uint32_t> nd, ids, rows, rsz, cols, racc, c2m;
  std::vector<double> cvals, inh, K, diag, b;
  std::vector<uint64_t> off{0};
  uint64_t dofs = 0;
  uint32_t mats = 0, nnz = 0;
  for (const Request *r : batch) {
    nd.insert(nd.end(), r->nd.begin(), r->nd.end());
    for (uint32_t g : r->ids) ids.push_back((uint32_t)(g + dofs));
    for (uint32_t g : r->rows) rows.push_back((uint32_t)(g + dofs));
    rsz.insert(rsz.end(), r->rsz.begin(), r->rsz.end());
    for (uint32_t g : r->cols) cols.push_back((uint32_t)(g + dofs));
    for (uint32_t a : r->racc) racc.push_back(a + nnz);
    cvals.insert(cvals.end(), r->cvals.begin(), r->cvals.end());
    inh.insert(inh.end(), r->inh.begin(), r->inh.end());
    K.insert(K.end(), r->K.begin(), r->K.end());
    for (uint32_t u : r->cell_to_mat) c2m.push_back(u + mats);
    diag.insert(diag.end(), r->diag.begin(), r->diag.end());
    b.insert(b.end(), r->b.begin(), r->b.end());
    dofs += r->n_dofs;
    off.push_back(dofs);
    mats += r->n_mats;
    nnz += (uint32_t)r->cols.size();
  }
  const Request *r0 = batch.front();
  const uint32_t n = (uint32_t)batch.size();
  std::vector<uint32_t> iters(n, 0);
  std::vector<int> st(n, GBFE_OK);
  std::vector<double> rn(n, 0.0), x(dofs, 0.0);
  gbfe_mesh *me = nullptr;
  gbfe_cons *cons = nullptr;
  gbfe_op *A = nullptr, *PC = nullptr;
  gbfe_mv *bv = nullptr, *X = nullptr;
  do {
    if ((rc = gbfe_mesh_upload(ctx, (uint32_t)nd.size(), nd.data(), ids.data(), dofs, &me))) break;
    if ((rc = gbfe_constraints_upload(me, (uint32_t)rows.size(), rows.data(), rsz.data(), cols.data(), racc.data(),
                                      cvals.data(), inh.data(), &cons)))
      break;
    if ((rc = gbfe_cellmat_upload_indexed(me, cons, mats, K.data(), c2m.data(), GBFE_PREC_FP64, &A))) break;
    if ((rc = gbfe_jacobi_upload(me, diag.data(), &PC))) break;
    if ((rc = gbfe_mv_create(me, 1, GBFE_F64, &bv))) break;
    if ((rc = gbfe_mv_copy_in(bv, b.data()))) break;
    if ((rc = gbfe_mv_create(me, 1, GBFE_F64, &X))) break;
    rc = gbfe_pcg_solve_batched(A, PC, bv, X, n, off.data(), r0->max_iter, r0->abs_tol, r0->rel_tol, r0->div_tol,
                                16, iters.data(), st.data(), rn.data());
    if (rc == GBFE_OK) rc = gbfe_mv_copy_out(X, x.data());
  } while (false);
  char msg[512] = {0};
  if (rc != GBFE_OK) gbfe_last_error(ctx, msg, sizeof msg);
  for (uint32_t i = 0; i < n; ++i) {
    Request *r = batch[i];
    if (rc != GBFE_OK) {
      r->status = rc;
      r->message = msg;
      continue;
    }
    r->status = st[i];
    r->iters = iters[i];
    r->x.assign(x.begin() + (ptrdiff_t)off[i], x.begin() + (ptrdiff_t)off[i + 1]);
  }
  publish(sv, batch);
  gbfe_mv_destroy(X);
  gbfe_mv_destroy(bv);
  gbfe_op_destroy(A);
  gbfe_op_destroy(PC);
  gbfe_constraints_destroy(cons);
  gbfe_mesh_destroy(me);
}

// two Poisson requests can share a batched solve
bool same_cg_params(const Request *a, const Request *b) {
  return a->kind == 1 && b->kind == 1 && a->max_iter == b->max_iter && a->abs_tol == b->abs_tol &&
         a->rel_tol == b->rel_tol && a->div_tol == b->div_tol;
}

// admit waiting requests while a slot is free and the footprint fits (lock held)
void admit_locked(gbfe_server *sv) {
  while (!sv->queue.empty()) {
    Request *r = sv->queue.front();
    if (r->cancel.load()) {
      sv->queue.pop_front();
      r->state = RQ_DONE;
      r->status = GBFE_ERR_CANCELLED;
      r->message = "cancelled while queued";
      r->t_done = now_s();
      sv->cv_done.notify_all();
      continue;
    }
    if (r->footprint > sv->budget) {
      sv->queue.pop_front();
      r->state = RQ_DONE;
      r->status = GBFE_ERR_ALLOC;
      r->message = "request footprint exceeds the server's HBM budget";
      r->t_done = now_s();
      ++sv->rejected;
      sv->cv_done.notify_all();
      continue;
    }
    if (sv->used + r->footprint > sv->budget) break;
    Slot *free_slot = nullptr;
    for (auto &s : sv->slots)
      if (!s.req) {
        free_slot = &s;
        break;
      }
    if (!free_slot) break;
    sv->queue.pop_front();
    sv->used += r->footprint;
    r->state = RQ_RUNNING;
    r->t_admit = now_s();
    free_slot->req = r;
    free_slot->batch.clear();
    ++sv->admitted;
    if (r->kind == 1) {
      // continuous batching: the compatible Poisson requests waiting behind it
      // join the same solve while the budget allows
      for (auto it = sv->queue.begin(); it != sv->queue.end() && free_slot->batch.size() + 1 < sv->max_poisson_batch;) {
        Request *q = *it;
        if (!q->cancel.load() && same_cg_params(r, q) && q->footprint <= sv->budget &&
            sv->used + q->footprint <= sv->budget) {
          if (free_slot->batch.empty()) free_slot->batch.push_back(r);
          free_slot->batch.push_back(q);
          sv->used += q->footprint;
          q->state = RQ_RUNNING;
          q->t_admit = r->t_admit;
          ++sv->admitted;
          it = sv->queue.erase(it);
        } else {
          ++it;
        }
      }
      if (!free_slot->batch.empty()) {
        ++sv->poisson_batches;
        sv->poisson_batched += free_slot->batch.size();
      }
    }
    sv->cv_work.notify_all();
  }
}

void worker(gbfe_server *sv, size_t slot_index) {
  Slot &slot = sv->slots[slot_index];
  cudaSetDevice(sv->device);
  // device blocks of finished requests are reused by the next ones on this
  // slot (no cudaFree, and its device-wide synchronisation, between requests)
  struct CacheScope {
    DevCache cache;
    explicit CacheScope(size_t cap) {
      cache.cap = cap;
      thread_dev_cache() = &cache;
    }
    ~CacheScope() {
      thread_dev_cache() = nullptr;
      cache.release();
    }
  } scope(std::max<uint64_t>(sv->budget / std::max<size_t>(1, sv->slots.size()), 1ull << 30));
  for (;;) {
    Request *r = nullptr;
    {
      std::unique_lock<std::mutex> lk(sv->mu);
      sv->cv_work.wait(lk, [&] { return sv->stop || slot.req != nullptr; });
      if (sv->stop && !slot.req) return;
      r = slot.req;
    }
    const bool urgent = r->kind != 0 && slot.hi;
    if (urgent) gbfe_ctx_set_stream(slot.ctx, slot.hi);
    std::vector<Request *> done;
    uint64_t footprint = 0;  // read now: a published request may be released by its caller
    {
      std::lock_guard<std::mutex> lk(sv->mu);
      done = slot.batch.empty() ? std::vector<Request *>{r} : slot.batch;
      for (Request *q : done) footprint += q->footprint;
    }
    if (done.size() > 1)
      run_poisson_batch(sv, slot.ctx, done);
    else
      run_request(sv, slot.ctx, r);
    gbfe_ctx_synchronize(slot.ctx);  // nothing of this request left on the slot's streams
    scope.cache.mark_safe();
    if (urgent) gbfe_ctx_set_stream(slot.ctx, nullptr);
    {
      std::lock_guard<std::mutex> lk(sv->mu);
      sv->used -= footprint;
      slot.req = nullptr;
      slot.batch.clear();
      admit_locked(sv);
      sv->cv_done.notify_all();
    }
  }
}

template <class T>
std::vector<T> copy_arr(const T *p, size_t n) {
  return p && n ? std::vector<T>(p, p + n) : std::vector<T>();
}

int submit_common(gbfe_server *sv, std::unique_ptr<Request> r, uint64_t *id_out) {
  std::lock_guard<std::mutex> lk(sv->mu);
  if (sv->stop) return GBFE_ERR_ARG;
  r->id = sv->next_id++;
  r->t_submit = now_s();
  Request *raw = r.get();
  sv->reqs[raw->id] = std::move(r);
  sv->queue.push_back(raw);
  admit_locked(sv);
  if (id_out) *id_out = raw->id;
  return GBFE_OK;
}

void fill_mesh(Request &r, const gbfe_mesh_desc *m) {
  r.nd = copy_arr(m->nd_per_cell, m->n_cells);
  uint64_t snd = 0;
  for (uint32_t v : r.nd) snd += v;
  r.ids = copy_arr(m->cell_dof_ids, snd);
  r.n_dofs = m->n_dofs;
  uint64_t nnz = 0;
  for (uint32_t i = 0; i < m->n_cons_rows; ++i) nnz = std::max<uint64_t>(nnz, (uint64_t)m->row_acc[i] + m->row_sizes[i]);
  r.rows = copy_arr(m->row_ids, m->n_cons_rows);
  r.rsz = copy_arr(m->row_sizes, m->n_cons_rows);
  r.racc = copy_arr(m->row_acc, m->n_cons_rows);
  r.inh = copy_arr(m->inhomogeneities, m->n_cons_rows);
  r.cols = copy_arr(m->col_ids, nnz);
  r.cvals = copy_arr(m->col_values, nnz);
}

}  // namespace

extern "C" {

int gbfe_server_create(int device, uint32_t slots, uint64_t hbm_budget_bytes, gbfe_server **out) {
  if (!out || slots == 0) return GBFE_ERR_ARG;
  *out = nullptr;
  auto *sv = new gbfe_server();
  sv->device = device;
  sv->budget = hbm_budget_bytes;
  sv->slots.resize(slots);
  for (auto &s : sv->slots) {
    const int rc = gbfe_ctx_create(device, &s.ctx);
    if (rc != GBFE_OK) {
      for (auto &t : sv->slots) {
        gbfe_ctx_destroy(t.ctx);
        if (t.hi) cudaStreamDestroy(t.hi);
      }
      delete sv;
      return rc;
    }
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess ||
        cudaStreamCreateWithPriority(&s.hi, cudaStreamNonBlocking, greatest) != cudaSuccess) {
      (void)cudaGetLastError();
      s.hi = nullptr;  // every request on the context's own stream
    }
  }
  for (size_t i = 0; i < sv->slots.size(); ++i) sv->slots[i].th = std::thread(worker, sv, i);
  *out = sv;
  return GBFE_OK;
}

int gbfe_server_destroy(gbfe_server *sv) {
  if (!sv) return GBFE_OK;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    for (Request *r : sv->queue) {
      r->state = RQ_DONE;
      r->status = GBFE_ERR_CANCELLED;
    }
    sv->queue.clear();
    sv->stop = true;
    sv->cv_work.notify_all();
  }
  for (auto &s : sv->slots)
    if (s.th.joinable()) s.th.join();
  for (auto &s : sv->slots) {
    gbfe_ctx_destroy(s.ctx);
    if (s.hi) cudaStreamDestroy(s.hi);
  }
  delete sv;
  return GBFE_OK;
}

int gbfe_server_submit_ks(gbfe_server *sv, const gbfe_mesh_desc *mesh, const double *H, const double *M,
                          const double *minv_diag, uint64_t blk_begin, uint64_t blk_n, const double *blk,
                          const double *X0, uint32_t m, const gbfe_ks_params *params, uint64_t *id_out) {
  if (!sv || !mesh || !H || !M || !minv_diag || !X0 || !params || m == 0) return GBFE_ERR_ARG;
  auto r = std::make_unique<Request>();
  r->kind = 0;
  fill_mesh(*r, mesh);
  uint64_t snd2 = 0;
  for (uint32_t v : r->nd) snd2 += (uint64_t)v * v;
  r->H = copy_arr(H, snd2);
  r->M = copy_arr(M, snd2);
  r->minv = copy_arr(minv_diag, r->n_dofs);
  r->blk_begin = blk_begin;
  r->blk_n = blk_n;
  r->blk = copy_arr(blk, blk_n * blk_n);
  r->X0 = copy_arr(X0, r->n_dofs * (uint64_t)m);
  r->m = m;
  r->ks = *params;
  // a start vector is copied like the other arrays (the caller may free it)
  if (params->use_lanczos && params->lanczos_start) {
    r->lanczos_start = copy_arr(params->lanczos_start, r->n_dofs);
    r->ks.lanczos_start = r->lanczos_start.data();
  } else {
    r->ks.lanczos_start = nullptr;
  }
  r->footprint = ks_footprint(*r);
  return submit_common(sv, std::move(r), id_out);
}

int gbfe_server_submit_poisson(gbfe_server *sv, const gbfe_mesh_desc *mesh, uint32_t n_mats, const double *mats,
                               const uint32_t *cell_to_mat, const double *jacobi_diag, const double *b,
                               uint32_t max_iter, double abs_tol, double rel_tol, double div_tol, uint64_t *id_out) {
  if (!sv || !mesh || !mats || !cell_to_mat || !jacobi_diag || !b || n_mats == 0) return GBFE_ERR_ARG;
  auto r = std::make_unique<Request>();
  r->kind = 1;
  fill_mesh(*r, mesh);
  r->cell_to_mat = copy_arr(cell_to_mat, r->nd.size());
  uint64_t tot = 0;
  std::vector<uint32_t> nd_of(n_mats, 0);
  for (size_t c = 0; c < r->nd.size(); ++c)
    if (cell_to_mat[c] < n_mats) nd_of[cell_to_mat[c]] = r->nd[c];
  for (uint32_t u = 0; u < n_mats; ++u) tot += (uint64_t)nd_of[u] * nd_of[u];
  r->K = copy_arr(mats, tot);
  r->n_mats = n_mats;
  r->diag = copy_arr(jacobi_diag, r->n_dofs);
  r->b = copy_arr(b, r->n_dofs);
  r->max_iter = max_iter;
  r->abs_tol = abs_tol;
  r->rel_tol = rel_tol;
  r->div_tol = div_tol;
  r->footprint = poisson_footprint(*r);
  return submit_common(sv, std::move(r), id_out);
}

int gbfe_server_cancel(gbfe_server *sv, uint64_t id) {
  if (!sv) return GBFE_ERR_ARG;
  std::lock_guard<std::mutex> lk(sv->mu);
  auto it = sv->reqs.find(id);
  if (it == sv->reqs.end()) return GBFE_ERR_ARG;
  it->second->cancel = 1;
  admit_locked(sv);  // drops it if still queued
  return GBFE_OK;
}

int gbfe_server_wait(gbfe_server *sv, uint64_t id, double timeout_s, gbfe_request_info *info) {
  if (!sv) return GBFE_ERR_ARG;
  std::unique_lock<std::mutex> lk(sv->mu);
  auto it = sv->reqs.find(id);
  if (it == sv->reqs.end()) return GBFE_ERR_ARG;
  Request *r = it->second.get();
  const bool done = sv->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s),
                                         [&] { return r->state == RQ_DONE; });
  if (!done) return GBFE_ERR_TIMEOUT;
  if (info) {
    info->status = r->status;
    info->t_submit = r->t_submit;
    info->t_admit = r->t_admit;
    info->t_done = r->t_done;
    info->passes_or_iters = r->kind == 0 ? r->passes : r->iters;
    info->footprint_bytes = r->footprint;
    snprintf(info->message, sizeof info->message, "%s", r->message.c_str());
  }
  return GBFE_OK;
}

int gbfe_server_result(gbfe_server *sv, uint64_t id, double *values, double *residuals) {
  if (!sv) return GBFE_ERR_ARG;
  std::lock_guard<std::mutex> lk(sv->mu);
  auto it = sv->reqs.find(id);
  if (it == sv->reqs.end() || it->second->state != RQ_DONE) return GBFE_ERR_ARG;
  Request *r = it->second.get();
  if (r->kind == 0) {
    if (values) std::copy(r->eig.begin(), r->eig.end(), values);
    if (residuals) std::copy(r->res.begin(), r->res.end(), residuals);
  } else if (values) {
    std::copy(r->x.begin(), r->x.end(), values);
  }
  return GBFE_OK;
}

int gbfe_server_release(gbfe_server *sv, uint64_t id) {
  if (!sv) return GBFE_ERR_ARG;
  std::lock_guard<std::mutex> lk(sv->mu);
  auto it = sv->reqs.find(id);
  if (it == sv->reqs.end() || it->second->state != RQ_DONE) return GBFE_ERR_ARG;
  sv->reqs.erase(it);
  return GBFE_OK;
}

int gbfe_server_stats(gbfe_server *sv, uint64_t *admitted, uint64_t *completed, uint64_t *rejected,
                      uint64_t *used_bytes, uint32_t *queued) {
  if (!sv) return GBFE_ERR_ARG;
  std::lock_guard<std::mutex> lk(sv->mu);
  if (admitted) *admitted = sv->admitted;
  if (completed) *completed = sv->completed;
  if (rejected) *rejected = sv->rejected;
  if (used_bytes) *used_bytes = sv->used;
  if (queued) *queued = (uint32_t)sv->queue.size();
  return GBFE_OK;
}

int gbfe_server_batch_stats(gbfe_server *sv, uint64_t *poisson_batches, uint64_t *poisson_batched_requests) {
  if (!sv) return GBFE_ERR_ARG;
  std::lock_guard<std::mutex> lk(sv->mu);
  if (poisson_batches) *poisson_batches = sv->poisson_batches;
  if (poisson_batched_requests) *poisson_batched_requests = sv->poisson_batched;
  return GBFE_OK;
}

int gbfe_server_set_max_batch(gbfe_server *sv, uint32_t max_poisson_batch) {
  if (!sv || max_poisson_batch == 0) return GBFE_ERR_ARG;
  std::lock_guard<std::mutex> lk(sv->mu);
  sv->max_poisson_batch = max_poisson_batch;
  return GBFE_OK;
}

int gbfe_server_inject_alloc_failures(gbfe_server *sv, int count) {
  if (!sv) return GBFE_ERR_ARG;
  std::lock_guard<std::mutex> lk(sv->mu);
  sv->inject_alloc_failures = count;
  return GBFE_OK;
}

}  // extern "C"
