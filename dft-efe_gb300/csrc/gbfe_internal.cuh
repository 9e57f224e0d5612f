// gbfe_internal.cuh -- device-resident state behind the C ABI in include/gbfe.h.
//
// HBM layout (all device buffers owned by the handle that created them):
//   mesh:  ids[sum nd]        cell-major cell->dof ids (uint32)
//          cell_off[C+1]      prefix sum of nd (uint32)
//          mat_off[C+1]       prefix sum of nd^2 (uint64)
//          slot_ptr[N+1], slot[sum nd]
//                             dof -> cell-slot transpose, slots of a dof in
//                             ascending (cell, local index) order, which is the
//                             order the reference's serial scatter adds them
//                             (FECellWiseDataOperations.t.cpp:87-151)
//   cons:  the reference CSR arrays + the column->row transpose
//          par_ptr[N+1], par_row[nnz], par_w[nnz] (rows of each parent column in
//          ascending constraint-row order, the order distributeChildToParent
//          adds them) + is_row[N] flags
//   op:    mats f64[sum nd^2] col-major per cell; optional split-BF16 hi/lo
//          copies; or diag f64[N]
//   mv:    data[N][m] row-major, vector index fastest
#pragma once
#include <cuda_runtime.h>
#include <cublas_v2.h>
#include <cusolverDn.h>
#include <cuda_bf16.h>

#include <cstdint>
#include <cstdio>
#include <atomic>
#include <map>
#include <tuple>
#include <memory>
#include <string>
#include <vector>
#include <stdexcept>

#include "../../include/gbfe.h"

namespace gbfe {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

#define GBFE_CUDA(call)                                                                      \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess)                                                                   \
      throw ::gbfe::Error(e_ == cudaErrorMemoryAllocation ? GBFE_ERR_ALLOC : GBFE_ERR_CUDA,  \
                          std::string(#call) + ": " + cudaGetErrorString(e_));               \
  } while (0)

#define GBFE_CUBLAS(call)                                                                    \
  do {                                                                                       \
    cublasStatus_t s_ = (call);                                                              \
    if (s_ != CUBLAS_STATUS_SUCCESS)                                                         \
      throw ::gbfe::Error(GBFE_ERR_CUDA, std::string(#call) + ": cublas status " +           \
                                             std::to_string((int)s_));                      \
  } while (0)

#define GBFE_CUSOLVER(call)                                                                  \
  do {                                                                                       \
    cusolverStatus_t s_ = (call);                                                            \
    if (s_ != CUSOLVER_STATUS_SUCCESS)                                                       \
      throw ::gbfe::Error(GBFE_ERR_CUDA, std::string(#call) + ": cusolver status " +         \
                                             std::to_string((int)s_));                      \
  } while (0)

#define GBFE_REQUIRE(cond, msg)                                                              \
  do {                                                                                       \
    if (!(cond)) throw ::gbfe::Error(GBFE_ERR_ARG, msg);                                     \
  } while (0)

// Devices a process may drive (the per-device flags and addresses below).
constexpr int kMaxDevices = 64;

// cudaFuncSetAttribute (the dynamic shared-memory opt-in of a kernel) is a
// property of a device's context, not of the process: a call site keeps one
// flag per device, so a context created later on another device sets the
// attribute there too.  The flags are atomic because server slot threads
// launch concurrently; two threads that both see "not done" both set the same
// value, which is harmless.  Not a stream operation, so it stays out of graph
// captures once it has run.
struct PerDeviceOnce {
  std::atomic<bool> done[kMaxDevices];
  template <class F>
  void run(int dev, F &&f) {
    if (dev < 0 || dev >= kMaxDevices) {
      f();
      return;
    }
    if (done[dev].load(std::memory_order_acquire)) return;
    f();
    done[dev].store(true, std::memory_order_release);
  }
};

// Device blocks kept for reuse by a thread that installs a cache (the serving
// workers): a block freed there is parked instead of handed to cudaFree,
// whose device-wide synchronisation would hold up the other slots' work.
// Parked blocks become reusable only at mark_safe(), which the owner calls
// once every stream that may still read them has been synchronised; blocks
// are reused by exact size.  Past `cap` parked bytes a free goes to cudaFree.
struct DevCache {
  std::multimap<size_t, void *> ready, parked;
  size_t bytes = 0, cap = 0;
  void mark_safe() {
    ready.insert(parked.begin(), parked.end());
    parked.clear();
  }
  void release() {
    for (auto &kv : ready) cudaFree(kv.second);
    for (auto &kv : parked) cudaFree(kv.second);
    ready.clear();
    parked.clear();
    bytes = 0;
  }
};
inline DevCache *&thread_dev_cache() {
  static thread_local DevCache *cache = nullptr;
  return cache;
}
inline cudaError_t dev_alloc(void **p, size_t bytes) {
  if (DevCache *c = thread_dev_cache()) {
    auto it = c->ready.find(bytes);
    if (it != c->ready.end()) {
      *p = it->second;
      c->ready.erase(it);
      c->bytes -= bytes;
      return cudaSuccess;
    }
  }
  return cudaMalloc(p, bytes);
}
inline void dev_free(void *p, size_t bytes) {
  DevCache *c = thread_dev_cache();
  if (c && c->bytes + bytes <= c->cap) {
    c->parked.emplace(bytes, p);
    c->bytes += bytes;
    return;
  }
  cudaFree(p);
}

// owning device buffer
template <class T>
struct DBuf {
  T *p = nullptr;
  size_t n = 0;
  bool borrowed = false;  // wraps memory owned by the caller: never freed here
  DBuf() = default;
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  ~DBuf() { reset(); }
  void reset() {
    if (p && !borrowed) dev_free(p, sizeof(T) * n);
    p = nullptr;
    n = 0;
    borrowed = false;
  }
  void wrap(T *ext, size_t count) {
    reset();
    p = ext;
    n = count;
    borrowed = true;
  }
  void alloc(size_t count) {
    if (count == n && p) return;
    reset();
    if (count) {
      void *q = nullptr;
      GBFE_CUDA(dev_alloc(&q, sizeof(T) * count));
      p = static_cast<T *>(q);
    }
    n = count;
  }
  // grow-only scratch
  void ensure(size_t count) {
    if (count > n) alloc(count);
  }
  void upload(const T *h, size_t count, cudaStream_t s) {
    alloc(count);
    if (count) GBFE_CUDA(cudaMemcpyAsync(p, h, sizeof(T) * count, cudaMemcpyHostToDevice, s));
  }
};

}  // namespace gbfe

// Per-kernel timing with CUDA events recorded on the launching stream
// (enabled by gbfe_ctx_set_profiling); resolved when the stats are read.
struct KernelStat {
  uint64_t launches = 0;
  double ms = 0.0, flops = 0.0, bytes = 0.0;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending;
};

// one timed kernel inside a captured graph (event-record nodes around it)
struct GraphProf {
  std::string name;
  cudaEvent_t e0, e1;
  double flops, bytes;
};

// autotuned launch shape of the persistent tensor-core kernel, keyed by
// (largest cell size of the launch group, 128-row tiles, vectors)
struct TcTune {
  uint32_t N = 0, stages = 0;
  float ms = 0.f;
  uint32_t occ = 2;   // resident CTAs per SM the kernel is compiled for (2 or 3)
  uint32_t nbuf = 0;  // TMEM accumulator buffers: 0 two where they fit, 1 one (more CTAs per SM)
  uint32_t pf = 0;    // X-row prefetch depth of the float4 gather (chunks, 0-3)
  uint32_t swap = 0;  // 1: vectors on the MMA's M extent, cell rows on N
};

// Pinned host staging for small host-to-device copies issued inside a solve:
// a copy from pageable memory synchronises the stream first, one from pinned
// memory does not.  `done` marks when the staged bytes may be overwritten.
struct PinnedSlot {
  void *h = nullptr;
  size_t cap = 0;
  cudaEvent_t done = nullptr;
  PinnedSlot() = default;
  PinnedSlot(const PinnedSlot &) = delete;
  PinnedSlot &operator=(const PinnedSlot &) = delete;
  ~PinnedSlot() {
    if (done) cudaEventDestroy(done);
    if (h) cudaFreeHost(h);
  }
};

struct gbfe_ctx {
  int device = 0;
  std::map<std::tuple<uint32_t, uint32_t, uint32_t>, TcTune> tc_tune;
  std::string tune_cache;    // file the tuned shapes are read from / appended to
  int profiling = 0;
  std::vector<GraphProf> *capture_prof = nullptr;  // set while a graph is captured with profiling on
  int use_graphs = 1;        // capture the Chebyshev recurrence into a CUDA graph
  std::map<std::string, KernelStat> kstats;
  std::vector<cudaEvent_t> event_free;  // recycled timing events of ProfScope
  std::vector<std::string> prof_only;   // profiling restricted to these scope names (empty: all)
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  // second stream for the split-BF16 size groups that do not wait on the
  // enrichment rows: forked from `stream` by fork_ev, joined by join_ev
  cudaStream_t side_stream = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  cudaEvent_t host_ev = nullptr;  // the host waits on this one, not on the stream, when work follows a download
  // instantiated filter-recurrence graphs no solve holds: the next capture of
  // the same shape updates one in place instead of instantiating anew
  std::vector<cudaGraphExec_t> fw_exec_pool;
  int split_groups = 1;      // 1: independent size groups of a cell product run concurrently
  cublasHandle_t cublas = nullptr;
  cusolverDnHandle_t cusolver = nullptr;
  std::string last_error;
  uint64_t launches = 0;
  int sm_count = 0;
  // shared scratch
  gbfe::DBuf<double> red;    // reduction partials
  gbfe::DBuf<double> small;  // m x m work matrices
  gbfe::DBuf<int> info;
  gbfe::DBuf<double> lwork;
  gbfe::DBuf<int> status;    // device status word written by bounded waits (0 = ok)
  int use_tc = 1;            // split-BF16 tcgen05 cell product for the mixed path
  int tc_version = 2;        // 2: persistent warp-specialised kernel; 1: one CTA per cell
  int tc_gather4 = 1;        // persistent kernel: 16-byte row gathers when the rows are aligned
  std::atomic<int> *cancel = nullptr;  // polled between passes / iterations when set
  int fp64_tc = 0;           // 1: FP64 applies use the sliced tensor-core product when built
  int fp64_tc_dense = 1;     // with fp64_tc: the Gram / rotation stages use the sliced products too
  int cc_major = 0;          // compute capability of the device
  int small_eig_host = 1;    // m x m eigenproblems of Rayleigh-Ritz on the host (m <= 128)
  int fuse_filter = 1;       // mixed filter: B^-1 in the tensor-core gather, step fused into the assembly
  gbfe::DBuf<int> oz_exp, oz_rexp;  // sliced products: column / row exponents
  gbfe::DBuf<int> oz_ipart;         // partial exponent maxima
  std::vector<std::unique_ptr<gbfe::DBuf<double>>> vec_pool;  // scoped m-vectors of a pass (LIFO)
  std::vector<std::unique_ptr<PinnedSlot>> vec_pin;            // their host staging
  PinnedSlot pin_small;                                        // m x m eigenvectors
  PinnedSlot pin_tab, pin_coef;  // the filter's coefficient tables (kept: cudaFreeHost synchronises the device)
  size_t vec_top = 0;
  gbfe::DBuf<double> oz_part;       // per-item Gram partials
  gbfe::DBuf<__nv_bfloat16> oz_tdig;  // slices of the rotation factor
  gbfe::DBuf<uint8_t> oz_dig;         // digit tiles of the Gram / rotation operands (each value cut once)
};

struct gbfe_mesh {
  gbfe_ctx *ctx = nullptr;
  uint64_t n_dofs = 0;
  uint32_t n_cells = 0;
  uint32_t nd_max = 0;
  uint32_t nd_min = 0;
  uint64_t total_cell_dofs = 0;  // sum nd
  uint64_t total_mat = 0;        // sum nd^2
  std::vector<uint32_t> h_nd;
  std::vector<uint32_t> h_cell_off;
  std::vector<uint64_t> h_mat_off;
  gbfe::DBuf<uint32_t> ids, cell_off, slot_ptr, slot, nd;
  gbfe::DBuf<uint64_t> mat_off;
  // size bins for variable-nd meshes: cells sorted by nd, grouped
  std::vector<uint32_t> bin_nd;       // nd of each bin
  std::vector<uint32_t> bin_begin;    // offset into bin_cells
  std::vector<uint32_t> bin_max_id;   // largest dof id in the cells of each bin
  gbfe::DBuf<uint32_t> bin_cells;     // cell ids grouped by bin
};

struct gbfe_cons {
  gbfe_mesh *mesh = nullptr;
  uint32_t n_rows = 0;
  uint64_t nnz = 0;
  bool pure_dirichlet = true;  // every row has 0 columns and 0 inhomogeneity
  gbfe::DBuf<uint32_t> row_ids, row_sizes, col_ids, row_acc;
  gbfe::DBuf<double> col_vals, inh;
  gbfe::DBuf<uint32_t> par_ptr, par_row;
  gbfe::DBuf<double> par_w;
  gbfe::DBuf<uint8_t> is_row;
};

enum OpKind { OP_CELL = 0, OP_DIAG = 1, OP_JACOBI = 2, OP_DIAG_BLOCK = 3 };

// Separable nonlocal part C^T V C (AtomCenterNonLocalOpContextFE): per cell
// c with np_c projectors the matrix C_c (np_c x nd_c, column-major, projector
// index fastest), a projector id per (cell, projector) slot, and a diagonal
// coupling V per projector.  Only cells with np_c > 0 are stored.
struct gbfe_nl {
  gbfe_mesh *mesh = nullptr;
  uint32_t n_proj = 0, n_cells_nl = 0, np_max = 0, n_slots = 0;
  gbfe::DBuf<uint32_t> cells;      // [n_cells_nl] cell index
  gbfe::DBuf<uint32_t> slot_off;   // [n_cells_nl + 1] first slot of each cell
  gbfe::DBuf<uint64_t> c_off;      // [n_cells_nl] offset of C_c in cmat
  gbfe::DBuf<uint32_t> pids;       // [n_slots] projector of each slot
  gbfe::DBuf<uint32_t> pslot_ptr;  // [n_proj + 1] slots of each projector, ascending
  gbfe::DBuf<uint32_t> pslot;      // [n_slots]
  gbfe::DBuf<double> cmat, v;
  gbfe::DBuf<float> cmat_f32, v_f32;
  mutable gbfe::DBuf<double> cx, w;  // [n_slots][m], [n_proj][m]
  mutable gbfe::DBuf<float> cx_f32, w_f32;
  mutable gbfe::DBuf<double> ycell;  // cell-wise result of the standalone apply
  mutable gbfe::DBuf<float> ycell_f32;
};

inline uint64_t gbfe_next_serial() {
  static std::atomic<uint64_t> n{0};
  return ++n;
}

struct gbfe_op {
  gbfe_mesh *mesh = nullptr;
  const gbfe_cons *cons = nullptr;
  const gbfe_nl *nl = nullptr;  // fused nonlocal part (cell operators)
  int kind = OP_CELL;
  int prec = GBFE_PREC_FP64;
  gbfe::DBuf<double> mats;            // f64 col-major per cell (or per distinct matrix)
  uint64_t mats_count = 0;            // entries in mats
  gbfe::DBuf<uint64_t> mat_off_own;   // per-cell offsets of an indexed operator
  gbfe::DBuf<__nv_bfloat16> mats_hi;  // split-BF16 hi/lo tiles (per cell, per K chunk)
  gbfe::DBuf<uint64_t> tc_aoff;       // element offset of each cell's tiles
  gbfe::DBuf<__nv_bfloat16> oz_mats;  // 8 integer slices per entry (FP64-accurate tensor product)
  gbfe::DBuf<uint64_t> oz_aoff;
  gbfe::DBuf<int> oz_row_exp;         // per cell row exponent of the slices
  mutable gbfe::DBuf<int> oz_xexp;    // per-vector exponent of the current X
  gbfe::DBuf<float> mats_f32;         // FP32 copy for the SIMT mixed apply
  gbfe::DBuf<double> diag;
  gbfe::DBuf<float> diag_f32;  // the diagonal rounded to FP32 (mixed-precision applies)
  gbfe::DBuf<double> fold_scale;  // per-dof factor of this B^-1 folded into A (0 on Dirichlet rows)
  uint64_t serial = gbfe_next_serial();  // identity (folded tiles name their B^-1 by it)
  mutable gbfe::DBuf<__nv_bfloat16> mats_hi_folded;  // split tiles of A diag(fold_scale of folded_for)
  mutable uint64_t folded_for = 0;
  uint64_t blk_begin = 0, blk_n = 0;  // OP_DIAG_BLOCK: dense block rows
  bool blk_cons = false;              // a constrained row lies inside the block
  gbfe::DBuf<double> blk;             // column-major blk_n x blk_n
  gbfe::DBuf<float> blk_f32;
  mutable gbfe::DBuf<float> blk_out_f32;  // block rows of B^-1 X for the fused filter
  mutable gbfe::DBuf<double> cellbuf;  // per-apply cell-wise result scratch (f64)
  mutable gbfe::DBuf<float> cellbuf_f32;
};

struct gbfe_mv {
  gbfe_mesh *mesh = nullptr;
  uint32_t m = 0;
  int dtype = GBFE_F64;
  gbfe::DBuf<double> d;
  gbfe::DBuf<float> f;
  size_t count() const { return (size_t)mesh->n_dofs * m; }
  void *ptr() const { return dtype == GBFE_F64 ? (void *)d.p : (void *)f.p; }
};

namespace gbfe {

// Division of an element index by the block width m without the
// multi-instruction integer division: q = (umulhi(n, mul) + n) >> shift
// (round-up multiplier), exact for n < 2^31; larger n fall back to '/'.
struct FastDiv {
  uint32_t d = 1, mul = 1, shift = 0;
  FastDiv() = default;
  explicit FastDiv(uint32_t div) : d(div ? div : 1) {
    shift = 0;
    while ((1ull << shift) < d) ++shift;
    mul = (uint32_t)(((1ull << 32) * ((1ull << shift) - d)) / d + 1);
  }
  // t -> (row, column)
  __device__ __forceinline__ void divmod(uint64_t t, uint64_t &q, uint32_t &r) const {
    if (t < (1ull << 31)) {
      const uint32_t n = (uint32_t)t;
      const uint32_t qq = (uint32_t)(((uint64_t)__umulhi(n, mul) + n) >> shift);
      q = qq;
      r = n - qq * d;
    } else {
      q = t / d;
      r = (uint32_t)(t - q * d);
    }
  }
};

// Per-column factors f[j] = (T)(s * w[j]) of one sweep over an N x m block,
// computed once per thread block into dynamic shared memory instead of once
// per element: GB300's FP64 pipe retires about two operations per SM clock,
// too few for a DMUL and a conversion per element of an FP32 sweep.
// col_factor_smem = the dynamic shared bytes of k factor arrays (0: the block
// width is too large, the kernel computes the factors per element).  The
// kernels take the choice as a template flag: with a runtime flag the
// compiler predicates the per-element FP64 branch into every iteration.
template <class T>
inline size_t col_factor_smem(uint32_t m, int k = 1) {
  const size_t b = (size_t)k * m * sizeof(T);
  return b <= 32 * 1024 ? b : 0;
}
template <class T>
__device__ __forceinline__ void load_col_factors(T *f, uint32_t m, double s, const double *__restrict__ w) {
  for (uint32_t j = threadIdx.x; j < m; j += blockDim.x) f[j] = (T)(s * w[j]);
}

inline unsigned grid_for(uint64_t n, unsigned block) {
  uint64_t g = (n + block - 1) / block;
  if (g > 0x7fffffffULL) g = 0x7fffffffULL;
  return (unsigned)(g ? g : 1);
}

inline void count_launch(gbfe_ctx *ctx, uint64_t n = 1) { ctx->launches += n; }
// the context's side stream and its fork / join events, created on first use
inline void ensure_side_stream(gbfe_ctx *ctx) {
  if (ctx->side_stream) return;
  GBFE_CUDA(cudaStreamCreateWithFlags(&ctx->side_stream, cudaStreamNonBlocking));
  GBFE_CUDA(cudaEventCreateWithFlags(&ctx->fork_ev, cudaEventDisableTiming));
  GBFE_CUDA(cudaEventCreateWithFlags(&ctx->join_ev, cudaEventDisableTiming));
}
inline void check_launch(gbfe_ctx *ctx, const char *name) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) throw Error(GBFE_ERR_CUDA, std::string(name) + ": " + cudaGetErrorString(e));
  count_launch(ctx);
}

// Brackets one launch with events when profiling is on.
struct ProfScope {
  gbfe_ctx *ctx;
  KernelStat *st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  const char *nm = nullptr;
  double fl = 0, by = 0;
  static cudaEvent_t get(gbfe_ctx *c) {
    cudaEvent_t e = nullptr;
    if (!c->event_free.empty()) {
      e = c->event_free.back();
      c->event_free.pop_back();
    } else {
      cudaEventCreate(&e);
    }
    return e;
  }
  static bool wanted(const gbfe_ctx *c, const char *name) {
    if (c->prof_only.empty()) return true;
    for (const auto &s : c->prof_only)
      if (s == name) return true;
    return false;
  }
  ProfScope(gbfe_ctx *c, const char *name, double flops, double bytes) : ctx(c), nm(name), fl(flops), by(bytes) {
    if (!ctx->profiling || !wanted(ctx, name)) return;
    e0 = get(ctx);
    e1 = get(ctx);
    if (ctx->capture_prof) {  // inside a graph: an event-record node, read after each replay
      cudaEventRecordWithFlags(e0, ctx->stream, cudaEventRecordExternal);
      return;
    }
    st = &ctx->kstats[name];
    st->flops += flops;
    st->bytes += bytes;
    cudaEventRecord(e0, ctx->stream);
  }
  ~ProfScope() {
    if (!e0) return;
    if (ctx->capture_prof && !st) {
      cudaEventRecordWithFlags(e1, ctx->stream, cudaEventRecordExternal);
      ctx->capture_prof->push_back(GraphProf{nm, e0, e1, fl, by});
      return;
    }
    cudaEventRecord(e1, ctx->stream);
    st->pending.emplace_back(e0, e1);
    st->launches++;
  }
};

// cell -> first entry of its matrix: the mesh's prefix sums, or the operator's
// own offsets when several cells share one stored matrix
inline const uint64_t *op_mat_off(const gbfe_op *op) {
  return op->mat_off_own.p ? op->mat_off_own.p : op->mesh->mat_off.p;
}

// ---- internal entry points shared between translation units
void constraints_p2c(gbfe_ctx *ctx, const gbfe_cons *c, gbfe_mv *x);
void apply_op(const gbfe_op *op, gbfe_mv *X, gbfe_mv *Y);
void apply_cell_mixed(const gbfe_op *op, gbfe_mv *X, gbfe_mv *Y);
void build_mixed_mats(gbfe_op *op);
void build_tc_mats(gbfe_op *op);
bool tc_supported(const gbfe_mesh *me);
void cell_apply_tc(const gbfe_op *op, const gbfe_mv *X, float *Yc, const __nv_bfloat16 *tiles = nullptr,
                   const float *xsub = nullptr, uint32_t sub_begin = 0, uint32_t sub_n = 0,
                   bool fork_recorded = false);
void build_tc_mats_folded(const gbfe_op *op, const double *kscale, gbfe::DBuf<__nv_bfloat16> &out);
// one step of the mixed Chebyshev recurrence in two launches:
//   R = alpha1 (A B^-1 RN - c RN) + alpha2 R + alpha1 eF2[j] Y
// (B^-1 applied in the tensor-core gather, the step fused into the assembly);
// returns false (nothing launched) where the operators do not allow it
bool filter_step_fused(const gbfe_op *A, const gbfe_op *BInv, gbfe_mv *RN, gbfe_mv *R, const double *coef,
                       const double *eF2, const gbfe_mv *Y);
// nonlocal part: W = V * (sum over slots of C_c X_c) and Yc += C_c^T W
// host -> device copy of n bytes through a pinned staging slot (no stream sync)
void h2d_staged(gbfe_ctx *ctx, PinnedSlot &slot, void *dst, const void *src, size_t n);
// Y = assembled cell-wise buffer Yc with the constraint epilogue of `cons`
void assemble_cells(gbfe_mesh *me, const gbfe_cons *cons, int dtype, const void *Yc, gbfe_mv *Y,
                    cudaStream_t stream = nullptr);
// AX = A X and BX = B X for two FP64 cell operators on the same mesh and
// constraints: the column exponents of X once, the two sliced products and
// assemblies on two streams (else two apply_op calls)
void apply_pair_f64(const gbfe_op *A, const gbfe_op *B, gbfe_mv *X, gbfe_mv *AX, gbfe_mv *BX);
void nonlocal_project(const gbfe_nl *nl, const gbfe_mv *X);
void nonlocal_add(const gbfe_nl *nl, uint32_t m, int dtype, void *Yc);
void autotune_tc(const gbfe_op *op, uint32_t m, std::vector<std::string> &log, std::vector<std::string> &fresh);
bool oz_supported(const gbfe_mesh *me);
// dense symmetric eigen-decomposition on the host (gbfe_host_eig.cpp)
int host_sym_eig(int n, double *a, double *w);
int host_cholesky(int n, double *a);
// keep the host pool's workers spinning (true) for the m x m block about to
// run, or let them sleep between blocks (false)
void host_pool_arm(bool on);
void host_trsm_lower(int n, const double *L, double *B);
void host_trsm_lower_t(int n, const double *L, double *B);
void host_sandwich(int n, const double *L, double *A);
// FP64-accurate sliced tensor-core products of the subspace stages (gbfe_ozgemm.cu)
bool oz_gemm_supported(gbfe_ctx *ctx, uint32_t m);
void oz_gram(gbfe_ctx *ctx, const double *const *A, uint32_t na, uint32_t ma, const double *B, uint32_t mb,
             uint64_t N, double *const *S, const int *bexp = nullptr);
// rows_ready: oz_rotate_rows already ran for these Y since they last changed
void oz_rotate(gbfe_ctx *ctx, const double *T, uint32_t m, uint32_t mo, const double *const *Y, double *const *out,
               uint32_t nops, uint64_t N, bool rows_ready = false);
// stream: where the launches go (default the context's stream; another
// stream is not profiled)
void oz_rotate_rows(gbfe_ctx *ctx, const double *const *Y, uint32_t m, uint32_t nops, uint64_t N,
                    bool pair12 = false, cudaStream_t stream = nullptr);
// X = Y T and R = HY T - MY T diag(eps) in one launch (2m <= 512)
bool oz_rotate_residual_supported(gbfe_ctx *ctx, uint32_t m);
void oz_rotate_residual(gbfe_ctx *ctx, const double *T, const double *eps, uint32_t m, const double *Y,
                        const double *HY, const double *MY, double *X, double *R, uint64_t N, bool rows_ready);
void build_oz_mats(gbfe_op *op);
// xexp: column exponents of X computed beforehand (nullptr: computed here)
void cell_apply_oz(const gbfe_op *op, const gbfe_mv *X, double *Yc, const int *xexp = nullptr,
                   cudaStream_t stream = nullptr);
const int *oz_column_exponents(const gbfe_op *op, const gbfe_mv *X);
// Yc (cell-wise, sum nd_c x m) = the operator's FP64 cell products of X, no
// constraints and no assembly (sliced tensor-core product in FP64 mode 1/2)
void cell_product_f64(const gbfe_op *op, gbfe_mv *X, double *Yc);

// vector kernels (solvers)
void axpby(gbfe_ctx *ctx, size_t n, double a, const gbfe_mv *x, double b, const gbfe_mv *y, gbfe_mv *z);
void col_dots(gbfe_ctx *ctx, const gbfe_mv *x, const gbfe_mv *y, double *host_out);

}  // namespace gbfe

// catch-all wrapper for the C ABI
template <class F>
static inline int gbfe_guard(gbfe_ctx *ctx, F &&f) {
  try {
    f();
    return GBFE_OK;
  } catch (const gbfe::Error &e) {
    if (ctx) ctx->last_error = e.what();
    return e.code;
  } catch (const std::bad_alloc &) {
    if (ctx) ctx->last_error = "host allocation failed";
    return GBFE_ERR_ALLOC;
  } catch (const std::exception &e) {
    if (ctx) ctx->last_error = e.what();
    return GBFE_ERR_ARG;
  }
}
