// gbfe_host_eig.cpp -- dense symmetric eigen-decomposition on the host for
// the small projected matrices of Rayleigh-Ritz (m x m, m <= a few hundred).
//
// The reference calls LAPACK dsyevd('V','L') here
// (RayleighRitzEigenSolver.t.cpp:233-301).  On the GPU that routine is a long
// chain of small launches with host round trips; for the m of the KS
// workloads one host core finishes the same decomposition sooner.  Method
// (Golub & Van Loan, Matrix Computations, sections 8.3.1 and 8.3.2):
//   1. Householder reduction T = Q^T A Q to tridiagonal form, Q accumulated
//      explicitly by applying the reflectors in reverse order;
//   2. implicit symmetric QR steps with the Wilkinson shift on the unreduced
//      trailing block, each a chase of Givens rotations G^T T G applied to the
//      tridiagonal held as two arrays and accumulated into Z = Q G_1 G_2 ...;
//      an off-diagonal entry is set to zero once it is below
//      eps (|t_ii| + |t_i+1,i+1|);
//   3. eigenvalues ascending with their eigenvector columns.
// Pure C++ (no intrinsics): identical code on x86 and Arm hosts.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <exception>
#include <functional>
#include <mutex>
#include <thread>
#include <utility>
#include <cstdint>
#include <numeric>
#include <vector>

namespace gbfe {

namespace {

// Fork-join pool for the row- and column-independent parts of the m x m block
// (the accumulation of the QR rotations into the eigenvectors, the triangular
// solves).  HOST_THREADS - 1 workers.  While the pool is armed (a caller about
// to run a whole m x m block: host_pool_arm) the workers spin on the job
// counter, so consecutive jobs start without a wake-up; otherwise a worker
// spins briefly after a job and then sleeps on a condition variable, so the
// pool burns no CPU time between blocks (on a host with a CPU quota, idle
// spinning is charged like work and can get the whole process throttled).  A
// job's split depends only on the problem size, never on timing, so results
// are the same whatever thread runs which part.
constexpr int HOST_THREADS = 4;

class HostPool {
 public:
  static HostPool &get() {
    static HostPool pool;
    return pool;
  }
  // f(part) for part = 0 .. parts-1, parts <= HOST_THREADS.  The caller runs
  // part 0 and then, like the workers, claims parts from a counter tagged with
  // the job's generation: a part no worker has started (one that is asleep or
  // was preempted) is run by the caller instead of waited for.
  void run(int parts, const std::function<void(int)> &f) {
    if (parts <= 1 || workers_.empty()) {
      for (int t = 0; t < parts; ++t) f(t);
      return;
    }
    std::lock_guard<std::mutex> serial(run_mu_);  // one job at a time
    uint64_t g;
    {
      std::lock_guard<std::mutex> lk(mu_);
      job_ = &f;
      parts_ = parts;
      pending_.store(parts, std::memory_order_relaxed);
      g = gen_.load(std::memory_order_relaxed) + 1;
      next_.store(g << 32, std::memory_order_relaxed);
      gen_.store(g, std::memory_order_release);
    }
    cv_.notify_all();
    claim_and_run(g, parts, f);
    // every part has been claimed; wait for the ones still running on workers
    // (they hold a reference to f, so f must stay alive until then), then
    // rethrow the first exception any part raised
    while (pending_.load(std::memory_order_acquire) != 0) std::this_thread::yield();
    std::exception_ptr err;
    {
      std::lock_guard<std::mutex> lk(err_mu_);
      std::swap(err, err_);
    }
    if (err) std::rethrow_exception(err);
  }
  void arm(bool on) {
    if (workers_.empty()) return;
    {
      std::lock_guard<std::mutex> lk(mu_);
      armed_.store(on, std::memory_order_release);
    }
    if (on) cv_.notify_all();
  }
  ~HostPool() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
      gen_.fetch_add(1, std::memory_order_release);
    }
    cv_.notify_all();
    for (auto &t : workers_) t.join();
  }

 private:
  HostPool() {
    const unsigned hw = std::thread::hardware_concurrency();
    const int n = hw >= 8 ? HOST_THREADS - 1 : 0;  // leave small hosts alone
    for (int i = 0; i < n; ++i) workers_.emplace_back([this, i] { loop(i + 1); });
  }
  void loop(int part) {
    uint64_t seen = 0;
    for (;;) {
      // spin while armed, else ~200 us after a job; then sleep until a job
      // comes or the pool is armed
      const auto t0 = std::chrono::steady_clock::now();
      while (gen_.load(std::memory_order_acquire) == seen &&
             (armed_.load(std::memory_order_acquire) ||
              std::chrono::steady_clock::now() - t0 < std::chrono::microseconds(200)))
        std::this_thread::yield();
      std::unique_lock<std::mutex> lk(mu_);
      cv_.wait(lk, [&] {
        return gen_.load(std::memory_order_acquire) != seen || armed_.load(std::memory_order_acquire);
      });
      if (gen_.load(std::memory_order_acquire) == seen) continue;  // armed, no job yet: spin
      seen = gen_.load(std::memory_order_acquire);
      if (stop_) return;
      const std::function<void(int)> *job = job_;
      const int parts = parts_;
      lk.unlock();
      claim_and_run(seen, parts, *job);
    }
  }
  // run unclaimed parts of job generation g until none is left; a claim is a
  // compare-and-swap on (generation << 32 | next part), so a thread holding a
  // finished job's pointer can never claim a part of the next job
  void claim_and_run(uint64_t g, int parts, const std::function<void(int)> &f) {
    for (;;) {
      uint64_t cur = next_.load(std::memory_order_acquire);
      if ((cur >> 32) != g || (int)(cur & 0xffffffffu) >= parts) return;
      if (!next_.compare_exchange_weak(cur, cur + 1, std::memory_order_acq_rel)) continue;
      // a part that throws still counts as done: the exception is kept for
      // run() to rethrow in the calling thread (never escapes a worker)
      try {
        f((int)(cur & 0xffffffffu));
      } catch (...) {
        std::lock_guard<std::mutex> lk(err_mu_);
        if (!err_) err_ = std::current_exception();
      }
      pending_.fetch_sub(1, std::memory_order_acq_rel);
    }
  }
  std::vector<std::thread> workers_;
  std::mutex mu_, run_mu_, err_mu_;
  std::exception_ptr err_;  // first exception of the current job
  std::condition_variable cv_;
  std::atomic<uint64_t> gen_{0};
  std::atomic<int> pending_{0};
  std::atomic<uint64_t> next_{0};
  std::atomic<bool> armed_{false};
  const std::function<void(int)> *job_ = nullptr;
  int parts_ = 0;
  bool stop_ = false;
};

// parts of an n-wide independent range worth a thread each
inline int host_parts(int n) { return n >= 48 ? HOST_THREADS : 1; }

}  // namespace

// a: n x n column-major; the lower triangle is read.  On success a holds the
// orthonormal eigenvectors (column j belongs to w[j]) and w the eigenvalues in
// ascending order.  Returns 0, or 1 if the QR iteration did not converge.
int host_sym_eig(int n, double *a, double *w) {
  if (n <= 0) return 0;
  const size_t N = (size_t)n;
  auto A = [&](std::vector<double> &M, int i, int j) -> double & { return M[(size_t)i + N * (size_t)j]; };
  std::vector<double> T(N * N), Z(N * N, 0.0), v(N), p(N), q(N);
  for (int j = 0; j < n; ++j)
    for (int i = j; i < n; ++i) A(T, i, j) = A(T, j, i) = a[(size_t)i + N * j];

  // ---- 1. Householder tridiagonalization; reflector k lives on rows k+1..n-1
  std::vector<double> refl(N * N, 0.0), beta(N, 0.0);
  for (int k = 0; k + 2 < n; ++k) {
    const int L = n - k - 1;
    double nx = 0.0;
    for (int i = 0; i < L; ++i) {
      v[i] = A(T, k + 1 + i, k);
      nx += v[i] * v[i];
    }
    nx = std::sqrt(nx);
    if (nx == 0.0) continue;
    const double alpha = v[0] >= 0.0 ? -nx : nx;
    v[0] -= alpha;
    double vv = 0.0;
    for (int i = 0; i < L; ++i) vv += v[i] * v[i];
    if (vv == 0.0) continue;
    const double b = 2.0 / vv;
    // p = b A22 v;  q = p - (b/2)(v^T p) v;  A22 -= v q^T + q v^T, on the
    // lower triangle of A22 only (symmetric: one pass down each column gives
    // both its axpy into p and its dot with v)
    for (int i = 0; i < L; ++i) p[i] = 0.0;
    for (int j = 0; j < L; ++j) {  // column-major: contiguous inner loops
      const double vj = b * v[j];
      const double *col = &A(T, k + 1, k + 1 + j);
      double dot = 0.0;
      for (int i = j + 1; i < L; ++i) {
        p[i] += col[i] * vj;
        dot += col[i] * v[i];
      }
      p[j] += col[j] * vj + b * dot;
    }
    double vp = 0.0;
    for (int i = 0; i < L; ++i) vp += v[i] * p[i];
    const double K = 0.5 * b * vp;
    for (int i = 0; i < L; ++i) q[i] = p[i] - K * v[i];
    for (int j = 0; j < L; ++j) {
      double *col = &A(T, k + 1, k + 1 + j);
      const double qj = q[j], vj = v[j];
      for (int i = j; i < L; ++i) col[i] -= v[i] * qj + q[i] * vj;
    }
    A(T, k + 1, k) = A(T, k, k + 1) = alpha;
    for (int i = 1; i < L; ++i) A(T, k + 1 + i, k) = A(T, k, k + 1 + i) = 0.0;
    for (int i = 0; i < L; ++i) refl[(size_t)k * N + i] = v[i];
    beta[k] = b;
  }
  // Q = H_0 H_1 ... H_{n-3}, built as H_k Q for k descending.  Column j is
  // touched by the reflectors k < j only, each column independently: the
  // columns are dealt round robin to the pool (column j costs ~j reflectors)
  for (int i = 0; i < n; ++i) A(Z, i, i) = 1.0;
  {
    const int parts = host_parts(n);
    HostPool::get().run(parts, [&](int part) {
      for (int j = 1 + part; j < n; j += parts)
        for (int k = std::min(j - 1, n - 3); k >= 0; --k) {
          if (beta[k] == 0.0) continue;
          const int L = n - k - 1;
          const double *vk = &refl[(size_t)k * N];
          double *z = &A(Z, k + 1, j);
          double s = 0.0;
          for (int i = 0; i < L; ++i) s += vk[i] * z[i];
          s *= beta[k];
          for (int i = 0; i < L; ++i) z[i] -= s * vk[i];
        }
    });
  }

  // ---- 2. implicit symmetric QR with Wilkinson shifts on the tridiagonal
  // held as arrays (diagonal d, off-diagonal e): one step on the unreduced
  // block [lo, hi] chases the bulge with rotations G_k on (k, k+1); with
  // G^T = [c -s; s c] the rows and columns of T and the columns of Z change as
  //   e[k-1] <- c e[k-1] - s bulge                 (the bulge is annihilated)
  //   d[k]   <- c^2 a - 2cs b + s^2 c'   d[k+1] <- s^2 a + 2cs b + c^2 c'
  //   e[k]   <- cs (a - c') + (c^2 - s^2) b      (a = d[k], b = e[k], c' = d[k+1])
  //   bulge  <- -s e[k+1],  e[k+1] <- c e[k+1]
  std::vector<double> d(N), e(N, 0.0);
  for (int i = 0; i < n; ++i) d[i] = A(T, i, i);
  for (int i = 0; i + 1 < n; ++i) e[i] = A(T, i + 1, i);
  const double eps = std::ldexp(1.0, -53);
  auto negligible = [&](int i) { return std::fabs(e[i]) <= eps * (std::fabs(d[i]) + std::fabs(d[i + 1])); };
  auto givens = [](double x, double z, double &c, double &s) {
    // [c -s; s c] [x; z] = [r; 0]
    if (z == 0.0) {
      c = 1.0;
      s = 0.0;
    } else if (std::fabs(z) > std::fabs(x)) {
      const double t = -x / z;
      s = 1.0 / std::sqrt(1.0 + t * t);
      c = s * t;
    } else {
      const double t = -z / x;
      c = 1.0 / std::sqrt(1.0 + t * t);
      s = c * t;
    }
  };
  std::vector<int> rot_k;
  std::vector<double> rot_cs;
  rot_k.reserve(N * 40);
  rot_cs.reserve(N * 80);
  int hi = n - 1;
  long iter = 0;
  const long max_iter = 60L * n;
  while (hi > 0) {
    if (negligible(hi - 1)) {
      e[hi - 1] = 0.0;
      --hi;
      continue;
    }
    if (++iter > max_iter) return 1;
    int lo = hi - 1;
    while (lo > 0 && !negligible(lo - 1)) --lo;
    if (lo > 0) e[lo - 1] = 0.0;
    const double tnn = d[hi], tn1 = e[hi - 1];
    const double dd = 0.5 * (d[hi - 1] - tnn);
    const double mu = tnn - tn1 * tn1 / (dd + (dd >= 0.0 ? 1.0 : -1.0) * std::hypot(dd, tn1));
    double x = d[lo] - mu, z = e[lo], bulge = 0.0;
    for (int k = lo; k < hi; ++k) {
      double c, s;
      givens(x, z, c, s);
      if (k > lo) e[k - 1] = c * e[k - 1] - s * bulge;
      const double a = d[k], b = e[k], cp = d[k + 1];
      const double cc = c * c, ss = s * s, cs = c * s;
      d[k] = cc * a - 2.0 * cs * b + ss * cp;
      d[k + 1] = ss * a + 2.0 * cs * b + cc * cp;
      e[k] = cs * (a - cp) + (cc - ss) * b;
      if (k + 1 < hi) {
        bulge = -s * e[k + 1];
        e[k + 1] = c * e[k + 1];
      }
      rot_k.push_back(k);
      rot_cs.push_back(c);
      rot_cs.push_back(s);
      x = e[k];
      z = bulge;
    }
  }
  for (int i = 0; i < n; ++i) A(T, i, i) = d[i];
  // Z <- Z G_1 G_2 ...: every row of Z sees the rotations in order, rows are
  // independent, so blocks of rows go to the pool (each block copied into a
  // small column-major tile so a rotation updates two contiguous columns)
  {
    const int parts = host_parts(n);
    const size_t nrot = rot_k.size();
    HostPool::get().run(parts, [&](int part) {
      const int r0 = (int)((int64_t)n * part / parts), r1 = (int)((int64_t)n * (part + 1) / parts);
      const int rb = r1 - r0;
      if (rb <= 0) return;
      std::vector<double> tile((size_t)rb * N);
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < rb; ++i) tile[(size_t)j * rb + i] = A(Z, r0 + i, j);
      for (size_t r = 0; r < nrot; ++r) {
        const int k = rot_k[r];
        const double c = rot_cs[2 * r], sn = rot_cs[2 * r + 1];
        double *zk = &tile[(size_t)k * rb], *zk1 = zk + rb;
        for (int i = 0; i < rb; ++i) {
          const double p = zk[i], q = zk1[i];
          zk[i] = c * p - sn * q;
          zk1[i] = sn * p + c * q;
        }
      }
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < rb; ++i) A(Z, r0 + i, j) = tile[(size_t)j * rb + i];
    });
  }

  // ---- 3. ascending order
  std::vector<int> ord(N);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int i, int j) { return A(T, i, i) < A(T, j, j); });
  for (int j = 0; j < n; ++j) {
    w[j] = A(T, ord[j], ord[j]);
    for (int i = 0; i < n; ++i) a[(size_t)i + N * j] = A(Z, i, ord[j]);
  }
  return 0;
}

// Cholesky factor of the symmetric positive definite a (n x n column-major,
// lower triangle read), in place: a = L with L L^T = A, upper triangle zeroed.
// Returns 0, or k + 1 when the leading minor of order k + 1 is not positive
// definite (LAPACK potrf's info).  Column-oriented (left-looking) elimination:
// every inner loop runs down a contiguous column.
void host_pool_arm(bool on) { HostPool::get().arm(on); }

int host_cholesky(int n, double *a) {
  const size_t N = (size_t)n;
  for (int k = 0; k < n; ++k) {
    double *ck = a + N * k;
    // column k -= sum_{j<k} L(k, j) L(k:n, j)
    for (int j = 0; j < k; ++j) {
      const double *cj = a + N * j;
      const double lkj = cj[k];
      if (lkj == 0.0) continue;
      for (int i = k; i < n; ++i) ck[i] -= lkj * cj[i];
    }
    const double d = ck[k];
    if (!(d > 0.0)) return k + 1;
    const double r = std::sqrt(d);
    ck[k] = r;
    const double inv = 1.0 / r;
    for (int i = k + 1; i < n; ++i) ck[i] *= inv;
    for (int i = 0; i < k; ++i) ck[i] = 0.0;
  }
  return 0;
}

// B <- L^-1 B for lower triangular L (both n x n column-major): forward
// substitution on every column of B, column-oriented
void host_trsm_lower(int n, const double *L, double *B) {
  const size_t N = (size_t)n;
  const int parts = host_parts(n);
  HostPool::get().run(parts, [&](int part) {
  for (int j = (int)((int64_t)n * part / parts); j < (int)((int64_t)n * (part + 1) / parts); ++j) {
    double *b = B + N * j;
    for (int k = 0; k < n; ++k) {
      const double *lk = L + N * k;
      const double x = b[k] / lk[k];
      b[k] = x;
      if (x == 0.0) continue;
      for (int i = k + 1; i < n; ++i) b[i] -= lk[i] * x;
    }
  }
  });
}

// B <- L^-T B for lower triangular L: back substitution with the rows of L^T
// (the columns of L), every dot product down a contiguous column
void host_trsm_lower_t(int n, const double *L, double *B) {
  const size_t N = (size_t)n;
  const int parts = host_parts(n);
  HostPool::get().run(parts, [&](int part) {
  for (int j = (int)((int64_t)n * part / parts); j < (int)((int64_t)n * (part + 1) / parts); ++j) {
    double *b = B + N * j;
    for (int k = n - 1; k >= 0; --k) {
      const double *lk = L + N * k;
      double s = b[k];
      for (int i = k + 1; i < n; ++i) s -= lk[i] * b[i];
      b[k] = s / lk[k];
    }
  }
  });
}

// A <- L^-1 A L^-T for symmetric A (full storage): W = L^-1 A, then
// L^-1 W^T = L^-1 A L^-T (A = A^T), symmetrised from its lower triangle
void host_sandwich(int n, const double *L, double *A) {
  const size_t N = (size_t)n;
  host_trsm_lower(n, L, A);
  for (int j = 0; j < n; ++j)
    for (int i = j + 1; i < n; ++i) std::swap(A[i + N * j], A[j + N * i]);
  host_trsm_lower(n, L, A);
  for (int j = 0; j < n; ++j)
    for (int i = j + 1; i < n; ++i) A[j + N * i] = A[i + N * j];
}

}  // namespace gbfe
