// ref_driver.cpp -- runs the reference's own (unmodified) CPU implementation
// of the hot path on inputs read from a directory, and writes the outputs.
// TEST INFRASTRUCTURE ONLY: it generates the golden vectors under
// tests/golden/; nothing in the product links it.
//
// Reference code exercised (compiled from its own sources):
//   ksdft::KohnShamOperatorContextFE<double,...,HOST,3>::apply
//       (ksdft/KohnShamOperatorContextFE.t.cpp:1326-1443)  for H, M and K
//   basis::ConstraintsInternal<double,HOST> (basis/ConstraintsInternal.cpp)
//   linearAlgebra::ResidualChebyshevFilterGEP (ChebyshevFilter.t.cpp:242-444)
//   linearAlgebra::ChebyshevFilter (ChebyshevFilter.t.cpp:39-135)
//   linearAlgebra::CGLinearSolver::solve (CGLinearSolver.t.cpp:68-313)
//   linearAlgebra::PreconditionerJacobi (PreconditionerJacobi.t.cpp)
//   basis::OrthoEFEOverlapInverseOpContextGLL::apply, direct branch
//       (OrthoEFEOverlapInverseOpContextGLL.t.cpp:1173-1305)
//   basis::AtomCenterNonLocalOpContextFE apply-side members
//       (AtomCenterNonLocalOpContextFE.t.cpp:36-265, :714-1045), standalone
//       and fused into the KS apply through an ONCV component
//       (KohnShamOperatorContextFE.t.cpp:1022-1080, :1177-1180)
// The M^-1 (GLL) operator below repeats the three calls of
// CFEOverlapInverseOpContextGLL::apply's diagonal branch
// (CFEOverlapInverseOpContextGLL.t.cpp:528-559) because that class's
// constructor needs the deal.II basis-data stack.
//
// Usage: ref_driver <dir>
//   inputs : meta.txt, nd.u32, ids.u32, H.f64, M.f64, K.f64, minv.f64,
//            jacdiag.f64, cons_rows.u32, cons_sizes.u32, cons_cols.u32,
//            cons_acc.u32, cons_vals.f64, cons_inh.f64, X.f64, eig.f64, b.f64
//            optional nonlocal part: nl_meta.txt (n_proj), nl_np.u32,
//            nl_pids.u32, nl_c.f64, nl_v.f64
//            optional enrichment block: efe_meta.txt (first enrichment id,
//            count), efe_blk.f64 (inverse enrichment overlap, column-major)
//   outputs: Y_H.f64, X_after.f64, Y_M.f64, Y_Minv.f64, Y_rfilter.f64,
//            Y_filter.f64, x_cg.f64, cg.txt; with the nonlocal inputs also
//            Y_nl.f64 (standalone) and Y_Hnl.f64 (H + nonlocal, fused); with
//            the enrichment block Y_Minv_efe.f64
#include <fstream>
#include <ksdft/KohnShamOperatorContextFE.h>
#include <basis/ConstraintsInternal.h>
#include <linearAlgebra/ChebyshevFilter.h>
#include <linearAlgebra/CGLinearSolver.h>
#include <linearAlgebra/PreconditionerJacobi.h>
#include <linearAlgebra/LinearSolverFunction.h>
#include <basis/OrthoEFEOverlapInverseOpContextGLL.h>
#include <cstdio>
#include <string>
#include <vector>

using namespace dftefe;
constexpr auto HOST = utils::MemorySpace::HOST;

template <class T>
static std::vector<T> read_bin(const std::string &path) {
  std::ifstream f(path, std::ios::binary | std::ios::ate);
  if (!f) return {};
  const std::streamsize n = f.tellg();
  f.seekg(0);
  std::vector<T> v(n / sizeof(T));
  f.read(reinterpret_cast<char *>(v.data()), n);
  return v;
}

template <class T>
static void write_bin(const std::string &path, const T *p, size_t n) {
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char *>(p), n * sizeof(T));
}

// ConstraintsLocal over the CSR arrays, forwarding to the reference's
// ConstraintsInternal<double, HOST>.
struct CsrConstraints : basis::ConstraintsLocal<double, HOST> {
  utils::MemoryStorage<size_type, HOST> rows, sizes, cols, acc;
  utils::MemoryStorage<double, HOST> vals, inh;
  void copyFrom(const basis::ConstraintsLocal<double, HOST> &) override {}
  void clear() override {}
  void setInhomogeneity(global_size_type, double) override {}
  void close() override {}
  bool isClosed() const override { return true; }
  bool isConstrained(global_size_type) const override { return false; }
  const std::vector<std::pair<global_size_type, double>> *getConstraintEntries(const global_size_type) const override {
    return nullptr;
  }
  bool isInhomogeneouslyConstrained(const global_size_type) const override { return false; }
  double getInhomogeneity(const global_size_type) const override { return 0.0; }
  void distributeChildToParent(linearAlgebra::MultiVector<double, HOST> &x, size_type b) const override {
    basis::ConstraintsInternal<double, HOST>::constraintsDistributeChildToParent(x, b, rows, sizes, cols, acc, vals,
                                                                                *x.getLinAlgOpContext());
  }
  void distributeParentToChild(linearAlgebra::MultiVector<double, HOST> &x, size_type b) const override {
    basis::ConstraintsInternal<double, HOST>::constraintsDistributeParentToChild(x, b, rows, sizes, cols, acc, vals,
                                                                                inh, *x.getLinAlgOpContext());
  }
  void setConstrainedNodesToZero(linearAlgebra::MultiVector<double, HOST> &x, size_type b) const override {
    basis::ConstraintsInternal<double, HOST>::constraintsSetConstrainedNodesToZero(x, b, rows);
  }
  void setConstrainedNodes(linearAlgebra::MultiVector<double, HOST> &x, size_type b, double a) const override {
    basis::ConstraintsInternal<double, HOST>::constraintsSetConstrainedNodes(x, b, rows, a);
  }
};

// A Hamiltonian component whose local part is a given set of cell matrices.
struct GivenCellMatrices : ksdft::Hamiltonian<double, HOST> {
  std::vector<double> mats;
  void getLocal(utils::MemoryStorage<double, HOST> &s) const override {
    s.resize(mats.size());
    s.copyFrom(mats);
  }
  void applyNonLocal(linearAlgebra::MultiVector<double, HOST> &, linearAlgebra::MultiVector<double, HOST> &, bool,
                     bool) const override {}
  bool hasLocalComponent() const override { return true; }
  bool hasNonLocalComponent() const override { return false; }
};

using Basis = basis::FEBasisManager<double, double, HOST, 3>;
using KSOp = ksdft::KohnShamOperatorContextFE<double, double, double, double, HOST, 3>;
using MV = linearAlgebra::MultiVector<double, HOST>;

// CFEOverlapInverseOpContextGLL::apply, diagonal branch
struct DiagInverseGLL : linearAlgebra::OperatorContext<double, double, HOST> {
  const Basis *basis;
  linearAlgebra::Vector<double, HOST> *diagInv;
  void apply(MV &X, MV &Y, bool, bool) const override {
    basis->getConstraints().distributeParentToChild(X, X.getNumberComponents());
    Y.setValue(0.0);
    linearAlgebra::blasLapack::khatriRaoProduct(linearAlgebra::blasLapack::Layout::ColMajor, 1,
                                                X.getNumberComponents(), diagInv->localSize(), diagInv->data(),
                                                X.data(), Y.data(), *(diagInv->getLinAlgOpContext()));
    basis->getConstraints().distributeChildToParent(Y, Y.getNumberComponents());
  }
};

struct PoissonFunction : linearAlgebra::LinearSolverFunction<double, double, HOST> {
  const linearAlgebra::OperatorContext<double, double, HOST> *A, *PC;
  MV *rhs, *guess, *solution;
  utils::mpi::MPIComm comm = utils::mpi::MPICommWorld;
  const linearAlgebra::OperatorContext<double, double, HOST> &getAxContext() const override { return *A; }
  const linearAlgebra::OperatorContext<double, double, HOST> &getPCContext() const override { return *PC; }
  void setSolution(const MV &x) override { *solution = x; }
  void getSolution(MV &s) override { s = *solution; }
  const MV &getRhs() const override { return *rhs; }
  const MV &getInitialGuess() const override { return *guess; }
  const utils::mpi::MPIComm &getMPIComm() const override { return comm; }
};

int main(int argc, char **argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: %s <dir>\n", argv[0]);
    return 2;
  }
  const std::string d = std::string(argv[1]) + "/";
  size_type N, C, m, degree, maxIter, nrhs;
  double wl, wu, uu, absTol, relTol, divTol;
  {
    std::ifstream meta(d + "meta.txt");
    meta >> N >> C >> m >> degree >> wl >> wu >> uu >> maxIter >> absTol >> relTol >> divTol >> nrhs;
    if (!meta) {
      fprintf(stderr, "bad meta.txt\n");
      return 2;
    }
  }
  auto ctx = std::make_shared<linearAlgebra::LinAlgOpContext<HOST>>(
      std::make_shared<linearAlgebra::blasLapack::BlasQueue<HOST>>(0),
      std::make_shared<linearAlgebra::blasLapack::LapackQueue<HOST>>(0));

  Basis basis;
  auto nd = read_bin<uint32_t>(d + "nd.u32");
  auto ids = read_bin<uint32_t>(d + "ids.u32");
  basis.nCells = C;
  basis.cellDofs.assign(nd.begin(), nd.end());
  std::vector<size_type> ids_st(ids.begin(), ids.end());
  basis.cellIds.resize(ids_st.size());
  basis.cellIds.copyFrom(ids_st);
  basis.pattern = std::make_shared<utils::mpi::MPIPatternP2P<HOST>>(N);

  CsrConstraints cons;
  {
    auto load_st = [&](const char *name, utils::MemoryStorage<size_type, HOST> &dst) {
      auto v = read_bin<uint32_t>(d + name);
      std::vector<size_type> s(v.begin(), v.end());
      dst.resize(s.size());
      if (!s.empty()) dst.copyFrom(s);
    };
    load_st("cons_rows.u32", cons.rows);
    load_st("cons_sizes.u32", cons.sizes);
    load_st("cons_cols.u32", cons.cols);
    load_st("cons_acc.u32", cons.acc);
    auto vals = read_bin<double>(d + "cons_vals.f64");
    auto inh = read_bin<double>(d + "cons_inh.f64");
    cons.vals.resize(vals.size());
    if (!vals.empty()) cons.vals.copyFrom(vals);
    cons.inh.resize(inh.size());
    if (!inh.empty()) cons.inh.copyFrom(inh);
  }
  basis.constraints = &cons;

  auto make_op = [&](const char *file) {
    auto comp = std::make_shared<GivenCellMatrices>();
    comp->mats = read_bin<double>(d + file);
    std::vector<KSOp::HamiltonianPtrVariant> hv{std::shared_ptr<ksdft::Hamiltonian<double, HOST>>(comp)};
    return std::make_unique<KSOp>(basis, hv, ctx, 1, std::max<size_type>(m, nrhs), true);
  };
  auto opH = make_op("H.f64");
  auto opM = make_op("M.f64");
  auto opK = make_op("K.f64");

  auto minv = read_bin<double>(d + "minv.f64");
  linearAlgebra::Vector<double, HOST> diagInv(basis.pattern, ctx);
  std::copy(minv.begin(), minv.end(), diagInv.data());
  DiagInverseGLL opMinv;
  opMinv.basis = &basis;
  opMinv.diagInv = &diagInv;

  auto X0 = read_bin<double>(d + "X.f64");
  auto eig = read_bin<double>(d + "eig.f64");
  auto load_mv = [&](MV &mv, const std::vector<double> &src) { std::copy(src.begin(), src.end(), mv.data()); };

  {  // applies
    MV X(basis.pattern, ctx, m, 0.0), Y(basis.pattern, ctx, m, 0.0);
    load_mv(X, X0);
    opH->apply(X, Y, true, false);
    write_bin(d + "Y_H.f64", Y.data(), (size_t)N * m);
    write_bin(d + "X_after.f64", X.data(), (size_t)N * m);
    load_mv(X, X0);
    opM->apply(X, Y, true, false);
    write_bin(d + "Y_M.f64", Y.data(), (size_t)N * m);
    load_mv(X, X0);
    opMinv.apply(X, Y, true, false);
    write_bin(d + "Y_Minv.f64", Y.data(), (size_t)N * m);
  }
#ifdef GBFE_REF_HAS_ORTHO_EFE_INVERSE
  {  // OrthoEFE inverse overlap (enriched meshes: the enrichment ids are the last ones)
    std::ifstream em(d + "efe_meta.txt");
    size_type enrBegin = 0, nEnr = 0;
    if (em >> enrBegin >> nEnr) {
      basis.ownedRanges = {{0, enrBegin}, {enrBegin, enrBegin + nEnr}};
      basis::EFEGlobalRanges gr;
      gr.ranges = basis.ownedRanges;
      auto blk = read_bin<double>(d + "efe_blk.f64");
      using EfeInv = basis::OrthoEFEOverlapInverseOpContextGLL<double, double, HOST, 3>;
      EfeInv opEfe(basis, gr, minv, nEnr, blk, ctx);
      MV X(basis.pattern, ctx, m, 0.0), Y(basis.pattern, ctx, m, 0.0);
      load_mv(X, X0);
      opEfe.apply(X, Y, true, false);
      write_bin(d + "Y_Minv_efe.f64", Y.data(), (size_t)N * m);
    }
  }
#endif
#ifdef GBFE_REF_HAS_NONLOCAL
  {  // nonlocal part: standalone and fused into the KS apply
    std::ifstream nm(d + "nl_meta.txt");
    size_type nProj = 0;
    if (nm >> nProj) {
      auto np = read_bin<uint32_t>(d + "nl_np.u32");
      auto pids = read_bin<uint32_t>(d + "nl_pids.u32");
      std::vector<size_type> np_st(np.begin(), np.end()), pid_st(pids.begin(), pids.end());
      auto cc = read_bin<double>(d + "nl_c.f64");
      auto vv = read_bin<double>(d + "nl_v.f64");
      using NLOp = basis::AtomCenterNonLocalOpContextFE<double, double, HOST, 3>;
      auto nl = std::make_shared<const NLOp>(basis, nProj, np_st, pid_st, cc, vv, 1, std::max<size_type>(m, nrhs), ctx);
      MV X(basis.pattern, ctx, m, 0.0), Y(basis.pattern, ctx, m, 0.0);
      load_mv(X, X0);
      nl->apply(X, Y, true, false);
      write_bin(d + "Y_nl.f64", Y.data(), (size_t)N * m);
      auto oncv = std::make_shared<ksdft::ElectrostaticONCVNonLocFE<double, double, double, double, HOST, 3>>();
      oncv->localMats = read_bin<double>(d + "H.f64");
      oncv->nonLocal = nl;
      std::vector<KSOp::HamiltonianPtrVariant> hv{std::shared_ptr<ksdft::Hamiltonian<double, HOST>>(oncv)};
      KSOp opHnl(basis, hv, ctx, 1, std::max<size_type>(m, nrhs), true);
      load_mv(X, X0);
      opHnl.apply(X, Y, true, false);
      write_bin(d + "Y_Hnl.f64", Y.data(), (size_t)N * m);
    }
  }
#endif
  {  // residual Chebyshev filter
    MV X(basis.pattern, ctx, m, 0.0), Y(basis.pattern, ctx, m, 0.0);
    load_mv(X, X0);
    std::vector<double> ev(eig.begin(), eig.end());
    linearAlgebra::ResidualChebyshevFilterGEP<double, double, HOST>(*opH, *opM, opMinv, ev, X, degree, wl, wu, uu, Y);
    write_bin(d + "Y_rfilter.f64", Y.data(), (size_t)N * m);
  }
  {  // standard Chebyshev filter
    MV X(basis.pattern, ctx, m, 0.0), Y(basis.pattern, ctx, m, 0.0);
    load_mv(X, X0);
    linearAlgebra::ChebyshevFilter<double, double, HOST>(*opH, opMinv, X, degree, wl, wu, uu, Y);
    write_bin(d + "Y_filter.f64", Y.data(), (size_t)N * m);
  }
  {  // Jacobi-preconditioned CG on K
    auto jd = read_bin<double>(d + "jacdiag.f64");
    linearAlgebra::Vector<double, HOST> diag(basis.pattern, ctx);
    std::copy(jd.begin(), jd.end(), diag.data());
    linearAlgebra::PreconditionerJacobi<double, double, HOST> pc(diag);
    auto bv = read_bin<double>(d + "b.f64");
    MV b(basis.pattern, ctx, nrhs, 0.0), x0(basis.pattern, ctx, nrhs, 0.0), sol(basis.pattern, ctx, nrhs, 0.0);
    load_mv(b, bv);
    PoissonFunction f;
    f.A = opK.get();
    f.PC = &pc;
    f.rhs = &b;
    f.guess = &x0;
    f.solution = &sol;
    linearAlgebra::CGLinearSolver<double, double, HOST> cg(maxIter, absTol, relTol, divTol);
    auto err = cg.solve(f);
    write_bin(d + "x_cg.f64", sol.data(), (size_t)N * nrhs);
    std::ofstream o(d + "cg.txt");
    o << (err.isSuccess ? 0 : 1) << "\n" << err.msg << "\n";
  }
  return 0;
}
