// p-multigrid preconditioner on the device.
//
// Mirrors (nekRS tree):
//   MGSolver_t::Run / runVcycle             src/solvers/elliptic/MG/MGSolver.cpp:150-193
//   pMGLevel smoothers / residual / transfers  src/solvers/elliptic/MG/ellipticMultiGridLevel.cpp:31-277
//   pMGLevel::setupSmoother, maxEigSmoothAx  src/solvers/elliptic/MG/ellipticMultiGridLevelSetup.cpp:109-453
//   ellipticMultiGridSetup                   src/solvers/elliptic/MG/ellipticMultiGridSetup.cpp:60-343
//   ellipticPreconditioner (MG branch)       src/solvers/elliptic/ellipticPreconditioner.cpp:55-62
// The whole hierarchy lives in HBM for the lifetime of the solver (meshes,
// geometric factors, FDM operators, halo maps).  The multigrid arithmetic
// runs in the precision T of `mgPrecision` (fp64 or fp32); the coarsest level
// is solved by Jacobi-PCG in T to `coarseTol` (default 1e-4) or smoothed.

#include "amg.hpp"
#include "mg_host.hpp"

#include <map>
#include <mutex>
#include <tuple>
#include "mg_kernels.hpp"

#include <cmath>
#include <cstring>

namespace nrsg {

struct MGState {
  virtual ~MGState() = default;
  virtual void apply(const double *r, double *z) = 0;
  virtual std::vector<double> info(const std::string &what) = 0;
  virtual void schwarz(int level, const double *u, double *Su) = 0;
  virtual void fdm(int level, const void *u, void *Su) = 0;
  virtual void coarse_launch() = 0;
  virtual bool graph_capturable() = 0;
  virtual long long level_size(int level) = 0;
  virtual int error() = 0;
  virtual void clear_error() = 0;
};
void MGDeleter::operator()(MGState *m) const { delete m; }

template <typename T> struct MGLevelDev {
  FieldLevel *L = nullptr;
  std::unique_ptr<FieldLevel> own;
  DevBuf<T> ggeo, D, invDegree;
  DevBuf<T> R, invDegreeFine;
  int Nf = 0;
  bool smoothed = true;
  DevBuf<T> invDiag;
  double rho = 0, lambda0 = 0, lambda1 = 0;
  int up = 2, down = 2;
  std::vector<double> upBetas, downBetas;
  DevBuf<T> Sx, Sy, Sz, invL, lam, wts, haloOut;  // invL (FP64 multigrid) or lam (FP32: 1/(lx+ly+lz) rebuilt)
  DevBuf<int> haloSrc, haloPartner;
  DevBuf<T> x, rhs, res;
  int axVariant = kAxVec;                      // FP32 axhelm variant (autotuner)
  std::vector<double> axMs;                    // autotuner: ms per launch of each variant, -1 not applicable / rejected
};

// Autotuner results shared by every solver of the process: (device, order, Poisson, elements) -> variant
namespace {
struct AxTuneCache {
  std::mutex m;
  std::map<std::tuple<int, int, int, long long>, std::pair<int, std::vector<double>>> best;
};
AxTuneCache &ax_tune_cache()
{
  static AxTuneCache c;
  return c;
}
} // namespace

template <typename T> struct MGImpl : public MGState {
  Elliptic &el;
  cudaStream_t &s; // the solver's stream (nrsg_elliptic_set_stream may replace it)
  MGPlan plan;
  std::vector<MGLevelDev<T>> lv;
  DevBuf<T> sRes, sRes2, sUpd, sTmp, rP, zP;
  DevBuf<T> cp, cz, cAp, cr;
  DevBuf<PcgScalars> csc;
  // persistent coarse solve (order-1 coarsest level)
  bool persistentCoarse = false;
  // algebraic multigrid coarse solve (coarseSolver = amg): one V-cycle on the assembled order-1 operator
  bool amgCoarse = false;
  AmgDevice<T> amg;
  DevBuf<int> amgRep, amgRowOf; // row -> representative E-vector node, E-vector node -> row (-1 masked)
  long long amgRows = 0;
  std::vector<double> amgInfo;  // rows and nonzeros per level, coarsest last
  static constexpr int kCoarseGridMax = 4096;
  DevBuf<double> cPartials;
  DevBuf<unsigned char> cState;
  // assembled coarse operator and its row vectors
  CoarseMatrix<T> cA;
  DevBuf<T> cx, cz2, cz3;
  DevBuf<T> cOnes;          // all-Neumann: ones on the coarsest level, for its rhs mean
  DevBuf<double> cSum;
  double cUnknowns = 0;     // sum of the coarsest level's invDegree = its assembled unknowns
  std::vector<int> coarseIters;
  T l0, l1;
  bool poisson;

  explicit MGImpl(Elliptic &e) : el(e), s(e.stream)
  {
    const Options &o = el.opt;
    plan = plan_levels(o, el.fine.N);
    l0 = (T)o.lambda0;
    l1 = (T)o.lambda1;
    poisson = o.poisson;
    const int nlev = (int)plan.orders.size();
    lv.resize(nlev);
    size_t nmax = 0;
    for (int l = 0; l < nlev; ++l) {
      auto &v = lv[l];
      if (l == 0) {
        v.L = &el.fine;
      } else {
        v.own.reset(new FieldLevel());
        v.own->build(plan.orders[l], el.fine.E, el.fine.VXh.data(), el.fine.EToVh.data(), el.fine.EToBh.data(),
                     nullptr, s);
        v.L = v.own.get();
        const FieldLevel &Lf = *lv[l - 1].L;
        v.Nf = Lf.N;
        std::vector<double> I; // I[f*Ncq + c] = l_c(z_f)
        lagrange_interp(v.L->z, Lf.z, I);
        const int Ncq = v.L->Nq, Nfq = Lf.Nq;
        std::vector<T> R((size_t)Ncq * Nfq);
        for (int c = 0; c < Ncq; ++c)
          for (int f = 0; f < Nfq; ++f) R[c * Nfq + f] = (T)I[f * Ncq + c];
        v.R.upload(R);
        std::vector<T> idf(Lf.gm.invDegree.begin(), Lf.gm.invDegree.end());
        v.invDegreeFine.upload(idf);
      }
      FieldLevel &L = *v.L;
      nmax = std::max(nmax, (size_t)L.Nlocal);
      v.ggeo.alloc(L.d_ggeo64.n);
      launch_copy_cast<double, T>((long long)L.d_ggeo64.n, L.d_ggeo64.p, v.ggeo.p, s);
      std::vector<T> D(L.Dh.begin(), L.Dh.end()), inv(L.gm.invDegree.begin(), L.gm.invDegree.end());
      v.D.upload(D);
      v.invDegree.upload(inv);
      v.x.alloc(L.Nlocal);
      v.rhs.alloc(L.Nlocal);
      v.res.alloc(L.Nlocal);
      const bool coarsest = (l == nlev - 1);
      v.smoothed = !coarsest || o.coarse == "smooth";
      if (plan.base == 0 || coarsest) {
        v.invDiag.alloc(L.Nlocal);
        launch_build_diag<T>(L.N, L.E, v.ggeo.p, v.D.p, l0, l1, poisson, v.invDiag.p, s);
        launch_gs<T>(L.ngroups, L.d_gsOff.p, L.d_gsIds.p, v.invDiag.p, s);
        launch_recip<T>(L.Nlocal, v.invDiag.p, s);
      }
    }
    sRes.alloc(nmax);
    sRes2.alloc(nmax);
    sUpd.alloc(nmax);
    sTmp.alloc(nmax);
    const FieldLevel &C = *lv.back().L;
    cp.alloc(C.Nlocal);
    cz.alloc(C.Nlocal);
    cAp.alloc(C.Nlocal);
    cr.alloc(C.Nlocal);
    csc.alloc(1);
    NRSG_CUDA(cudaMemsetAsync(csc.p, 0, sizeof(PcgScalars), s));
    if (el.allNeumann) {
      cOnes.alloc(C.Nlocal);
      launch_fill<T>(C.Nlocal, T(1), cOnes.p, s);
      cSum.alloc(1);
      cUnknowns = 0;
      for (double w : C.gm.invDegree) cUnknowns += w;
    }
    amgCoarse = o.coarse == "amg";
    if (amgCoarse && C.N != 1)
      throw Error(NRSG_ERR_BAD_CONFIG, "coarseSolver = amg needs an order-1 coarsest level");
    if (amgCoarse && el.allNeumann)
      throw Error(NRSG_ERR_BAD_CONFIG, "coarseSolver = amg does not take all-Neumann problems (coarseSolver = jpcg)");
    persistentCoarse = (C.N == 1) && o.coarse != "smooth" && !amgCoarse && o.coarsePersistent;
    if ((o.galerkin || o.semfem) && !persistentCoarse && !amgCoarse)
      throw Error(NRSG_ERR_BAD_CONFIG, "coarseGridDiscretization FEM+Galerkin / SEMFEM needs an order-1 coarsest level "
                                       "solved on its assembled operator (coarseSolver = jpcg or amg)");
    if (amgCoarse) build_amg(C);
    if (persistentCoarse) {
      cPartials.alloc(6 * kCoarseGridMax);
      cState.alloc(coarse_state_bytes());
      NRSG_CUDA(cudaMemsetAsync(cState.p, 0, coarse_state_bytes(), s));
      build_coarse_matrix(C);
    }
    if (!std::is_same<T, double>::value) {
      rP.alloc(el.fine.Nlocal);
      zP.alloc(el.fine.Nlocal);
    }
    // smoothers: FDM operators, lambda_max, Chebyshev degrees
    for (int l = 0; l < nlev; ++l) {
      auto &v = lv[l];
      if (!v.smoothed) continue;
      if (plan.base != 0) build_fdm(v);
      autotune_ax(v);
      v.rho = max_eig(v, o.seed + (unsigned long long)l);
      v.lambda1 = o.maxEigFactor * v.rho;
      v.lambda0 = o.minEigFactor * v.rho;
      const int ord = plan.orders[l];
      const bool coarsest = (l == nlev - 1);
      v.up = v.down = coarsest ? 3 : o.chebyDegree;
      auto itd = plan.down.find(ord), itu = plan.up.find(ord);
      if (!o.schedule.empty()) {
        if (itd != plan.down.end() && itd->second > -1) v.down = itd->second;
        if (itu != plan.up.end() && itu->second > -1) v.up = itu->second;
      }
      if (plan.kind == 2) {
        v.upBetas = opt4_betas(v.up);
        v.downBetas = opt4_betas(v.down);
      } else {
        v.upBetas.assign(std::max(v.up, 1), 1.0);
        v.downBetas.assign(std::max(v.down, 1), 1.0);
      }
    }
    NRSG_CUDA(cudaStreamSynchronize(s));
  }

  // --------------------------------------------------------------- setup
  // Assembled operator of the coarsest level in ELL form (rows padded to the
  // widest row with zero entries on the row itself), its inverse diagonal, a
  // representative E-vector node per row and the row of each E-vector node.
  void build_coarse_matrix(const FieldLevel &C)
  {
    CsrMatrix A;
    assemble_coarse(C, A);
    std::vector<int> rep(A.nrow);
    for (long long r = 0; r < A.nrow; ++r) rep[r] = C.gm.ids[C.gm.off[r]];
    coarse_matrix_setup<T>(A.nrow, A.rowPtr.data(), A.col.data(), A.val.data(), C.Nlocal, A.rowOfNode.data(),
                           rep.data(), cA);
    const long long nv = std::max(A.nrow, 1LL);
    cx.alloc(nv);
    cz2.alloc(nv);
    cz3.alloc(nv);
  }

  // the algebraic multigrid hierarchy of the assembled coarsest operator and its row maps
  void build_amg(const FieldLevel &C)
  {
    CsrMatrix A;
    assemble_coarse(C, A);
    AmgHierarchy H;
    amg_build(A.nrow, A.rowPtr.data(), A.col.data(), A.val.data(), H);
    if (!H.invertible) throw Error(NRSG_ERR_INVALID, "algebraic multigrid: singular coarsest operator");
    amg_upload<T>(H, amg);
    std::vector<int> rep(A.nrow), rowOf(A.rowOfNode.size());
    for (long long r = 0; r < A.nrow; ++r) rep[r] = C.gm.ids[C.gm.off[r]];
    for (size_t i = 0; i < rowOf.size(); ++i) rowOf[i] = (int)A.rowOfNode[i];
    amgRep.upload(rep);
    amgRowOf.upload(rowOf);
    amgRows = A.nrow;
    amgInfo.clear();
    for (const auto &L : H.levels) {
      amgInfo.push_back(L.A.n);
      amgInfo.push_back((double)L.A.ci.size());
    }
    amgInfo.push_back(H.coarse.n);
    amgInfo.push_back((double)H.coarse.ci.size());
    if (amgRows > 0) {
      amgB.alloc(amgRows);
      amgX.alloc(amgRows);
      amgR.alloc(amgRows);
    }
  }
  DevBuf<T> amgB;

  // one V-cycle on the assembled unknowns: b (E-vector, assembled) -> rows -> V-cycle -> x (E-vector)
  void amg_coarse(const T *b, T *x)
  {
    launch_rows_gather<T>(amgRows, amgRep.p, b, amgB.p, s);
    const T *xr = amg_vcycle<T>(amg, amgB.p, s);
    if (el.opt.amgIterations > 1) {
      NRSG_CUDA(cudaMemcpyAsync(amgX.p, xr, sizeof(T) * amgRows, cudaMemcpyDeviceToDevice, s));
      amg_more_cycles<T>(amg, amgB.p, amgX.p, amgR.p, el.opt.amgIterations, s);
      xr = amgX.p;
    }
    launch_rows_scatter<T>((long long)amgRowOf.n, amgRowOf.p, xr, x, s);
  }
  DevBuf<T> amgX, amgR;

  void assemble_coarse(const FieldLevel &C, CsrMatrix &A)
  {
    if (el.opt.galerkin) {
      // B^T A_fine B from the finest level's FP32 operator (ellipticMultiGridSetup.cpp:260-261)
      const std::vector<double> gf = el.fine.d_ggeo64.download();
      std::vector<double> Ae;
      galerkin_element_matrices(el.fine.N, el.fine.E, el.fine.Dh, el.fine.z, gf.data(), el.opt.lambda0,
                                el.opt.lambda1, el.opt.poisson, Ae);
      assemble_rows(8, C.E, Ae, C.gm, A);
    } else if (el.opt.semfem) {
      // SEMFEMSolver_t on the coarsest level (ellipticMultiGridSetup.cpp:219-250)
      std::vector<double> X, Y, Z;
      trilinear_nodes(C.N, C.E, C.VXh.data(), C.z, X, Y, Z);
      semfem_assemble(C.N, C.E, X.data(), Y.data(), Z.data(), C.gm, C.maskIds, el.opt.lambda0, A);
    } else {
      const std::vector<double> gg = C.d_ggeo64.download();
      assemble_level(C.N, C.E, C.Dh, gg.data(), el.opt.lambda0, el.opt.lambda1, el.opt.poisson, C.gm, A);
    }
  }

  void build_fdm(MGLevelDev<T> &v)
  {
    const FieldLevel &L = *v.L;
    const int nl = L.N + 3, npe = nl * nl * nl;
    const long long E = L.E;
    const FdmLengths len = fdm_lengths(el.fine, el.fine.um);
    const bool recip = !std::is_same<T, double>::value;
    std::vector<T> Sx((size_t)E * nl * nl), Sy((size_t)E * nl * nl), Sz((size_t)E * nl * nl);
    std::vector<T> iL(recip ? 0 : (size_t)E * npe), lm(recip ? (size_t)E * 3 * nl : 0);
#pragma omp parallel for
    for (long long e = 0; e < E; ++e) {
      const int *bc = &L.EToBh[e * 6];
      // (left, right) faces per direction in nekRS face order: r: 4,2  s: 1,3  t: 0,5
      const int lb[3] = {bc[4], bc[1], bc[0]}, rb[3] = {bc[2], bc[3], bc[5]};
      std::vector<double> S[3], lam[3];
      for (int d = 0; d < 3; ++d)
        fdm_1d_operator(L, lb[d], rb[d], len.left[3 * e + d], len.mid[3 * e + d], len.right[3 * e + d], S[d], lam[d]);
      for (int q = 0; q < nl * nl; ++q) {
        Sx[e * nl * nl + q] = (T)S[0][q];
        Sy[e * nl * nl + q] = (T)S[1][q];
        Sz[e * nl * nl + q] = (T)S[2][q];
      }
      if (recip) {
        for (int d = 0; d < 3; ++d)
          for (int i = 0; i < nl; ++i) lm[(e * 3 + d) * nl + i] = (T)lam[d][i];
      } else {
        for (int k = 0; k < nl; ++k)
          for (int j = 0; j < nl; ++j)
            for (int i = 0; i < nl; ++i) {
              const double dsum = lam[0][i] + lam[1][j] + lam[2][k];
              iL[e * npe + i + nl * (j + nl * k)] = (T)(dsum > 1e-5 ? 1.0 / dsum : 0.0);
            }
      }
    }
    v.Sx.upload(Sx);
    v.Sy.upload(Sy);
    v.Sz.upload(Sz);
    if (recip) v.lam.upload(lm);
    else v.invL.upload(iL);
    std::vector<int> src, partner;
    std::vector<double> w;
    fdm_halo_maps(L, src, partner, w);
    v.haloSrc.upload(src);
    v.haloPartner.upload(partner);
    // ASM weights its combined overlap result by the overlap weights
    // (generate_weights); RAS restricts each element's own nodes with the
    // level's inverse degree (fusedFDM with p_restrict gets elliptic->o_invDegree,
    // ellipticMultiGridSchwarz.cpp:1069-1077, fusedFDM.c:209-215)
    std::vector<T> wt;
    if (plan.base == 2)
      wt.assign(L.gm.invDegree.begin(), L.gm.invDegree.end());
    else
      wt.assign(w.begin(), w.end());
    v.wts.upload(wt);
    if (plan.base == 1) v.haloOut.alloc(src.size());
  }

  double read(const double *d)
  {
    double h = 0;
    NRSG_CUDA(cudaMemcpyAsync(&h, d, sizeof(double), cudaMemcpyDeviceToHost, s));
    NRSG_CUDA(cudaStreamSynchronize(s));
    return h;
  }

  // rho(S A) by 10 Arnoldi steps with a seeded start vector (maxEigSmoothAx)
  double max_eig(MGLevelDev<T> &v, unsigned long long seed)
  {
    FieldLevel &L = *v.L;
    const long long n = L.Nlocal;
    const int k = (int)std::min<long long>(10, n);
    DevBuf<double> V((size_t)(k + 1) * n), vx(n);
    DevBuf<T> tq(n), ta(n);
    DevBuf<int> uoff, uids;
    uoff.upload(L.um.devOff);
    uids.upload(L.um.devIds);
    launch_random_fill(n, seed, vx.p, s);
    launch_gs<double>((long long)L.um.devOff.size() - 1, uoff.p, uids.p, vx.p, s);
    launch_mask<double>((long long)L.maskIds.size(), L.d_mask.p, vx.p, s);
    double *out = &el.d_scal.p->pad;
    const double *w = L.d_invDegree64.p;
    launch_wdot<double>(n, w, vx.p, nullptr, out, el.red, 4, s);
    const double nv = std::sqrt(read(out));
    auto Vj = [&](int j) { return V.p + (size_t)j * n; };
    launch_scale_copy<double>(n, 1.0 / nv, vx.p, Vj(0), s);
    std::vector<double> H((size_t)k * k, 0.0);
    int keff = k;
    for (int j = 0; j < k; ++j) {
      launch_copy_cast<double, T>(n, Vj(j), tq.p, s);
      level_op(v, tq.p, ta.p);
      apply_S(v, ta.p, tq.p);
      launch_copy_cast<T, double>(n, tq.p, Vj(j + 1), s);
      for (int i = 0; i <= j; ++i) {
        launch_wdot<double>(n, w, Vj(i), Vj(j + 1), out, el.red, 4, s);
        const double hij = read(out);
        launch_axpby<double>(n, -hij, Vj(i), 1.0, Vj(j + 1), s);
        H[i + (size_t)j * k] = hij;
      }
      if (j + 1 < k) {
        launch_wdot<double>(n, w, Vj(j + 1), nullptr, out, el.red, 4, s);
        const double nj = std::sqrt(read(out));
        // invariant subspace (e.g. a level with a single free node): the
        // leading (j+1) x (j+1) block already holds the exact eigenvalues
        if (!(nj > 1e-13 * std::fabs(H[j + (size_t)j * k]))) {
          keff = j + 1;
          break;
        }
        launch_scale_copy<double>(n, 1.0 / nj, Vj(j + 1), Vj(j + 1), s);
        H[j + 1 + (size_t)j * k] = nj;
      }
    }
    NRSG_CUDA(cudaStreamSynchronize(s));
    std::vector<double> Hk((size_t)keff * keff);
    for (int c = 0; c < keff; ++c)
      for (int r = 0; r < keff; ++r) Hk[r + (size_t)keff * c] = H[r + (size_t)k * c];
    return hessenberg_spectral_radius(keff, Hk);
  }

  // --------------------------------------------------------------- operators
  void level_op(MGLevelDev<T> &v, const T *q, T *Aq)
  {
    FieldLevel &L = *v.L;
    bool done = false;
    if constexpr (std::is_same<T, float>::value) {
      if (el.opt.axConst) done = launch_ax_const(L.N, L.E, v.ggeo.p, v.D.p, l0, l1, poisson, q, Aq, s);
      if (!done) done = el.opt.axPipeline && launch_ax_pipe(L.N, L.E, v.ggeo.p, v.D.p, l0, l1, poisson, q, Aq, s);
    }
    if constexpr (std::is_same<T, float>::value) {
      if (!done) done = launch_ax_f32_variant(v.axVariant, L.N, L.E, v.ggeo.p, v.D.p, l0, l1, poisson, q, Aq, s);
    }
    if (!done) launch_ax_stored<T>(L.N, L.E, v.ggeo.p, v.D.p, l0, l1, poisson, q, Aq, s);
    launch_gs_mask<T>(L.gsPlan, Aq, true, s);
  }

  // Autotuner (FP32 levels): the interchangeable axhelm variants are run on this level's geometric
  // factors and a reproducible test vector; a variant whose output differs from the default kernel's
  // in any bit is rejected (the reference's benchmarker accepts 400 eps: kernelBenchmarker.cpp:68-119,
  // benchmarkAx.cpp:268-307); the others are timed with CUDA events (2 warm-up, 5 timed launches) and
  // the fastest is kept.  Results are cached per (device, order, Poisson, elements).
  void autotune_ax(MGLevelDev<T> &v)
  {
    if constexpr (std::is_same<T, float>::value) {
      FieldLevel &L = *v.L;
      const std::string &want = el.opt.axKernel;
      if (el.opt.axConst) v.axVariant = kAxConst; // the older switches force a variant
      else if (el.opt.axPipeline) v.axVariant = kAxPipe;
      else if (want == "vec") v.axVariant = kAxVec;
      else if (want == "plain") v.axVariant = kAxPlain;
      else if (want == "epb2") v.axVariant = kAxEpb2;
      else if (want == "pipe") v.axVariant = kAxPipe;
      else if (want == "const") v.axVariant = kAxConst;
      else if (want == "constpf") v.axVariant = kAxConstPf;
      if (want != "auto" || el.opt.axConst || el.opt.axPipeline) return;
      int dev = 0;
      NRSG_CUDA(cudaGetDevice(&dev));
      const auto key = std::make_tuple(dev, L.N, poisson ? 1 : 0, L.E);
      auto &cache = ax_tune_cache();
      {
        std::lock_guard<std::mutex> lock(cache.m);
        auto it = cache.best.find(key);
        if (it != cache.best.end()) {
          v.axVariant = it->second.first;
          v.axMs = it->second.second;
          return;
        }
      }
      const long long n = L.Nlocal;
      float *q = v.x.p, *ref = v.res.p, *out = v.rhs.p;
      launch_hash_fill(n, 0x5eedull + (unsigned long long)L.N, q, s);
      launch_ax_f32_variant(kAxVec, L.N, L.E, v.ggeo.p, v.D.p, l0, l1, poisson, q, ref, s);
      DevBuf<unsigned> bad(1);
      cudaEvent_t e0, e1;
      NRSG_CUDA(cudaEventCreate(&e0));
      NRSG_CUDA(cudaEventCreate(&e1));
      std::vector<double> ms(kAxVariants, -1.0);
      int best = kAxVec;
      for (int c = 0; c < kAxVariants; ++c) {
        NRSG_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(unsigned), s));
        if (!launch_ax_f32_variant(c, L.N, L.E, v.ggeo.p, v.D.p, l0, l1, poisson, q, out, s)) continue;
        launch_count_mismatch(n, ref, out, bad.p, s);
        unsigned h = 0;
        NRSG_CUDA(cudaMemcpyAsync(&h, bad.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
        NRSG_CUDA(cudaStreamSynchronize(s));
        if (h != 0) continue; // not bit-identical: rejected
        for (int w = 0; w < 2; ++w) launch_ax_f32_variant(c, L.N, L.E, v.ggeo.p, v.D.p, l0, l1, poisson, q, out, s);
        NRSG_CUDA(cudaEventRecord(e0, s));
        for (int w = 0; w < 5; ++w) launch_ax_f32_variant(c, L.N, L.E, v.ggeo.p, v.D.p, l0, l1, poisson, q, out, s);
        NRSG_CUDA(cudaEventRecord(e1, s));
        NRSG_CUDA(cudaEventSynchronize(e1));
        float t = 0;
        NRSG_CUDA(cudaEventElapsedTime(&t, e0, e1));
        ms[c] = t / 5.0;
        if (ms[c] < ms[best] || ms[best] < 0) best = c;
      }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      if (ax_pipe_error(s)) best = kAxVec; // a bulk copy of the pipelined variant did not complete in time
      v.axVariant = best;
      v.axMs = ms;
      std::lock_guard<std::mutex> lock(cache.m);
      cache.best[key] = {best, ms};
    }
  }

  // the fused FDM of one level: FP16 tensor-core transforms (option fdmPrecision = fp16) where they
  // apply (FP32 multigrid, order 7, RAS), TF32 tensor-core transforms (fdmPrecision = tf32; FP32
  // multigrid, orders 3, 5, 7; tcgen05.mma for order-7 RAS unless fdmMma = sync, mma.sync otherwise),
  // the FP32 kernels otherwise
  void run_fdm(MGLevelDev<T> &v, const T *u, T *Su)
  {
    FieldLevel &L = *v.L;
    const bool ras = plan.base == 2;
    if constexpr (std::is_same<T, float>::value) {
      if (el.opt.fdmFp16 && ras && L.N == 7 &&
          launch_fdm8h(L.E, u, v.haloSrc.p, v.Sx.p, v.Sy.p, v.Sz.p, v.lam.p, v.wts.p, Su, s))
        return;
      if (el.opt.fdmTf32 && el.opt.fdmTcgen05 && ras && L.N == 7 &&
          launch_fdm_tc(L.E, u, v.haloSrc.p, v.Sx.p, v.Sy.p, v.Sz.p, v.lam.p, v.wts.p, Su, s))
        return;
      if (el.opt.fdmTf32 && launch_fdm_tf32(L.N, L.E, ras, u, v.haloSrc.p, v.Sx.p, v.Sy.p, v.Sz.p, v.lam.p,
                                            v.wts.p, Su, v.haloOut.p, s))
        return;
    }
    launch_fdm<T>(L.N, L.E, ras, u, v.haloSrc.p, v.Sx.p, v.Sy.p, v.Sz.p, v.invL.p, v.lam.p, v.wts.p, Su, v.haloOut.p,
                  s, el.opt.fdmGeneric);
  }

  // Schwarz: FDM (+ ASM combine) -> gs -> mask; u and Su must not alias
  void schwarz_apply(MGLevelDev<T> &v, const T *u, T *Su)
  {
    FieldLevel &L = *v.L;
    const bool ras = plan.base == 2;
    run_fdm(v, u, Su);
    if (!ras) launch_asm_combine<T>(L.N, L.E, v.haloPartner.p, v.haloOut.p, v.wts.p, Su, s);
    launch_gs_mask<T>(L.gsPlan, Su, true, s);
  }

  void apply_S(MGLevelDev<T> &v, const T *r, T *Sr)
  {
    const long long n = v.L->Nlocal;
    if (plan.base == 0) {
      launch_axmyz<T>(n, v.invDiag.p, r, Sr, s);
    } else if (r == Sr) {
      NRSG_CUDA(cudaMemcpyAsync(sTmp.p, r, sizeof(T) * n, cudaMemcpyDeviceToDevice, s));
      schwarz_apply(v, sTmp.p, Sr);
    } else {
      schwarz_apply(v, r, Sr);
    }
  }

  void smooth_cheby1(MGLevelDev<T> &v, const T *r, T *x, bool xIsZero)
  {
    const int degree = xIsZero ? v.down : v.up;
    if (degree == 0) return;
    const long long n = v.L->Nlocal;
    const T theta = (T)(0.5 * (v.lambda1 + v.lambda0));
    const T delta = (T)(0.5 * (v.lambda1 - v.lambda0));
    const T invTheta = (T)1.0 / theta;
    const T sigma = theta / delta;
    T rho_n = (T)1.0 / sigma;
    T *res = sRes.p, *Ad = sRes2.p, *d = sUpd.p;
    if (xIsZero) launch_fill<T>(n, T(0), x, s);
    if (!xIsZero) {
      level_op(v, x, res);
      launch_axpby<T>(n, T(1), r, T(-1), res, s);
    } else {
      NRSG_CUDA(cudaMemcpyAsync(res, r, sizeof(T) * n, cudaMemcpyDeviceToDevice, s));
    }
    apply_S(v, res, res);
    launch_scale_copy<T>(n, invTheta, res, d, s);
    for (int k = 1; k < degree; ++k) {
      level_op(v, d, Ad);
      apply_S(v, Ad, Ad);
      const T rhoSave = rho_n;
      rho_n = (T)1.0 / ((T)2.0 * sigma - rho_n);
      const T rCoeff = (T)2.0 * rho_n / delta;
      const T dCoeff = rho_n * rhoSave;
      launch_cheby1_update<T>(n, dCoeff, rCoeff, Ad, d, res, x, s);
    }
    launch_axpby<T>(n, T(1), d, T(1), x, s);
    launch_mask<T>((long long)v.L->maskIds.size(), v.L->d_mask.p, x, s);
  }

  // 4th-kind / optimal 4th-kind Chebyshev over S (ellipticMultiGridLevel.cpp
  // smoothChebyshevFourthKind).  With x = 0 on entry the first S is applied to
  // r itself and the first update writes x = beta d (no zero fill, no copy of
  // r).  No mask at the end: d is a combination of S outputs (masked) and x of
  // masked vectors, so their masked entries are already 0.
  void smooth_cheby4(MGLevelDev<T> &v, const T *r, T *x, bool xIsZero)
  {
    const int degree = xIsZero ? v.down : v.up;
    if (degree == 0) {
      if (xIsZero) launch_fill<T>(v.L->Nlocal, T(0), x, s);
      return;
    }
    const auto &betas = xIsZero ? v.downBetas : v.upBetas;
    const long long n = v.L->Nlocal;
    T *res = sRes.p, *Ad = sRes2.p, *d = sUpd.p;
    const double rho = v.lambda1;
    const T *rcur = r;
    const bool xzero = xIsZero;
    if (!xIsZero) {
      level_op(v, x, res);
      launch_axpby<T>(n, T(1), r, T(-1), res, s);
      rcur = res;
    }
    // x += beta_k d_k is applied where d_k is formed (the same updates, in the same order, as applying it in
    // the next step's residual update and once more after the loop)
    apply_S(v, rcur, Ad);
    launch_cheby4_dx<T>(n, (T)(4.0 / (3.0 * rho)), Ad, T(0), d, (T)betas[0], x, true, xzero, s);
    for (int k = 1; k < degree; ++k) {
      level_op(v, d, Ad);
      launch_cheby4_res<T>(n, Ad, rcur, res, s);
      rcur = res;
      apply_S(v, res, Ad);
      const T dCoeff = (T)((2.0 * k - 1.0) / (2.0 * k + 3.0));
      const T rCoeff = (T)((8.0 * k + 4.0) / ((2.0 * k + 3.0) * rho));
      launch_cheby4_dx<T>(n, rCoeff, Ad, dCoeff, d, (T)betas[k], x, false, false, s);
    }
  }

  void smooth(MGLevelDev<T> &v, const T *r, T *x, bool xIsZero)
  {
    if (plan.kind == 0)
      smooth_cheby1(v, r, x, xIsZero);
    else
      smooth_cheby4(v, r, x, xIsZero);
  }

  // all-Neumann problems: the assembled coarse operator annihilates constants and
  // the Krylov coarse solve needs a consistent right-hand side, so the rhs's
  // mean over the assembled unknowns (invDegree-weighted E-vector mean) is
  // removed first (the reference's BoomerAMG instead smooths on its coarsest
  // level when told of the null space, hypreWrapper.cpp:143-147)
  void project_coarse_rhs(MGLevelDev<T> &v, T *b)
  {
    const long long n = v.L->Nlocal;
    launch_wdot<T>(n, v.invDegree.p, b, cOnes.p, cSum.p, el.red, 5, s);
    launch_sub_mean<T>(n, cSum.p, cUnknowns, b, s);
  }

  int coarse_pcg(MGLevelDev<T> &v, const T *b, T *x)
  {
    FieldLevel &L = *v.L;
    if (persistentCoarse) {
      if (el.capturing && cA.grid > 1) {
        el.capture_split(); // a cooperative coarse solve is launched between the iteration's graph segments
        return 0;
      }
      if (el.allNeumann) project_coarse_rhs(v, const_cast<T *>(b));
      coarse_pcg_persistent<T>(cA, b, x, cx.p, cz2.p, cz3.p, cPartials.p, cState.p, kCoarseGridMax,
                               el.opt.coarseTol, el.opt.coarseMaxIter, s, el.opt.coarseSpinLimit,
                               (unsigned)el.opt.coarseBarrierExtra);
      return 0;
    }
    const long long n = L.Nlocal;
    const Options &o = el.opt;
    const T *w = v.invDegree.p;
    PcgScalars *sc = csc.p;
    if (el.allNeumann) project_coarse_rhs(v, const_cast<T *>(b));
    launch_fill<T>(n, T(0), x, s);
    NRSG_CUDA(cudaMemcpyAsync(cr.p, b, sizeof(T) * n, cudaMemcpyDeviceToDevice, s));
    launch_fill<T>(n, T(0), cp.p, s);
    launch_wdot<T>(n, w, cr.p, nullptr, &sc->rdotr, el.red, 5, s);
    const double r0 = std::sqrt(read(&sc->rdotr));
    if (r0 == 0) return 0;
    const double tol = o.coarseTol * r0;
    double rn = r0;
    int it = 0;
    while (rn > tol && it < o.coarseMaxIter) {
      ++it;
      launch_pcg_rdotz<T>(n, w, v.invDiag.p, cr.p, cz.p, sc, el.red, 5, s);
      launch_pcg_p<T>(n, cz.p, cp.p, sc, it == 1, s);
      level_op(v, cp.p, cAp.p);
      launch_wdot<T>(n, w, cp.p, cAp.p, &sc->pAp, el.red, 6, s);
      launch_pcg_xr<T>(n, w, cp.p, cAp.p, x, cr.p, sc, el.red, 7, s);
      rn = std::sqrt(read(&sc->rdotr));
    }
    coarseIters.push_back(it);
    return it;
  }

  void vcycle(int k)
  {
    auto &v = lv[k];
    const int base = (int)lv.size() - 1;
    if (k == base) {
      if (el.opt.coarse == "smooth")
        smooth(v, v.rhs.p, v.x.p, true);
      else if (amgCoarse)
        amg_coarse(v.rhs.p, v.x.p);
      else
        coarse_pcg(v, v.rhs.p, v.x.p);
      return;
    }
    auto &c = lv[k + 1];
    const long long n = v.L->Nlocal;
    smooth(v, v.rhs.p, v.x.p, true);
    level_op(v, v.x.p, v.res.p);
    launch_axpby<T>(n, T(1), v.rhs.p, T(-1), v.res.p, s);
    // coarsen: res *= invDegree(fine), restrict, gs, mask
    launch_axmy<T>(n, c.invDegreeFine.p, v.res.p, s);
    launch_coarsen<T>(v.L->N, c.L->N, c.L->E, c.R.p, v.res.p, c.rhs.p, s);
    launch_gs_mask<T>(c.L->gsPlan, c.rhs.p, true, s);
    vcycle(k + 1);
    launch_prolong<T>(v.L->N, c.L->N, c.L->E, c.R.p, c.x.p, v.x.p, s);
    smooth(v, v.rhs.p, v.x.p, false);
  }

  // --------------------------------------------------------------- interface
  void apply(const double *r, double *z) override
  {
    auto &v0 = lv[0];
    const long long n = el.fine.Nlocal;
    if (std::is_same<T, double>::value) {
      NRSG_CUDA(cudaMemcpyAsync(v0.rhs.p, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
      vcycle(0);
      NRSG_CUDA(cudaMemcpyAsync(z, v0.x.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    } else {
      launch_copy_cast<double, T>(n, r, v0.rhs.p, s);
      vcycle(0);
      launch_copy_cast<T, double>(n, v0.x.p, z, s);
    }
  }

  std::vector<double> info(const std::string &what) override
  {
    std::vector<double> out;
    if (what == "mg.levels")
      for (auto &v : lv) out.push_back(v.L->N);
    else if (what == "mg.rho")
      for (auto &v : lv) {
        if (v.smoothed) out.push_back(v.rho);
      }
    else if (what == "mg.coarseIters") {
      if (persistentCoarse) {
        std::vector<unsigned char> h(coarse_state_bytes());
        NRSG_CUDA(cudaStreamSynchronize(s));
        NRSG_CUDA(cudaMemcpy(h.data(), cState.p, h.size(), cudaMemcpyDeviceToHost));
        int it = 0;
        coarse_state_read(h.data(), &it, nullptr, nullptr);
        out.push_back(it);
      } else {
        out.assign(coarseIters.begin(), coarseIters.end());
      }
    } else if (what == "mg.coarseError") {
      double e = 0;
      if (persistentCoarse) {
        std::vector<unsigned char> h(coarse_state_bytes());
        NRSG_CUDA(cudaStreamSynchronize(s));
        NRSG_CUDA(cudaMemcpy(h.data(), cState.p, h.size(), cudaMemcpyDeviceToHost));
        e = coarse_state_read(h.data(), nullptr, nullptr, nullptr);
      }
      out.push_back(e);
    }
    else if (what == "mg.degrees")
      for (auto &v : lv) {
        if (v.smoothed) { out.push_back(v.down); out.push_back(v.up); }
      }
    else if (what == "mg.bytes")
      out.push_back((double)sizeof(T)); // multigrid precision
    else if (what == "mg.axKernel") {
      // per smoothed level: the axhelm variant in use (0 vec, 1 plain, 2 epb2, 3 pipe, 4 const)
      for (auto &v : lv)
        if (v.smoothed) out.push_back((double)v.axVariant);
    } else if (what == "mg.axTimes") {
      // per smoothed level and variant: autotuner ms per launch (-1: not applicable or rejected)
      for (auto &v : lv)
        if (v.smoothed)
          for (int c = 0; c < kAxVariants; ++c) out.push_back(c < (int)v.axMs.size() ? v.axMs[c] : -1.0);
    } else if (what == "mg.amgLevels") {
      out = amgInfo;
    } else if (what == "mg.coarseMatrix") {
      // rows, ELL width, stored nonzeros, row blocks (CTAs), rows per block, matrix in shared memory,
      // thread-block cluster size (0: one CTA or a cooperative launch)
      if (persistentCoarse)
        out = {(double)cA.nrow, (double)cA.width, (double)cA.nnz, (double)cA.grid, (double)cA.chunk,
               cA.matInSmem ? 1.0 : 0.0, (double)cA.cluster};
    } else
      throw Error(NRSG_ERR_INVALID, "unknown array '" + what + "'");
    return out;
  }

  long long level_size(int level) override { return lv.at(level).L->Nlocal; }

  void clear_error() override
  {
    if (persistentCoarse) coarse_state_clear(cState.p, s);
  }
  int error() override
  {
    if (std::is_same<T, float>::value && el.opt.axPipeline && ax_pipe_error(s)) return 2;
    if (std::is_same<T, float>::value && el.opt.fdmTf32 && el.opt.fdmTcgen05 && fdm_tc_error(s)) return 3;
    if (!persistentCoarse) return 0;
    std::vector<unsigned char> h(coarse_state_bytes());
    NRSG_CUDA(cudaMemcpyAsync(h.data(), cState.p, h.size(), cudaMemcpyDeviceToHost, s));
    NRSG_CUDA(cudaStreamSynchronize(s));
    return coarse_state_read(h.data(), nullptr, nullptr, nullptr);
  }

  // one fused FDM launch of level `level` on buffers of the multigrid
  // precision (RAS: weighted own nodes; ASM: own nodes and the halo results)
  void fdm(int level, const void *u, void *Su) override
  {
    auto &v = lv.at(level);
    if (plan.base == 0 || !v.smoothed) throw Error(NRSG_ERR_INVALID, "level has no Schwarz smoother");
    run_fdm(v, (const T *)u, (T *)Su);
  }

  void coarse_launch() override
  {
    auto &c = lv.back();
    coarse_pcg(c, c.rhs.p, c.x.p);
  }
  // host-driven coarse iterations read the device between launches: not capturable
  bool graph_capturable() override { return persistentCoarse || amgCoarse || el.opt.coarse == "smooth"; }

  void schwarz(int level, const double *u, double *Su) override
  {
    auto &v = lv.at(level);
    const long long n = v.L->Nlocal;
    launch_copy_cast<double, T>(n, u, sRes.p, s);
    apply_S(v, sRes.p, sRes2.p);
    launch_copy_cast<T, double>(n, sRes2.p, Su, s);
    NRSG_CUDA(cudaStreamSynchronize(s));
  }
};

void Elliptic::mg_setup()
{
  if (opt.mgPrecision == "fp32" || opt.mgPrecision == "mixed")
    mg.reset(new MGImpl<float>(*this));
  else if (opt.mgPrecision == "fp64")
    mg.reset(new MGImpl<double>(*this));
  else
    throw Error(NRSG_ERR_BAD_CONFIG, "mgPrecision must be fp64, fp32 or mixed");
}
void Elliptic::mg_apply(const double *r, double *zz)
{
  if (!mg) throw Error(NRSG_ERR_BAD_CONFIG, "multigrid not set up");
  mg->apply(r, zz);
}
void Elliptic::mg_release() { mg.reset(); }
int Elliptic::mg_error() { return mg ? mg->error() : 0; }
void Elliptic::mg_clear_error()
{
  if (mg) mg->clear_error();
}
std::vector<double> Elliptic::mg_get(const std::string &name)
{
  if (!mg) throw Error(NRSG_ERR_INVALID, "no multigrid preconditioner");
  return mg->info(name);
}
long long Elliptic::mg_level_size(int level)
{
  if (!mg) throw Error(NRSG_ERR_INVALID, "no multigrid preconditioner");
  return mg->level_size(level);
}
void Elliptic::mg_coarse_launch()
{
  if (mg) mg->coarse_launch();
}
bool Elliptic::mg_graph_capturable() { return mg && mg->graph_capturable(); }

void Elliptic::mg_fdm(int level, const void *u, void *Su)
{
  if (!mg) throw Error(NRSG_ERR_INVALID, "no multigrid preconditioner");
  mg->fdm(level, u, Su);
}
void Elliptic::mg_schwarz(int level, const double *u, double *Su)
{
  if (!mg) throw Error(NRSG_ERR_INVALID, "no multigrid preconditioner");
  mg->schwarz(level, u, Su);
}

} // namespace nrsg
