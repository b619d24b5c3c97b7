// ORACLE — test infrastructure only (see oracle_mesh.cpp header).
//
// p-multigrid preconditioner, restated from (nekRS tree):
//   level schedule        src/solvers/elliptic/MG/determineMGLevels.cpp:5-98,
//                         src/solvers/elliptic/MG/parseMultigridSchedule.cpp:7-131
//   V-cycle               src/solvers/elliptic/MG/MGSolver.cpp:150-193
//   smoothers             src/solvers/elliptic/MG/ellipticMultiGridLevel.cpp:37-277
//   smoother setup        src/solvers/elliptic/MG/ellipticMultiGridLevelSetup.cpp:109-180
//   lambda_max (Arnoldi)  src/solvers/elliptic/MG/ellipticMultiGridLevelSetup.cpp:292-453
//   transfer operators    ellipticMultiGridLevelSetup.cpp:238-258, kernels/elliptic/
//                         ellipticPreconCoarsenHex3D.c, ellipticPreconProlongateHex3D.c
//   Schwarz / FDM         src/solvers/elliptic/MG/ellipticMultiGridSchwarz.cpp:41-1156,
//                         kernels/elliptic/preFDM.c, fusedFDM.c, postFDM.c
//   opt. 4th-kind betas   src/solvers/elliptic/MG/optimalCoeffs.cpp (Lottes, arXiv:2202.08830)
// The coarsest level is solved by Jacobi-PCG to a relative tolerance
// (default 1e-4) in the MG precision, or only smoothed (coarseSolver=smooth).
// Generalized symmetric eigenproblems (LAPACK dsygv in the reference) use a
// cyclic Jacobi eigensolver (B is diagonal for the lumped 1-D mass); the
// Hessenberg eigenvalues (dgeev) use a shifted QR iteration.

#include "oracle_internal.hpp"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <map>
#include <sstream>
#include <stdexcept>

namespace orc {

// ---------------------------------------------------------------------------
// small dense linear algebra
// ---------------------------------------------------------------------------
// symmetric Jacobi eigensolver: A (n x n, row-major, symmetric) -> eigenvalues, V columns
static void jacobi_eig(int n, std::vector<double> A, std::vector<double> &lam, std::vector<double> &V)
{
  V.assign(n * n, 0.0);
  for (int i = 0; i < n; ++i) V[i * n + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) off += A[p * n + q] * A[p * n + q];
    if (off < 1e-300) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = A[p * n + q];
        if (std::fabs(apq) < 1e-300) continue;
        const double theta = (A[q * n + q] - A[p * n + p]) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {
          const double akp = A[k * n + p], akq = A[k * n + q];
          A[k * n + p] = c * akp - s * akq;
          A[k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          const double apk = A[p * n + k], aqk = A[q * n + k];
          A[p * n + k] = c * apk - s * aqk;
          A[q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double vkp = V[k * n + p], vkq = V[k * n + q];
          V[k * n + p] = c * vkp - s * vkq;
          V[k * n + q] = s * vkp + c * vkq;
        }
      }
  }
  lam.resize(n);
  for (int i = 0; i < n; ++i) lam[i] = A[i * n + i];
}

// eigenvalues of a real upper-Hessenberg matrix (column-major H(i,j) = H[i + j*n]) by shifted QR
static std::vector<std::complex<double>> hessenberg_eigs(int n, std::vector<double> Hc)
{
  // row-major working copy
  std::vector<double> a(n * n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) a[i * n + j] = Hc[i + j * n];
  std::vector<std::complex<double>> ev;
  int hi = n - 1;
  int iter = 0;
  while (hi >= 0 && iter < 10000) {
    if (hi == 0) { ev.push_back(a[0]); --hi; continue; }
    // find small subdiagonal
    int l = hi;
    while (l > 0) {
      const double s = std::fabs(a[(l - 1) * n + l - 1]) + std::fabs(a[l * n + l]);
      if (std::fabs(a[l * n + l - 1]) <= 1e-15 * (s == 0 ? 1.0 : s)) break;
      --l;
    }
    if (l == hi) { ev.push_back(a[hi * n + hi]); --hi; iter = 0; continue; }
    if (l == hi - 1) {
      const double p = a[(hi - 1) * n + hi - 1], q = a[(hi - 1) * n + hi], r = a[hi * n + hi - 1], s = a[hi * n + hi];
      const double tr = p + s, det = p * s - q * r;
      const std::complex<double> disc = std::sqrt(std::complex<double>(tr * tr / 4 - det, 0));
      ev.push_back(tr / 2 + disc);
      ev.push_back(tr / 2 - disc);
      hi -= 2;
      iter = 0;
      continue;
    }
    // Wilkinson shift from the trailing 2x2, single-shift QR by Givens on [l..hi]
    const double p = a[(hi - 1) * n + hi - 1], q = a[(hi - 1) * n + hi], r = a[hi * n + hi - 1], s = a[hi * n + hi];
    const double tr = p + s, det = p * s - q * r;
    const double d = tr * tr / 4 - det;
    double mu = s;
    if (d >= 0) {
      const double r1 = tr / 2 + std::sqrt(d), r2 = tr / 2 - std::sqrt(d);
      mu = (std::fabs(r1 - s) < std::fabs(r2 - s)) ? r1 : r2;
    }
    if (iter % 11 == 10) mu += std::fabs(a[hi * n + hi - 1]); // exceptional shift
    for (int i = l; i <= hi; ++i) a[i * n + i] -= mu;
    std::vector<double> cs(hi - l), sn(hi - l);
    for (int k = l; k < hi; ++k) {
      const double x = a[k * n + k], y = a[(k + 1) * n + k];
      const double h = std::hypot(x, y);
      const double c = h == 0 ? 1.0 : x / h, sg = h == 0 ? 0.0 : y / h;
      cs[k - l] = c;
      sn[k - l] = sg;
      for (int j = k; j < n; ++j) {
        const double t1 = a[k * n + j], t2 = a[(k + 1) * n + j];
        a[k * n + j] = c * t1 + sg * t2;
        a[(k + 1) * n + j] = -sg * t1 + c * t2;
      }
    }
    for (int k = l; k < hi; ++k) {
      const double c = cs[k - l], sg = sn[k - l];
      for (int i = 0; i <= std::min(hi, k + 2); ++i) {
        const double t1 = a[i * n + k], t2 = a[i * n + k + 1];
        a[i * n + k] = c * t1 + sg * t2;
        a[i * n + k + 1] = -sg * t1 + c * t2;
      }
    }
    for (int i = l; i <= hi; ++i) a[i * n + i] += mu;
    ++iter;
  }
  return ev;
}

static const std::vector<double> &opt_betas(int degree)
{
  // Optimal 4th-kind Chebyshev coefficients (Lottes, arXiv:2202.08830), degrees 1..8.
  static const std::vector<std::vector<double>> tab = {
      {},
      {1.12500000000000},
      {1.02387287570313, 1.26408905371085},
      {1.00842544782028, 1.08867839208730, 1.33753125909618},
      {1.00391310427285, 1.04035811188593, 1.14863498546254, 1.38268869241000},
      {1.00212930146164, 1.02173711549260, 1.07872433192603, 1.19810065292663, 1.41322542791682},
      {1.00128517255940, 1.01304293035233, 1.04678215124113, 1.11616489419675, 1.23829020218444, 1.43524297106744},
      {1.00083464397912, 1.00843949430122, 1.03008707768713, 1.07408384092003, 1.15036186707366, 1.27116474046139,
       1.45186658649364},
      {1.00057246631197, 1.00577427662415, 1.02050187922941, 1.05019803444565, 1.10115572984941, 1.18086042806856,
       1.29838585382576, 1.46486073151099},
  };
  if (degree < 0 || degree >= (int)tab.size()) throw std::runtime_error("opt. 4th-kind Chebyshev degree must be 0..8");
  return tab[degree];
}

// ---------------------------------------------------------------------------
// schedule
// ---------------------------------------------------------------------------
static std::vector<std::string> split(const std::string &s, char c)
{
  std::vector<std::string> out;
  std::string cur;
  for (char ch : s) {
    if (ch == c) { out.push_back(cur); cur.clear(); }
    else if (ch != ' ') cur.push_back(ch);
  }
  out.push_back(cur);
  return out;
}

struct Schedule {
  std::vector<int> levels;                 // down leg orders, finest first
  std::map<std::pair<int, bool>, int> deg; // (order, downLeg) -> degree
};

static Schedule parse_schedule(const std::string &sched, int N, int defaultDegree)
{
  Schedule S;
  const int INVALID = -1000000;
  int minOrder = 1 << 30, prev = 1 << 30;
  auto entries = split(sched, ',');
  for (auto &en : entries)
    for (auto &tok : split(en, '+'))
      if (tok.rfind("p=", 0) == 0) minOrder = std::min(minOrder, std::stoi(tok.substr(2)));
  bool down = true;
  for (auto &en : entries) {
    int order = INVALID, degree = INVALID;
    for (auto &tok : split(en, '+')) {
      if (tok.rfind("p=", 0) == 0) {
        order = std::stoi(tok.substr(2));
        if (order > prev) down = false;
        if (down) S.levels.push_back(order);
        prev = order;
      } else if (tok.rfind("degree=", 0) == 0) {
        degree = std::stoi(tok.substr(7));
      } else if (!tok.empty()) {
        throw std::runtime_error("unknown token in pMGSchedule: " + tok);
      }
    }
    if (order == INVALID) throw std::runtime_error("order not specified in " + en);
    if (degree == INVALID && order != minOrder) degree = defaultDegree;
    S.deg[{order, down}] = degree;
  }
  if (S.levels.empty() || S.levels.front() != N) throw std::runtime_error("finest pMG degree must match N");
  return S;
}

static std::vector<int> default_levels(int N, bool schwarz)
{
  static const std::map<int, std::vector<int>> sch = {{1, {1}}, {2, {2, 1}}, {3, {3, 1}}, {4, {4, 2, 1}}, {5, {5, 3, 1}},
                                                      {6, {6, 3, 1}}, {7, {7, 3, 1}}, {8, {8, 5, 1}}, {9, {9, 5, 1}}};
  static const std::map<int, std::vector<int>> jac = {{1, {1}}, {2, {2, 1}}, {3, {3, 1}}, {4, {4, 2, 1}},
                                                      {5, {5, 3, 1}}, {6, {6, 4, 2, 1}}, {7, {7, 5, 3, 1}},
                                                      {8, {8, 6, 4, 1}}, {9, {9, 7, 5, 1}}};
  return schwarz ? sch.at(N) : jac.at(N);
}

// ---------------------------------------------------------------------------
// MG state
// ---------------------------------------------------------------------------
template <typename T> struct FDMData {
  int Nqe = 0, Npe = 0;
  std::vector<T> Sx, Sy, Sz, invL, wts;
  std::vector<int> extOff, extIds;   // masked extended-mesh gather groups
  std::vector<T> work1, work2;
  std::vector<T> Sext, out;          // per-call result buffers, kept between calls
};

template <typename T> struct MGLevel {
  Level *L = nullptr;              // mesh data (the fine level points at Elliptic::fine)
  std::unique_ptr<Level> own;
  std::vector<T> ggeo, D, invDegree;
  // transfer from the next finer level
  std::vector<T> R;                // [Ncq][Nfq]: R[c][f] = l_c(z_f)
  std::vector<T> invDegreeFine;
  int Nf = 0;
  // smoother
  bool smoothed = true;
  std::string base;                // jac | asm | ras
  std::string kind;                // cheby | fourth | fourthopt
  std::vector<T> invDiag;
  double rho = 0, lambda0 = 0, lambda1 = 0;
  int up = 2, down = 2;
  std::vector<double> upBetas, downBetas;
  FDMData<T> fdm;
  std::vector<T> x, rhs, res;
};

template <typename T> struct MGT {
  std::vector<MGLevel<T>> levels;
  std::vector<T> sRes, sRes2, sUpd;      // smoother scratch (pMGLevel::o_smoother*)
  std::vector<T> rP, zP;                 // pfloat copies of r, z
  Options o;
  bool poisson = true;
  T lambda0 = 1, lambda1 = 0;
  bool allNeumann = false;               // singular coarse system: project its right-hand side
  // coarse PCG scratch
  std::vector<T> cp, cz, cAp, cr;
  std::vector<int> coarseIters;
  // Galerkin coarse operator (CSR over the coarsest level's masked gather groups)
  std::vector<long long> gRowPtr, gCol, gRowOfNode;
  std::vector<T> gVal, gInvDiag;
  std::vector<long long> gRep;
};

struct MG {
  bool fp32 = false;
  MGT<double> d;
  MGT<float> f;
  std::vector<double> rho;  // per smoothed level
  std::vector<int> degrees;
};

// operator on a level in precision T: Ax -> mask -> gs (ellipticOperator, pfloat)
template <typename T> static void level_op(MGT<T> &M, MGLevel<T> &lv, const T *q, T *Aq)
{
  ax_stored<T>(*lv.L, lv.ggeo.data(), lv.D.data(), M.lambda0, M.lambda1, M.poisson, q, Aq);
  apply_mask(*lv.L, Aq);
  gs_add(*lv.L, Aq);
}

// ---------------------------------------------------------------------------
// FDM / Schwarz setup (ellipticMultiGridSchwarz.cpp)
// ---------------------------------------------------------------------------
struct Lengths {
  std::vector<double> lx, ly, lz, mx, my, mz, rx, ry, rz;
};

// element lengths on the finest mesh (compute_element_lengths / harmonic_mean_element_length)
static Lengths element_lengths(const Level &F)
{
  const int Nq = F.Nq;
  const long long E = F.E;
  Lengths Ls;
  for (auto *v : {&Ls.lx, &Ls.ly, &Ls.lz, &Ls.mx, &Ls.my, &Ls.mz, &Ls.rx, &Ls.ry, &Ls.rz}) v->assign(E, 0.0);
  const int nx = (Nq == 2) ? Nq : Nq - 1;
  const int start = (Nq == 2) ? 0 : 1;
  const double *w = F.w.data();
  for (long long e = 0; e < E; ++e) {
    const long long o = e * F.Np;
    auto dist2 = [&](long long a, long long b) {
      const double dx = F.x[a] - F.x[b], dy = F.y[a] - F.y[b], dz = F.zc[a] - F.zc[b];
      return dx * dx + dy * dy + dz * dz;
    };
    double l2 = 0, ws = 0;
    for (int k = start; k < nx; ++k)
      for (int j = start; j < nx; ++j) {
        const double wt = (Nq == 2) ? 1.0 : w[j - 1] * w[k - 1];
        l2 += wt / dist2(o + (Nq - 1) + j * Nq + k * Nq * Nq, o + 0 + j * Nq + k * Nq * Nq);
        ws += wt;
      }
    Ls.mx[e] = 1.0 / std::sqrt(l2 / ws);
    l2 = ws = 0;
    for (int k = start; k < nx; ++k)
      for (int i = start; i < nx; ++i) {
        const double wt = (Nq == 2) ? 1.0 : w[i - 1] * w[k - 1];
        l2 += wt / dist2(o + i + (Nq - 1) * Nq + k * Nq * Nq, o + i + 0 * Nq + k * Nq * Nq);
        ws += wt;
      }
    Ls.my[e] = 1.0 / std::sqrt(l2 / ws);
    l2 = ws = 0;
    for (int j = start; j < nx; ++j)
      for (int i = start; i < nx; ++i) {
        const double wt = (Nq == 2) ? 1.0 : w[i - 1] * w[j - 1];
        l2 += wt / dist2(o + i + j * Nq + (Nq - 1) * Nq * Nq, o + i + j * Nq);
        ws += wt;
      }
    Ls.mz[e] = 1.0 / std::sqrt(l2 / ws);
  }
  if (Nq == 2) {
    Ls.lx = Ls.rx = Ls.mx;
    Ls.ly = Ls.ry = Ls.my;
    Ls.lz = Ls.rz = Ls.mz;
    return Ls;
  }
  // neighbour lengths through an (unmasked) gather-scatter of face values
  std::vector<double> l(F.Nlocal, 0.0);
  const int N = F.N;
  for (long long e = 0; e < E; ++e) {
    const long long o = e * F.Np;
    for (int j = 1; j < N; ++j)
      for (int k = 1; k < N; ++k) {
        l[o + k * Nq + j * Nq * Nq] = Ls.mx[e];
        l[o + Nq - 1 + k * Nq + j * Nq * Nq] = Ls.mx[e];
        l[o + k + 0 * Nq + j * Nq * Nq] = Ls.my[e];
        l[o + k + (Nq - 1) * Nq + j * Nq * Nq] = Ls.my[e];
        l[o + k + j * Nq] = Ls.mz[e];
        l[o + k + j * Nq + (Nq - 1) * Nq * Nq] = Ls.mz[e];
      }
  }
  std::vector<int> off, gid;
  std::vector<double> inv;
  ogs_setup(F.Nlocal, F.ids.data(), off, gid, inv);
  for (size_t g = 0; g + 1 < off.size(); ++g) {
    if (off[g] + 1 == off[g + 1]) continue;
    double v = 0;
    for (int q = off[g]; q < off[g + 1]; ++q) v += l[gid[q]];
    for (int q = off[g]; q < off[g + 1]; ++q) l[gid[q]] = v;
  }
  const double tol = 1e-12;
  for (long long e = 0; e < E; ++e) {
    const long long o = e * F.Np;
    Ls.lx[e] = l[o + 1 * Nq + 1 * Nq * Nq] - Ls.mx[e];
    Ls.rx[e] = l[o + Nq - 1 + 1 * Nq + 1 * Nq * Nq] - Ls.mx[e];
    Ls.ly[e] = l[o + 1 + 1 * Nq * Nq] - Ls.my[e];
    Ls.ry[e] = l[o + 1 + (Nq - 1) * Nq + 1 * Nq * Nq] - Ls.my[e];
    Ls.lz[e] = l[o + 1 + Nq] - Ls.mz[e];
    Ls.rz[e] = l[o + 1 + Nq + (Nq - 1) * Nq * Nq] - Ls.mz[e];
    auto fix = [&](double &v, double m) {
      if (std::fabs(v) < tol || v < -tol) v = m;
    };
    fix(Ls.lx[e], Ls.mx[e]);
    fix(Ls.ly[e], Ls.my[e]);
    fix(Ls.lz[e], Ls.mz[e]);
    fix(Ls.rx[e], Ls.mx[e]);
    fix(Ls.ry[e], Ls.my[e]);
    fix(Ls.rz[e], Ls.mz[e]);
  }
  return Ls;
}

// 1-D stiffness / mass on the extended (n+3) grid and their generalized
// eigenvectors; returns S column-major (S[r + nl*c]) with Dirichlet rows zeroed.
static void fdm_1d(const Level &L, int lbc, int rbc, double ll, double lm, double lr, std::vector<double> &S,
                   std::vector<double> &lam)
{
  const int n = L.N, nq = n + 1, nl = n + 3;
  std::vector<double> ah(nq * nq);
  for (int i = 0; i < nq; ++i)
    for (int j = 0; j < nq; ++j) {
      double v = 0;
      for (int k = 0; k < nq; ++k) v += L.D[k * nq + i] * L.w[k] * L.D[k * nq + j];
      ah[i + nq * j] = v;
    }
  auto AH = [&](int i, int j) { return ah[i + nq * j]; };
  std::vector<double> a(nl * nl, 0.0), b(nl * nl, 0.0);
  auto A = [&](int i, int j) -> double & { return a[i + nl * j]; };
  auto B = [&](int i, int j) -> double & { return b[i + nl * j]; };
  const int i0 = (lbc == 1) ? 1 : 0;
  const int i1 = (rbc == 1) ? n - 1 : n;
  double fac = 2.0 / lm;
  A(1, 1) = 1.0;
  A(n + 1, n + 1) = 1.0;
  for (int j = i0; j <= i1; ++j)
    for (int i = i0; i <= i1; ++i) A(i + 1, j + 1) = fac * AH(i, j);
  if (lbc == 0) {
    fac = 2.0 / ll;
    A(0, 0) = fac * AH(n - 1, n - 1);
    A(1, 0) = fac * AH(n, n - 1);
    A(0, 1) = fac * AH(n - 1, n);
    A(1, 1) = A(1, 1) + fac * AH(n, n);
  } else {
    A(0, 0) = 1.0;
  }
  if (rbc == 0) {
    fac = 2.0 / lr;
    A(n + 1, n + 1) = A(n + 1, n + 1) + fac * AH(0, 0);
    A(n + 2, n + 1) = fac * AH(1, 0);
    A(n + 1, n + 2) = fac * AH(0, 1);
    A(n + 2, n + 2) = fac * AH(1, 1);
  } else {
    A(n + 2, n + 2) = 1.0;
  }
  fac = 0.5 * lm;
  B(1, 1) = 1.0;
  B(n + 1, n + 1) = 1.0;
  for (int i = i0; i <= i1; ++i) B(i + 1, i + 1) = fac * L.w[i];
  if (lbc == 0) {
    fac = 0.5 * ll;
    B(0, 0) = fac * L.w[n - 1];
    B(1, 1) = B(1, 1) + fac * L.w[n];
  } else {
    B(0, 0) = 1.0;
  }
  if (rbc == 0) {
    fac = 0.5 * lr;
    B(n + 1, n + 1) = B(n + 1, n + 1) + fac * L.w[0];
    B(n + 2, n + 2) = fac * L.w[1];
  } else {
    B(n + 2, n + 2) = 1.0;
  }
  // A s = lambda B s with diagonal B: C = B^-1/2 A B^-1/2 (symmetric), s = B^-1/2 q
  std::vector<double> binv(nl), C(nl * nl);
  for (int i = 0; i < nl; ++i) binv[i] = 1.0 / std::sqrt(B(i, i));
  for (int i = 0; i < nl; ++i)
    for (int j = 0; j < nl; ++j) C[i * nl + j] = binv[i] * 0.5 * (A(i, j) + A(j, i)) * binv[j];
  std::vector<double> Q;
  jacobi_eig(nl, C, lam, Q);
  S.assign(nl * nl, 0.0);
  for (int r = 0; r < nl; ++r)
    for (int c = 0; c < nl; ++c) S[r + nl * c] = binv[r] * Q[r * nl + c];
  auto row_zero = [&](int r) {
    for (int c = 0; c < nl; ++c) S[r + nl * c] = 0.0;
  };
  if (lbc > 0) row_zero(0);
  if (lbc == 1) row_zero(1);
  if (rbc > 0) row_zero(nl - 1);
  if (rbc == 1) row_zero(nl - 2);
}

// extended-mesh gather groups: edges of the (Nq+2)^3 element and Dirichlet nodes masked
static void ext_gather(const Level &L, std::vector<int> &off, std::vector<int> &gid)
{
  const int Ne = L.N + 2, nqe = Ne + 1;
  const long long npe = (long long)nqe * nqe * nqe, nloc = L.E * npe;
  std::vector<long long> ids(nloc);
  global_ids(Ne, L.E, L.EToV.data(), ids.data());
  std::vector<int> uoff, ugid;
  std::vector<double> uinv;
  ogs_setup(nloc, ids.data(), uoff, ugid, uinv);
  std::vector<int> mask;
  dirichlet_mask(Ne, L.E, L.EToB.data(), uoff, ugid, mask);
  std::vector<char> masked(nloc, 0);
  for (int m : mask) masked[m] = 1;
  for (long long e = 0; e < L.E; ++e)
    for (int k = 0; k < nqe; ++k)
      for (int j = 0; j < nqe; ++j)
        for (int i = 0; i < nqe; ++i) {
          const int ext = (i == 0 || i == nqe - 1) + (j == 0 || j == nqe - 1) + (k == 0 || k == nqe - 1);
          if (ext >= 2) masked[e * npe + i + nqe * (j + nqe * k)] = 1;
        }
  for (long long q = 0; q < nloc; ++q)
    if (masked[q]) ids[q] = 0;
  std::vector<double> inv;
  ogs_setup(nloc, ids.data(), off, gid, inv);
}

template <typename T> static void gs_groups(const std::vector<int> &off, const std::vector<int> &gid, T *q)
{
  const long long ng = (long long)off.size() - 1;
#pragma omp parallel for schedule(static)
  for (long long g = 0; g < ng; ++g) {
    if (off[g] + 1 == off[g + 1]) continue;
    T v = 0;
    for (int m = off[g]; m < off[g + 1]; ++m) v += q[gid[m]];
    for (int m = off[g]; m < off[g + 1]; ++m) q[gid[m]] = v;
  }
}

// arr1 face layers (l1 and its mirror) = f1*arr1 + f2*arr2 (layers l2), face-interior points only
template <typename T> static void extrude(T *a1, int l1, T f1, const T *a2, int l2, T f2, long long E, int nx)
{
  auto I = [&](int r, int s, int t, long long e) { return r + nx * (s + nx * (t + nx * e)); };
  for (long long e = 0; e < E; ++e) {
    for (int k = 1; k < nx - 1; ++k)
      for (int j = 1; j < nx - 1; ++j) {
        a1[I(l1, j, k, e)] = f1 * a1[I(l1, j, k, e)] + f2 * a2[I(l2, j, k, e)];
        a1[I(nx - l1 - 1, j, k, e)] = f1 * a1[I(nx - l1 - 1, j, k, e)] + f2 * a2[I(nx - l2 - 1, j, k, e)];
      }
    for (int k = 1; k < nx - 1; ++k)
      for (int i = 1; i < nx - 1; ++i) {
        a1[I(i, l1, k, e)] = f1 * a1[I(i, l1, k, e)] + f2 * a2[I(i, l2, k, e)];
        a1[I(i, nx - l1 - 1, k, e)] = f1 * a1[I(i, nx - l1 - 1, k, e)] + f2 * a2[I(i, nx - l2 - 1, k, e)];
      }
    for (int j = 1; j < nx - 1; ++j)
      for (int i = 1; i < nx - 1; ++i) {
        a1[I(i, j, l1, e)] = f1 * a1[I(i, j, l1, e)] + f2 * a2[I(i, j, l2, e)];
        a1[I(i, j, nx - l1 - 1, e)] = f1 * a1[I(i, j, nx - l1 - 1, e)] + f2 * a2[I(i, j, nx - l2 - 1, e)];
      }
  }
}

template <typename T> static void fdm_setup(MGLevel<T> &lv, const Level &fineL)
{
  const Level &L = *lv.L;
  auto &F = lv.fdm;
  const int nl = L.N + 3;
  F.Nqe = nl;
  F.Npe = nl * nl * nl;
  const long long E = L.E;
  Lengths Ls = element_lengths(fineL);
  F.Sx.resize((size_t)E * nl * nl);
  F.Sy.resize((size_t)E * nl * nl);
  F.Sz.resize((size_t)E * nl * nl);
  F.invL.resize((size_t)E * F.Npe);
  for (long long e = 0; e < E; ++e) {
    const int *bc = &L.EToB[e * 6];
    const int lbr = bc[4], rbr = bc[2], lbs = bc[1], rbs = bc[3], lbt = bc[0], rbt = bc[5];
    std::vector<double> Sx, Sy, Sz, lr, ls, lt;
    fdm_1d(L, lbr, rbr, Ls.lx[e], Ls.mx[e], Ls.rx[e], Sx, lr);
    fdm_1d(L, lbs, rbs, Ls.ly[e], Ls.my[e], Ls.ry[e], Sy, ls);
    fdm_1d(L, lbt, rbt, Ls.lz[e], Ls.mz[e], Ls.rz[e], Sz, lt);
    // stored as op[i + j*nl] = S(j, i)
    for (int i = 0; i < nl; ++i)
      for (int j = 0; j < nl; ++j) {
        F.Sx[e * nl * nl + i + j * nl] = (T)Sx[j + i * nl];
        F.Sy[e * nl * nl + i + j * nl] = (T)Sy[j + i * nl];
        F.Sz[e * nl * nl + i + j * nl] = (T)Sz[j + i * nl];
      }
    long long l = 0;
    for (int k = 0; k < nl; ++k)
      for (int j = 0; j < nl; ++j)
        for (int i = 0; i < nl; ++i) {
          const double d = lr[i] + ls[j] + lt[k];
          F.invL[e * F.Npe + l++] = (T)(d > 1e-5 ? 1.0 / d : 0.0);
        }
  }
  ext_gather(L, F.extOff, F.extIds);
  F.work1.assign((size_t)E * F.Npe, 0);
  F.work2.assign((size_t)E * F.Npe, 0);
  // weights (generate_weights)
  std::vector<T> w1((size_t)E * F.Npe, 1), w2((size_t)E * F.Npe, 1);
  extrude<T>(w2.data(), 0, 0, w1.data(), 0, 1, E, nl);
  gs_groups(F.extOff, F.extIds, w1.data());
  extrude<T>(w1.data(), 0, 1, w2.data(), 0, -1, E, nl);
  extrude<T>(w1.data(), 2, 1, w1.data(), 0, 1, E, nl);
  F.wts.resize(L.Nlocal);
  const int nq = L.Nq;
  for (long long e = 0; e < E; ++e)
    for (int k = 0; k < nq; ++k)
      for (int j = 0; j < nq; ++j)
        for (int i = 0; i < nq; ++i)
          F.wts[e * L.Np + i + nq * (j + nq * k)] = w1[e * F.Npe + (i + 1) + nl * ((j + 1) + nl * (k + 1))];
  gs_add(L, F.wts.data());
  for (auto &v : F.wts) v = (T)1 / v;
}

// Schwarz smoother Su = S(u) (pMGLevel::smoothSchwarz): preFDM -> ext gs ->
// fusedFDM -> [ASM: ext gs -> postFDM] -> gs -> mask.  u and Su may alias.
constexpr int kMaxNpe = 12 * 12 * 12; // (N+3)^3 for N <= 9
template <typename T> static void smooth_schwarz(MGT<T> &M, MGLevel<T> &lv, const T *u, T *Su)
{
  const Level &L = *lv.L;
  auto &F = lv.fdm;
  const int nq = L.Nq, nl = F.Nqe, npe = F.Npe, np = L.Np;
  const long long E = L.E;
  const bool ras = lv.base == "ras";
  T *w1 = F.work1.data(), *w2 = F.work2.data();
  auto X = [&](int i, int j, int k) { return i + nl * (j + nl * k); };
  // preFDM
  #pragma omp parallel for schedule(static)
  for (long long e = 0; e < E; ++e) {
    T *we = w1 + e * npe;
    const T *ue = u + e * np;
    for (int k = 0; k < nl; ++k)
      for (int j = 0; j < nl; ++j)
        for (int i = 0; i < nl; ++i) {
          const bool in = i >= 1 && i < nl - 1 && j >= 1 && j < nl - 1 && k >= 1 && k < nl - 1;
          we[X(i, j, k)] = in ? ue[(i - 1) + nq * ((j - 1) + nq * (k - 1))] : T(0);
        }
    auto U = [&](int i, int j, int k) { return ue[(i - 1) + nq * ((j - 1) + nq * (k - 1))]; };
    for (int a = 1; a < nl - 1; ++a)
      for (int b = 1; b < nl - 1; ++b) {
        we[X(0, a, b)] = U(2, a, b);
        we[X(nl - 1, a, b)] = U(nl - 3, a, b);
        we[X(a, 0, b)] = U(a, 2, b);
        we[X(a, nl - 1, b)] = U(a, nl - 3, b);
        we[X(a, b, 0)] = U(a, b, 2);
        we[X(a, b, nl - 1)] = U(a, b, nl - 3);
      }
  }
  gs_groups(F.extOff, F.extIds, w1);
  if (!ras && F.Sext.size() != (size_t)E * npe) F.Sext.resize((size_t)E * npe);
  if (F.out.size() != (size_t)E * np) F.out.resize((size_t)E * np);
  std::vector<T> &Sext = F.Sext, &out = F.out; // every entry is written below before it is read
  #pragma omp parallel for schedule(static)
  for (long long e = 0; e < E; ++e) {
    T *we = w1 + e * npe;
    for (int a = 1; a < nl - 1; ++a)
      for (int b = 1; b < nl - 1; ++b) {
        we[X(0, a, b)] -= we[X(2, a, b)];
        we[X(nl - 1, a, b)] -= we[X(nl - 3, a, b)];
        we[X(a, 0, b)] -= we[X(a, 2, b)];
        we[X(a, nl - 1, b)] -= we[X(a, nl - 3, b)];
        we[X(a, b, 0)] -= we[X(a, b, 2)];
        we[X(a, b, nl - 1)] -= we[X(a, b, nl - 3)];
      }
    const T *sx = &F.Sx[e * nl * nl], *sy = &F.Sy[e * nl * nl], *sz = &F.Sz[e * nl * nl];
    // S(r,c) = op[c + r*nl]
    auto SX = [&](int r, int c) { return sx[c + r * nl]; };
    auto SY = [&](int r, int c) { return sy[c + r * nl]; };
    auto SZ = [&](int r, int c) { return sz[c + r * nl]; };
    T t1[kMaxNpe], t2[kMaxNpe];
    // forward: S^T along x, y, z; scale by invL; back: S along x, y, z.  Each
    // output is sum_l S(.,.) v(l) accumulated for l ascending from 0 (the
    // order of fusedFDM.c); the loops run the outputs innermost so that they
    // vectorise without changing any output's summation order.
    const int nl2 = nl * nl;
    for (int q = 0; q < npe; ++q) t1[q] = 0;
    for (int k = 0; k < nl; ++k)
      for (int j = 0; j < nl; ++j)
        for (int l = 0; l < nl; ++l) {
          const T w = we[X(l, j, k)];
          T *o = t1 + X(0, j, k);
          const T *srow = sx + l * nl; // SX(l, i) = sx[i + l nl]
          for (int i = 0; i < nl; ++i) o[i] += srow[i] * w;
        }
    for (int q = 0; q < npe; ++q) t2[q] = 0;
    for (int k = 0; k < nl; ++k)
      for (int j = 0; j < nl; ++j)
        for (int l = 0; l < nl; ++l) {
          const T c = SY(l, j);
          T *o = t2 + X(0, j, k);
          const T *v = t1 + X(0, l, k);
          for (int i = 0; i < nl; ++i) o[i] += c * v[i];
        }
    for (int q = 0; q < npe; ++q) t1[q] = 0;
    for (int k = 0; k < nl; ++k)
      for (int l = 0; l < nl; ++l) {
        const T c = SZ(l, k);
        T *o = t1 + k * nl2;
        const T *v = t2 + l * nl2;
        for (int ij = 0; ij < nl2; ++ij) o[ij] += c * v[ij];
      }
    for (int q = 0; q < npe; ++q) t1[q] = t1[q] * F.invL[e * npe + q];
    for (int q = 0; q < npe; ++q) t2[q] = 0;
    for (int k = 0; k < nl; ++k)
      for (int j = 0; j < nl; ++j)
        for (int l = 0; l < nl; ++l) {
          const T w = t1[X(l, j, k)];
          T *o = t2 + X(0, j, k);
          for (int i = 0; i < nl; ++i) o[i] += SX(i, l) * w;
        }
    for (int q = 0; q < npe; ++q) t1[q] = 0;
    for (int k = 0; k < nl; ++k)
      for (int j = 0; j < nl; ++j)
        for (int l = 0; l < nl; ++l) {
          const T c = SY(j, l);
          T *o = t1 + X(0, j, k);
          const T *v = t2 + X(0, l, k);
          for (int i = 0; i < nl; ++i) o[i] += c * v[i];
        }
    for (int q = 0; q < npe; ++q) t2[q] = 0;
    for (int k = 0; k < nl; ++k)
      for (int l = 0; l < nl; ++l) {
        const T c = SZ(k, l);
        T *o = t2 + k * nl2;
        const T *v = t1 + l * nl2;
        for (int ij = 0; ij < nl2; ++ij) o[ij] += c * v[ij];
      }
    if (ras) {
      // restrict with the level's inverse degree (the weights argument of
      // fusedFDM, elliptic->o_invDegree: ellipticMultiGridSchwarz.cpp:1069-1077,
      // fusedFDM.c:209-215)
      for (int k = 0; k < nq; ++k)
        for (int j = 0; j < nq; ++j)
          for (int i = 0; i < nq; ++i) {
            const long long id = e * np + i + nq * (j + nq * k);
            out[id] = t2[X(i + 1, j + 1, k + 1)] * lv.invDegree[id];
          }
    } else {
      std::memcpy(&Sext[e * npe], t2, sizeof(T) * npe);
      // keep this element's own face-layer results for the overlap combine
      for (int a = 1; a < nl - 1; ++a)
        for (int b = 1; b < nl - 1; ++b)
          for (int side = 0; side < 2; ++side) {
            const int f = side ? nl - 1 : 0;
            we[X(f, a, b)] = t2[X(f, a, b)];
            we[X(a, f, b)] = t2[X(a, f, b)];
            we[X(a, b, f)] = t2[X(a, b, f)];
          }
    }
  }
  if (!ras) {
    gs_groups(F.extOff, F.extIds, Sext.data());
    #pragma omp parallel for schedule(static)
    for (long long e = 0; e < E; ++e) {
      T *s = &Sext[e * npe];
      const T *own = w1 + e * npe;
      // face layers: (sum over the overlap) - own = the neighbour's contribution
      for (int a = 1; a < nl - 1; ++a)
        for (int b = 1; b < nl - 1; ++b)
          for (int side = 0; side < 2; ++side) {
            const int f = side ? nl - 1 : 0;
            s[X(f, a, b)] -= own[X(f, a, b)];
            s[X(a, f, b)] -= own[X(a, f, b)];
            s[X(a, b, f)] -= own[X(a, b, f)];
          }
      // add it onto the first interior layer inside the element
      for (int a = 1; a < nl - 1; ++a)
        for (int b = 1; b < nl - 1; ++b) {
          s[X(2, a, b)] += s[X(0, a, b)];
          s[X(nl - 3, a, b)] += s[X(nl - 1, a, b)];
          s[X(a, 2, b)] += s[X(a, 0, b)];
          s[X(a, nl - 3, b)] += s[X(a, nl - 1, b)];
          s[X(a, b, 2)] += s[X(a, b, 0)];
          s[X(a, b, nl - 3)] += s[X(a, b, nl - 1)];
        }
      for (int k = 0; k < nq; ++k)
        for (int j = 0; j < nq; ++j)
          for (int i = 0; i < nq; ++i) {
            const long long id = e * np + i + nq * (j + nq * k);
            out[id] = s[X(i + 1, j + 1, k + 1)] * F.wts[id];
          }
    }
  }
  gs_add(L, out.data());
  apply_mask(L, out.data());
  std::memcpy(Su, out.data(), sizeof(T) * L.Nlocal);
}

// smoother S applied to r (pMGLevel::smoother)
template <typename T> static void apply_S(MGT<T> &M, MGLevel<T> &lv, const T *r, T *Sr)
{
  const long long n = lv.L->Nlocal;
  if (lv.base == "jac") {
    #pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i) Sr[i] = lv.invDiag[i] * r[i];
  } else {
    smooth_schwarz(M, lv, r, Sr);
  }
}

// ---------------------------------------------------------------------------
// Chebyshev smoothers
// ---------------------------------------------------------------------------
template <typename T> static void smooth_cheby1(MGT<T> &M, MGLevel<T> &lv, const T *r, T *x, bool xIsZero)
{
  const int degree = xIsZero ? lv.down : lv.up;
  if (degree == 0) return;
  const long long n = lv.L->Nlocal;
  const T theta = (T)(0.5 * (lv.lambda1 + lv.lambda0));
  const T delta = (T)(0.5 * (lv.lambda1 - lv.lambda0));
  const T invTheta = (T)1.0 / theta;
  const T sigma = theta / delta;
  T rho_n = (T)1.0 / sigma;
  T *res = M.sRes.data(), *Ad = M.sRes2.data(), *d = M.sUpd.data();
  if (xIsZero) std::fill(x, x + n, T(0));
  if (!xIsZero) {
    level_op(M, lv, x, res);
    #pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i) res[i] = (T)1 * r[i] + (T)(-1) * res[i];
  } else {
    std::memcpy(res, r, sizeof(T) * n);
  }
  apply_S(M, lv, res, res);
  #pragma omp parallel for schedule(static)
  for (long long i = 0; i < n; ++i) d[i] = invTheta * res[i];
  for (int k = 1; k < degree; ++k) {
    level_op(M, lv, d, Ad);
    apply_S(M, lv, Ad, Ad);
    const T rhoSave = rho_n;
    rho_n = (T)1.0 / ((T)2.0 * sigma - rho_n);
    const T rCoeff = (T)2.0 * rho_n / delta;
    const T dCoeff = rho_n * rhoSave;
    #pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i) {
      x[i] = x[i] + d[i];
      res[i] = res[i] - Ad[i];
      d[i] = dCoeff * d[i] + rCoeff * res[i];
    }
  }
  #pragma omp parallel for schedule(static)
  for (long long i = 0; i < n; ++i) x[i] = (T)1 * d[i] + (T)1 * x[i];
  apply_mask(*lv.L, x);
}

template <typename T> static void smooth_cheby4(MGT<T> &M, MGLevel<T> &lv, const T *r, T *x, bool xIsZero)
{
  const int degree = xIsZero ? lv.down : lv.up;
  if (degree == 0) return;
  const auto &betas = xIsZero ? lv.downBetas : lv.upBetas;
  const long long n = lv.L->Nlocal;
  T *res = M.sRes.data(), *Ad = M.sRes2.data(), *d = M.sUpd.data();
  const double rho = lv.lambda1;
  if (xIsZero) {
    std::fill(x, x + n, T(0));
    std::memcpy(res, r, sizeof(T) * n);
  } else {
    level_op(M, lv, x, res);
    #pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i) res[i] = r[i] - res[i];
  }
  apply_S(M, lv, res, Ad);
  const T c0 = (T)(4.0 / (3.0 * rho));
  #pragma omp parallel for schedule(static)
  for (long long i = 0; i < n; ++i) d[i] = c0 * Ad[i];
  for (int k = 1; k < degree; ++k) {
    level_op(M, lv, d, Ad);
    const T beta = (T)betas[k - 1];
    #pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i) {
      x[i] = x[i] + beta * d[i];
      res[i] = res[i] - Ad[i];
    }
    apply_S(M, lv, res, Ad);
    const T dCoeff = (T)((2.0 * k - 1.0) / (2.0 * k + 3.0));
    const T rCoeff = (T)((8.0 * k + 4.0) / ((2.0 * k + 3.0) * rho));
    #pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i) d[i] = rCoeff * Ad[i] + dCoeff * d[i];
  }
  const T bl = (T)betas.back();
  #pragma omp parallel for schedule(static)
  for (long long i = 0; i < n; ++i) x[i] = bl * d[i] + x[i];
  apply_mask(*lv.L, x);
}

template <typename T> static void smooth(MGT<T> &M, MGLevel<T> &lv, const T *r, T *x, bool xIsZero)
{
  if (lv.kind == "cheby")
    smooth_cheby1(M, lv, r, x, xIsZero);
  else
    smooth_cheby4(M, lv, r, x, xIsZero);
}

// ---------------------------------------------------------------------------
// transfers
// ---------------------------------------------------------------------------
// qc = (R x R x R) qf with R[c][f]; the reference's serial kernel accumulates in dfloat
template <typename T> static void coarsen_apply(const MGLevel<T> &lc, const T *qf, T *qc)
{
  const int Nfq = lc.Nf + 1, Ncq = lc.L->Nq;
  const long long E = lc.L->E;
  const long long npf = (long long)Nfq * Nfq * Nfq, npc = (long long)Ncq * Ncq * Ncq;
#pragma omp parallel
  {
  std::vector<double> t1((size_t)Nfq * Nfq * Ncq), t2((size_t)Nfq * Ncq * Ncq); // per-thread scratch
#pragma omp for schedule(static)
  for (long long e = 0; e < E; ++e) {
    const T *f = qf + e * npf;
    // along k
    for (int j = 0; j < Nfq; ++j)
      for (int i = 0; i < Nfq; ++i)
        for (int c = 0; c < Ncq; ++c) {
          double v = 0;
          for (int k = 0; k < Nfq; ++k) v += (double)lc.R[c * Nfq + k] * (double)f[i + Nfq * (j + Nfq * k)];
          t1[i + Nfq * (j + Nfq * c)] = v;
        }
    // along j
    for (int c = 0; c < Ncq; ++c)
      for (int b = 0; b < Ncq; ++b)
        for (int i = 0; i < Nfq; ++i) {
          double v = 0;
          for (int j = 0; j < Nfq; ++j) v += (double)lc.R[b * Nfq + j] * t1[i + Nfq * (j + Nfq * c)];
          t2[i + Nfq * (b + Ncq * c)] = v;
        }
    for (int c = 0; c < Ncq; ++c)
      for (int b = 0; b < Ncq; ++b)
        for (int a = 0; a < Ncq; ++a) {
          double v = 0;
          for (int i = 0; i < Nfq; ++i) v += (double)lc.R[a * Nfq + i] * t2[i + Nfq * (b + Ncq * c)];
          qc[e * npc + a + Ncq * (b + Ncq * c)] = (T)v;
        }
  }
  }
}

// qf += (P x P x P) qc with P = R^T
template <typename T> static void prolong_apply(const MGLevel<T> &lc, const T *qc, T *qf)
{
  const int Nfq = lc.Nf + 1, Ncq = lc.L->Nq;
  const long long E = lc.L->E;
  const long long npf = (long long)Nfq * Nfq * Nfq, npc = (long long)Ncq * Ncq * Ncq;
#pragma omp parallel
  {
  std::vector<double> t1((size_t)Ncq * Ncq * Nfq), t2((size_t)Ncq * Nfq * Nfq); // per-thread scratch
#pragma omp for schedule(static)
  for (long long e = 0; e < E; ++e) {
    const T *c = qc + e * npc;
    for (int b = 0; b < Ncq; ++b)
      for (int a = 0; a < Ncq; ++a)
        for (int k = 0; k < Nfq; ++k) {
          double v = 0;
          for (int cc = 0; cc < Ncq; ++cc) v += (double)lc.R[cc * Nfq + k] * (double)c[a + Ncq * (b + Ncq * cc)];
          t1[a + Ncq * (b + Ncq * k)] = v;
        }
    for (int k = 0; k < Nfq; ++k)
      for (int j = 0; j < Nfq; ++j)
        for (int a = 0; a < Ncq; ++a) {
          double v = 0;
          for (int b = 0; b < Ncq; ++b) v += (double)lc.R[b * Nfq + j] * t1[a + Ncq * (b + Ncq * k)];
          t2[a + Ncq * (j + Nfq * k)] = v;
        }
    for (int k = 0; k < Nfq; ++k)
      for (int j = 0; j < Nfq; ++j)
        for (int i = 0; i < Nfq; ++i) {
          double v = 0;
          for (int a = 0; a < Ncq; ++a) v += (double)lc.R[a * Nfq + i] * t2[a + Ncq * (j + Nfq * k)];
          qf[e * npf + i + Nfq * (j + Nfq * k)] += (T)v;
        }
  }
  }
}

template <typename T> static void level_coarsen(MGT<T> &M, MGLevel<T> &lc, T *resFine, T *rhsC)
{
  const long long nf = (long long)lc.L->E * (lc.Nf + 1) * (lc.Nf + 1) * (lc.Nf + 1);
  for (long long i = 0; i < nf; ++i) resFine[i] = lc.invDegreeFine[i] * resFine[i];
  coarsen_apply(lc, resFine, rhsC);
  gs_add(*lc.L, rhsC);
  apply_mask(*lc.L, rhsC);
}

// ---------------------------------------------------------------------------
// coarse solve: Jacobi-PCG in precision T to a relative tolerance
// ---------------------------------------------------------------------------
template <typename T> static int coarse_pcg(MGT<T> &M, MGLevel<T> &lv, const T *b, T *x)
{
  const Level &L = *lv.L;
  const long long n = L.Nlocal;
  const T *w = lv.invDegree.data();
  T *r = M.cr.data(), *p = M.cp.data(), *z = M.cz.data(), *Ap = M.cAp.data();
  std::fill(x, x + n, T(0));
  std::memcpy(r, b, sizeof(T) * n);
  std::fill(p, p + n, T(0));
  if (M.allNeumann) {
    // all-Neumann: the assembled coarse operator annihilates constants; remove the rhs's component along
    // them (its mean over the assembled unknowns) so that the Krylov solve sees a consistent system
    double sw = 0, swb = 0;
    for (long long i = 0; i < n; ++i) {
      sw += (double)w[i];
      swb += (double)w[i] * (double)r[i];
    }
    const T mean = (T)(swb / sw);
    for (long long i = 0; i < n; ++i) r[i] -= mean;
  }
  const double r0 = std::sqrt((double)wdot<T>(n, w, r, r));
  if (r0 == 0) return 0;
  const double tol = M.o.coarseTol * r0;
  double rdotz1 = 0, rdotz2 = 0;
  int it = 0;
  double rn = r0;
  while (rn > tol && it < M.o.coarseMaxIter) {
    ++it;
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i) z[i] = lv.invDiag[i] * r[i];
    rdotz2 = rdotz1;
    rdotz1 = (double)wdot<T>(n, w, r, z);
    const double beta = (it == 1) ? 0.0 : rdotz1 / rdotz2;
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i) p[i] = z[i] + (T)beta * p[i];
    level_op(M, lv, p, Ap);
    const double pAp = (double)wdot<T>(n, w, p, Ap);
    const T alpha = (T)(rdotz1 / (pAp + 1e-300));
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i) {
      x[i] += alpha * p[i];
      r[i] -= alpha * Ap[i];
    }
    rn = std::sqrt((double)wdot<T>(n, w, r, r));
  }
  M.coarseIters.push_back(it);
  return it;
}

// coarse solve on the Galerkin matrix: the same Jacobi-PCG on its rows
// (rhs of a row = the assembled E-vector value of one of its nodes; the
// solution is scattered back to every node of the row, 0 on masked nodes)
template <typename T> static int coarse_pcg_csr(MGT<T> &M, MGLevel<T> &lv, const T *b, T *x)
{
  const long long nr = (long long)M.gRowPtr.size() - 1, n = lv.L->Nlocal;
  std::vector<T> xr(nr, 0), r(nr), p(nr, 0), z(nr), Ap(nr);
  for (long long i = 0; i < nr; ++i) r[i] = b[M.gRep[i]];
  if (M.allNeumann) {
    double sr = 0;
    for (long long i = 0; i < nr; ++i) sr += (double)r[i];
    const T mean = (T)(sr / (double)nr);
    for (long long i = 0; i < nr; ++i) r[i] -= mean;
  }
  auto dot = [&](const std::vector<T> &a, const std::vector<T> &c) {
    double s = 0;
    for (long long i = 0; i < nr; ++i) s += (double)a[i] * (double)c[i];
    return s;
  };
  const double r0 = std::sqrt(dot(r, r));
  int it = 0;
  if (r0 > 0) {
    const double tol = M.o.coarseTol * r0;
    double rdotz1 = 0, rdotz2 = 0, rn = r0;
    while (rn > tol && it < M.o.coarseMaxIter) {
      ++it;
      for (long long i = 0; i < nr; ++i) z[i] = M.gInvDiag[i] * r[i];
      rdotz2 = rdotz1;
      rdotz1 = dot(r, z);
      const double beta = (it == 1) ? 0.0 : rdotz1 / rdotz2;
      for (long long i = 0; i < nr; ++i) p[i] = z[i] + (T)beta * p[i];
      for (long long i = 0; i < nr; ++i) {
        T s = 0;
        for (long long t = M.gRowPtr[i]; t < M.gRowPtr[i + 1]; ++t) s += M.gVal[t] * p[M.gCol[t]];
        Ap[i] = s;
      }
      const T alpha = (T)(rdotz1 / (dot(p, Ap) + 1e-300));
      for (long long i = 0; i < nr; ++i) {
        xr[i] += alpha * p[i];
        r[i] -= alpha * Ap[i];
      }
      rn = std::sqrt(dot(r, r));
    }
  }
  for (long long i = 0; i < n; ++i) x[i] = M.gRowOfNode[i] < 0 ? T(0) : xr[M.gRowOfNode[i]];
  M.coarseIters.push_back(it);
  return it;
}

// ---------------------------------------------------------------------------
// V-cycle
// ---------------------------------------------------------------------------
template <typename T> static void vcycle(MGT<T> &M, int k)
{
  auto &lv = M.levels[k];
  const int base = (int)M.levels.size() - 1;
  if (k == base) {
    if (M.o.coarse == "smooth")
      smooth(M, lv, lv.rhs.data(), lv.x.data(), true);
    else if (M.o.galerkin || M.o.semfem)
      coarse_pcg_csr(M, lv, lv.rhs.data(), lv.x.data());
    else
      coarse_pcg(M, lv, lv.rhs.data(), lv.x.data());
    return;
  }
  auto &lc = M.levels[k + 1];
  smooth(M, lv, lv.rhs.data(), lv.x.data(), true);
  // residual: res = rhs - A x
  level_op(M, lv, lv.x.data(), lv.res.data());
  const long long n = lv.L->Nlocal;
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < n; ++i) lv.res[i] = (T)1 * lv.rhs[i] + (T)(-1) * lv.res[i];
  level_coarsen(M, lc, lv.res.data(), lc.rhs.data());
  vcycle(M, k + 1);
  prolong_apply(lc, lc.x.data(), lv.x.data());
  smooth(M, lv, lv.rhs.data(), lv.x.data(), false);
}

// ---------------------------------------------------------------------------
// setup
// ---------------------------------------------------------------------------
static uint64_t smix(uint64_t x)
{
  x += 0x9E3779B97F4A7C15ull;
  uint64_t z = x;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// rho(S A) by k = 10 Arnoldi steps (maxEigSmoothAx), FP64 vectors, operator and smoother in T
template <typename T> static double max_eig(MGT<T> &M, MGLevel<T> &lv, unsigned long long seed)
{
  const Level &L = *lv.L;
  const long long n = L.Nlocal;
  const int k = (int)std::min<long long>(10, n);
  // seeded start vector in [0,1), summed over the unmasked handle, masked
  std::vector<double> v(n);
  for (long long i = 0; i < n; ++i) v[i] = (double)(smix(seed ^ smix((uint64_t)i)) >> 11) * (1.0 / 9007199254740992.0);
  {
    std::vector<int> off, gid;
    std::vector<double> inv;
    ogs_setup(n, L.ids.data(), off, gid, inv);
    gs_groups(off, gid, v.data());
  }
  for (int m : L.maskIds) v[m] = 0;
  const double *w = L.invDegree.data();
  std::vector<std::vector<double>> V(k + 1, std::vector<double>(n));
  std::vector<double> H(k * k, 0.0);
  const double nv = std::sqrt(wdot<double>(n, w, v.data(), v.data()));
  for (long long i = 0; i < n; ++i) V[0][i] = 1.0 / nv * v[i];
  std::vector<T> vp(n), avp(n);
  int keff = k;
  for (int j = 0; j < k; ++j) {
    for (long long i = 0; i < n; ++i) vp[i] = (T)V[j][i];
    level_op(M, lv, vp.data(), avp.data());
    apply_S(M, lv, avp.data(), vp.data());
    for (long long i = 0; i < n; ++i) V[j + 1][i] = (double)vp[i];
    for (int i = 0; i <= j; ++i) {
      const double hij = wdot<double>(n, w, V[i].data(), V[j + 1].data());
      for (long long q = 0; q < n; ++q) V[j + 1][q] = -hij * V[i][q] + 1.0 * V[j + 1][q];
      H[i + j * k] = hij;
    }
    if (j + 1 < k) {
      const double nj = std::sqrt(wdot<double>(n, w, V[j + 1].data(), V[j + 1].data()));
      // breakdown: invariant subspace reached, keep the leading block (the
      // reference would hand NaN entries to dgeev and abort)
      if (!(nj > 1e-13 * std::fabs(H[j + j * k]))) {
        keff = j + 1;
        break;
      }
      for (long long q = 0; q < n; ++q) V[j + 1][q] *= 1.0 / nj;
      H[j + 1 + j * k] = nj;
    }
  }
  std::vector<double> Hk((size_t)keff * keff);
  for (int c = 0; c < keff; ++c)
    for (int r = 0; r < keff; ++r) Hk[r + keff * c] = H[r + k * c];
  double rho = 0;
  for (auto &ev : hessenberg_eigs(keff, Hk)) rho = std::max(rho, std::abs(ev));
  return rho;
}

template <typename T> static void build_mg(Elliptic &el, MGT<T> &M, MG &mg)
{
  const Options &o = el.o;
  M.o = o;
  M.poisson = o.poisson;
  M.allNeumann = el.allNeumann;
  M.lambda0 = (T)o.lambda0;
  M.lambda1 = (T)o.lambda1;
  // smoother family
  std::string base = "jac";
  if (o.smoother.find("ras") != std::string::npos) base = "ras";
  else if (o.smoother.find("asm") != std::string::npos) base = "asm";
  std::string kind = "cheby";
  if (o.smoother.find("fourthopt") != std::string::npos) kind = "fourthopt";
  else if (o.smoother.find("fourth") != std::string::npos) kind = "fourth";
  const int N = el.fine.N;
  std::vector<int> orders;
  Schedule S;
  const bool haveSched = !o.schedule.empty();
  if (haveSched) {
    S = parse_schedule(o.schedule, N, o.chebyDegree);
    orders = S.levels;
  } else {
    orders = default_levels(N, base != "jac");
  }
  const int nlev = (int)orders.size();
  M.levels.resize(nlev);
  for (int l = 0; l < nlev; ++l) {
    auto &lv = M.levels[l];
    if (l == 0) {
      lv.L = &el.fine;
    } else {
      lv.own.reset(new Level());
      build_level(*lv.own, orders[l], el.fine.E, el.fine.VX.data(), el.fine.EToV.data(), el.fine.EToB.data());
      lv.L = lv.own.get();
      lv.Nf = orders[l - 1];
      // R[c][f] = l_c(z_f): transpose of the coarse->fine interpolation
      const Level &Lf = *M.levels[l - 1].L;
      std::vector<double> I((size_t)Lf.Nq * lv.L->Nq);
      interp_matrix(lv.L->Nq, lv.L->z.data(), Lf.Nq, Lf.z.data(), I.data());
      lv.R.resize(I.size());
      for (int c = 0; c < lv.L->Nq; ++c)
        for (int f = 0; f < Lf.Nq; ++f) lv.R[c * Lf.Nq + f] = (T)I[f * lv.L->Nq + c];
      lv.invDegreeFine.assign(Lf.invDegree.begin(), Lf.invDegree.end());
    }
    const Level &L = *lv.L;
    lv.ggeo.assign(L.ggeo.begin(), L.ggeo.end());
    lv.D.assign(L.D.begin(), L.D.end());
    lv.invDegree.assign(L.invDegree.begin(), L.invDegree.end());
    lv.x.assign(L.Nlocal, 0);
    lv.rhs.assign(L.Nlocal, 0);
    lv.res.assign(L.Nlocal, 0);
    lv.base = base;
    lv.kind = kind;
    const bool coarsest = (l == nlev - 1);
    lv.smoothed = !coarsest || o.coarse == "smooth";
    // Jacobi diagonal (pfloat, ellipticUpdateJacobi mgLevel branch); also used by the coarse PCG
    if (base == "jac" || coarsest) {
      lv.invDiag.resize(L.Nlocal);
      build_diag<T>(L, lv.ggeo.data(), lv.D.data(), M.lambda0, M.lambda1, M.poisson, lv.invDiag.data());
      gs_add(L, lv.invDiag.data());
      for (auto &v : lv.invDiag) v = (T)1 / v;
    }
  }
  if (o.galerkin || o.semfem) {
    const Level &C = *M.levels.back().L;
    if (C.N != 1) throw std::runtime_error("the Galerkin / SEMFEM coarse operator needs an order-1 coarsest level");
    std::vector<double> vals;
    if (o.semfem)
      assemble_semfem(C, (double)M.lambda0, M.gRowPtr, M.gCol, vals);
    else
      assemble_galerkin(el.fine, C, (double)M.lambda0, (double)M.lambda1, M.poisson, M.gRowPtr, M.gCol, vals);
    const long long nr = (long long)M.gRowPtr.size() - 1;
    M.gVal.assign(vals.begin(), vals.end());
    M.gInvDiag.assign(nr, T(0));
    for (long long i = 0; i < nr; ++i)
      for (long long t = M.gRowPtr[i]; t < M.gRowPtr[i + 1]; ++t)
        if (M.gCol[t] == i) M.gInvDiag[i] = (T)(1.0 / vals[t]);
    M.gRowOfNode.assign(C.Nlocal, -1);
    M.gRep.assign(nr, 0);
    for (long long g = 0; g < nr; ++g) {
      M.gRep[g] = C.gsIds[C.gsOff[g]];
      for (int t = C.gsOff[g]; t < C.gsOff[g + 1]; ++t) M.gRowOfNode[C.gsIds[t]] = g;
    }
  }
  size_t nmax = 0;
  for (auto &lv : M.levels) nmax = std::max(nmax, (size_t)lv.L->Nlocal);
  M.sRes.assign(nmax, 0);
  M.sRes2.assign(nmax, 0);
  M.sUpd.assign(nmax, 0);
  const auto &cl = *M.levels.back().L;
  M.cp.assign(cl.Nlocal, 0);
  M.cz.assign(cl.Nlocal, 0);
  M.cAp.assign(cl.Nlocal, 0);
  M.cr.assign(cl.Nlocal, 0);
  for (int l = 0; l < nlev; ++l) {
    auto &lv = M.levels[l];
    if (!lv.smoothed) continue;
    if (lv.base != "jac") fdm_setup(lv, el.fine);
    lv.rho = max_eig(M, lv, o.seed + (unsigned long long)l);
    lv.lambda1 = o.maxEigFactor * lv.rho;
    lv.lambda0 = o.minEigFactor * lv.rho;
    const bool coarsest = (l == nlev - 1);
    lv.up = lv.down = coarsest ? 3 : o.chebyDegree;
    if (haveSched) {
      auto itU = S.deg.find({orders[l], false});
      auto itD = S.deg.find({orders[l], true});
      if (itU != S.deg.end() && itU->second > -1) lv.up = itU->second;
      if (itD != S.deg.end() && itD->second > -1) lv.down = itD->second;
    }
    if (lv.kind == "fourthopt") {
      lv.upBetas = opt_betas(lv.up);
      lv.downBetas = opt_betas(lv.down);
    } else {
      lv.upBetas.assign(std::max(lv.up, 1), 1.0);
      lv.downBetas.assign(std::max(lv.down, 1), 1.0);
    }
    mg.rho.push_back(lv.rho);
    mg.degrees.push_back(lv.down);
    mg.degrees.push_back(lv.up);
  }
  M.rP.assign(el.fine.Nlocal, 0);
  M.zP.assign(el.fine.Nlocal, 0);
}

void mg_setup(Elliptic &el)
{
  el.mg = std::make_shared<MG>();
  // "mixed" keeps the FP32 multigrid of the reference's pfloat build (the FP32-pair fine operator is a GPU
  // implementation detail of the FP64 operator)
  el.mg->fp32 = (el.o.mgPrecision == "fp32" || el.o.mgPrecision == "mixed");
  if (el.mg->fp32)
    build_mg<float>(el, el.mg->f, *el.mg);
  else
    build_mg<double>(el, el.mg->d, *el.mg);
}

template <typename T> static void run_mg(MGT<T> &M, const double *r, double *z, long long n)
{
  auto &l0 = M.levels[0];
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < n; ++i) {
    l0.rhs[i] = (T)r[i];
    l0.x[i] = 0;
  }
  vcycle(M, 0);
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < n; ++i) z[i] = (double)l0.x[i];
}

void mg_apply(Elliptic &el, const double *r, double *z)
{
  if (el.mg->fp32)
    run_mg(el.mg->f, r, z, el.fine.Nlocal);
  else
    run_mg(el.mg->d, r, z, el.fine.Nlocal);
}

std::vector<double> mg_info(const Elliptic &el, const std::string &what)
{
  std::vector<double> out;
  if (!el.mg) return out;
  if (what == "rho") return el.mg->rho;
  if (what == "levels") {
    if (el.mg->fp32)
      for (auto &lv : el.mg->f.levels) out.push_back(lv.L->N);
    else
      for (auto &lv : el.mg->d.levels) out.push_back(lv.L->N);
  }
  if (what == "coarseIters") {
    const auto &v = el.mg->fp32 ? el.mg->f.coarseIters : el.mg->d.coarseIters;
    out.assign(v.begin(), v.end());
  }
  if (what == "degrees") out.assign(el.mg->degrees.begin(), el.mg->degrees.end());
  return out;
}

// single-operator hooks for parity tests (precision of the MG)
void mg_level_smooth_schwarz(Elliptic &el, int level, const double *u, double *Su)
{
  auto go = [&](auto &M) {
    using T = typename std::decay<decltype(M.sRes)>::type::value_type;
    auto &lv = M.levels[level];
    const long long n = lv.L->Nlocal;
    std::vector<T> a(u, u + n), b(n);
    smooth_schwarz(M, lv, a.data(), b.data());
    for (long long i = 0; i < n; ++i) Su[i] = b[i];
  };
  if (el.mg->fp32) go(el.mg->f);
  else go(el.mg->d);
}

long long mg_level_size(Elliptic &el, int level)
{
  if (el.mg->fp32) return el.mg->f.levels.at(level).L->Nlocal;
  return el.mg->d.levels.at(level).L->Nlocal;
}

} // namespace orc

namespace orc {
// ---------------------------------------------------------------------------
// accessors for parity tests
// ---------------------------------------------------------------------------
std::vector<double> mg_level_array(Elliptic &el, int level, const std::string &name)
{
  std::vector<double> out;
  auto go = [&](auto &M) {
    auto &lv = M.levels.at(level);
    auto put = [&](const auto &v) { out.assign(v.begin(), v.end()); };
    if (name == "R") put(lv.R);
    else if (name == "Sx") put(lv.fdm.Sx);
    else if (name == "Sy") put(lv.fdm.Sy);
    else if (name == "Sz") put(lv.fdm.Sz);
    else if (name == "invL") put(lv.fdm.invL);
    else if (name == "wts") put(lv.fdm.wts);
    else if (name == "extOff") put(lv.fdm.extOff);
    else if (name == "extIds") put(lv.fdm.extIds);
    else if (name == "ids") put(lv.L->ids);
    else if (name == "gsOff") put(lv.L->gsOff);
    else if (name == "gsIds") put(lv.L->gsIds);
    else if (name == "maskIds") put(lv.L->maskIds);
    else if (name == "invDegree") put(lv.L->invDegree);
    else if (name == "invDiag") put(lv.invDiag);
    else if (name == "ggeo") put(lv.L->ggeo);
    else throw std::runtime_error("unknown MG array " + name);
  };
  if (el.mg->fp32) go(el.mg->f);
  else go(el.mg->d);
  return out;
}

void mg_level_transfer(Elliptic &el, int level, bool restrict_, const double *in, double *out)
{
  auto go = [&](auto &M) {
    using T = typename std::decay<decltype(M.sRes)>::type::value_type;
    auto &lc = M.levels.at(level);
    const int Nfq = lc.Nf + 1, Ncq = lc.L->Nq;
    const long long nf = lc.L->E * Nfq * Nfq * Nfq, nc = lc.L->E * Ncq * Ncq * Ncq;
    if (restrict_) {
      std::vector<T> a(in, in + nf), b(nc);
      coarsen_apply(lc, a.data(), b.data());
      for (long long i = 0; i < nc; ++i) out[i] = b[i];
    } else {
      std::vector<T> a(in, in + nc), b(out, out + nf);
      prolong_apply(lc, a.data(), b.data());
      for (long long i = 0; i < nf; ++i) out[i] = b[i];
    }
  };
  if (el.mg->fp32) go(el.mg->f);
  else go(el.mg->d);
}
} // namespace orc

namespace orc {
double hessenberg_rho_public(int n, const double *Hcol)
{
  std::vector<double> H(Hcol, Hcol + (size_t)n * n);
  double r = 0;
  for (auto &ev : hessenberg_eigs(n, H)) r = std::max(r, std::abs(ev));
  return r;
}
} // namespace orc
