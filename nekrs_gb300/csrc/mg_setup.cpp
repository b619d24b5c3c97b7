// Host-side p-multigrid setup: level schedule, FDM (Schwarz) operators,
// neighbour-halo maps, the Hessenberg eigenvalue problem of the Arnoldi
// lambda_max estimate and the assembled coarse operator.
//
// Reference behaviour (nekRS tree):
//   schedule / default levels   src/solvers/elliptic/MG/parseMultigridSchedule.cpp:7-131,
//                               src/solvers/elliptic/MG/determineMGLevels.cpp:5-98
//   element lengths             ellipticMultiGridSchwarz.cpp:58-247
//   1-D stiffness / mass / eig  ellipticMultiGridSchwarz.cpp:265-580 (LAPACK dsygv there)
//   FDM operators, invL         ellipticMultiGridSchwarz.cpp:582-663
//   extended mesh + overlap     ellipticMultiGridSchwarz.cpp:665-742 (ext. numbering,
//                               edges masked), preFDM/postFDM kernels
//   overlap weights             ellipticMultiGridSchwarz.cpp:792-834 (generate_weights)
//   lambda_max eigenvalues      ellipticMultiGridLevelSetup.cpp:260-290 (LAPACK dgeev there)
//   assembled coarse operator   ellipticBuildFEM.cpp:73-300 (ellipticBuildFEMHex3D)

#include "mg_host.hpp"

#include <algorithm>
#include <cmath>
#include <complex>
#include <map>
#include <stdexcept>

namespace nrsg {

// ---------------------------------------------------------------------------
// schedule
// ---------------------------------------------------------------------------
static std::vector<std::string> tokens(const std::string &s, char sep)
{
  std::vector<std::string> out(1);
  for (char c : s) {
    if (c == sep) out.emplace_back();
    else if (c != ' ' && c != '\t') out.back().push_back(c);
  }
  return out;
}

MGPlan plan_levels(const Options &o, int N)
{
  MGPlan P;
  P.base = o.smoother.find("ras") != std::string::npos   ? 2
           : o.smoother.find("asm") != std::string::npos ? 1
                                                         : 0;
  P.kind = o.smoother.find("fourthopt") != std::string::npos ? 2
           : o.smoother.find("fourth") != std::string::npos  ? 1
                                                             : 0;
  if (o.schedule.empty()) {
    static const int schw[10][3] = {{0}, {1}, {2, 1}, {3, 1}, {4, 2, 1}, {5, 3, 1}, {6, 3, 1}, {7, 3, 1}, {8, 5, 1}, {9, 5, 1}};
    static const int jac[10][4] = {{0},          {1},          {2, 1},       {3, 1},       {4, 2, 1},
                                   {5, 3, 1},    {6, 4, 2, 1}, {7, 5, 3, 1}, {8, 6, 4, 1}, {9, 7, 5, 1}};
    const int *row = P.base ? schw[N] : jac[N];
    const int len = P.base ? 3 : 4;
    for (int q = 0; q < len && row[q] > 0; ++q) {
      P.orders.push_back(row[q]);
      if (row[q] == 1) break;
    }
    for (int ord : P.orders) {
      P.down[ord] = o.chebyDegree;
      P.up[ord] = o.chebyDegree;
    }
    return P;
  }
  int minOrder = 1 << 30;
  const auto entries = tokens(o.schedule, ',');
  for (const auto &en : entries)
    for (const auto &tk : tokens(en, '+'))
      if (tk.rfind("p=", 0) == 0) minOrder = std::min(minOrder, std::stoi(tk.substr(2)));
  bool down = true;
  int prev = 1 << 30;
  std::map<int, int> dn, upm;
  for (const auto &en : entries) {
    int order = -1, degree = -1;
    for (const auto &tk : tokens(en, '+')) {
      if (tk.rfind("p=", 0) == 0) {
        order = std::stoi(tk.substr(2));
        if (order > prev) down = false;
        if (down) P.orders.push_back(order);
        prev = order;
      } else if (tk.rfind("degree=", 0) == 0) {
        degree = std::stoi(tk.substr(7));
      } else if (!tk.empty()) {
        throw Error(NRSG_ERR_BAD_CONFIG, "unknown token '" + tk + "' in pMGSchedule");
      }
    }
    if (order < 1) throw Error(NRSG_ERR_BAD_CONFIG, "pMGSchedule entry without a valid order: " + en);
    if (degree < 0 && order != minOrder) degree = o.chebyDegree;
    (down ? dn : upm)[order] = degree;
  }
  std::vector<int> d1, u1;
  for (auto &kv : dn)
    if (kv.first > minOrder) d1.push_back(kv.first);
  for (auto &kv : upm)
    if (kv.first > minOrder) u1.push_back(kv.first);
  if (d1 != u1) throw Error(NRSG_ERR_BAD_CONFIG, "pMGSchedule: down leg and up leg orders must be identical");
  if (P.orders.empty() || P.orders.front() != N)
    throw Error(NRSG_ERR_BAD_CONFIG, "pMGSchedule: finest order must equal the polynomial order");
  P.down = dn;
  P.up = upm;
  return P;
}

const std::vector<double> &opt4_betas(int degree)
{
  // Optimal 4th-kind Chebyshev coefficients of Lottes (arXiv:2202.08830), degrees 1..8.
  static const std::vector<double> b[9] = {
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
       1.29838585382576, 1.46486073151099}};
  if (degree < 0 || degree > 8) throw Error(NRSG_ERR_BAD_CONFIG, "fourthOptCheby degree must be 0..8");
  return b[degree];
}

// ---------------------------------------------------------------------------
// element lengths: harmonic mean of the distances across the element in
// each reference direction, weighted by GLL weights (the reference indexes
// the weights with a shift of one), from the finest mesh; neighbour lengths
// from the face neighbour (through the unmasked gather groups), falling back
// to the element's own length on domain boundaries.
// ---------------------------------------------------------------------------
static void trilinear_point(const double *v, double r, double s, double t, double X[3])
{
  const double a[2] = {0.5 * (1 - r), 0.5 * (1 + r)}, b[2] = {0.5 * (1 - s), 0.5 * (1 + s)},
               c[2] = {0.5 * (1 - t), 0.5 * (1 + t)};
  X[0] = X[1] = X[2] = 0;
  for (int q = 0; q < 8; ++q) {
    const double wq = a[q & 1] * b[(q >> 1) & 1] * c[q >> 2];
    for (int d = 0; d < 3; ++d) X[d] += wq * v[3 * q + d];
  }
}

FdmLengths fdm_lengths(const FieldLevel &F, const GatherMap &unmaskedFine)
{
  const int Nq = F.Nq, N = F.N;
  const long long E = F.E;
  FdmLengths L;
  L.mid.assign(3 * E, 0.0);
  L.left.assign(3 * E, 0.0);
  L.right.assign(3 * E, 0.0);
  const int nx = (Nq == 2) ? Nq : Nq - 1;
  const int st = (Nq == 2) ? 0 : 1;
#pragma omp parallel for
  for (long long e = 0; e < E; ++e) {
    const double *v = &F.VXh[e * 24];
    for (int dir = 0; dir < 3; ++dir) {
      double acc = 0, ws = 0;
      for (int b = st; b < nx; ++b)
        for (int a = st; a < nx; ++a) {
          const double wt = (Nq == 2) ? 1.0 : F.w[a - 1] * F.w[b - 1];
          double P0[3], P1[3];
          const double za = F.z[a], zb = F.z[b];
          if (dir == 0) { trilinear_point(v, -1, za, zb, P0); trilinear_point(v, 1, za, zb, P1); }
          else if (dir == 1) { trilinear_point(v, za, -1, zb, P0); trilinear_point(v, za, 1, zb, P1); }
          else { trilinear_point(v, za, zb, -1, P0); trilinear_point(v, za, zb, 1, P1); }
          const double d2 = (P1[0] - P0[0]) * (P1[0] - P0[0]) + (P1[1] - P0[1]) * (P1[1] - P0[1]) +
                            (P1[2] - P0[2]) * (P1[2] - P0[2]);
          acc += wt / d2;
          ws += wt;
        }
      L.mid[3 * e + dir] = 1.0 / std::sqrt(acc / ws);
    }
  }
  if (Nq == 2) {
    L.left = L.mid;
    L.right = L.mid;
    return L;
  }
  // group of each node (unmasked); a face-interior probe node has exactly one partner across the face
  std::vector<int> groupOf(F.Nlocal, -1);
  for (size_t g = 0; g + 1 < unmaskedFine.off.size(); ++g)
    for (int q = unmaskedFine.off[g]; q < unmaskedFine.off[g + 1]; ++q) groupOf[unmaskedFine.ids[q]] = (int)g;
  auto partner_elem = [&](long long node) -> long long {
    const int g = groupOf[node];
    if (g < 0) return -1;
    for (int q = unmaskedFine.off[g]; q < unmaskedFine.off[g + 1]; ++q)
      if (unmaskedFine.ids[q] != node) return unmaskedFine.ids[q] / F.Np;
    return -1;
  };
  (void)N;
  const double tol = 1e-12;
  for (long long e = 0; e < E; ++e) {
    const long long o = e * F.Np;
    // probe nodes: (0,1,1) (Nq-1,1,1) (1,0,1) (1,Nq-1,1) (1,1,0) (1,1,Nq-1)
    const long long probe[6] = {o + Nq + Nq * Nq,         o + Nq - 1 + Nq + Nq * Nq, o + 1 + Nq * Nq,
                                o + 1 + (Nq - 1) * Nq + Nq * Nq, o + 1 + Nq,      o + 1 + Nq + (long long)(Nq - 1) * Nq * Nq};
    for (int s = 0; s < 6; ++s) {
      const int dir = s / 2;
      const long long pe = partner_elem(probe[s]);
      double v = (pe >= 0) ? L.mid[3 * pe + dir] : 0.0;
      if (std::fabs(v) < tol || v < -tol) v = L.mid[3 * e + dir];
      (s % 2 ? L.right : L.left)[3 * e + dir] = v;
    }
  }
  return L;
}

// ---------------------------------------------------------------------------
// 1-D generalized eigenproblem on the extended (N+3) grid.  B is diagonal, so
// with C = B^-1/2 A B^-1/2 = Q diag(lam) Q^T the B-orthonormal eigenvectors
// are B^-1/2 Q.  C is diagonalised by cyclic Jacobi rotations.
// ---------------------------------------------------------------------------
static void sym_eig(int n, std::vector<double> &C, std::vector<double> &lam, std::vector<double> &Q)
{
  Q.assign(n * n, 0.0);
  for (int i = 0; i < n; ++i) Q[i + n * i] = 1.0;
  auto c = [&](int i, int j) -> double & { return C[i + n * j]; };
  for (int sweep = 0; sweep < 64; ++sweep) {
    double offd = 0, diag = 0;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) (i == j ? diag : offd) += c(i, j) * c(i, j);
    if (offd <= 1e-32 * diag || offd == 0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        if (c(p, q) == 0.0) continue;
        const double tau = (c(q, q) - c(p, p)) / (2 * c(p, q));
        const double t = (tau >= 0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1 + tau * tau));
        const double cs = 1 / std::sqrt(1 + t * t), sn = t * cs;
        for (int k = 0; k < n; ++k) { // columns p, q
          const double a = c(k, p), b = c(k, q);
          c(k, p) = cs * a - sn * b;
          c(k, q) = sn * a + cs * b;
        }
        for (int k = 0; k < n; ++k) { // rows p, q
          const double a = c(p, k), b = c(q, k);
          c(p, k) = cs * a - sn * b;
          c(q, k) = sn * a + cs * b;
        }
        for (int k = 0; k < n; ++k) {
          const double a = Q[k + n * p], b = Q[k + n * q];
          Q[k + n * p] = cs * a - sn * b;
          Q[k + n * q] = sn * a + cs * b;
        }
      }
  }
  lam.resize(n);
  for (int i = 0; i < n; ++i) lam[i] = c(i, i);
}

void fdm_1d_operator(const FieldLevel &L, int lbc, int rbc, double ll, double lm, double lr, std::vector<double> &S,
                     std::vector<double> &lam)
{
  const int n = L.N, nq = n + 1, nl = n + 3;
  // reference stiffness Dhat^T W Dhat
  std::vector<double> ah(nq * nq, 0.0);
  for (int j = 0; j < nq; ++j)
    for (int i = 0; i < nq; ++i) {
      double v = 0;
      for (int k = 0; k < nq; ++k) v += L.Dh[k * nq + i] * L.w[k] * L.Dh[k * nq + j];
      ah[i + nq * j] = v;
    }
  std::vector<double> A(nl * nl, 0.0), Bd(nl, 0.0);
  auto a = [&](int i, int j) -> double & { return A[i + nl * j]; };
  const int lo = (lbc == NRSG_BC_DIRICHLET) ? 1 : 0, hi = (rbc == NRSG_BC_DIRICHLET) ? n - 1 : n;
  a(1, 1) = 1.0;
  a(n + 1, n + 1) = 1.0;
  for (int j = lo; j <= hi; ++j)
    for (int i = lo; i <= hi; ++i) a(i + 1, j + 1) = (2.0 / lm) * ah[i + nq * j];
  if (lbc == 0) {
    const double f = 2.0 / ll;
    a(0, 0) = f * ah[(n - 1) + nq * (n - 1)];
    a(1, 0) = f * ah[n + nq * (n - 1)];
    a(0, 1) = f * ah[(n - 1) + nq * n];
    a(1, 1) += f * ah[n + nq * n];
  } else {
    a(0, 0) = 1.0;
  }
  if (rbc == 0) {
    const double f = 2.0 / lr;
    a(n + 1, n + 1) += f * ah[0];
    a(n + 2, n + 1) = f * ah[1];
    a(n + 1, n + 2) = f * ah[nq];
    a(n + 2, n + 2) = f * ah[1 + nq];
  } else {
    a(n + 2, n + 2) = 1.0;
  }
  Bd[1] = 1.0;
  Bd[n + 1] = 1.0;
  for (int i = lo; i <= hi; ++i) Bd[i + 1] = 0.5 * lm * L.w[i];
  if (lbc == 0) {
    Bd[0] = 0.5 * ll * L.w[n - 1];
    Bd[1] += 0.5 * ll * L.w[n];
  } else {
    Bd[0] = 1.0;
  }
  if (rbc == 0) {
    Bd[n + 1] += 0.5 * lr * L.w[0];
    Bd[n + 2] = 0.5 * lr * L.w[1];
  } else {
    Bd[n + 2] = 1.0;
  }
  std::vector<double> isq(nl), C(nl * nl), Q;
  for (int i = 0; i < nl; ++i) isq[i] = 1.0 / std::sqrt(Bd[i]);
  for (int j = 0; j < nl; ++j)
    for (int i = 0; i < nl; ++i) C[i + nl * j] = isq[i] * 0.5 * (a(i, j) + a(j, i)) * isq[j];
  sym_eig(nl, C, lam, Q);
  S.assign(nl * nl, 0.0);
  for (int c = 0; c < nl; ++c)
    for (int r = 0; r < nl; ++r) S[r + nl * c] = isq[r] * Q[r + nl * c];
  auto zero_row = [&](int r) {
    for (int c = 0; c < nl; ++c) S[r + nl * c] = 0.0;
  };
  if (lbc > 0) zero_row(0);
  if (lbc == NRSG_BC_DIRICHLET) zero_row(1);
  if (rbc > 0) zero_row(nl - 1);
  if (rbc == NRSG_BC_DIRICHLET) zero_row(nl - 2);
}

// ---------------------------------------------------------------------------
// halo maps.  The reference overlaps neighbouring elements through the
// numbering of the order N+2 "extended" mesh with element edges masked: an
// extended face-interior point is shared by exactly the two elements on that
// face.  Halo point (e, f, a, b) of element e stands for the neighbour's node
// next to the shared face; its partner is the neighbour's halo point with the
// same extended id.
// ---------------------------------------------------------------------------
static inline int halo_adj_node(int f, int a, int b, int Nq)
{
  const int N = Nq - 1;
  switch (f) {
  case 0: return 1 + Nq * (a + Nq * b);
  case 1: return (N - 1) + Nq * (a + Nq * b);
  case 2: return a + Nq * (1 + Nq * b);
  case 3: return a + Nq * ((N - 1) + Nq * b);
  case 4: return a + Nq * (b + Nq * 1);
  default: return a + Nq * (b + Nq * (N - 1));
  }
}

void fdm_halo_maps(const FieldLevel &L, std::vector<int> &haloSrc, std::vector<int> &haloPartner,
                   std::vector<double> &wts)
{
  const int Nq = L.Nq, Ne = L.N + 2, nl = Ne + 1, NF = Nq * Nq;
  const long long E = L.E, npe = (long long)nl * nl * nl;
  std::vector<long long> ext;
  nek_global_ids(Ne, E, L.EToVh.data(), ext);
  // extended id of each halo point
  const long long nh = E * 6 * NF;
  std::vector<long long> hid(nh);
  long long idmin = std::numeric_limits<long long>::max(), idmax = 0;
  for (long long e = 0; e < E; ++e)
    for (int f = 0; f < 6; ++f)
      for (int b = 0; b < Nq; ++b)
        for (int a = 0; a < Nq; ++a) {
          int i, j, k;
          switch (f) {
          case 0: i = 0; j = a + 1; k = b + 1; break;
          case 1: i = nl - 1; j = a + 1; k = b + 1; break;
          case 2: i = a + 1; j = 0; k = b + 1; break;
          case 3: i = a + 1; j = nl - 1; k = b + 1; break;
          case 4: i = a + 1; j = b + 1; k = 0; break;
          default: i = a + 1; j = b + 1; k = nl - 1; break;
          }
          const long long id = ext[e * npe + i + nl * (j + (long long)nl * k)];
          hid[(e * 6 + f) * NF + a + Nq * b] = id;
          idmin = std::min(idmin, id);
          idmax = std::max(idmax, id);
        }
  ext.clear();
  ext.shrink_to_fit();
  haloPartner.assign(nh, -1);
  haloSrc.assign(nh, -1);
  {
    std::vector<long long> first(idmax - idmin + 1, -1);
    for (long long h = 0; h < nh; ++h) {
      long long &fh = first[hid[h] - idmin];
      if (fh < 0) {
        fh = h;
      } else {
        haloPartner[h] = (int)fh;
        haloPartner[fh] = (int)h;
      }
    }
  }
  for (long long h = 0; h < nh; ++h) {
    const long long ph = haloPartner[h];
    if (ph < 0) continue;
    const long long pe = ph / (6 * NF);
    const int pf = (int)((ph / NF) % 6), pp = (int)(ph % NF);
    haloSrc[h] = (int)(pe * L.Np + halo_adj_node(pf, pp % Nq, pp / Nq, Nq));
  }
  // overlap weights: 1 / (number of subdomains covering the node), summed over shared copies
  wts.assign(L.Nlocal, 1.0);
  for (long long h = 0; h < nh; ++h)
    if (haloPartner[h] >= 0) {
      const long long e = h / (6 * NF);
      const int f = (int)((h / NF) % 6), p = (int)(h % NF);
      wts[e * L.Np + halo_adj_node(f, p % Nq, p / Nq, Nq)] += 1.0;
    }
  for (size_t g = 0; g + 1 < L.gm.off.size(); ++g) {
    const int s = L.gm.off[g], t = L.gm.off[g + 1];
    if (s + 1 == t) continue;
    double v = 0;
    for (int q = s; q < t; ++q) v += wts[L.gm.ids[q]];
    for (int q = s; q < t; ++q) wts[L.gm.ids[q]] = v;
  }
  for (auto &v : wts) v = 1.0 / v;
}

// ---------------------------------------------------------------------------
// spectral radius of a small upper-Hessenberg matrix (column-major H(i,j) =
// H[i + n*j]): Francis double-shift QR on the host.
// ---------------------------------------------------------------------------
double hessenberg_spectral_radius(int n, const std::vector<double> &Hcol)
{
  std::vector<double> h(n * n);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) h[i * n + j] = Hcol[i + n * j];
  auto H = [&](int i, int j) -> double & { return h[i * n + j]; };
  double rho = 0;
  int hi = n - 1, its = 0;
  while (hi >= 0) {
    if (hi == 0) { rho = std::max(rho, std::fabs(H(0, 0))); break; }
    int l = hi;
    for (; l > 0; --l) {
      const double s = std::fabs(H(l - 1, l - 1)) + std::fabs(H(l, l));
      if (std::fabs(H(l, l - 1)) <= 1e-14 * (s > 0 ? s : 1.0)) { H(l, l - 1) = 0; break; }
    }
    if (l == hi) { rho = std::max(rho, std::fabs(H(hi, hi))); --hi; its = 0; continue; }
    const double a = H(hi - 1, hi - 1), b = H(hi - 1, hi), c = H(hi, hi - 1), d = H(hi, hi);
    if (l == hi - 1) {
      const double tr = a + d, det = a * d - b * c, disc = tr * tr / 4 - det;
      if (disc >= 0) {
        rho = std::max(rho, std::max(std::fabs(tr / 2 + std::sqrt(disc)), std::fabs(tr / 2 - std::sqrt(disc))));
      } else {
        rho = std::max(rho, std::sqrt(std::max(det, 0.0)));
      }
      hi -= 2;
      its = 0;
      continue;
    }
    if (++its > 200) throw Error(NRSG_ERR_BREAKDOWN, "Hessenberg QR did not converge");
    // double shift: x^2 - s x + t with s = a + d, t = ad - bc (exceptional shifts every 10 steps)
    double s = a + d, t = a * d - b * c;
    if (its % 10 == 0) {
      const double w = std::fabs(H(hi, hi - 1)) + std::fabs(H(hi - 1, hi - 2));
      s = 1.5 * w;
      t = w * w;
    }
    double x = H(l, l) * H(l, l) + H(l, l + 1) * H(l + 1, l) - s * H(l, l) + t;
    double y = H(l + 1, l) * (H(l, l) + H(l + 1, l + 1) - s);
    double z = (l + 2 <= hi) ? H(l + 1, l) * H(l + 2, l + 1) : 0.0;
    for (int k = l; k <= hi - 1; ++k) {
      const int nr = (k + 2 <= hi) ? 3 : 2;
      double v[3] = {x, y, z};
      const double alpha = -std::copysign(std::sqrt(x * x + y * y + (nr == 3 ? z * z : 0.0)), x);
      v[0] -= alpha;
      double vn = v[0] * v[0] + v[1] * v[1] + (nr == 3 ? v[2] * v[2] : 0.0);
      if (vn > 0) {
        const int c0 = std::max(l, k - 1);
        for (int j = c0; j < n; ++j) {
          double sum = v[0] * H(k, j) + v[1] * H(k + 1, j) + (nr == 3 ? v[2] * H(k + 2, j) : 0.0);
          sum = 2 * sum / vn;
          H(k, j) -= sum * v[0];
          H(k + 1, j) -= sum * v[1];
          if (nr == 3) H(k + 2, j) -= sum * v[2];
        }
        const int r1 = std::min(hi, k + 3);
        for (int i = 0; i <= r1; ++i) {
          double sum = v[0] * H(i, k) + v[1] * H(i, k + 1) + (nr == 3 ? v[2] * H(i, k + 2) : 0.0);
          sum = 2 * sum / vn;
          H(i, k) -= sum * v[0];
          H(i, k + 1) -= sum * v[1];
          if (nr == 3) H(i, k + 2) -= sum * v[2];
        }
      }
      x = H(k + 1, k);
      y = (k + 2 <= hi) ? H(k + 2, k) : 0.0;
      z = (k + 3 <= hi) ? H(k + 3, k) : 0.0;
    }
  }
  return rho;
}

// ---------------------------------------------------------------------------
// Assembled level operator (the coarse-solver matrix).  The reference builds
// it in ellipticBuildFEMHex3D (src/solvers/elliptic/MG/ellipticBuildFEM.cpp:
// 73-230): per element the SEM stiffness matrix from ggeo and D, masked rows
// and columns skipped, rows and columns numbered by the masked gather groups,
// duplicates summed, exact zeros dropped.  Here each element matrix is the sum over quadrature
// points q of the outer products of the gradient stencils at q
// (A_nm = sum_q sum_ab Dg_a(q,n) G_ab(q) Dg_b(q,m), Dg_a(q,n) = D[q_a][n_a]
// where n and q agree off direction a), times lambda0, plus lambda1 JW on the
// diagonal of a Helmholtz operator.  Row r sums its members' contributions in
// ascending E-vector order, which is ascending element order: an element adds
// at most once to an entry, so the summation order is fixed.
// ---------------------------------------------------------------------------
void assemble_level(int N, long long E, const std::vector<double> &Dh, const double *ggeo, double lam0, double lam1,
                    bool poisson, const GatherMap &gm, CsrMatrix &A)
{
  const int nq = N + 1, np = nq * nq * nq, ns = 3 * nq;
  // element matrices [e][n][m]
  std::vector<double> Ae((size_t)E * np * np, 0.0);
#pragma omp parallel for schedule(static)
  for (long long e = 0; e < E; ++e) {
    double *M = &Ae[(size_t)e * np * np];
    const double *g = ggeo + (size_t)e * 7 * np;
    std::vector<int> sn(ns);
    std::vector<double> sc(ns);
    for (int k = 0; k < nq; ++k)
      for (int j = 0; j < nq; ++j)
        for (int i = 0; i < nq; ++i) {
          const int q = i + nq * (j + nq * k);
          for (int m = 0; m < nq; ++m) {
            sn[m] = m + nq * (j + nq * k);
            sc[m] = Dh[i * nq + m];
            sn[nq + m] = i + nq * (m + nq * k);
            sc[nq + m] = Dh[j * nq + m];
            sn[2 * nq + m] = i + nq * (j + nq * m);
            sc[2 * nq + m] = Dh[k * nq + m];
          }
          const double G[3][3] = {{g[0 * np + q], g[1 * np + q], g[4 * np + q]},
                                  {g[1 * np + q], g[2 * np + q], g[3 * np + q]},
                                  {g[4 * np + q], g[3 * np + q], g[5 * np + q]}};
          for (int a = 0; a < ns; ++a) {
            const double ca = sc[a];
            if (ca == 0.0) continue;
            const int na = sn[a], da = a / nq;
            for (int b = 0; b < ns; ++b) {
              const double cb = sc[b];
              if (cb == 0.0) continue;
              M[na * np + sn[b]] += lam0 * (ca * G[da][b / nq] * cb);
            }
          }
        }
    if (!poisson)
      for (int n = 0; n < np; ++n) M[n * np + n] += lam1 * g[6 * np + n];
  }
  assemble_rows(np, E, Ae, gm, A);
}

// Element matrices M[e][m][n] (row m, column n) into the CSR operator whose
// rows are the masked gather groups; masked rows / columns and exact zeros
// are dropped, duplicates summed in element order.
void assemble_rows(int np, long long E, const std::vector<double> &Ae, const GatherMap &gm, CsrMatrix &A)
{
  const long long nloc = E * np;
  A.nrow = (long long)gm.off.size() - 1;
  A.rowOfNode.assign(nloc, -1);
  for (long long g = 0; g < A.nrow; ++g)
    for (int q = gm.off[g]; q < gm.off[g + 1]; ++q) A.rowOfNode[gm.ids[q]] = g;
  // rows: members in ascending E-vector order, then element columns
  std::vector<std::vector<std::pair<long long, double>>> rows(A.nrow);
#pragma omp parallel for schedule(dynamic, 256)
  for (long long r = 0; r < A.nrow; ++r) {
    auto &row = rows[r];
    for (int q = gm.off[r]; q < gm.off[r + 1]; ++q) {
      const long long i = gm.ids[q], e = i / np;
      const int n = (int)(i % np);
      const double *M = &Ae[(size_t)e * np * np + (size_t)n * np];
      for (int m = 0; m < np; ++m) {
        const long long c = A.rowOfNode[e * np + m];
        if (c < 0 || M[m] == 0.0) continue; // masked column, or an exact zero (dropped as the reference does)
        size_t t = 0;
        while (t < row.size() && row[t].first != c) ++t;
        if (t == row.size()) row.push_back({c, 0.0});
        row[t].second += M[m];
      }
    }
    std::sort(row.begin(), row.end(), [](const auto &x, const auto &y) { return x.first < y.first; });
  }
  A.rowPtr.assign(A.nrow + 1, 0);
  for (long long r = 0; r < A.nrow; ++r) A.rowPtr[r + 1] = A.rowPtr[r] + (long long)rows[r].size();
  A.col.resize(A.rowPtr[A.nrow]);
  A.val.resize(A.rowPtr[A.nrow]);
  for (long long r = 0; r < A.nrow; ++r)
    for (size_t t = 0; t < rows[r].size(); ++t) {
      A.col[A.rowPtr[r] + t] = rows[r][t].first;
      A.val[A.rowPtr[r] + t] = rows[r][t].second;
    }
}

// Galerkin coarse operator (ellipticBuildFEMGalerkinHex3D,
// src/solvers/elliptic/MG/ellipticBuildFEM.cpp:384-520): per element, the
// fine-level FP32 operator applied to each trilinear basis function sampled
// at the fine GLL nodes (ellipticGenerateCoarseBasisHex3D :344-382; the
// reference runs its pfloat ellipticAx on all elements at once), projected
// on every basis function in FP64: M[e][m][n] = sum_k (double)(A_f b_n)_k b_m(k).
// The FP32 operator follows the serial ellipticPartialAxCoeffHex3D order.
void galerkin_element_matrices(int Nf, long long E, const std::vector<double> &Dh, const std::vector<double> &z,
                               const double *ggeo, double lam0, double lam1, bool poisson, std::vector<double> &Ae)
{
  const int nq = Nf + 1, np = nq * nq * nq;
  std::vector<double> b((size_t)8 * np);
  for (int c = 0; c < 8; ++c)
    for (int k = 0; k < nq; ++k)
      for (int j = 0; j < nq; ++j)
        for (int i = 0; i < nq; ++i) {
          const double zr = (c & 1) ? 0.5 * (1 + z[i]) : 0.5 * (1 - z[i]);
          const double zs = (c & 2) ? 0.5 * (1 + z[j]) : 0.5 * (1 - z[j]);
          const double zt = (c & 4) ? 0.5 * (1 + z[k]) : 0.5 * (1 - z[k]);
          b[(size_t)c * np + i + nq * (j + nq * k)] = zr * zs * zt;
        }
  std::vector<float> D32(Dh.begin(), Dh.end());
  Ae.assign((size_t)E * 64, 0.0);
  const float l0 = (float)lam0, l1 = (float)lam1;
#pragma omp parallel for schedule(static)
  for (long long e = 0; e < E; ++e) {
    std::vector<float> g32((size_t)7 * np), q(np), Aq(np), Gr(np), Gs(np), Gt(np);
    for (size_t t = 0; t < g32.size(); ++t) g32[t] = (float)ggeo[(size_t)e * 7 * np + t];
    for (int c = 0; c < 8; ++c) {
      for (int t = 0; t < np; ++t) q[t] = (float)b[(size_t)c * np + t];
      for (int k = 0; k < nq; ++k)
        for (int j = 0; j < nq; ++j)
          for (int i = 0; i < nq; ++i) {
            const int n = i + nq * (j + nq * k);
            float qr = 0, qs = 0, qt = 0;
            for (int m = 0; m < nq; ++m) {
              qr += D32[i * nq + m] * q[m + nq * (j + nq * k)];
              qs += D32[j * nq + m] * q[i + nq * (m + nq * k)];
              qt += D32[k * nq + m] * q[i + nq * (j + nq * m)];
            }
            const float G00 = g32[0 * np + n], G01 = g32[1 * np + n], G11 = g32[2 * np + n];
            const float G12 = g32[3 * np + n], G02 = g32[4 * np + n], G22 = g32[5 * np + n];
            float a = G00 * qr;
            a += G01 * qs;
            a += G02 * qt;
            float bb = G01 * qr;
            bb += G11 * qs;
            bb += G12 * qt;
            float cc = G02 * qr;
            cc += G12 * qs;
            cc += G22 * qt;
            Gr[n] = l0 * a;
            Gs[n] = l0 * bb;
            Gt[n] = l0 * cc;
          }
      for (int k = 0; k < nq; ++k)
        for (int j = 0; j < nq; ++j)
          for (int i = 0; i < nq; ++i) {
            const int n = i + nq * (j + nq * k);
            const float r0 = poisson ? 0.f : g32[6 * np + n] * l1 * q[n];
            float ar = 0, as = 0, at = 0;
            for (int m = 0; m < nq; ++m) {
              ar += D32[m * nq + i] * Gr[m + nq * (j + nq * k)];
              as += D32[m * nq + j] * Gs[i + nq * (m + nq * k)];
              at += D32[m * nq + k] * Gt[i + nq * (j + nq * m)];
            }
            Aq[n] = ar + as + at + r0;
          }
      for (int m = 0; m < 8; ++m) {
        double val = 0;
        for (int t = 0; t < np; ++t) val += (double)Aq[t] * b[(size_t)m * np + t];
        Ae[(size_t)e * 64 + m * 8 + c] = val;
      }
    }
  }
}

// SEMFEM operator (SEMFEMSolver_t::build, src/solvers/elliptic/
// SEMFEMSolverBuild.cpp:218-335 with fem_assembly_host :551-700): the
// linear-tetrahedron Poisson stiffness on the level's GLL sub-grid. Every
// sub-hexahedron of every element is covered by its eight corner tetrahedra
// (mesh_connectivity :859-940: each corner and its three edge neighbours), each
// integrated with the 4-point rule of weight 1/24 (:12-34) using the signed
// Jacobian determinant of the corner map; lambda0 scales everything (the
// reference takes the first entry of its coefficient, no mass term). Entries
// between unmasked nodes accumulate in FP32 in the reference's loop order
// (element, sub-hex z / y / x, tetrahedron, i, j); rows are the level's masked
// gather groups.
void semfem_assemble(int N, long long E, const double *x, const double *y, const double *z, const GatherMap &gm,
                     const std::vector<int> &maskIds, double lam0, CsrMatrix &A)
{
  const int nq = N + 1, np = nq * nq * nq;
  static const int vc[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0}, {0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
  static const int tm[8][4] = {{0, 2, 1, 4}, {1, 0, 3, 5}, {2, 6, 3, 0}, {3, 2, 7, 1},
                               {4, 5, 6, 0}, {5, 7, 4, 1}, {6, 7, 2, 4}, {7, 3, 6, 5}};
  static const double dphi[4][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {-1, -1, -1}};
  A.nrow = (long long)gm.off.size() - 1;
  A.rowOfNode.assign((size_t)E * np, -1);
  for (long long g = 0; g < A.nrow; ++g)
    for (int q = gm.off[g]; q < gm.off[g + 1]; ++q) A.rowOfNode[gm.ids[q]] = g;
  // element-interior nodes carry no global id (they are gathered with nothing) but are unknowns of the
  // SEMFEM system (the reference numbers every unmasked node): one row each, after the shared rows
  std::vector<char> masked((size_t)E * np, 0);
  for (int m : maskIds) masked[m] = 1;
  for (long long i = 0; i < E * np; ++i)
    if (A.rowOfNode[i] < 0 && !masked[i]) A.rowOfNode[i] = A.nrow++;
  std::vector<std::vector<std::pair<long long, float>>> rows(A.nrow);
  for (long long e = 0; e < E; ++e)
    for (int sz = 0; sz < nq - 1; ++sz)
      for (int sy = 0; sy < nq - 1; ++sy)
        for (int sx = 0; sx < nq - 1; ++sx) {
          int idx[8];
          for (int v = 0; v < 8; ++v) idx[v] = (sx + vc[v][0]) + (sy + vc[v][1]) * nq + (sz + vc[v][2]) * nq * nq;
          for (int t = 0; t < 8; ++t) {
            double xt[3][4];
            for (int k = 0; k < 4; ++k) {
              const long long node = e * np + idx[tm[t][k]];
              xt[0][k] = x[node];
              xt[1][k] = y[node];
              xt[2][k] = z[node];
            }
            double J[3][3];
            for (int a = 0; a < 3; ++a)
              for (int b = 0; b < 3; ++b) {
                J[a][b] = 0.0;
                for (int k = 0; k < 4; ++k) J[a][b] += xt[a][k] * dphi[k][b];
              }
            const double det = J[0][0] * (J[1][1] * J[2][2] - J[2][1] * J[1][2]) -
                               J[0][1] * (J[1][0] * J[2][2] - J[2][0] * J[1][2]) +
                               J[0][2] * (J[1][0] * J[2][1] - J[2][0] * J[1][1]);
            const double id = 1.0 / det;
            double Ji[3][3];
            Ji[0][0] = id * (J[1][1] * J[2][2] - J[2][1] * J[1][2]);
            Ji[0][1] = id * (J[0][2] * J[2][1] - J[2][2] * J[0][1]);
            Ji[0][2] = id * (J[0][1] * J[1][2] - J[1][1] * J[0][2]);
            Ji[1][0] = id * (J[1][2] * J[2][0] - J[2][2] * J[1][0]);
            Ji[1][1] = id * (J[0][0] * J[2][2] - J[2][0] * J[0][2]);
            Ji[1][2] = id * (J[0][2] * J[1][0] - J[1][2] * J[0][0]);
            Ji[2][0] = id * (J[1][0] * J[2][1] - J[2][0] * J[1][1]);
            Ji[2][1] = id * (J[0][1] * J[2][0] - J[2][1] * J[0][0]);
            Ji[2][2] = id * (J[0][0] * J[1][1] - J[1][0] * J[0][1]);
            // the integrand is constant on a tetrahedron: each of the 4 points adds the same term
            double Al[4][4] = {};
            for (int q = 0; q < 4; ++q)
              for (int i = 0; i < 4; ++i)
                for (int j = 0; j < 4; ++j) {
                  double f = 0.0;
                  for (int al = 0; al < 3; ++al) {
                    double a = 0.0, b = 0.0;
                    for (int be = 0; be < 3; ++be) {
                      a += dphi[i][be] * Ji[be][al];
                      b += dphi[j][be] * Ji[be][al];
                    }
                    f += a * b;
                  }
                  Al[i][j] += f * det * (1.0 / 24.0);
                }
            for (int i = 0; i < 4; ++i)
              for (int j = 0; j < 4; ++j) {
                const long long r = A.rowOfNode[e * np + idx[tm[t][i]]], c = A.rowOfNode[e * np + idx[tm[t][j]]];
                if (r < 0 || c < 0) continue;
                auto &row = rows[r];
                size_t k = 0;
                while (k < row.size() && row[k].first != c) ++k;
                if (k == row.size()) row.push_back({c, 0.0f});
                row[k].second += lam0 * Al[i][j];
              }
          }
        }
  A.rowPtr.assign(A.nrow + 1, 0);
  for (long long r = 0; r < A.nrow; ++r) {
    auto &row = rows[r];
    std::sort(row.begin(), row.end(), [](const auto &a, const auto &b) { return a.first < b.first; });
    long long kept = 0;
    for (auto &p : row) kept += std::fabs((double)p.second) > 0.0;
    A.rowPtr[r + 1] = A.rowPtr[r] + kept;
  }
  A.col.resize(A.rowPtr[A.nrow]);
  A.val.resize(A.rowPtr[A.nrow]);
  for (long long r = 0; r < A.nrow; ++r) {
    long long t = A.rowPtr[r];
    for (auto &p : rows[r])
      if (std::fabs((double)p.second) > 0.0) {
        A.col[t] = p.first;
        A.val[t] = p.second;
        ++t;
      }
  }
}

} // namespace nrsg
