// Host-side setup of the elliptic solve: 1-D basis, Nek5000 global
// numbering, gather maps, Dirichlet mask and the options parser.
//
// Reference behaviour followed (files relative to the nekRS tree):
//   GLL nodes / weights, D, interpolation   src/mesh/meshBasis1D.cpp:99-153,249-280
//   global numbering                        3rd_party/nek5000/core/navier8.f:2004-2350 (setvert3d)
//   gather maps / invDegree                 3rd_party/gslib/ogs/src/ogsSetup.cpp:111-397
//   Dirichlet mask                          src/solvers/elliptic/ellipticOgs.cpp:4-134
//   .par keys                               src/setup/parReader.cpp, doc/parHelp.txt:80-120

#include "nrsg_internal.hpp"

#include <algorithm>
#include <array>
#include <cctype>
#include <cmath>
#include <cstring>
#include <numeric>
#include <sstream>

namespace nrsg {

// ---------------------------------------------------------------------------
// 1-D basis: GLL nodes are the roots of (1-x^2) P_N'(x), found by Newton
// iteration from Chebyshev-Lobatto guesses; weights 2/(N(N+1) P_N^2).
// ---------------------------------------------------------------------------
static void legendre_pair(int n, double x, double &pn, double &pnm1)
{
  double a = 1.0, b = x;
  if (n == 0) { pn = 1.0; pnm1 = 0.0; return; }
  for (int k = 2; k <= n; ++k) {
    const double c = ((2 * k - 1) * x * b - (k - 1) * a) / k;
    a = b;
    b = c;
  }
  pn = b;
  pnm1 = a;
}

void gll_nodes(int N, std::vector<double> &z, std::vector<double> &w)
{
  z.assign(N + 1, 0.0);
  w.assign(N + 1, 0.0);
  z[0] = -1.0;
  z[N] = 1.0;
  for (int i = 1; i <= N / 2; ++i) {
    double x = -std::cos(M_PI * i / N);
    for (int it = 0; it < 64; ++it) {
      double pn, pm;
      legendre_pair(N, x, pn, pm);
      // P_N'(x) = N (P_{N-1} - x P_N)/(1-x^2); Newton on f = P_{N-1} - x P_N
      const double f = pm - x * pn;
      // f' = P'_{N-1} - P_N - x P'_N  evaluated through the identity f' = -(N+1) P_N
      const double df = -(N + 1.0) * pn;
      const double dx = f / df;
      x -= dx;
      if (std::fabs(dx) < 1e-17) break;
    }
    z[i] = x;
    z[N - i] = -x;
  }
  if (N % 2 == 0) z[N / 2] = 0.0;
  for (int i = 0; i <= N; ++i) {
    double pn, pm;
    legendre_pair(N, z[i], pn, pm);
    w[i] = 2.0 / (N * (N + 1.0) * pn * pn);
  }
}

void diff_matrix(const std::vector<double> &z, std::vector<double> &D)
{
  const int n = (int)z.size();
  std::vector<double> c(n, 1.0);
  for (int j = 0; j < n; ++j)
    for (int k = 0; k < n; ++k)
      if (k != j) c[j] *= (z[j] - z[k]);
  D.assign(n * n, 0.0);
  for (int i = 0; i < n; ++i) {
    double s = 0;
    for (int j = 0; j < n; ++j) {
      if (j == i) continue;
      D[i * n + j] = c[i] / (c[j] * (z[i] - z[j]));
      s += D[i * n + j];
    }
    D[i * n + i] = -s; // rows of D annihilate constants exactly
  }
}

void lagrange_interp(const std::vector<double> &zin, const std::vector<double> &zout, std::vector<double> &I)
{
  const int ni = (int)zin.size(), no = (int)zout.size();
  I.assign(no * ni, 0.0);
  for (int o = 0; o < no; ++o)
    for (int j = 0; j < ni; ++j) {
      double v = 1.0;
      for (int k = 0; k < ni; ++k)
        if (k != j) v *= (zout[o] - zin[k]) / (zin[j] - zin[k]);
      I[o * ni + j] = v;
    }
}

void trilinear_nodes(int N, long long E, const double *VX, const std::vector<double> &z1, std::vector<double> &x,
                     std::vector<double> &y, std::vector<double> &zz)
{
  const int nq = N + 1;
  const long long np = (long long)nq * nq * nq;
  x.resize(E * np);
  y.resize(E * np);
  zz.resize(E * np);
#pragma omp parallel for
  for (long long e = 0; e < E; ++e) {
    const double *v = VX + e * 24;
    for (int k = 0; k < nq; ++k)
      for (int j = 0; j < nq; ++j)
        for (int i = 0; i < nq; ++i) {
          const double a[2] = {0.5 * (1 - z1[i]), 0.5 * (1 + z1[i])};
          const double b[2] = {0.5 * (1 - z1[j]), 0.5 * (1 + z1[j])};
          const double c[2] = {0.5 * (1 - z1[k]), 0.5 * (1 + z1[k])};
          double X[3] = {0, 0, 0};
          for (int q = 0; q < 8; ++q) {
            const double wq = a[q & 1] * b[(q >> 1) & 1] * c[q >> 2];
            for (int d = 0; d < 3; ++d) X[d] += wq * v[q * 3 + d];
          }
          const long long id = e * np + i + nq * (j + nq * k);
          x[id] = X[0];
          y[id] = X[1];
          zz[id] = X[2];
        }
  }
}

// ---------------------------------------------------------------------------
// Nek5000 numbering (setvert3d with ifcenter = false): corners carry the
// vertex ids; the n-2 interior nodes of each unique edge and the (n-2)^2
// interior nodes of each unique face get consecutive ids after the vertices,
// edges and faces being ranked lexicographically by their sorted vertex
// tuples; each edge / face is traversed from its smallest vertex id exactly
// as setvert3d does, so shared nodes receive identical ids.  Element
// interiors stay 0 (they take no part in the gather-scatter).
// ---------------------------------------------------------------------------
namespace {
struct EdgeKey {
  long long a, b;
  bool operator<(const EdgeKey &o) const { return a < o.a || (a == o.a && b < o.b); }
  bool operator==(const EdgeKey &o) const { return a == o.a && b == o.b; }
};
struct FaceKey {
  long long a, b, c;
  bool operator<(const FaceKey &o) const
  {
    if (a != o.a) return a < o.a;
    if (b != o.b) return b < o.b;
    return c < o.c;
  }
  bool operator==(const FaceKey &o) const { return a == o.a && b == o.b && c == o.c; }
};
template <typename K> std::vector<long long> dense_rank(const std::vector<K> &keys, long long &nunique)
{
  std::vector<long long> idx(keys.size());
  std::iota(idx.begin(), idx.end(), 0);
  std::sort(idx.begin(), idx.end(), [&](long long u, long long v) { return keys[u] < keys[v]; });
  std::vector<long long> rank(keys.size());
  long long r = 0;
  for (size_t q = 0; q < idx.size(); ++q) {
    if (q == 0 || !(keys[idx[q]] == keys[idx[q - 1]])) ++r;
    rank[idx[q]] = r; // 1-based
  }
  nunique = r;
  return rank;
}
} // namespace

void nek_global_ids(int N, long long E, const long long *EToV, std::vector<long long> &ids)
{
  const int n = N + 1;
  const long long np = (long long)n * n * n;
  ids.assign(E * np, 0);
  auto at = [&](long long e, int i, int j, int k) -> long long & { return ids[e * np + i + n * (j + (long long)n * k)]; };
  long long vmax = 0;
  for (long long q = 0; q < 8 * E; ++q) vmax = std::max(vmax, EToV[q]);
  const int L = n - 1;
  for (long long e = 0; e < E; ++e)
    for (int v = 0; v < 8; ++v) at(e, (v & 1) * L, ((v >> 1) & 1) * L, (v >> 2) * L) = EToV[8 * e + v];
  if (n == 2) return;
  long long base = vmax;

  // 12 edges per element: 4 along r (varying j,k), 4 along s (varying i,k), 4 along t (varying i,j)
  // edge e*12+q: start corner and direction
  struct EdgeDef { int v0, v1, dir; };
  static const EdgeDef edef[12] = {{0, 1, 0}, {2, 3, 0}, {4, 5, 0}, {6, 7, 0}, {0, 2, 1}, {1, 3, 1},
                                   {4, 6, 1}, {5, 7, 1}, {0, 4, 2}, {1, 5, 2}, {2, 6, 2}, {3, 7, 2}};
  std::vector<EdgeKey> ek(12 * E);
  for (long long e = 0; e < E; ++e)
    for (int q = 0; q < 12; ++q) {
      long long a = EToV[8 * e + edef[q].v0], b = EToV[8 * e + edef[q].v1];
      ek[12 * e + q] = {std::min(a, b), std::max(a, b)};
    }
  long long nEdges = 0;
  std::vector<long long> erank = dense_rank(ek, nEdges);
  const long long ne = n - 2;
#pragma omp parallel for
  for (long long e = 0; e < E; ++e)
    for (int q = 0; q < 12; ++q) {
      const int v0 = edef[q].v0;
      const int i0 = (v0 & 1) * L, j0 = ((v0 >> 1) & 1) * L, k0 = (v0 >> 2) * L;
      const long long first = base + ne * (erank[12 * e + q] - 1);
      const bool forward = EToV[8 * e + edef[q].v0] < EToV[8 * e + edef[q].v1];
      for (int s = 1; s <= n - 2; ++s) {
        const long long id = forward ? first + s : first + 1 + ne - s;
        if (edef[q].dir == 0) at(e, s, j0, k0) = id;
        else if (edef[q].dir == 1) at(e, i0, s, k0) = id;
        else at(e, i0, j0, s) = id;
      }
    }
  base += nEdges * ne;

  // 6 faces per element in Nek's symmetric order x-, x+, y-, y+, z-, z+;
  // (p,q) run over the face with p the first and q the second in-plane axis.
  static const int fcorner[6][4] = {{0, 2, 4, 6}, {1, 3, 5, 7}, {0, 1, 4, 5}, {2, 3, 6, 7}, {0, 1, 2, 3}, {4, 5, 6, 7}};
  std::vector<FaceKey> fk(6 * E);
  for (long long e = 0; e < E; ++e)
    for (int f = 0; f < 6; ++f) {
      std::array<long long, 4> c;
      for (int q = 0; q < 4; ++q) c[q] = EToV[8 * e + fcorner[f][q]];
      std::sort(c.begin(), c.end());
      fk[6 * e + f] = {c[0], c[1], c[2]};
    }
  long long nFaces = 0;
  std::vector<long long> frank = dense_rank(fk, nFaces);
  const long long nf = (long long)(n - 2) * (n - 2);
#pragma omp parallel for
  for (long long e = 0; e < E; ++e)
    for (int f = 0; f < 6; ++f) {
      auto node = [&](int p, int q) -> long long & {
        switch (f) {
        case 0: return at(e, 0, p, q);
        case 1: return at(e, L, p, q);
        case 2: return at(e, p, 0, q);
        case 3: return at(e, p, L, q);
        case 4: return at(e, p, q, 0);
        default: return at(e, p, q, L);
        }
      };
      const long long c00 = node(0, 0), c10 = node(L, 0), c01 = node(0, L), c11 = node(L, L);
      // start at the smallest corner; walk first towards the smaller of its two neighbours
      int ps = 1, qs = 1;
      bool pFast;
      const long long m = std::min(std::min(c00, c10), std::min(c01, c11));
      if (m == c00) { pFast = c10 < c01; }
      else if (m == c10) { ps = -1; pFast = c00 < c11; }
      else if (m == c01) { qs = -1; pFast = c11 < c00; }
      else { ps = -1; qs = -1; pFast = c01 < c10; }
      const long long first = base + nf * (frank[6 * e + f] - 1);
      long long cnt = 0;
      for (int outer = 1; outer < n - 1; ++outer)
        for (int inner = 1; inner < n - 1; ++inner) {
          const int a = pFast ? inner : outer; // position along p
          const int b = pFast ? outer : inner; // position along q
          const int p = ps > 0 ? a : L - a;
          const int q = qs > 0 ? b : L - b;
          node(p, q) = first + (++cnt);
        }
    }
}

// ---------------------------------------------------------------------------
// Gather maps by counting sort: O(N).  Groups are ordered by their smallest
// local index and list members in ascending local order, which is the CSR
// ogsSetup produces for one rank; a group's sum therefore runs in the same
// order as the reference kernel.
// ---------------------------------------------------------------------------
void build_gather(const std::vector<long long> &ids, GatherMap &gm)
{
  const long long n = (long long)ids.size();
  long long maxId = 0;
  for (long long v : ids) maxId = std::max(maxId, std::llabs(v));
  std::vector<int> groupOfId(maxId + 1, -1);
  std::vector<int> count;
  std::vector<int> groupOfNode(n, -1);
  for (long long i = 0; i < n; ++i) {
    const long long id = std::llabs(ids[i]);
    if (id == 0) continue;
    int &g = groupOfId[id];
    if (g < 0) { g = (int)count.size(); count.push_back(0); }
    groupOfNode[i] = g;
    count[g]++;
  }
  const size_t ng = count.size();
  gm.off.assign(ng + 1, 0);
  for (size_t g = 0; g < ng; ++g) gm.off[g + 1] = gm.off[g] + count[g];
  gm.ids.assign(gm.off[ng], 0);
  std::vector<int> fill(gm.off.begin(), gm.off.end() - 1);
  for (long long i = 0; i < n; ++i)
    if (groupOfNode[i] >= 0) gm.ids[fill[groupOfNode[i]]++] = (int)i;
  gm.invDegree.assign(n, 1.0);
  gm.devOff.clear();
  gm.devIds.clear();
  gm.devOff.push_back(0);
  for (size_t g = 0; g < ng; ++g) {
    const int m = gm.off[g + 1] - gm.off[g];
    for (int q = gm.off[g]; q < gm.off[g + 1]; ++q) gm.invDegree[gm.ids[q]] = 1.0 / m;
    if (m >= 2) {
      for (int q = gm.off[g]; q < gm.off[g + 1]; ++q) gm.devIds.push_back(gm.ids[q]);
      gm.devOff.push_back((int)gm.devIds.size());
    }
  }
}

void dirichlet_nodes(int N, long long E, const int *EToB, const GatherMap &um, std::vector<int> &maskIds)
{
  const int n = N + 1;
  const long long np = (long long)n * n * n;
  const int none = 1 << 20;
  std::vector<int> flag(E * np, none);
  for (long long e = 0; e < E; ++e)
    for (int f = 0; f < 6; ++f) {
      const int bc = EToB[6 * e + f];
      if (bc <= 0) continue;
      for (int b = 0; b < n; ++b)
        for (int a = 0; a < n; ++a) {
          // nekRS face order: t-, s-, r+, s+, r-, t+
          int i = a, j = b, k = 0;
          if (f == 1) { i = a; j = 0; k = b; }
          else if (f == 2) { i = n - 1; j = a; k = b; }
          else if (f == 3) { i = a; j = n - 1; k = b; }
          else if (f == 4) { i = 0; j = a; k = b; }
          else if (f == 5) { i = a; j = b; k = n - 1; }
          int &v = flag[e * np + i + n * (j + (long long)n * k)];
          v = std::min(v, bc);
        }
    }
  for (size_t g = 0; g + 1 < um.off.size(); ++g) {
    int v = none;
    for (int q = um.off[g]; q < um.off[g + 1]; ++q) v = std::min(v, flag[um.ids[q]]);
    for (int q = um.off[g]; q < um.off[g + 1]; ++q) flag[um.ids[q]] = v;
  }
  maskIds.clear();
  for (long long i = 0; i < E * np; ++i)
    if (flag[i] == NRSG_BC_DIRICHLET) maskIds.push_back((int)i);
}

// ---------------------------------------------------------------------------
// Options
// ---------------------------------------------------------------------------
static std::string lc(std::string s)
{
  for (auto &c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}
static std::string strip(const std::string &s)
{
  const auto a = s.find_first_not_of(" \t\r\n");
  if (a == std::string::npos) return "";
  const auto b = s.find_last_not_of(" \t\r\n");
  return s.substr(a, b - a + 1);
}

Options parse_options(const char *text)
{
  Options o;
  bool axSet = false;
  std::string t = text ? text : "";
  std::replace(t.begin(), t.end(), ';', '\n');
  std::istringstream in(t);
  std::string line;
  while (std::getline(in, line)) {
    const auto hash = line.find('#');
    if (hash != std::string::npos) line = line.substr(0, hash);
    const auto eq = line.find('=');
    if (eq == std::string::npos) continue;
    const std::string key = lc(strip(line.substr(0, eq)));
    const std::string v = lc(strip(line.substr(eq + 1)));
    try {
      if (key == "solver") {
        const std::string head = v.substr(0, v.find('+'));
        const bool flex = v.find("flexible") != std::string::npos;
        if (head == "pcg") o.solver = flex ? "pfcg" : "pcg";
        else if (head == "pfcg" || head == "fcg") o.solver = "pfcg";
        else if (head == "pgmres" || head == "gmres") o.solver = flex ? "pfgmres" : "pgmres";
        else if (head == "pfgmres" || head == "fgmres") o.solver = "pfgmres";
        else throw Error(NRSG_ERR_BAD_CONFIG, "unknown solver '" + v + "'");
        const auto p = v.find("nvector=");
        if (p != std::string::npos) o.nVector = std::stoi(v.substr(p + 8));
        if (v.find("block") != std::string::npos) o.nfields = 3;
      } else if (key == "residualtol") {
        o.tol = std::stod(v.substr(0, v.find('+')));
        o.relative = v.find("relative") != std::string::npos;
      } else if (key == "relative") o.relative = std::stoi(v) != 0;
      else if (key == "maxiterations") o.maxIter = std::stoi(v);
      else if (key == "preconditioner") {
        if (v != "none" && v != "jacobi" && v != "multigrid" && v != "semfem")
          throw Error(NRSG_ERR_BAD_CONFIG, "unknown preconditioner '" + v + "'");
        o.precon = v;
      } else if (key == "smoothertype") o.smoother = v;
      else if (key == "chebyshevdegree") o.chebyDegree = std::stoi(v);
      else if (key == "mineigenvalueboundfactor") o.minEigFactor = std::stod(v);
      else if (key == "maxeigenvalueboundfactor") o.maxEigFactor = std::stod(v);
      else if (key == "pmgschedule") o.schedule = v;
      else if (key == "coarsesolver") {
        if (v != "jpcg" && v != "smooth" && v != "amg")
          throw Error(NRSG_ERR_BAD_CONFIG, "coarseSolver must be jpcg, amg or smooth");
        o.coarse = v;
      }
      else if (key == "amgiterations") {
        o.amgIterations = std::stoi(v);
        if (o.amgIterations < 1 || o.amgIterations > 16) throw Error(NRSG_ERR_BAD_CONFIG, "amgIterations must be 1..16");
      }
      else if (key == "coarsegriddiscretization") {
        o.galerkin = (v == "fem+galerkin" || v == "galerkin");
        o.semfem = (v == "semfem");
        if (!o.galerkin && !o.semfem && v != "fem")
          throw Error(NRSG_ERR_BAD_CONFIG, "coarseGridDiscretization '" + v + "' (fem | fem+galerkin | semfem)");
      } else if (key == "galerkincoarseoperator") o.galerkin = (v == "true" || v == "1" || v == "yes");
      else if (key == "coarsetol") o.coarseTol = std::stod(v);
      else if (key == "coarsemaxiterations") o.coarseMaxIter = std::stoi(v);
      else if (key == "coarsepersistent") o.coarsePersistent = std::stoi(v) != 0;
      else if (key == "coarsespinlimit") {
        o.coarseSpinLimit = std::stoll(v);
        if (o.coarseSpinLimit < 64) throw Error(NRSG_ERR_BAD_CONFIG, "coarseSpinLimit must be >= 64");
      }
      else if (key == "coarsebarrierextra") {
        o.coarseBarrierExtra = std::stoi(v);
        if (o.coarseBarrierExtra < 0) throw Error(NRSG_ERR_BAD_CONFIG, "coarseBarrierExtra must be >= 0");
      }
      else if (key == "cudagraphs") o.graphs = std::stoi(v) != 0;
      else if (key == "axpipeline") o.axPipeline = std::stoi(v) != 0;
      else if (key == "axconst") o.axConst = std::stoi(v) != 0;
      else if (key == "nfields") o.nfields = std::stoi(v);
      else if (key == "stressformulation") o.stress = (v == "true" || v == "1" || v == "yes");
      else if (key == "initialguess") {
        if (v == "projectionaconj" || v == "projection-aconj") o.projection = 2;
        else if (v == "projection") o.projection = 1;
        else if (v == "none" || v == "previous") o.projection = 0;
        else throw Error(NRSG_ERR_BAD_CONFIG, "unknown initialGuess '" + v + "'");
      } else if (key == "residualprojectionvectors") o.projVecs = std::stoi(v);
      else if (key == "residualprojectionstart") o.projStart = std::stoi(v);
      else if (key == "mgprecision") o.mgPrecision = v;
      else if (key == "axkernel") {
        if (v != "auto" && v != "vec" && v != "plain" && v != "epb2" && v != "pipe" && v != "const" && v != "constpf")
          throw Error(NRSG_ERR_BAD_CONFIG, "axKernel must be auto, vec, plain, epb2, pipe, const or constpf");
        o.axKernel = v;
      }
      else if (key == "fdmprecision") {
        if (v != "fp32" && v != "fp16" && v != "tf32")
          throw Error(NRSG_ERR_BAD_CONFIG, "fdmPrecision must be fp32, fp16 or tf32");
        o.fdmFp16 = (v == "fp16");
        o.fdmTf32 = (v == "tf32");
      }
      else if (key == "fdmmma") {
        if (v != "tcgen05" && v != "sync") throw Error(NRSG_ERR_BAD_CONFIG, "fdmMma must be tcgen05 or sync");
        o.fdmTcgen05 = (v == "tcgen05");
      }
      else if (key == "fdmkernel") {
        if (v != "auto" && v != "generic") throw Error(NRSG_ERR_BAD_CONFIG, "fdmKernel must be auto or generic");
        o.fdmGeneric = (v == "generic");
      }
      else if (key == "axprecision") {
        if (v != "fp64" && v != "fp32x2") throw Error(NRSG_ERR_BAD_CONFIG, "axPrecision must be fp64 or fp32x2");
        o.axPrecision = v;
        axSet = true;
      }
      else if (key == "poisson") o.poisson = std::stoi(v) != 0;
      else if (key == "lambda0") o.lambda0 = std::stod(v);
      else if (key == "lambda1") o.lambda1 = std::stod(v);
      else if (key == "elementmap") o.trilinear = (v == "trilinear");
      else if (key == "trilinearlambda0") {
        if (v != "all" && v != "t") throw Error(NRSG_ERR_BAD_CONFIG, "trilinearLambda0 must be t or all");
        o.trilinearLambda0All = (v == "all");
      }
      else if (key == "seed") o.seed = std::stoull(v);
      else throw Error(NRSG_ERR_BAD_CONFIG, "unknown option '" + key + "'");
    } catch (const std::invalid_argument &) {
      throw Error(NRSG_ERR_BAD_CONFIG, "bad value for '" + key + "': " + v);
    } catch (const std::out_of_range &) {
      throw Error(NRSG_ERR_BAD_CONFIG, "bad value for '" + key + "': " + v);
    }
  }
  // mixed precision: FP32 multigrid under an FP64-accurate FP32-pair fine operator
  if (o.mgPrecision == "mixed" && !axSet && !o.trilinear) o.axPrecision = "fp32x2";
  if (o.mgPrecision != "fp64" && o.mgPrecision != "fp32" && o.mgPrecision != "mixed")
    throw Error(NRSG_ERR_BAD_CONFIG, "mgPrecision must be fp64, fp32 or mixed");
  if (o.tol <= 0 || o.maxIter < 1) throw Error(NRSG_ERR_BAD_CONFIG, "residualTol and maxIterations must be positive");
  if (!o.poisson && o.precon == "multigrid" && o.smoother.find("jac") == std::string::npos)
    throw Error(NRSG_ERR_BAD_CONFIG, "Non-Poisson type equations require Jacobi multigrid smoother");
  return o;
}

} // namespace nrsg
