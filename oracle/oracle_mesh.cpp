// ORACLE — test infrastructure only.
//
// CPU restatement of nekRS's mesh-side setup for the pressure/Helmholtz
// elliptic solve: GLL basis, Kershaw box vertices, trilinear node
// coordinates, geometric factors, Nek5000 global numbering (setvert3d),
// ogs local gather maps and the Dirichlet mask.  Only tests/, the smoke
// entry point and the CPU-baseline leg of bench.py may load this code; the
// product library never links or calls it.
//
// Parity pins: integer maps are checked for self-consistency against node
// coordinates (same id <=> same physical point) and against the reference's
// invariants; floating point operators are pinned against the reference's
// own serial kernels compiled from their sources into oracle/_ref (see
// oracle/Makefile) and against committed golden fixtures.

#include "oracle.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <numeric>
#include <stdexcept>

namespace orc {

// ---------------------------------------------------------------------------
// 1-D basis.  nekRS computes GLL nodes with a Golub-Welsch Jacobi-Gauss
// solve and D / interpolation through Vandermonde right-solves
// (src/mesh/meshBasis1D.cpp:99-153,249-280).  The restatement uses closed
// forms, which agree with those to rounding: the interior nodes are the
// roots of P_N'(x) found by Newton's method on f = P_{N-1} - x P_N (a
// multiple of (1 - x^2) P_N'/N) with f' = -(N+1) P_N at the root, from
// Chebyshev-Lobatto guesses; weights 2/(N(N+1) P_N^2); D from the node
// products c_j = prod_{k != j} (z_j - z_k).  The FP64 solve compares the
// device bit for bit with this oracle, so these are the same operations, in
// the same order, as the device library's host setup.
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

void gll(int N, double *z, double *w)
{
  for (int i = 0; i <= N; ++i) z[i] = 0.0;
  z[0] = -1.0;
  z[N] = 1.0;
  for (int i = 1; i <= N / 2; ++i) {
    double x = -std::cos(M_PI * i / N);
    for (int it = 0; it < 64; ++it) {
      double pn, pm;
      legendre_pair(N, x, pn, pm);
      const double f = pm - x * pn;
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

void dmatrix(int N, const double *z, double *D)
{
  const int nq = N + 1;
  std::vector<double> c(nq, 1.0);
  for (int j = 0; j < nq; ++j)
    for (int k = 0; k < nq; ++k)
      if (k != j) c[j] *= (z[j] - z[k]);
  for (int i = 0; i < nq; ++i) {
    double s = 0;
    for (int j = 0; j < nq; ++j) {
      if (j == i) continue;
      D[i * nq + j] = c[i] / (c[j] * (z[i] - z[j]));
      s += D[i * nq + j];
    }
    D[i * nq + i] = -s;
  }
}

static void bary_weights(int n, const double *z, double *lam)
{
  for (int j = 0; j < n; ++j) {
    double prod = 1.0;
    for (int k = 0; k < n; ++k)
      if (k != j) prod *= (z[j] - z[k]);
    lam[j] = 1.0 / prod;
  }
}

void interp_matrix(int nin, const double *zin, int nout, const double *zout, double *I)
{
  std::vector<double> lam(nin);
  bary_weights(nin, zin, lam.data());
  for (int o = 0; o < nout; ++o) {
    int hit = -1;
    for (int j = 0; j < nin; ++j)
      if (std::fabs(zout[o] - zin[j]) < 1e-15) hit = j;
    if (hit >= 0) {
      for (int j = 0; j < nin; ++j) I[o * nin + j] = (j == hit) ? 1.0 : 0.0;
      continue;
    }
    double den = 0.0;
    for (int j = 0; j < nin; ++j) den += lam[j] / (zout[o] - zin[j]);
    for (int j = 0; j < nin; ++j) I[o * nin + j] = (lam[j] / (zout[o] - zin[j])) / den;
  }
}

// ---------------------------------------------------------------------------
// Kershaw vertex map, restated from examples/kershaw/kershaw.usr:107-188
// (right/left/step/kershaw) and applied to box vertices as in usrdat
// (kershaw.usr:191-225).  The box is [0,1]^3 (the reference's final
// rescale to [-0.5,0.5], kershaw.usr:84-90, is a translation and is omitted).
// ---------------------------------------------------------------------------
static double k_right(double eps, double x) { return (x <= 0.5) ? (2.0 - eps) * x : 1.0 + eps * (x - 1.0); }
static double k_left(double eps, double x) { return 1.0 - k_right(eps, 1.0 - x); }
static double k_step(double a, double b, double x)
{
  if (x <= 0.0) return a;
  if (x >= 1.0) return b;
  return a + (b - a) * x;
}

void kershaw_map(double epsy, double epsz, double x, double y, double z, double &xx, double &yy, double &zz)
{
  xx = x;
  const int layer = (int)(x * 6.0);
  const double lambda = (x - layer / 6.0) * 6.0;
  if (layer == 0) {
    yy = k_left(epsy, y);
    zz = k_left(epsz, z);
  } else if (layer == 1 || layer == 4) {
    yy = k_step(k_left(epsy, y), k_right(epsy, y), lambda);
    zz = k_step(k_left(epsz, z), k_right(epsz, z), lambda);
  } else if (layer == 2) {
    const double t = lambda / 2.0;
    yy = k_step(k_right(epsy, y), k_left(epsy, y), t);
    zz = k_step(k_right(epsz, z), k_left(epsz, z), t);
  } else if (layer == 3) {
    const double t = (1.0 + lambda) / 2.0;
    yy = k_step(k_right(epsy, y), k_left(epsy, y), t);
    zz = k_step(k_right(epsz, z), k_left(epsz, z), t);
  } else {
    yy = k_right(epsy, y);
    zz = k_right(epsz, z);
  }
}

void box_mesh(int nx, int ny, int nz, double eps, double *VX, long long *EToV, int *EToB, int allDirichlet)
{
  // Elements are numbered x fastest (genbox order).  Vertices are in
  // hypercube order v = i + 2j + 4k inside an element; global vertex ids
  // are 1-based lexicographic lattice ids.
  const long long sx = nx + 1, sy = ny + 1;
  for (int ez = 0; ez < nz; ++ez)
    for (int ey = 0; ey < ny; ++ey)
      for (int ex = 0; ex < nx; ++ex) {
        const long long e = ex + (long long)nx * (ey + (long long)ny * ez);
        for (int v = 0; v < 8; ++v) {
          const int a = v & 1, b = (v >> 1) & 1, c = (v >> 2) & 1;
          const long long ix = ex + a, iy = ey + b, iz = ez + c;
          EToV[e * 8 + v] = 1 + ix + sx * (iy + sy * iz);
          double xx, yy, zz;
          kershaw_map(eps, eps, (double)ix / nx, (double)iy / ny, (double)iz / nz, xx, yy, zz);
          VX[(e * 8 + v) * 3 + 0] = xx;
          VX[(e * 8 + v) * 3 + 1] = yy;
          VX[(e * 8 + v) * 3 + 2] = zz;
        }
        // nekRS face order: 0:t-,1:s-,2:r+,3:s+,4:r-,5:t+ (meshBasisHex3D.cpp:53-82)
        int bc[6] = {ez == 0, ey == 0, ex == nx - 1, ey == ny - 1, ex == 0, ez == nz - 1};
        for (int f = 0; f < 6; ++f) EToB[e * 6 + f] = bc[f] ? (allDirichlet ? 1 : 4) : 0;
      }
}

// Trilinear node coordinates from the 8 vertices (straight-sided hexes, as
// Nek5000 builds xm1 for elements without curved sides); blending weights
// (hr hs) ht and fused multiply-adds in vertex order, as the device does.
void trilinear_coords(int N, long long E, const double *VX, const double *z1, double *x, double *y, double *z)
{
  const int nq = N + 1, np = nq * nq * nq;
#pragma omp parallel for schedule(static)
  for (long long e = 0; e < E; ++e)
    for (int k = 0; k < nq; ++k)
      for (int j = 0; j < nq; ++j)
        for (int i = 0; i < nq; ++i) {
          const double r = z1[i], s = z1[j], t = z1[k];
          const double hr[2] = {0.5 * (1 - r), 0.5 * (1 + r)};
          const double hs[2] = {0.5 * (1 - s), 0.5 * (1 + s)};
          const double ht[2] = {0.5 * (1 - t), 0.5 * (1 + t)};
          double X = 0, Y = 0, Z = 0;
          for (int v = 0; v < 8; ++v) {
            const double wv = hr[v & 1] * hs[(v >> 1) & 1] * ht[(v >> 2) & 1];
            X = std::fma(wv, VX[(e * 8 + v) * 3 + 0], X);
            Y = std::fma(wv, VX[(e * 8 + v) * 3 + 1], Y);
            Z = std::fma(wv, VX[(e * 8 + v) * 3 + 2], Z);
          }
          const long long id = e * np + i + nq * (j + nq * k);
          x[id] = X;
          y[id] = Y;
          z[id] = Z;
        }
}

// Geometric factors, restated from kernels/mesh/geometricFactorsHex3D.okl:77-139.
// ggeo layout [e][7][Np] with G00,G01,G11,G12,G02,G22,GWJ (mesh3D.h:96-102).
// Every multiply-add is an explicit std::fma or a separately rounded product,
// in the order of the device kernel (geofac_kernel), so that the FP64
// factors are bit-identical to the device's.
void geometric_factors(int N, long long E, const double *D, const double *w, const double *x, const double *y,
                       const double *z, double *ggeo, double *J_out)
{
  const int nq = N + 1, np = nq * nq * nq;
#pragma omp parallel for schedule(static)
  for (long long e = 0; e < E; ++e) {
    const double *xe = x + e * np, *ye = y + e * np, *ze = z + e * np;
    for (int k = 0; k < nq; ++k)
      for (int j = 0; j < nq; ++j)
        for (int i = 0; i < nq; ++i) {
          double xr = 0, xs = 0, xt = 0, yr = 0, ys = 0, yt = 0, zr = 0, zs = 0, zt = 0;
          for (int m = 0; m < nq; ++m) {
            const int ir = m + nq * (j + nq * k), is = i + nq * (m + nq * k), it = i + nq * (j + nq * m);
            xr = std::fma(D[i * nq + m], xe[ir], xr);
            xs = std::fma(D[j * nq + m], xe[is], xs);
            xt = std::fma(D[k * nq + m], xe[it], xt);
            yr = std::fma(D[i * nq + m], ye[ir], yr);
            ys = std::fma(D[j * nq + m], ye[is], ys);
            yt = std::fma(D[k * nq + m], ye[it], yt);
            zr = std::fma(D[i * nq + m], ze[ir], zr);
            zs = std::fma(D[j * nq + m], ze[is], zs);
            zt = std::fma(D[k * nq + m], ze[it], zt);
          }
          // 2x2 minors a b - c d as fma(a, b, -(c d)) (the device kernel's operation order)
          auto minor2 = [](double a, double b, double c, double d) { return std::fma(a, b, -(c * d)); };
          const double cx = minor2(ys, zt, zs, yt), cy = minor2(xs, zt, zs, xt), cz = minor2(xs, yt, ys, xt);
          const double J = std::fma(zr, cz, std::fma(-yr, cy, xr * cx));
          const double Ji = 1.0 / J;
          const double JW = J * w[i] * w[j] * w[k];
          const double rx = cx * Ji, ry = -cy * Ji, rz = cz * Ji;
          const double sx = -minor2(yr, zt, zr, yt) * Ji, sy = minor2(xr, zt, zr, xt) * Ji,
                       sz = -minor2(xr, yt, yr, xt) * Ji;
          const double tx = minor2(yr, zs, zr, ys) * Ji, ty = -minor2(xr, zs, zr, xs) * Ji,
                       tz = minor2(xr, ys, yr, xs) * Ji;
          auto dot3 = [](double a0, double b0, double a1, double b1, double a2, double b2) {
            return std::fma(a2, b2, std::fma(a1, b1, a0 * b0));
          };
          const int n = i + nq * (j + nq * k);
          double *g = ggeo + e * 7 * np;
          g[0 * np + n] = JW * dot3(rx, rx, ry, ry, rz, rz);
          g[1 * np + n] = JW * dot3(rx, sx, ry, sy, rz, sz);
          g[2 * np + n] = JW * dot3(sx, sx, sy, sy, sz, sz);
          g[3 * np + n] = JW * dot3(sx, tx, sy, ty, sz, tz);
          g[4 * np + n] = JW * dot3(rx, tx, ry, ty, rz, tz);
          g[5 * np + n] = JW * dot3(tx, tx, ty, ty, tz, tz);
          g[6 * np + n] = JW;
          if (J_out) J_out[e * np + n] = J;
        }
  }
}

// ---------------------------------------------------------------------------
// Nek5000 global numbering with interiors excluded, restated from setvert3d
// (3rd_party/nek5000/core/navier8.f:2004-2350), single rank.  Vertex ids come
// from the caller (the reference takes them from parRSB).  Unique edges and
// faces are ranked lexicographically by their sorted vertex tuples
// (gbtuple_rank8 / i8rank_vecn, navier8.f:1790-1830,1934-1998).
// ---------------------------------------------------------------------------
void global_ids(int N, long long E, const long long *EToV, long long *ids)
{
  const int nx = N + 1;
  const long long nxyz = (long long)nx * nx * nx;
  auto gid = [&](long long e, int a, int b, int c) -> long long & { return ids[e * nxyz + a + nx * (b + nx * c)]; };

  long long ngvv = 0;
  for (long long i = 0; i < E * 8; ++i) ngvv = std::max(ngvv, EToV[i]);
  for (long long i = 0; i < E * nxyz; ++i) ids[i] = 0;
  for (long long e = 0; e < E; ++e)
    for (int v = 0; v < 8; ++v) gid(e, (v & 1) * (nx - 1), ((v >> 1) & 1) * (nx - 1), ((v >> 2) & 1) * (nx - 1)) = EToV[e * 8 + v];
  long long ngv = ngvv;
  if (nx == 2) return;

  // --- edges: 12 per element, order r-edges (j,k), s-edges (i,k), t-edges (i,j)
  std::vector<std::pair<long long, long long>> etup(12 * E);
  for (long long e = 0; e < E; ++e) {
    const long long *V = EToV + e * 8;
    int q = 0;
    for (int c = 0; c < 2; ++c)
      for (int b = 0; b < 2; ++b) etup[12 * e + q++] = {V[0 + 2 * b + 4 * c], V[1 + 2 * b + 4 * c]};
    for (int c = 0; c < 2; ++c)
      for (int a = 0; a < 2; ++a) etup[12 * e + q++] = {V[a + 0 + 4 * c], V[a + 2 + 4 * c]};
    for (int b = 0; b < 2; ++b)
      for (int a = 0; a < 2; ++a) etup[12 * e + q++] = {V[a + 2 * b + 0], V[a + 2 * b + 4]};
  }
  for (auto &t : etup)
    if (t.first > t.second) std::swap(t.first, t.second);
  std::vector<std::pair<long long, long long>> eu(etup);
  std::sort(eu.begin(), eu.end());
  eu.erase(std::unique(eu.begin(), eu.end()), eu.end());
  auto erank = [&](const std::pair<long long, long long> &t) {
    return (long long)(std::lower_bound(eu.begin(), eu.end(), t) - eu.begin()) + 1;
  };
  const long long n_on_edge = nx - 2;
  const long long n_unique_edges = (long long)eu.size();
  for (long long e = 0; e < E; ++e) {
    int q = 0;
    // edges along r
    for (int c = 0; c < 2; ++c)
      for (int b = 0; b < 2; ++b) {
        const long long igv = ngv + n_on_edge * (erank(etup[12 * e + q++]) - 1);
        const int bb = b * (nx - 1), cc = c * (nx - 1);
        const bool fwd = gid(e, 0, bb, cc) < gid(e, nx - 1, bb, cc);
        for (int a = 1; a < nx - 1; ++a) gid(e, a, bb, cc) = fwd ? igv + a : igv + 1 + n_on_edge - a;
      }
    for (int c = 0; c < 2; ++c)
      for (int a = 0; a < 2; ++a) {
        const long long igv = ngv + n_on_edge * (erank(etup[12 * e + q++]) - 1);
        const int aa = a * (nx - 1), cc = c * (nx - 1);
        const bool fwd = gid(e, aa, 0, cc) < gid(e, aa, nx - 1, cc);
        for (int b = 1; b < nx - 1; ++b) gid(e, aa, b, cc) = fwd ? igv + b : igv + 1 + n_on_edge - b;
      }
    for (int b = 0; b < 2; ++b)
      for (int a = 0; a < 2; ++a) {
        const long long igv = ngv + n_on_edge * (erank(etup[12 * e + q++]) - 1);
        const int aa = a * (nx - 1), bb = b * (nx - 1);
        const bool fwd = gid(e, aa, bb, 0) < gid(e, aa, bb, nx - 1);
        for (int c = 1; c < nx - 1; ++c) gid(e, aa, bb, c) = fwd ? igv + c : igv + 1 + n_on_edge - c;
      }
  }
  ngv += n_unique_edges * n_on_edge;

  // --- faces (symmetric numbering 1..6: x-,x+,y-,y+,z-,z+), keyed by the 3
  // smallest corner vertex ids (TOPOL ICFACE table).
  static const int icface[6][4] = {{0, 2, 4, 6}, {1, 3, 5, 7}, {0, 1, 4, 5}, {2, 3, 6, 7}, {0, 1, 2, 3}, {4, 5, 6, 7}};
  typedef std::array<long long, 3> T3;
  std::vector<T3> ftup(6 * E);
  for (long long e = 0; e < E; ++e)
    for (int f = 0; f < 6; ++f) {
      long long c4[4];
      for (int q = 0; q < 4; ++q) c4[q] = EToV[e * 8 + icface[f][q]];
      std::sort(c4, c4 + 4);
      ftup[6 * e + f] = {c4[0], c4[1], c4[2]};
    }
  std::vector<T3> fu(ftup);
  std::sort(fu.begin(), fu.end());
  fu.erase(std::unique(fu.begin(), fu.end()), fu.end());
  const long long n_unique_faces = (long long)fu.size();
  const long long n_on_face = (long long)(nx - 2) * (nx - 2);
  for (long long e = 0; e < E; ++e)
    for (int f = 0; f < 6; ++f) {
      const long long fnum = (long long)(std::lower_bound(fu.begin(), fu.end(), ftup[6 * e + f]) - fu.begin()) + 1;
      // face-local (p,q) -> element (a,b,c); p plays Nek's "i" loop, q its "j" loop
      auto pt = [&](int p, int q) -> long long & {
        switch (f) {
        case 0: return gid(e, 0, p, q);
        case 1: return gid(e, nx - 1, p, q);
        case 2: return gid(e, p, 0, q);
        case 3: return gid(e, p, nx - 1, q);
        case 4: return gid(e, p, q, 0);
        default: return gid(e, p, q, nx - 1);
        }
      };
      const long long g1 = pt(0, 0), g2 = pt(nx - 1, 0), g3 = pt(0, nx - 1), g4 = pt(nx - 1, nx - 1);
      const long long gv[4] = {g1, g2, g3, g4};
      int imin = 0;
      for (int q = 1; q < 4; ++q)
        if (gv[q] < gv[imin]) imin = q;
      int idir = 1, jdir = 1;
      bool ifij = false;
      if (imin == 0) { idir = 1; jdir = 1; ifij = g2 < g3; }
      else if (imin == 1) { idir = -1; jdir = 1; ifij = g1 < g4; }
      else if (imin == 2) { idir = 1; jdir = -1; ifij = g4 < g1; }
      else { idir = -1; jdir = -1; ifij = g3 < g2; }
      const int p0 = idir > 0 ? 0 : nx - 1, ps = idir;
      const int q0 = jdir > 0 ? 0 : nx - 1, qs = jdir;
      const long long ig0 = ngv + n_on_face * (fnum - 1);
      long long kk = 0, l = 0;
      const long long nxx = (long long)nx * nx;
      auto visit = [&](int p, int q) {
        ++kk;
        if (kk > nx && kk < nxx - nx && kk % nx != 1 && kk % nx != 0) {
          ++l;
          pt(p, q) = l + ig0;
        }
      };
      if (ifij) {
        for (int qq = 0; qq < nx; ++qq)
          for (int pp = 0; pp < nx; ++pp) visit(p0 + ps * pp, q0 + qs * qq);
      } else {
        for (int pp = 0; pp < nx; ++pp)
          for (int qq = 0; qq < nx; ++qq) visit(p0 + ps * pp, q0 + qs * qq);
      }
    }
  // interiors stay 0 (set_vert is called with ifcenter = .false.)
  (void)n_unique_faces;
}

// ---------------------------------------------------------------------------
// ogs local gather maps, restated from ogsSetup (3rd_party/gslib/ogs/src/
// ogsSetup.cpp:111-397) on one rank: nodes with id 0 are excluded; nodes
// are grouped by |id|; groups are numbered in order of their smallest local
// index; within a group local indices ascend.  invDegree = 1/multiplicity
// (1 for excluded nodes).
// ---------------------------------------------------------------------------
void ogs_setup(long long Nlocal, const long long *ids, std::vector<int> &offsets, std::vector<int> &gids,
               std::vector<double> &invDegree)
{
  struct Node { long long base; long long local; };
  std::vector<Node> nodes;
  nodes.reserve(Nlocal);
  for (long long i = 0; i < Nlocal; ++i)
    if (ids[i] != 0) nodes.push_back({std::llabs(ids[i]), i});
  std::sort(nodes.begin(), nodes.end(), [](const Node &a, const Node &b) {
    if (a.base != b.base) return a.base < b.base;
    return a.local < b.local;
  });
  // group id in sorted order, and each group's first (= smallest) local index
  std::vector<long long> groupOf(nodes.size());
  std::vector<std::pair<long long, long long>> groups; // (min local, sorted group index)
  long long g = -1;
  for (size_t i = 0; i < nodes.size(); ++i) {
    if (i == 0 || nodes[i].base != nodes[i - 1].base) {
      ++g;
      groups.push_back({nodes[i].local, g});
    }
    groupOf[i] = g;
  }
  std::sort(groups.begin(), groups.end());
  std::vector<long long> order(groups.size());
  for (size_t k = 0; k < groups.size(); ++k) order[groups[k].second] = (long long)k;
  std::vector<int> counts(groups.size(), 0);
  for (size_t i = 0; i < nodes.size(); ++i) counts[order[groupOf[i]]]++;
  offsets.assign(groups.size() + 1, 0);
  for (size_t k = 0; k < groups.size(); ++k) offsets[k + 1] = offsets[k] + counts[k];
  gids.assign(nodes.size(), 0);
  std::vector<int> fill(groups.size(), 0);
  // nodes are sorted by (base, local) so members land in ascending local order
  for (size_t i = 0; i < nodes.size(); ++i) {
    const long long k = order[groupOf[i]];
    gids[offsets[k] + fill[k]++] = (int)nodes[i].local;
  }
  invDegree.assign(Nlocal, 1.0);
  for (size_t k = 0; k < groups.size(); ++k) {
    const int m = offsets[k + 1] - offsets[k];
    for (int q = offsets[k]; q < offsets[k + 1]; ++q) invDegree[gids[q]] = 1.0 / m;
  }
}

// Dirichlet mask, restated from ellipticOgs (src/solvers/elliptic/ellipticOgs.cpp:4-134):
// node flag = min over faces of the face BC (DIRICHLET=1 wins), min-reduced
// over the unmasked gather groups; mask ids ascend by local index.
void dirichlet_mask(int N, long long E, const int *EToB, const std::vector<int> &offsets, const std::vector<int> &gids,
                    std::vector<int> &maskIds)
{
  const int nq = N + 1, np = nq * nq * nq;
  const int large = 1 << 20;
  std::vector<int> mapB((size_t)E * np, large);
  for (long long e = 0; e < E; ++e)
    for (int f = 0; f < 6; ++f) {
      const int bc = EToB[e * 6 + f];
      if (bc <= 0) continue;
      for (int b = 0; b < nq; ++b)
        for (int a = 0; a < nq; ++a) {
          int i, j, k;
          switch (f) {
          case 0: i = a; j = b; k = 0; break;
          case 1: i = a; j = 0; k = b; break;
          case 2: i = nq - 1; j = a; k = b; break;
          case 3: i = a; j = nq - 1; k = b; break;
          case 4: i = 0; j = a; k = b; break;
          default: i = a; j = b; k = nq - 1; break;
          }
          int &m = mapB[e * np + i + nq * (j + nq * k)];
          m = std::min(m, bc);
        }
    }
  for (size_t g = 0; g + 1 < offsets.size(); ++g) {
    int v = large;
    for (int q = offsets[g]; q < offsets[g + 1]; ++q) v = std::min(v, mapB[gids[q]]);
    for (int q = offsets[g]; q < offsets[g + 1]; ++q) mapB[gids[q]] = v;
  }
  maskIds.clear();
  for (long long n = 0; n < E * np; ++n)
    if (mapB[n] == 1) maskIds.push_back((int)n);
}

} // namespace orc
