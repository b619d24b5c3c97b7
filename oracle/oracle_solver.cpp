// ORACLE — test infrastructure only (see oracle_mesh.cpp header).
//
// CPU restatement of the elliptic operator and Krylov drivers:
//   ellipticAx / ellipticOperator   src/solvers/elliptic/ellipticOperator.cpp:31-172
//   Ax kernel (stored geometry)     kernels/elliptic/ellipticPartialAxCoeffHex3D.c:1-98
//   Ax kernel (trilinear geometry)  kernels/elliptic/ellipticPartialAxTrilinearHex3D.okl:2-186
//   Jacobi diagonal                 kernels/elliptic/ellipticBlockBuildDiagonalHex3D.okl:27-117,
//                                   src/solvers/elliptic/ellipticUpdateJacobi.cpp:32-89
//   local gather-scatter            3rd_party/gslib/ogs/okl/gatherScatterMany.okl
//   ellipticSolve                   src/solvers/elliptic/ellipticSolve.cpp:32-190
//   pcg / flexible pcg              src/solvers/elliptic/linearSolver/PCG.cpp:33-203
//   pgmres / flexible pgmres        src/solvers/elliptic/linearSolver/PGMRES.cpp:31-340
// The multigrid preconditioner lives in oracle_mg.cpp.
//
// Bit-identical FP64 path.  The plain FP64 solve (stored geometry; Jacobi or
// no preconditioner; PCG, flexible PCG, GMRES, flexible GMRES; solution
// projection) performs exactly the device library's floating-point
// operations in the device's order: weighted sums through wsum() (one fused
// multiply-add per entry on 32 interleaved lanes of 1024-entry chunks, a lane
// tree, then a blocked pairwise tree over the chunk sums), std::fma wherever
// the device uses a fused multiply-add, and
// separately rounded products elsewhere.  The oracle is compiled without
// contraction (-ffp-contract=off), so the same source rounds the same way on
// every host.  The reference-order operator (ax_stored, the order of the
// reference's serial kernel) is kept and pinned bit for bit against that
// kernel; the device-order operator (ax_stored_dev) differs from it only by
// fused rounding.

#include "oracle_internal.hpp"

#include <algorithm>
#include <cmath>
#include <map>
#include <cstdio>
#include <cstring>
#include <sstream>
#include <stdexcept>

namespace orc {

// ---------------------------------------------------------------------------
// options: "key=value" pairs separated by ';' or newlines; keys follow the
// .par [PRESSURE] section names (doc/parHelp.txt:80-120).
// ---------------------------------------------------------------------------
static std::string lower(std::string s)
{
  for (auto &c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}
static std::string trim(const std::string &s)
{
  size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
  return a == std::string::npos ? "" : s.substr(a, b - a + 1);
}

Options parse_options(const std::string &text)
{
  Options o;
  std::string t = text;
  for (auto &c : t)
    if (c == ';') c = '\n';
  std::istringstream in(t);
  std::string line;
  while (std::getline(in, line)) {
    const auto eq = line.find('=');
    if (eq == std::string::npos) continue;
    const std::string key = lower(trim(line.substr(0, eq)));
    const std::string val = trim(line.substr(eq + 1));
    const std::string lv = lower(val);
    if (key == "solver") {
      // pcg, pfcg (= pcg+flexible), pgmres+nvector=15, pfgmres
      o.solver = lv.substr(0, lv.find('+'));
      if (lv.find("flexible") != std::string::npos && o.solver == "pcg") o.solver = "pfcg";
      const auto nv = lv.find("nvector=");
      if (nv != std::string::npos) o.nVector = std::stoi(lv.substr(nv + 8));
    } else if (key == "residualtol") {
      o.tol = std::stod(lv.substr(0, lv.find('+')));
      o.relative = lv.find("relative") != std::string::npos;
    } else if (key == "relative") o.relative = std::stoi(lv) != 0;
    else if (key == "maxiterations") o.maxIter = std::stoi(lv);
    else if (key == "preconditioner") o.precon = lv;
    else if (key == "smoothertype") o.smoother = lv;
    else if (key == "chebyshevdegree") o.chebyDegree = std::stoi(lv);
    else if (key == "mineigenvalueboundfactor") o.minEigFactor = std::stod(lv);
    else if (key == "maxeigenvalueboundfactor") o.maxEigFactor = std::stod(lv);
    else if (key == "pmgschedule") o.schedule = lv;
    else if (key == "coarsesolver") o.coarse = lv;
    else if (key == "coarsegriddiscretization") {
      o.galerkin = (lv == "fem+galerkin" || lv == "galerkin");
      o.semfem = (lv == "semfem");
    }
    else if (key == "galerkincoarseoperator") o.galerkin = (lv == "true" || lv == "1" || lv == "yes");
    else if (key == "coarsetol") o.coarseTol = std::stod(lv);
    else if (key == "coarsemaxiterations") o.coarseMaxIter = std::stoi(lv);
    else if (key == "mgprecision") o.mgPrecision = lv;
    else if (key == "poisson") o.poisson = std::stoi(lv) != 0;
    else if (key == "lambda0") o.lambda0 = std::stod(lv);
    else if (key == "lambda1") o.lambda1 = std::stod(lv);
    else if (key == "elementmap") o.trilinear = (lv == "trilinear");
    else if (key == "trilinearlambda0") o.trilinearLambda0All = (lv == "all");
    else if (key == "seed") o.seed = std::stoull(lv);
    else if (key == "initialguess")
      o.projection = (lv == "projectionaconj" || lv == "projection-aconj") ? 2 : (lv == "projection" ? 1 : 0);
    else if (key == "residualprojectionvectors") o.projVecs = std::stoi(lv);
    else if (key == "residualprojectionstart") o.projStart = std::stoi(lv);
  }
  return o;
}

// ---------------------------------------------------------------------------
// Level construction (mesh data for one polynomial order)
// ---------------------------------------------------------------------------
void build_level(Level &L, int N, long long E, const double *VX, const long long *EToV, const int *EToB)
{
  L.N = N;
  L.Nq = N + 1;
  L.Np = L.Nq * L.Nq * L.Nq;
  L.E = E;
  L.Nlocal = E * L.Np;
  L.z.resize(L.Nq);
  L.w.resize(L.Nq);
  gll(N, L.z.data(), L.w.data());
  L.D.resize(L.Nq * L.Nq);
  dmatrix(N, L.z.data(), L.D.data());
  L.x.resize(L.Nlocal);
  L.y.resize(L.Nlocal);
  L.zc.resize(L.Nlocal);
  trilinear_coords(N, E, VX, L.z.data(), L.x.data(), L.y.data(), L.zc.data());
  L.ggeo.resize((size_t)7 * L.Nlocal);
  geometric_factors(N, E, L.D.data(), L.w.data(), L.x.data(), L.y.data(), L.zc.data(), L.ggeo.data(), nullptr);
  L.ids.resize(L.Nlocal);
  global_ids(N, E, EToV, L.ids.data());
  // unmasked handle (mesh->ogs) for the BC min-reduction, then the masked one
  std::vector<int> off, gid;
  std::vector<double> invd;
  ogs_setup(L.Nlocal, L.ids.data(), off, gid, invd);
  dirichlet_mask(N, E, EToB, off, gid, L.maskIds);
  L.maskedIds = L.ids;
  for (int m : L.maskIds) L.maskedIds[m] = 0;
  ogs_setup(L.Nlocal, L.maskedIds.data(), L.gsOff, L.gsIds, L.invDegree);
  L.volume = 0;
  for (long long e = 0; e < E; ++e)
    for (int n = 0; n < L.Np; ++n) L.volume += L.ggeo[(size_t)e * 7 * L.Np + 6 * L.Np + n];
  L.VX.assign(VX, VX + E * 24);
  L.EToB.assign(EToB, EToB + E * 6);
  L.EToV.assign(EToV, EToV + E * 8);
}

// ---------------------------------------------------------------------------
// Ax, stored geometric factors.  Same operation order as the serial kernel
// ellipticPartialAxCoeffHex3D.c:27-96 (qr,qs,qt by DT; G*grad*lambda0; D^T).
// ---------------------------------------------------------------------------
template <typename T>
void ax_stored(const Level &L, const T *ggeo, const T *D, T lambda0, T lambda1, bool poisson, const T *q, T *Aq)
{
  const int nq = L.Nq, np = L.Np;
#pragma omp parallel for
  for (long long e = 0; e < L.E; ++e) {
    T Gr[1000], Gs[1000], Gt[1000]; // Np <= 10^3
    const T *qe = q + e * np;
    const T *g = ggeo + (size_t)e * 7 * np;
    for (int k = 0; k < nq; ++k)
      for (int j = 0; j < nq; ++j)
        for (int i = 0; i < nq; ++i) {
          const int n = i + nq * (j + nq * k);
          T qr = 0, qs = 0, qt = 0;
          for (int m = 0; m < nq; ++m) {
            qr += D[i * nq + m] * qe[m + nq * (j + nq * k)];
            qs += D[j * nq + m] * qe[i + nq * (m + nq * k)];
            qt += D[k * nq + m] * qe[i + nq * (j + nq * m)];
          }
          const T G00 = g[0 * np + n], G01 = g[1 * np + n], G11 = g[2 * np + n];
          const T G12 = g[3 * np + n], G02 = g[4 * np + n], G22 = g[5 * np + n];
          T a = G00 * qr; a += G01 * qs; a += G02 * qt;
          T b = G01 * qr; b += G11 * qs; b += G12 * qt;
          T c = G02 * qr; c += G12 * qs; c += G22 * qt;
          Gr[n] = lambda0 * a;
          Gs[n] = lambda0 * b;
          Gt[n] = lambda0 * c;
        }
    for (int k = 0; k < nq; ++k)
      for (int j = 0; j < nq; ++j)
        for (int i = 0; i < nq; ++i) {
          const int n = i + nq * (j + nq * k);
          T r0 = 0;
          if (!poisson) r0 = g[6 * np + n] * lambda1 * qe[n];
          T ar = 0, as = 0, at = 0;
          for (int m = 0; m < nq; ++m) {
            ar += D[m * nq + i] * Gr[m + nq * (j + nq * k)];
            as += D[m * nq + j] * Gs[i + nq * (m + nq * k)];
            at += D[m * nq + k] * Gt[i + nq * (j + nq * m)];
          }
          Aq[e * np + n] = ar + as + at + r0;
        }
  }
}

// Ax in FP64 in the device kernel's operation order (ax_stored_kernel<double>
// and ax_trilinear_kernel<double>): per k-plane, qt, qr, qs as fused
// multiply-add chains over m; G q as l0 fma(Gc, qt, fma(Gb, qs, Ga qr)); then
// for m ascending auk += D[m][j] Gs(i,m,k), Aq(i,j,m) += D[k][m] Gt(i,j,k),
// auk += D[m][i] Gr(m,j,k), all fused; Aq(i,j,k) += auk at the end of plane k.
// gf(e, i, j, k, G[7]) supplies G00, G01, G11, G12, G02, G22, GWJ of a node;
// l0rs scales the r and s fluxes, l0t the t flux.
template <typename GF>
static void ax_dev(const Level &L, const double *D, double l0rs, double l0t, double lambda1, bool poisson,
                   const double *q, double *Aq, const GF &gf)
{
  const int nq = L.Nq, np = L.Np, nq2 = nq * nq;
  auto gflux = [&](double l0, double Ga, double Gb, double Gc, double qr, double qs, double qt) {
    return l0 * std::fma(Gc, qt, std::fma(Gb, qs, Ga * qr));
  };
#pragma omp parallel for
  for (long long e = 0; e < L.E; ++e) {
    double Gr[100], Gs[100], Gt[100], auk[100], rAq[1000]; // Nq <= 10
    for (int t = 0; t < np; ++t) rAq[t] = 0.0;
    const double *qe = q + e * np;
    for (int k = 0; k < nq; ++k) {
      for (int j = 0; j < nq; ++j)
        for (int i = 0; i < nq; ++i) {
          const int n = i + nq * (j + nq * k), t = i + nq * j;
          double qt = 0, qr = 0, qs = 0;
          for (int m = 0; m < nq; ++m) qt = std::fma(D[k * nq + m], qe[t + nq2 * m], qt);
          for (int m = 0; m < nq; ++m) {
            qr = std::fma(D[i * nq + m], qe[m + nq * j + nq2 * k], qr);
            qs = std::fma(D[j * nq + m], qe[i + nq * m + nq2 * k], qs);
          }
          double G[7];
          gf(e, i, j, k, G);
          const double G00 = G[0], G01 = G[1], G11 = G[2], G12 = G[3], G02 = G[4], G22 = G[5];
          Gr[t] = gflux(l0rs, G00, G01, G02, qr, qs, qt);
          Gs[t] = gflux(l0rs, G01, G11, G12, qr, qs, qt);
          Gt[t] = gflux(l0t, G02, G12, G22, qr, qs, qt);
          auk[t] = poisson ? 0.0 : G[6] * lambda1 * qe[n];
        }
      for (int j = 0; j < nq; ++j)
        for (int i = 0; i < nq; ++i) {
          const int t = i + nq * j;
          double a = auk[t];
          for (int m = 0; m < nq; ++m) {
            a = std::fma(D[m * nq + j], Gs[i + nq * m], a);
            rAq[t + nq2 * m] = std::fma(D[k * nq + m], Gt[t], rAq[t + nq2 * m]);
            a = std::fma(D[m * nq + i], Gr[m + nq * j], a);
          }
          rAq[t + nq2 * k] += a;
        }
    }
    std::copy(rAq, rAq + np, Aq + e * np);
  }
}

void ax_stored_dev(const Level &L, const double *ggeo, const double *D, double lambda0, double lambda1, bool poisson,
                   const double *q, double *Aq)
{
  const int nq = L.Nq, np = L.Np;
  ax_dev(L, D, lambda0, lambda0, lambda1, poisson, q, Aq, [&](long long e, int i, int j, int k, double *G) {
    const double *g = ggeo + (size_t)e * 7 * np;
    const int n = i + nq * (j + nq * k);
    for (int c = 0; c < 7; ++c) G[c] = g[c * np + n];
  });
}

// Ax with geometric factors rebuilt from the 8 trilinear vertices
// (ellipticPartialAxTrilinearHex3D.okl:50-120), in the device kernel's
// operation order.  Vertex input is in hypercube order.  The reference
// scales the t-flux alone by lambda0 (lines 154-157), which is the default
// here; option trilinearLambda0 = all scales all three fluxes.
void ax_trilinear(const Level &L, double lambda0, double lambda1, bool poisson, bool lambda0All, const double *q,
                  double *Aq)
{
  // CCW vertex order used by the reference kernel: 0:(-,-,-) 1:(+,-,-) 2:(+,+,-) 3:(-,+,-), 4..7 at t=+1
  static const int ccw[8] = {0, 1, 3, 2, 4, 5, 7, 6};
  auto gf = [&](long long e, int i, int j, int k, double *G) {
    double xe[8], ye[8], ze[8];
    for (int v = 0; v < 8; ++v) {
      xe[v] = L.VX[(e * 8 + ccw[v]) * 3 + 0];
      ye[v] = L.VX[(e * 8 + ccw[v]) * 3 + 1];
      ze[v] = L.VX[(e * 8 + ccw[v]) * 3 + 2];
    }
    const double rn = L.z[i], sn = L.z[j], tn = L.z[k];
    const double am = (1 - tn) * (1 - sn), ap = (1 - tn) * (1 + sn), bm = (1 + tn) * (1 - sn), bp = (1 + tn) * (1 + sn);
    const double cm = (1 - tn) * (1 - rn), cp = (1 - tn) * (1 + rn), dm = (1 + tn) * (1 - rn), dp = (1 + tn) * (1 + rn);
    const double fm = (1 - rn) * (1 - sn), fp = (1 + rn) * (1 - sn), hp = (1 + rn) * (1 + sn), hm = (1 - rn) * (1 + sn);
    auto comb = [](double a0, double d0, double a1, double d1, double a2, double d2, double a3, double d3) {
      return 0.125 * std::fma(a3, d3, std::fma(a2, d2, std::fma(a1, d1, a0 * d0)));
    };
    auto dr = [&](const double *X) { return comb(am, X[1] - X[0], ap, X[2] - X[3], bm, X[5] - X[4], bp, X[6] - X[7]); };
    auto ds = [&](const double *X) { return comb(cm, X[3] - X[0], cp, X[2] - X[1], dm, X[7] - X[4], dp, X[6] - X[5]); };
    auto dt = [&](const double *X) { return comb(fm, X[4] - X[0], fp, X[5] - X[1], hp, X[6] - X[2], hm, X[7] - X[3]); };
    const double xr = dr(xe), xs = ds(xe), xt = dt(xe);
    const double yr = dr(ye), ys = ds(ye), yt = dt(ye);
    const double zr = dr(ze), zs = ds(ze), zt = dt(ze);
    auto minor2 = [](double a, double b, double c, double d) { return std::fma(a, b, -(c * d)); };
    const double rx = minor2(ys, zt, zs, yt), ry = -minor2(xs, zt, zs, xt), rz = minor2(xs, yt, ys, xt);
    const double sx = -minor2(yr, zt, zr, yt), sy = minor2(xr, zt, zr, xt), sz = -minor2(xr, yt, yr, xt);
    const double tx = minor2(yr, zs, zr, ys), ty = -minor2(xr, zs, zr, xs), tz = minor2(xr, ys, yr, xs);
    const double J = std::fma(zr, rz, std::fma(yr, ry, xr * rx));
    const double W = L.w[i] * L.w[j] * L.w[k];
    const double sc = W / J;
    auto dot3 = [](double a0, double b0, double a1, double b1, double a2, double b2) {
      return std::fma(a2, b2, std::fma(a1, b1, a0 * b0));
    };
    G[0] = sc * dot3(rx, rx, ry, ry, rz, rz);
    G[1] = sc * dot3(rx, sx, ry, sy, rz, sz);
    G[2] = sc * dot3(sx, sx, sy, sy, sz, sz);
    G[3] = sc * dot3(sx, tx, sy, ty, sz, tz);
    G[4] = sc * dot3(rx, tx, ry, ty, rz, tz);
    G[5] = sc * dot3(tx, tx, ty, ty, tz, tz);
    G[6] = W * J;
  };
  ax_dev(L, L.D.data(), lambda0All ? lambda0 : 1.0, lambda0, lambda1, poisson, q, Aq, gf);
}

// diag(A_L) per element (ellipticBlockBuildDiagonalHex3D.okl:61-107), single field.
template <typename T>
void build_diag(const Level &L, const T *ggeo, const T *D, T lambda0, T lambda1, bool poisson, T *diag)
{
  const int nq = L.Nq, np = L.Np;
#pragma omp parallel for
  for (long long e = 0; e < L.E; ++e) {
    const T *g = ggeo + (size_t)e * 7 * np;
    for (int k = 0; k < nq; ++k)
      for (int j = 0; j < nq; ++j)
        for (int i = 0; i < nq; ++i) {
          const int n = i + nq * (j + nq * k);
          T r = 0;
          const T grs = g[1 * np + n], grt = g[4 * np + n], gst = g[3 * np + n];
          if constexpr (sizeof(T) == 8) {
            // the device kernel's order: fma(((2 g) l0) Da, Db, r), fma((g l0) Dm, Dm, r)
            auto cross = [&](double g0, double Da, double Db) { r = std::fma(2.0 * g0 * lambda0 * Da, Db, r); };
            auto line = [&](double g0, double Dm) { r = std::fma(g0 * lambda0 * Dm, Dm, r); };
            cross(grs, D[i * nq + i], D[j * nq + j]);
            cross(grt, D[i * nq + i], D[k * nq + k]);
            cross(gst, D[j * nq + j], D[k * nq + k]);
            for (int m = 0; m < nq; ++m) {
              line(g[0 * np + m + nq * (j + nq * k)], D[m * nq + i]);
              line(g[2 * np + i + nq * (m + nq * k)], D[m * nq + j]);
              line(g[5 * np + i + nq * (j + nq * m)], D[m * nq + k]);
            }
            if (!poisson) r = std::fma(g[6 * np + n], lambda1, r);
            diag[e * np + n] = r;
            continue;
          }
          r += (T)2.0 * grs * lambda0 * D[i * nq + i] * D[j * nq + j];
          r += (T)2.0 * grt * lambda0 * D[i * nq + i] * D[k * nq + k];
          r += (T)2.0 * gst * lambda0 * D[j * nq + j] * D[k * nq + k];
          for (int m = 0; m < nq; ++m) {
            r += g[0 * np + m + nq * (j + nq * k)] * lambda0 * D[m * nq + i] * D[m * nq + i];
            r += g[2 * np + i + nq * (m + nq * k)] * lambda0 * D[m * nq + j] * D[m * nq + j];
            r += g[5 * np + i + nq * (j + nq * m)] * lambda0 * D[m * nq + k] * D[m * nq + k];
          }
          if (!poisson) r += g[6 * np + n] * lambda1;
          diag[e * np + n] = r;
        }
  }
}

template <typename T> void gs_add(const Level &L, T *q)
{
  const long long ng = (long long)L.gsOff.size() - 1;
#pragma omp parallel for
  for (long long g = 0; g < ng; ++g) {
    const int s = L.gsOff[g], t = L.gsOff[g + 1];
    if (s + 1 == t) continue;
    T v = 0;
    for (int m = s; m < t; ++m) v += q[L.gsIds[m]];
    for (int m = s; m < t; ++m) q[L.gsIds[m]] = v;
  }
}

template <typename T> void apply_mask(const Level &L, T *q)
{
  const long long nm = (long long)L.maskIds.size();
#pragma omp parallel for schedule(static)
  for (long long k = 0; k < nm; ++k) q[L.maskIds[k]] = 0;
}

// Weighted inner product in the device's summation order (wsum): entry
// factors (w_i a_i rounded, b_i), so the argument order matters.
template <typename T> T wdot(long long n, const T *w, const T *a, const T *b)
{
  return (T)wsum(n, [&](long long i, double &x, double &y) {
    x = (double)w[i] * (double)a[i];
    y = (double)b[i];
  });
}

// explicit instantiations used by the MG code
template void ax_stored<double>(const Level &, const double *, const double *, double, double, bool, const double *, double *);
template void ax_stored<float>(const Level &, const float *, const float *, float, float, bool, const float *, float *);
template void build_diag<double>(const Level &, const double *, const double *, double, double, bool, double *);
template void build_diag<float>(const Level &, const float *, const float *, float, float, bool, float *);
template void gs_add<double>(const Level &, double *);
template void gs_add<float>(const Level &, float *);
template void apply_mask<double>(const Level &, double *);
template void apply_mask<float>(const Level &, float *);
template double wdot<double>(long long, const double *, const double *, const double *);
template float wdot<float>(long long, const float *, const float *, const float *);

// ---------------------------------------------------------------------------
// Elliptic solver state
// ---------------------------------------------------------------------------
void Elliptic::setup(int N, long long E, const double *VX, const long long *EToV, const int *EToB, const std::string &opt)
{
  o = parse_options(opt);
  build_level(fine, N, E, VX, EToV, EToB);
  // ellipticSetup.cpp:187-205: a Poisson problem with no face other than Neumann (4) has a constant null space
  allNeumann = false;
  if (o.poisson) {
    allNeumann = true;
    for (long long i = 0; i < E * 6; ++i)
      if (EToB[i] > 0 && EToB[i] != 4) allNeumann = false;
  }
  if (o.precon == "jacobi") {
    invDiag.resize(fine.Nlocal);
    build_diag<double>(fine, fine.ggeo.data(), fine.D.data(), o.lambda0, o.lambda1, o.poisson, invDiag.data());
    gs_add(fine, invDiag.data());
    for (auto &v : invDiag) v = 1.0 / v;
  } else if (o.precon == "multigrid") {
    mg_setup(*this);
  }
}

void Elliptic::ax(const double *q, double *Aq) const
{
  if (o.trilinear)
    ax_trilinear(fine, o.lambda0, o.lambda1, o.poisson, o.trilinearLambda0All, q, Aq);
  else
    ax_stored_dev(fine, fine.ggeo.data(), fine.D.data(), o.lambda0, o.lambda1, o.poisson, q, Aq);
}

void Elliptic::ax_ref(const double *q, double *Aq) const
{
  ax_stored<double>(fine, fine.ggeo.data(), fine.D.data(), o.lambda0, o.lambda1, o.poisson, q, Aq);
}

void Elliptic::op(const double *q, double *Aq) const
{
  ax(q, Aq);
  apply_mask(fine, Aq);
  gs_add(fine, Aq);
}

void Elliptic::precond(const double *r, double *z)
{
  const long long n = fine.Nlocal;
  if (o.precon == "jacobi") {
    #pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i) z[i] = r[i] * invDiag[i];
  } else if (o.precon == "multigrid") {
    mg_apply(*this, r, z);
  } else {
    std::memcpy(z, r, sizeof(double) * n);
  }
  if (allNeumann) zero_mean(z); // ellipticPreconditioner.cpp:82-83
}

// ellipticZeroMean (ellipticZeroMean.cpp:31-44): q -= sum(q) / (E Np)
void Elliptic::zero_mean(double *q) const
{
  const long long n = fine.Nlocal;
  const double s = wsum(n, [&](long long i, double &x, double &y) {
    x = q[i];
    y = 1.0;
  });
  const double mean = s / (double)n;
  #pragma omp parallel for schedule(static)
  for (long long i = 0; i < n; ++i) q[i] += -mean;
}

double Elliptic::norm(const double *r) const
{
  // res0Norm = weightedNorm2Many * sqrt(resNormFactor) (ellipticSolve.cpp:130-139)
  return std::sqrt(wdot<double>(fine.Nlocal, fine.invDegree.data(), r, r)) * std::sqrt(1.0 / fine.volume);
}

// PCG / flexible PCG (PCG.cpp:86-203)
int Elliptic::pcg(double *r, double *x, double tol, int maxit, double &rnorm)
{
  const long long n = fine.Nlocal;
  const double *w = fine.invDegree.data();
  const bool flexible = (o.solver == "pfcg");
  std::vector<double> p(n, 0.0), z(n), Ap(n);
  double rdotz1 = 0, alpha = 0;
  int it = 0;
  do {
    ++it;
    const double rdotz2 = rdotz1;
    if (o.precon != "none") {
      precond(r, z.data());
      rdotz1 = wdot<double>(n, w, r, z.data());
    } else {
      std::memcpy(z.data(), r, sizeof(double) * n);
      // (PCG.cpp:129 reuses the scaled residual norm here; the restatement
      // uses (r,r)_w, which is what unpreconditioned CG needs)
      rdotz1 = wdot<double>(n, w, r, r);
    }
    double beta = 0;
    if (it > 1) {
      beta = rdotz1 / rdotz2;
      if (flexible) {
        const double zdotAp = wdot<double>(n, w, z.data(), Ap.data());
        beta = -alpha * zdotAp / rdotz2;
      }
    }
    #pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i) p[i] = std::fma(beta, p[i], z[i]);
    op(p.data(), Ap.data());
    const double pAp = wdot<double>(n, w, p.data(), Ap.data());
    alpha = rdotz1 / (pAp + 1e-300);
    #pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i) {
      r[i] = std::fma(-alpha, Ap[i], r[i]);
      x[i] = std::fma(alpha, p[i], x[i]);
    }
    const double rdotr = wdot<double>(n, w, r, r);
    // rdotr = sqrt(update() * resNormFactor) (PCG.cpp:189)
    rnorm = std::sqrt(rdotr * (1.0 / fine.volume));
    history.push_back(rnorm);
    if (std::isnan(rnorm)) { status = 3; break; }
  } while (rnorm > tol && it < maxit);
  return it;
}

// ellipticSolve (ellipticSolve.cpp:32-190), x0 taken from x on input.
// ---------------------------------------------------------------------------
// Solution projection (initial guess from previous solutions), restated from
// SolutionProjection (src/solvers/elliptic/ellipticSolutionProjection.cpp):
// pre() (:143-182, :262-272) projects the residual onto the stored basis,
// post() (:183-221, :273-279) adds the new solution to the basis and
// A-orthonormalises it by one classical Gram-Schmidt pass with the
// dependence test of updateProjectionSpace (:40-140); accumulate.okl and
// multiScaledAddwOffset.okl give the summation orders.  Weighted inner
// products use invDegree.
// ---------------------------------------------------------------------------
void Elliptic::proj_update_space()
{
  const long long n = fine.Nlocal;
  const int m = projM;
  if (m <= 0) return;
  const bool classic = o.projection == 1;
  const double *w = fine.invDegree.data();
  const double *b = &projBB[(size_t)(classic ? m - 1 : 0) * n];
  std::vector<double> alpha(m);
  for (int k = 0; k < m; ++k) alpha[k] = wdot<double>(n, w, b, &projXX[(size_t)k * n]);
  const double normOrig = alpha[m - 1];
  double *xm = &projXX[(size_t)(m - 1) * n];
  #pragma omp parallel for schedule(static)
  for (long long i = 0; i < n; ++i) {
    double v = xm[i];
    for (int k = 0; k < m - 1; ++k) v = std::fma(-alpha[k], projXX[(size_t)k * n + i], v);
    xm[i] = v;
  }
  if (classic) {
    double *bm = &projBB[(size_t)(m - 1) * n];
    #pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i) {
      double v = bm[i];
      for (int k = 0; k < m - 1; ++k) v = std::fma(-alpha[k], projBB[(size_t)k * n + i], v);
      bm[i] = v;
    }
  }
  double sumAlpha = 0;
  for (int k = 0; k < m - 1; ++k) sumAlpha += alpha[k] * alpha[k];
  const double normNew = std::sqrt(normOrig - sumAlpha);
  if (normNew / normOrig > 1e-7) {
    const double sc = 1.0 / normNew;
    #pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i) xm[i] *= sc;
    if (classic)
      #pragma omp parallel for schedule(static)
      for (long long i = 0; i < n; ++i) projBB[(size_t)(m - 1) * n + i] *= sc;
  } else {
    --projM; // linearly dependent: discard
  }
}

void Elliptic::proj_pre(double *r)
{
  const long long n = fine.Nlocal;
  ++projStep;
  if (projStep < o.projStart || projM <= 0) return;
  const double *w = fine.invDegree.data();
  const int m = projM;
  std::vector<double> alpha(m);
  for (int k = 0; k < m; ++k) alpha[k] = wdot<double>(n, w, r, &projXX[(size_t)k * n]);
  #pragma omp parallel for schedule(static)
  for (long long i = 0; i < n; ++i) {
    double v = alpha[0] * projXX[i];
    for (int k = 1; k < m; ++k) v = std::fma(alpha[k], projXX[(size_t)k * n + i], v);
    projXbar[i] = v;
  }
  std::vector<double> t(n);
  if (o.projection == 1) {
    #pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i) {
      double v = alpha[0] * projBB[i];
      for (int k = 1; k < m; ++k) v = std::fma(alpha[k], projBB[(size_t)k * n + i], v);
      t[i] = v;
    }
  } else {
    op(projXbar.data(), t.data());
  }
  #pragma omp parallel for schedule(static)
  for (long long i = 0; i < n; ++i) r[i] = -1.0 * t[i] + 1.0 * r[i];
}

void Elliptic::proj_post(double *x)
{
  const long long n = fine.Nlocal;
  if (projStep < o.projStart) return;
  const int maxv = o.projVecs;
  if (projM == 0) {
    projM = 1;
    std::copy(x, x + n, projXX.begin());
  } else if (projM == maxv) {
    projM = 1;
    #pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i) x[i] = 1.0 * projXbar[i] + 1.0 * x[i];
    std::copy(x, x + n, projXX.begin());
  } else {
    ++projM;
    std::copy(x, x + n, projXX.begin() + (size_t)(projM - 1) * n);
    #pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i) x[i] = 1.0 * projXbar[i] + 1.0 * x[i];
  }
  const int prev = projM;
  const int bOff = o.projection == 1 ? projM - 1 : 0;
  op(&projXX[(size_t)(projM - 1) * n], &projBB[(size_t)bOff * n]);
  proj_update_space();
  if (projM < prev) { // the new vector was dependent: restart the space from x
    projM = 1;
    std::copy(x, x + n, projXX.begin());
    op(projXX.data(), projBB.data());
    proj_update_space();
  }
}

int Elliptic::solve(double *r, double *x, double &res0, double &res)
{
  const long long n = fine.Nlocal;
  std::vector<double> Ax0(n), x0(x, x + n);
  ax(x, Ax0.data());
  #pragma omp parallel for schedule(static)
  for (long long i = 0; i < n; ++i) r[i] = -Ax0[i] + r[i];
  if (allNeumann) zero_mean(r); // ellipticSolve.cpp:101
  apply_mask(fine, r);
  gs_add(fine, r);
  #pragma omp parallel for schedule(static)
  for (long long i = 0; i < n; ++i) x[i] = 0;
  if (o.projection) {
    if (projXX.empty()) {
      projXX.assign((size_t)o.projVecs * n, 0.0);
      projBB.assign((size_t)(o.projection == 1 ? o.projVecs : 1) * n, 0.0);
      projXbar.assign(n, 0.0);
    }
    proj_pre(r);
  }
  res0 = norm(r);
  double tol = o.tol;
  if (o.relative) tol *= res0;
  res = res0;
  history.clear();
  status = 0;
  int iters = 0;
  if (o.solver == "pcg" || o.solver == "pfcg")
    iters = pcg(r, x, tol, o.maxIter, res);
  else
    iters = pgmres(r, x, tol, o.maxIter, res);
  if (o.projection) proj_post(x);
  #pragma omp parallel for schedule(static)
  for (long long i = 0; i < n; ++i) x[i] += x0[i];
  if (allNeumann) zero_mean(x); // ellipticSolve.cpp:188-189
  if (std::isnan(res)) status = 3;
  else if (iters >= o.maxIter && res > tol) status = 1;
  return iters;
}

// Restarted (flexible) GMRES restated from PGMRES.cpp:111-340 and the
// gmresUpdate helper (PGMRES.cpp:70-107): classical Gram-Schmidt through one
// weighted multi-dot per step, Givens rotations on the host, right
// preconditioning (flexible keeps every Z_i), true residual at each restart.
int Elliptic::pgmres(double *r, double *x, double tol, int maxit, double &rdotr)
{
  const long long n = fine.Nlocal;
  const double *wt = fine.invDegree.data();
  const int nr = o.nVector;
  const bool flexible = (o.solver == "pfgmres");
  const int ld = nr + 1;
  std::vector<std::vector<double>> V(nr, std::vector<double>(n)), Z(flexible ? nr : 1, std::vector<double>(n));
  std::vector<double> H(ld * ld, 0.0), sn(nr), cs(nr), s(nr + 1), y(nr);
  std::vector<double> w(n), b(r, r + n), Ax(n), ztmp(n), tmp(n);
  const double sqrtFac = std::sqrt(1.0 / fine.volume);
  double nrm = rdotr / sqrtFac;
  double error = rdotr;
  auto update = [&](int m) {
    for (int k = m - 1; k >= 0; --k) {
      y[k] = s[k];
      for (int j = k + 1; j < m; ++j) y[k] -= H[k + j * ld] * y[j];
      y[k] /= H[k + k * ld];
    }
    if (flexible) {
      for (long long q = 0; q < n; ++q) {
        double v = x[q];
        for (int k = 0; k < m; ++k) v = std::fma(y[k], Z[k][q], v);
        x[q] = v;
      }
    } else {
      for (long long q = 0; q < n; ++q) {
        double v = 0;
        for (int k = 0; k < m; ++k) v = std::fma(y[k], V[k][q], v);
        ztmp[q] = v;
      }
      precond(ztmp.data(), tmp.data());
      for (long long q = 0; q < n; ++q) x[q] = tmp[q] + x[q];
    }
  };
  int iter = 0;
  for (iter = 0; iter < maxit;) {
    s[0] = nrm;
    const double inrm = 1.0 / nrm;
    for (long long q = 0; q < n; ++q) V[0][q] = inrm * r[q];
    for (int i = 0; i < nr; ++i) {
      std::vector<double> &Mv = flexible ? Z[i] : Z[0];
      precond(V[i].data(), Mv.data());
      op(Mv.data(), w.data());
      for (int k = 0; k <= i; ++k) y[k] = wdot<double>(n, wt, w.data(), V[k].data());
      for (long long q = 0; q < n; ++q) {
        double v = w[q];
        for (int k = 0; k <= i; ++k) v = std::fma(-y[k], V[k][q], v);
        w[q] = v;
      }
      const double nw = std::sqrt(wdot<double>(n, wt, w.data(), w.data()));
      H[i + 1 + i * ld] = nw;
      if (i < nr - 1) {
        const double inw = 1.0 / nw;
        for (long long q = 0; q < n; ++q) V[i + 1][q] = inw * w[q];
      }
      for (int k = 0; k <= i; ++k) H[k + i * ld] = y[k];
      for (int k = 0; k < i; ++k) {
        const double h1 = H[k + i * ld], h2 = H[k + 1 + i * ld];
        H[k + i * ld] = cs[k] * h1 + sn[k] * h2;
        H[k + 1 + i * ld] = -sn[k] * h1 + cs[k] * h2;
      }
      const double h1 = H[i + i * ld], h2 = H[i + 1 + i * ld];
      const double hr = std::sqrt(h1 * h1 + h2 * h2);
      cs[i] = h1 / hr;
      sn[i] = h2 / hr;
      H[i + i * ld] = cs[i] * h1 + sn[i] * h2;
      H[i + 1 + i * ld] = 0;
      s[i + 1] = -sn[i] * s[i];
      s[i] = cs[i] * s[i];
      ++iter;
      error = std::fabs(s[i + 1]) * sqrtFac;
      rdotr = error;
      history.push_back(error);
      if (std::isnan(error)) { status = 3; return iter; }
      if (error < tol || iter == maxit) {
        update(i + 1);
        break;
      }
    }
    if (error < tol || iter == maxit) break;
    update(nr);
    op(x, Ax.data());
    for (long long q = 0; q < n; ++q) r[q] = b[q] - Ax[q];
    nrm = std::sqrt(wdot<double>(n, wt, r, r));
    error = nrm * sqrtFac;
    rdotr = error;
    if (error <= tol) return iter;
  }
  return iter;
}

} // namespace orc

namespace orc {

// ---------------------------------------------------------------------------
// Assembled level operator, following ellipticBuildFEMHex3D
// (src/solvers/elliptic/MG/ellipticBuildFEM.cpp:73-300): per element and per
// unmasked node pair (n, m) the stiffness entry is built term by term from
// ggeo and D (rr, rs/sr, rt/tr, ss, st/ts, tt; lines 152-212), entries with
// |val| > 0 are kept (line 227), rows/columns are the masked gather groups
// (lines 98-117), entries are sorted by (row, column) and duplicates summed
// (lines 258-297; summed here in element order).  The reference builds the
// Poisson matrix (lambda1 = 0, line 90); a Helmholtz operator here adds
// lambda1 JW on the diagonal, the same operator the level smoother applies.
// ---------------------------------------------------------------------------
void assemble_fem(const Level &L, double lambda0, double lambda1, bool poisson, std::vector<long long> &rowPtr,
                  std::vector<long long> &cols, std::vector<double> &vals)
{
  const int nq = L.Nq, np = L.Np;
  const double *D = L.D.data(); // D[i*nq + j] = l_j'(z_i)
  std::vector<long long> num(L.Nlocal, -1);
  const long long ng = (long long)L.gsOff.size() - 1;
  for (long long g = 0; g < ng; ++g)
    for (int q = L.gsOff[g]; q < L.gsOff[g + 1]; ++q) num[L.gsIds[q]] = g;
  struct NZ { long long row, col, e; double val; };
  std::vector<NZ> nz;
  for (long long e = 0; e < L.E; ++e) {
    const double *g = &L.ggeo[(size_t)e * 7 * np];
    auto G = [&](int c, int i, int j, int k) { return g[c * np + i + nq * (j + nq * k)]; };
    for (int nzc = 0; nzc < nq; ++nzc)
      for (int ny = 0; ny < nq; ++ny)
        for (int nx = 0; nx < nq; ++nx) {
          const int idn = nx + nq * (ny + nq * nzc);
          if (num[e * np + idn] < 0) continue;
          for (int mz = 0; mz < nq; ++mz)
            for (int my = 0; my < nq; ++my)
              for (int mx = 0; mx < nq; ++mx) {
                const int idm = mx + nq * (my + nq * mz);
                if (num[e * np + idm] < 0) continue;
                double val = 0;
                if (ny == my && nzc == mz)
                  for (int k = 0; k < nq; ++k) val += G(0, k, ny, nzc) * D[k * nq + nx] * D[k * nq + mx];
                if (nzc == mz) {
                  val += G(1, mx, ny, nzc) * D[mx * nq + nx] * D[ny * nq + my];
                  val += G(1, nx, my, nzc) * D[nx * nq + mx] * D[my * nq + ny];
                }
                if (ny == my) {
                  val += G(4, mx, ny, nzc) * D[mx * nq + nx] * D[nzc * nq + mz];
                  val += G(4, nx, ny, mz) * D[nx * nq + mx] * D[mz * nq + nzc];
                }
                if (nx == mx && nzc == mz)
                  for (int k = 0; k < nq; ++k) val += G(2, nx, k, nzc) * D[k * nq + ny] * D[k * nq + my];
                if (nx == mx) {
                  val += G(3, nx, my, nzc) * D[my * nq + ny] * D[nzc * nq + mz];
                  val += G(3, nx, ny, mz) * D[ny * nq + my] * D[mz * nq + nzc];
                }
                if (nx == mx && ny == my)
                  for (int k = 0; k < nq; ++k) val += G(5, nx, ny, k) * D[k * nq + nzc] * D[k * nq + mz];
                double v = lambda0 * val;
                if (!poisson && idn == idm) v += lambda1 * G(6, nx, ny, nzc);
                if (std::fabs(v) > 0.0) nz.push_back({num[e * np + idn], num[e * np + idm], e, v});
              }
        }
  }
  std::stable_sort(nz.begin(), nz.end(), [](const NZ &a, const NZ &b) {
    return a.row != b.row ? a.row < b.row : a.col < b.col;
  });
  rowPtr.assign(ng + 1, 0);
  cols.clear();
  vals.clear();
  for (size_t i = 0; i < nz.size(); ++i) {
    if (!cols.empty() && i > 0 && nz[i].row == nz[i - 1].row && nz[i].col == nz[i - 1].col) {
      vals.back() += nz[i].val;
      continue;
    }
    cols.push_back(nz[i].col);
    vals.push_back(nz[i].val);
    rowPtr[nz[i].row + 1]++;
  }
  for (long long r = 0; r < ng; ++r) rowPtr[r + 1] += rowPtr[r];
}

// ---------------------------------------------------------------------------
// Galerkin coarse operator, following ellipticBuildFEMGalerkinHex3D
// (src/solvers/elliptic/MG/ellipticBuildFEM.cpp:384-520): the eight trilinear
// basis functions sampled at the fine GLL nodes (ellipticGenerateCoarseBasisHex3D
// :344-382), each copied into every element and run through the fine level's
// pfloat operator (ellipticAx, all elements at once), then projected on each
// basis function in dfloat (lines 465-495); masked rows / columns skipped,
// |val| > dropTol (0) kept, row = the projected function m, column = the
// applied function n; sorted and duplicates summed as assemble_fem.
// ---------------------------------------------------------------------------
void assemble_galerkin(const Level &F, const Level &C, double lambda0, double lambda1, bool poisson,
                       std::vector<long long> &rowPtr, std::vector<long long> &cols, std::vector<double> &vals)
{
  const int nqf = F.Nq, npf = F.Np;
  std::vector<double> b((size_t)8 * npf);
  for (int jj = 1; jj <= 8; ++jj)
    for (int k = 0; k < nqf; ++k)
      for (int j = 0; j < nqf; ++j)
        for (int i = 0; i < nqf; ++i) {
          const double zr = (jj % 2 == 0) ? 0.5 * (1 + F.z[i]) : 0.5 * (1 - F.z[i]);
          const double zs = (jj == 3 || jj == 4 || jj == 7 || jj == 8) ? 0.5 * (1 + F.z[j]) : 0.5 * (1 - F.z[j]);
          const double zt = (jj > 4) ? 0.5 * (1 + F.z[k]) : 0.5 * (1 - F.z[k]);
          b[(size_t)(jj - 1) * npf + i + nqf * (j + nqf * k)] = zr * zs * zt;
        }
  std::vector<float> g32(F.ggeo.begin(), F.ggeo.end()), D32(F.D.begin(), F.D.end());
  std::vector<float> q(F.Nlocal), Aq(F.Nlocal);
  std::vector<std::vector<float>> AqAll(8);
  for (int n = 0; n < 8; ++n) {
    for (long long e = 0; e < F.E; ++e)
      for (int t = 0; t < npf; ++t) q[e * npf + t] = (float)b[(size_t)n * npf + t];
    ax_stored<float>(F, g32.data(), D32.data(), (float)lambda0, (float)lambda1, poisson, q.data(), Aq.data());
    AqAll[n] = Aq;
  }
  std::vector<long long> num(C.Nlocal, -1);
  const long long ng = (long long)C.gsOff.size() - 1;
  for (long long g = 0; g < ng; ++g)
    for (int t = C.gsOff[g]; t < C.gsOff[g + 1]; ++t) num[C.gsIds[t]] = g;
  struct NZ { long long row, col; double val; };
  std::vector<NZ> nz;
  for (long long e = 0; e < C.E; ++e)
    for (int n = 0; n < 8; ++n) {
      if (num[e * 8 + n] < 0) continue;
      for (int m = 0; m < 8; ++m) {
        if (num[e * 8 + m] < 0) continue;
        double val = 0;
        for (int t = 0; t < npf; ++t) val += (double)AqAll[n][e * npf + t] * b[(size_t)m * npf + t];
        if (std::fabs(val) > 0.0) nz.push_back({num[e * 8 + m], num[e * 8 + n], val});
      }
    }
  std::stable_sort(nz.begin(), nz.end(), [](const NZ &a, const NZ &c) {
    return a.row != c.row ? a.row < c.row : a.col < c.col;
  });
  rowPtr.assign(ng + 1, 0);
  cols.clear();
  vals.clear();
  for (size_t i = 0; i < nz.size(); ++i) {
    if (i > 0 && nz[i].row == nz[i - 1].row && nz[i].col == nz[i - 1].col) {
      vals.back() += nz[i].val;
      continue;
    }
    cols.push_back(nz[i].col);
    vals.push_back(nz[i].val);
    rowPtr[nz[i].row + 1]++;
  }
  for (long long r = 0; r < ng; ++r) rowPtr[r + 1] += rowPtr[r];
}

// ---------------------------------------------------------------------------
// SEMFEM operator, following SEMFEMSolver_t::build / fem_assembly_host
// (src/solvers/elliptic/SEMFEMSolverBuild.cpp:218-335, 551-700): on every
// sub-hexahedron of the level's GLL grid the eight corner tetrahedra
// (mesh_connectivity :859-940), P1 stiffness by the 4-point rule (weights
// 1/24, :12-34) with the signed determinant of the tetrahedron map,
// lambda0 * A_loc added in FP32 entry by entry in the loop order element,
// sub-hex (z, y, x), tetrahedron, i, j; exact zeros dropped (dropTol 0).
// ---------------------------------------------------------------------------
void assemble_semfem(const Level &L, double lambda0, std::vector<long long> &rowPtr, std::vector<long long> &cols,
                     std::vector<double> &vals)
{
  const int nq = L.Nq, np = L.Np;
  const int corner[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0}, {0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
  const int tet[8][4] = {{0, 2, 1, 4}, {1, 0, 3, 5}, {2, 6, 3, 0}, {3, 2, 7, 1},
                         {4, 5, 6, 0}, {5, 7, 4, 1}, {6, 7, 2, 4}, {7, 3, 6, 5}};
  // reference-tetrahedron basis gradients: r, s, t, 1 - r - s - t
  const double grad[4][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {-1, -1, -1}};
  std::vector<long long> num(L.Nlocal, -1);
  long long ng = (long long)L.gsOff.size() - 1;
  for (long long g = 0; g < ng; ++g)
    for (int t = L.gsOff[g]; t < L.gsOff[g + 1]; ++t) num[L.gsIds[t]] = g;
  // every unmasked node is an unknown (matrix_distribution :337-420 ranks all of them); element-interior
  // nodes, which no gather group holds, follow the shared ones in E-vector order
  std::vector<char> isMasked(L.Nlocal, 0);
  for (int m : L.maskIds) isMasked[m] = 1;
  for (long long i = 0; i < L.Nlocal; ++i)
    if (num[i] < 0 && !isMasked[i]) num[i] = ng++;
  std::map<std::pair<long long, long long>, float> entries;
  for (long long e = 0; e < L.E; ++e)
    for (int sz = 0; sz + 1 < nq; ++sz)
      for (int sy = 0; sy + 1 < nq; ++sy)
        for (int sx = 0; sx + 1 < nq; ++sx)
          for (int t = 0; t < 8; ++t) {
            long long node[4];
            double X[3][4];
            for (int k = 0; k < 4; ++k) {
              const int *c = corner[tet[t][k]];
              node[k] = e * np + (sx + c[0]) + nq * ((sy + c[1]) + nq * (sz + c[2]));
              X[0][k] = L.x[node[k]];
              X[1][k] = L.y[node[k]];
              X[2][k] = L.zc[node[k]];
            }
            double J[3][3];
            for (int a = 0; a < 3; ++a)
              for (int b = 0; b < 3; ++b) {
                J[a][b] = 0;
                for (int k = 0; k < 4; ++k) J[a][b] += X[a][k] * grad[k][b];
              }
            const double det = J[0][0] * (J[1][1] * J[2][2] - J[2][1] * J[1][2]) -
                               J[0][1] * (J[1][0] * J[2][2] - J[2][0] * J[1][2]) +
                               J[0][2] * (J[1][0] * J[2][1] - J[2][0] * J[1][1]);
            const double inv = 1.0 / det;
            const double Ji[3][3] = {{inv * (J[1][1] * J[2][2] - J[2][1] * J[1][2]), inv * (J[0][2] * J[2][1] - J[2][2] * J[0][1]),
                                      inv * (J[0][1] * J[1][2] - J[1][1] * J[0][2])},
                                     {inv * (J[1][2] * J[2][0] - J[2][2] * J[1][0]), inv * (J[0][0] * J[2][2] - J[2][0] * J[0][2]),
                                      inv * (J[0][2] * J[1][0] - J[1][2] * J[0][0])},
                                     {inv * (J[1][0] * J[2][1] - J[2][0] * J[1][1]), inv * (J[0][1] * J[2][0] - J[2][1] * J[0][0]),
                                      inv * (J[0][0] * J[1][1] - J[1][0] * J[0][1])}};
            double Aloc[4][4] = {};
            for (int q = 0; q < 4; ++q)
              for (int i = 0; i < 4; ++i)
                for (int j = 0; j < 4; ++j) {
                  double f = 0;
                  for (int al = 0; al < 3; ++al) {
                    double a = 0, b = 0;
                    for (int be = 0; be < 3; ++be) {
                      a += grad[i][be] * Ji[be][al];
                      b += grad[j][be] * Ji[be][al];
                    }
                    f += a * b;
                  }
                  Aloc[i][j] += f * det * (1.0 / 24.0);
                }
            for (int i = 0; i < 4; ++i)
              for (int j = 0; j < 4; ++j) {
                const long long r = num[node[i]], c = num[node[j]];
                if (r < 0 || c < 0) continue;
                float &v = entries[{r, c}];
                v += lambda0 * Aloc[i][j];
              }
          }
  rowPtr.assign(ng + 1, 0);
  cols.clear();
  vals.clear();
  for (const auto &kv : entries) {
    if (!(std::fabs((double)kv.second) > 0.0)) continue;
    cols.push_back(kv.first.second);
    vals.push_back(kv.second);
    rowPtr[kv.first.first + 1]++;
  }
  for (long long r = 0; r < ng; ++r) rowPtr[r + 1] += rowPtr[r];
}

} // namespace orc
