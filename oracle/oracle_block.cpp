// ORACLE — test infrastructure only (see oracle_mesh.cpp header).
//
// Block (vector) Helmholtz restated for the parity tests: Nfields fields at
// fieldOffset = Nlocal, per-node coefficients lambda0 / lambda1 (p_lambda = 1,
// loffset 0 or Nlocal) or scalar ones.
//   block axhelm   kernels/elliptic/ellipticBlockPartialAxCoeffHex3D.c:1-146
//   stress axhelm  kernels/elliptic/ellipticStressPartialAxCoeffHex3D.c:1-170
//                  on the volume factors vgeo (mesh3D.h:82-93, from
//                  geometricFactorsHex3D as the oracle's ggeo)
//   block diagonal kernels/elliptic/ellipticBlockBuildDiagonalHex3D.okl:30-110
//                  (also the stress form's Jacobi, ellipticUpdateJacobi.cpp:63)
//   solve          ellipticSolve.cpp:32-190 with PCG.cpp:86-203 and
//                  ellipticBlockUpdatePCG.c over Nfields fields, norms
//                  weightedNorm2Many (sum over fields, invDegree per node);
//                  zero-normal boundaries below (BlockSolver's op and residual).
#include "oracle_internal.hpp"

#include <cmath>
#include <cstring>

namespace orc {

struct BlockSpec {
  int nf = 1;
  bool stress = false, poisson = false;
  long long loffset = 0;
  const double *lam0 = nullptr, *lam1 = nullptr; // null: scalar l0 / l1
  double l0 = 1, l1 = 0;
  double c0(long long id, int f) const { return lam0 ? lam0[id + f * loffset] : l0; }
  double c1(long long id, int f) const { return lam1 ? lam1[id + f * loffset] : l1; }
};

// vgeo [E][12][Np]: rx ry rz sx sy sz tx ty tz J JW 1/JW
void vgeo_factors(const Level &L, std::vector<double> &vg)
{
  const int nq = L.Nq, np = L.Np;
  vg.assign((size_t)L.E * 12 * np, 0.0);
  const double *D = L.D.data();
  for (long long e = 0; e < L.E; ++e) {
    const double *xe = &L.x[e * np], *ye = &L.y[e * np], *ze = &L.zc[e * np];
    for (int k = 0; k < nq; ++k)
      for (int j = 0; j < nq; ++j)
        for (int i = 0; i < nq; ++i) {
          double xr = 0, xs = 0, xt = 0, yr = 0, ys = 0, yt = 0, zr = 0, zs = 0, zt = 0;
          for (int m = 0; m < nq; ++m) {
            const int ir = m + nq * (j + nq * k), is = i + nq * (m + nq * k), it = i + nq * (j + nq * m);
            xr += D[i * nq + m] * xe[ir];
            xs += D[j * nq + m] * xe[is];
            xt += D[k * nq + m] * xe[it];
            yr += D[i * nq + m] * ye[ir];
            ys += D[j * nq + m] * ye[is];
            yt += D[k * nq + m] * ye[it];
            zr += D[i * nq + m] * ze[ir];
            zs += D[j * nq + m] * ze[is];
            zt += D[k * nq + m] * ze[it];
          }
          const double J = xr * (ys * zt - zs * yt) - yr * (xs * zt - zs * xt) + zr * (xs * yt - ys * xt);
          const double Ji = 1.0 / J;
          const double JW = J * L.w[i] * L.w[j] * L.w[k];
          const int n = i + nq * (j + nq * k);
          double *g = &vg[(size_t)e * 12 * np];
          g[0 * np + n] = (ys * zt - zs * yt) * Ji;
          g[1 * np + n] = -(xs * zt - zs * xt) * Ji;
          g[2 * np + n] = (xs * yt - ys * xt) * Ji;
          g[3 * np + n] = -(yr * zt - zr * yt) * Ji;
          g[4 * np + n] = (xr * zt - zr * xt) * Ji;
          g[5 * np + n] = -(xr * yt - yr * xt) * Ji;
          g[6 * np + n] = (yr * zs - zr * ys) * Ji;
          g[7 * np + n] = -(xr * zs - zr * xs) * Ji;
          g[8 * np + n] = (xr * ys - yr * xs) * Ji;
          g[9 * np + n] = J;
          g[10 * np + n] = JW;
          g[11 * np + n] = 1.0 / JW;
        }
  }
}

// ellipticBlockPartialAxCoeffHex3D: per field, lambda0 inside the gradient
// term, GwJ lambda1 q added last
void block_ax(const Level &L, const BlockSpec &S, const double *q, double *Aq)
{
  const int nq = L.Nq, np = L.Np;
  const long long off = L.Nlocal;
  const double *D = L.D.data();
#pragma omp parallel for
  for (long long e = 0; e < L.E; ++e) {
    std::vector<double> Gr(np), Gs(np), Gt(np);
    const double *g = &L.ggeo[(size_t)e * 7 * np];
    for (int f = 0; f < S.nf; ++f) {
      const double *qe = q + f * off + e * np;
      for (int k = 0; k < nq; ++k)
        for (int j = 0; j < nq; ++j)
          for (int i = 0; i < nq; ++i) {
            const int n = i + nq * (j + nq * k);
            double qr = 0, qs = 0, qt = 0;
            for (int m = 0; m < nq; ++m) {
              qr += D[i * nq + m] * qe[m + nq * (j + nq * k)];
              qs += D[j * nq + m] * qe[i + nq * (m + nq * k)];
              qt += D[k * nq + m] * qe[i + nq * (j + nq * m)];
            }
            const double G00 = g[0 * np + n], G01 = g[1 * np + n], G11 = g[2 * np + n];
            const double G12 = g[3 * np + n], G02 = g[4 * np + n], G22 = g[5 * np + n];
            const double lam = S.c0(e * np + n, f);
            Gr[n] = lam * (G00 * qr + G01 * qs + G02 * qt);
            Gs[n] = lam * (G01 * qr + G11 * qs + G12 * qt);
            Gt[n] = lam * (G02 * qr + G12 * qs + G22 * qt);
          }
      for (int k = 0; k < nq; ++k)
        for (int j = 0; j < nq; ++j)
          for (int i = 0; i < nq; ++i) {
            const int n = i + nq * (j + nq * k);
            const double a0 = S.poisson ? 0.0 : g[6 * np + n] * S.c1(e * np + n, f) * qe[n];
            double ar = 0, as = 0, at = 0;
            for (int m = 0; m < nq; ++m) ar += D[m * nq + i] * Gr[m + nq * (j + nq * k)];
            for (int m = 0; m < nq; ++m) as += D[m * nq + j] * Gs[i + nq * (m + nq * k)];
            for (int m = 0; m < nq; ++m) at += D[m * nq + k] * Gt[i + nq * (j + nq * m)];
            Aq[f * off + e * np + n] = ar + as + at + a0;
          }
    }
  }
}

// ellipticStressPartialAxCoeffHex3D: symmetric-gradient (stress) operator,
// the three fields coupled
void stress_ax(const Level &L, const BlockSpec &S, const std::vector<double> &vg, const double *q, double *Aq)
{
  const int nq = L.Nq, np = L.Np;
  const long long off = L.Nlocal;
  const double *D = L.D.data();
#pragma omp parallel for
  for (long long e = 0; e < L.E; ++e) {
    std::vector<double> SU[3], SV[3], SW[3];
    for (int d = 0; d < 3; ++d) SU[d].resize(np), SV[d].resize(np), SW[d].resize(np);
    const double *U = q + e * np, *V = q + off + e * np, *W = q + 2 * off + e * np;
    const double *g = &vg[(size_t)e * 12 * np];
    for (int k = 0; k < nq; ++k)
      for (int j = 0; j < nq; ++j)
        for (int i = 0; i < nq; ++i) {
          const int n = i + nq * (j + nq * k);
          double ur = 0, us = 0, ut = 0, vr = 0, vs = 0, vt = 0, wr = 0, ws = 0, wt = 0;
          for (int m = 0; m < nq; ++m) {
            const double Dim = D[i * nq + m], Djm = D[j * nq + m], Dkm = D[k * nq + m];
            const int ir = m + nq * (j + nq * k), is = i + nq * (m + nq * k), it = i + nq * (j + nq * m);
            ur += Dim * U[ir];
            us += Djm * U[is];
            ut += Dkm * U[it];
            vr += Dim * V[ir];
            vs += Djm * V[is];
            vt += Dkm * V[it];
            wr += Dim * W[ir];
            ws += Djm * W[is];
            wt += Dkm * W[it];
          }
          const double rx = g[0 * np + n], ry = g[1 * np + n], rz = g[2 * np + n];
          const double sx = g[3 * np + n], sy = g[4 * np + n], sz = g[5 * np + n];
          const double tx = g[6 * np + n], ty = g[7 * np + n], tz = g[8 * np + n];
          const double JW = g[10 * np + n];
          const long long id = e * np + n;
          const double ul = S.c0(id, 0), vl = S.c0(id, 1), wl = S.c0(id, 2);
          const double dudx = rx * ur + sx * us + tx * ut, dudy = ry * ur + sy * us + ty * ut,
                       dudz = rz * ur + sz * us + tz * ut;
          const double dvdx = rx * vr + sx * vs + tx * vt, dvdy = ry * vr + sy * vs + ty * vt,
                       dvdz = rz * vr + sz * vs + tz * vt;
          const double dwdx = rx * wr + sx * ws + tx * wt, dwdy = ry * wr + sy * ws + ty * wt,
                       dwdz = rz * wr + sz * ws + tz * wt;
          const double s11 = ul * JW * (dudx + dudx), s12 = ul * JW * (dudy + dvdx), s13 = ul * JW * (dudz + dwdx);
          const double s21 = vl * JW * (dvdx + dudy), s22 = vl * JW * (dvdy + dvdy), s23 = vl * JW * (dvdz + dwdy);
          const double s31 = wl * JW * (dwdx + dudz), s32 = wl * JW * (dwdy + dvdz), s33 = wl * JW * (dwdz + dwdz);
          SU[0][n] = rx * s11 + ry * s12 + rz * s13;
          SU[1][n] = sx * s11 + sy * s12 + sz * s13;
          SU[2][n] = tx * s11 + ty * s12 + tz * s13;
          SV[0][n] = rx * s21 + ry * s22 + rz * s23;
          SV[1][n] = sx * s21 + sy * s22 + sz * s23;
          SV[2][n] = tx * s21 + ty * s22 + tz * s23;
          SW[0][n] = rx * s31 + ry * s32 + rz * s33;
          SW[1][n] = sx * s31 + sy * s32 + sz * s33;
          SW[2][n] = tx * s31 + ty * s32 + tz * s33;
        }
    for (int k = 0; k < nq; ++k)
      for (int j = 0; j < nq; ++j)
        for (int i = 0; i < nq; ++i) {
          const int n = i + nq * (j + nq * k);
          double au = 0, av = 0, aw = 0;
          for (int m = 0; m < nq; ++m) {
            const double Dim = D[m * nq + i], Djm = D[m * nq + j], Dkm = D[m * nq + k];
            const int ir = m + nq * (j + nq * k), is = i + nq * (m + nq * k), it = i + nq * (j + nq * m);
            au += Dim * SU[0][ir];
            au += Djm * SU[1][is];
            au += Dkm * SU[2][it];
            av += Dim * SV[0][ir];
            av += Djm * SV[1][is];
            av += Dkm * SV[2][it];
            aw += Dim * SW[0][ir];
            aw += Djm * SW[1][is];
            aw += Dkm * SW[2][it];
          }
          const long long id = e * np + n;
          const double JW = g[10 * np + n];
          Aq[id] = au + S.c1(id, 0) * JW * U[n];
          Aq[off + id] = av + S.c1(id, 1) * JW * V[n];
          Aq[2 * off + id] = aw + S.c1(id, 2) * JW * W[n];
        }
  }
}

// ellipticBlockBuildDiagonalHex3D (per field; lambda0 per node)
void block_diag(const Level &L, const BlockSpec &S, double *diag)
{
  const int nq = L.Nq, np = L.Np;
  const double *D = L.D.data();
#pragma omp parallel for
  for (long long e = 0; e < L.E; ++e) {
    const double *g = &L.ggeo[(size_t)e * 7 * np];
    for (int f = 0; f < S.nf; ++f)
      for (int k = 0; k < nq; ++k)
        for (int j = 0; j < nq; ++j)
          for (int i = 0; i < nq; ++i) {
            const int n = i + nq * (j + nq * k);
            const long long id = e * np + n;
            const double lam = S.c0(id, f);
            double r = 0;
            r += 2.0 * g[1 * np + n] * lam * D[i * nq + i] * D[j * nq + j];
            r += 2.0 * g[4 * np + n] * lam * D[i * nq + i] * D[k * nq + k];
            r += 2.0 * g[3 * np + n] * lam * D[j * nq + j] * D[k * nq + k];
            for (int m = 0; m < nq; ++m) {
              const int a = m + nq * (j + nq * k), b = i + nq * (m + nq * k), c = i + nq * (j + nq * m);
              r += g[0 * np + a] * S.c0(e * np + a, f) * D[m * nq + i] * D[m * nq + i];
              r += g[2 * np + b] * S.c0(e * np + b, f) * D[m * nq + j] * D[m * nq + j];
              r += g[5 * np + c] * S.c0(e * np + c, f) * D[m * nq + k] * D[m * nq + k];
            }
            if (!S.poisson) r += g[6 * np + n] * S.c1(id, f);
            diag[f * L.Nlocal + id] = r;
          }
  }
}

// ---------------------------------------------------------------------------
// Zero-normal (symmetry) condition on boundaries of any orientation, face type
// ZERO_NORMAL = 2 (elliptic.h:44-49; only the block solver takes it,
// ellipticSetup.cpp:94-110), restated from
//   face normals   kernels/mesh/surfaceGeometricFactorsHex3D.okl: the normal
//                  of faces t-, s-, r+, s+, r-, t+ is -grad t, -grad s,
//                  +grad r, +grad s, -grad r, +grad t, normalised
//   node types     src/bdry/createEToBV.cpp: min over the faces through a
//                  node (face types > 0), ogsMin, "none" -> 0; taken from the
//                  first field's types (setup.cpp:810-817)
//   mask           kernels/nrs/initializeZeroNormalMask.okl: (0, 1, 1) at
//                  zero-normal nodes, (1, 1, 1) elsewhere
//   normals        applyDirichlet.cpp:7-33 createZeroNormalMask:
//                  averageNormalBcType.okl (sum of the zero-normal faces'
//                  normals and their count per node, per element in face
//                  order) + ogsAdd, then fixZeroNormalMask.okl (the averaged
//                  normal, its tangents t1 = (-ny, nx, 0) / |.| or (1, 0, 0)
//                  when |nz| ~ 1, t2 = n x t1 normalised; its tolerance 1
//                  makes this branch the only one taken)
//   application    kernels/nrs/applyZeroNormalMask.okl (per element, face by
//                  face, each face node: U = (U.n) maskN n + (U.t1) maskT1 t1 +
//                  (U.t2) maskT2 t2), called first in ellipticApplyMask
//                  (ellipticApplyMask.cpp:19-23), i.e. before the Dirichlet
//                  mask and the gather-scatter
// ---------------------------------------------------------------------------
struct ZeroNormal {
  bool active = false;
  int nq = 0, np = 0;
  long long E = 0, Nlocal = 0;
  std::vector<int> EToB0;    // [e][6]
  std::vector<double> sgeo;  // [e][f][nq * nq][9]: n, t1, t2 of zero-normal faces
  std::vector<double> mask;  // [3][Nlocal]
};

static int face_volume_node(int nq, int f, int a, int b)
{
  int i, j, k;
  switch (f) {
  case 0: i = a; j = b; k = 0; break;
  case 1: i = a; j = 0; k = b; break;
  case 2: i = nq - 1; j = a; k = b; break;
  case 3: i = a; j = nq - 1; k = b; break;
  case 4: i = 0; j = a; k = b; break;
  default: i = a; j = b; k = nq - 1; break;
  }
  return i + nq * (j + nq * k);
}

// unit outward normal of face f at volume node n of element e (the reference's surface factors)
static void face_normal(const Level &L, long long e, int f, int n, double out[3])
{
  const int nq = L.Nq, np = L.Np;
  const int i = n % nq, j = (n / nq) % nq, k = n / (nq * nq);
  const double *xe = &L.x[e * np], *ye = &L.y[e * np], *ze = &L.zc[e * np], *D = L.D.data();
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
  auto minor2 = [](double a, double b, double c, double d) { return std::fma(a, b, -(c * d)); };
  const double cx = minor2(ys, zt, zs, yt), cy = minor2(xs, zt, zs, xt), cz = minor2(xs, yt, ys, xt);
  const double J = std::fma(zr, cz, std::fma(-yr, cy, xr * cx));
  const double Ji = 1.0 / J;
  double g[3];
  switch (f) {
  case 0:
  case 5: // t
    g[0] = minor2(yr, zs, zr, ys) * Ji, g[1] = -minor2(xr, zs, zr, xs) * Ji, g[2] = minor2(xr, ys, yr, xs) * Ji;
    break;
  case 1:
  case 3: // s
    g[0] = -minor2(yr, zt, zr, yt) * Ji, g[1] = minor2(xr, zt, zr, xt) * Ji, g[2] = -minor2(xr, yt, yr, xt) * Ji;
    break;
  default: // r
    g[0] = cx * Ji, g[1] = -cy * Ji, g[2] = cz * Ji;
    break;
  }
  const double sgn = (f == 0 || f == 1 || f == 4) ? -1.0 : 1.0;
  double nx = sgn * g[0], ny = sgn * g[1], nz = sgn * g[2];
  const double sJ = std::sqrt(nx * nx + ny * ny + nz * nz);
  const double invSJ = 1.0 / sJ;
  out[0] = nx * invSJ;
  out[1] = ny * invSJ;
  out[2] = nz * invSJ;
}

void build_zero_normal(const Level &L, const int *EToB0, ZeroNormal &Z)
{
  const int nq = L.Nq, np = L.Np, nfp = nq * nq;
  Z = ZeroNormal();
  Z.nq = nq;
  Z.np = np;
  Z.E = L.E;
  Z.Nlocal = L.Nlocal;
  Z.EToB0.assign(EToB0, EToB0 + L.E * 6);
  for (long long q = 0; q < L.E * 6; ++q)
    if (EToB0[q] == 2) Z.active = true;
  if (!Z.active) return;
  std::vector<int> off, gid;
  std::vector<double> invd;
  ogs_setup(L.Nlocal, L.ids.data(), off, gid, invd);
  // createEToBV
  const int large = 1 << 20;
  std::vector<int> bv((size_t)L.Nlocal, large);
  for (long long e = 0; e < L.E; ++e)
    for (int f = 0; f < 6; ++f) {
      const int bc = EToB0[e * 6 + f];
      if (bc <= 0) continue;
      for (int n = 0; n < nfp; ++n) {
        int &v = bv[e * np + face_volume_node(nq, f, n % nq, n / nq)];
        v = std::min(v, bc);
      }
    }
  for (size_t g = 0; g + 1 < off.size(); ++g) {
    int v = large;
    for (int q = off[g]; q < off[g + 1]; ++q) v = std::min(v, bv[gid[q]]);
    for (int q = off[g]; q < off[g + 1]; ++q) bv[gid[q]] = v;
  }
  for (auto &v : bv)
    if (v == large) v = 0;
  // initializeZeroNormalMask
  Z.mask.assign((size_t)3 * L.Nlocal, 1.0);
  for (long long id = 0; id < L.Nlocal; ++id)
    if (bv[id] == 2) Z.mask[id] = 0.0;
  // averageNormalBcType + ogsAdd over the four fields
  std::vector<double> nrm((size_t)4 * L.Nlocal, 0.0);
  const long long off4 = L.Nlocal;
  for (long long e = 0; e < L.E; ++e)
    for (int f = 0; f < 6; ++f) {
      if (EToB0[e * 6 + f] != 2) continue;
      for (int n = 0; n < nfp; ++n) {
        const int vn = face_volume_node(nq, f, n % nq, n / nq);
        const long long id = e * np + vn;
        double fnv[3];
        face_normal(L, e, f, vn, fnv);
        nrm[id + 0 * off4] += fnv[0];
        nrm[id + 1 * off4] += fnv[1];
        nrm[id + 2 * off4] += fnv[2];
        nrm[id + 3 * off4] += 1;
      }
    }
  for (int c = 0; c < 4; ++c)
    for (size_t g = 0; g + 1 < off.size(); ++g) {
      double v = 0;
      for (int q = off[g]; q < off[g + 1]; ++q) v += nrm[gid[q] + c * off4];
      for (int q = off[g]; q < off[g + 1]; ++q) nrm[gid[q] + c * off4] = v;
    }
  // fixZeroNormalMask
  Z.sgeo.assign((size_t)L.E * 6 * nfp * 9, 0.0);
  for (long long e = 0; e < L.E; ++e)
    for (int f = 0; f < 6; ++f) {
      if (EToB0[e * 6 + f] != 2) continue;
      for (int n = 0; n < nfp; ++n) {
        const long long id = e * np + face_volume_node(nq, f, n % nq, n / nq);
        double vx = nrm[id], vy = nrm[id + off4], vz = nrm[id + 2 * off4];
        const double invCount = 1.0 / nrm[id + 3 * off4];
        vx *= invCount;
        vy *= invCount;
        vz *= invCount;
        const double mag = std::sqrt(vx * vx + vy * vy + vz * vz);
        const double invMag = 1.0 / mag;
        const double nx = vx * invMag, ny = vy * invMag, nz = vz * invMag;
        double t1x, t1y, t1z;
        if (std::fabs(std::fabs(nz) - 1.0) < 1e-4) {
          t1x = 1.0, t1y = 0.0, t1z = 0.0;
        } else {
          const double m2 = std::sqrt(nx * nx + ny * ny);
          t1x = -ny / m2, t1y = nx / m2, t1z = 0.0;
        }
        double t2x = ny * t1z - nz * t1y, t2y = nz * t1x - nx * t1z, t2z = nx * t1y - ny * t1x;
        const double inv2 = 1.0 / std::sqrt(t2x * t2x + t2y * t2y + t2z * t2z);
        t2x *= inv2;
        t2y *= inv2;
        t2z *= inv2;
        double *sg = &Z.sgeo[(((size_t)e * 6 + f) * nfp + n) * 9];
        sg[0] = nx, sg[1] = ny, sg[2] = nz;
        sg[3] = t1x, sg[4] = t1y, sg[5] = t1z;
        sg[6] = t2x, sg[7] = t2y, sg[8] = t2z;
      }
    }
}

// applyZeroNormalMask on three fields at offset Nlocal
void apply_zero_normal(const ZeroNormal &Z, double *U)
{
  if (!Z.active) return;
  const int nfp = Z.nq * Z.nq;
  const long long off = Z.Nlocal;
  for (long long e = 0; e < Z.E; ++e)
    for (int f = 0; f < 6; ++f) {
      if (Z.EToB0[e * 6 + f] != 2) continue;
      for (int n = 0; n < nfp; ++n) {
        const long long id = e * Z.np + face_volume_node(Z.nq, f, n % Z.nq, n / Z.nq);
        const double *sg = &Z.sgeo[(((size_t)e * 6 + f) * nfp + n) * 9];
        const double mN = Z.mask[id], mT1 = Z.mask[id + off], mT2 = Z.mask[id + 2 * off];
        const double u = U[id], v = U[id + off], w = U[id + 2 * off];
        const double Rn = (u * sg[0] + v * sg[1] + w * sg[2]) * mN;
        const double R1 = (u * sg[3] + v * sg[4] + w * sg[5]) * mT1;
        const double R2 = (u * sg[6] + v * sg[7] + w * sg[8]) * mT2;
        U[id] = Rn * sg[0] + R1 * sg[3] + R2 * sg[6];
        U[id + off] = Rn * sg[1] + R1 * sg[4] + R2 * sg[7];
        U[id + 2 * off] = Rn * sg[2] + R1 * sg[5] + R2 * sg[8];
      }
    }
}

struct BlockSolver {
  const Level &L;
  BlockSpec S;
  std::vector<double> vg, invDiag, w;
  bool jacobi;
  // per-field boundary types (elliptic->EToB with Nfields sections): the mask and gather groups of field f
  std::vector<Level> fieldLevels;
  ZeroNormal zn; // zero-normal faces among the first field's types (three fields)
  const Level &FL(int f) const { return fieldLevels.empty() ? L : fieldLevels[f]; }
  BlockSolver(const Level &L_, const BlockSpec &S_, bool jac, const int *EToBfields = nullptr)
      : L(L_), S(S_), jacobi(jac)
  {
    if (EToBfields) {
      fieldLevels.resize(S.nf);
      for (int f = 0; f < S.nf; ++f)
        build_level(fieldLevels[f], L.N, L.E, L.VX.data(), L.EToV.data(), EToBfields + (size_t)f * L.E * 6);
      if (S.nf == 3) build_zero_normal(L, EToBfields, zn);
    }
    if (S.stress) vgeo_factors(L, vg);
    const long long n = L.Nlocal * S.nf;
    w.resize(n);
    for (int f = 0; f < S.nf; ++f)
      for (long long i = 0; i < L.Nlocal; ++i) w[f * L.Nlocal + i] = L.invDegree[i];
    if (jacobi) {
      invDiag.resize(n);
      block_diag(L, S, invDiag.data());
      for (int f = 0; f < S.nf; ++f) gs_add(FL(f), invDiag.data() + f * L.Nlocal);
      for (long long i = 0; i < n; ++i) invDiag[i] = 1.0 / invDiag[i];
    }
  }
  void ax(const double *q, double *Aq) const
  {
    if (S.stress) stress_ax(L, S, vg, q, Aq);
    else block_ax(L, S, q, Aq);
  }
  void op(const double *q, double *Aq) const
  {
    ax(q, Aq);
    apply_zero_normal(zn, Aq);
    for (int f = 0; f < S.nf; ++f) {
      apply_mask(FL(f), Aq + f * L.Nlocal);
      gs_add(FL(f), Aq + f * L.Nlocal);
    }
  }
  double norm(const double *r) const
  {
    return std::sqrt(wdot<double>(L.Nlocal * S.nf, w.data(), r, r) / L.volume);
  }
  // ellipticSolve + PCG over all fields
  int solve(double *r, double *x, double tol, bool relative, int maxit, double &res0, double &res, int &status) const
  {
    const long long n = L.Nlocal * S.nf;
    std::vector<double> x0(x, x + n), Ax0(n), p(n, 0.0), z(n), Ap(n);
    ax(x, Ax0.data());
    for (long long i = 0; i < n; ++i) r[i] = -Ax0[i] + r[i];
    apply_zero_normal(zn, r);
    for (int f = 0; f < S.nf; ++f) {
      apply_mask(FL(f), r + f * L.Nlocal);
      gs_add(FL(f), r + f * L.Nlocal);
    }
    for (long long i = 0; i < n; ++i) x[i] = 0;
    res0 = norm(r);
    if (relative) tol *= res0;
    res = res0;
    status = 0;
    double rdotz1 = 0, alpha = 0;
    int it = 0;
    if (res0 > tol) do {
        ++it;
        const double rdotz2 = rdotz1;
        if (jacobi)
          for (long long i = 0; i < n; ++i) z[i] = r[i] * invDiag[i];
        else
          std::memcpy(z.data(), r, sizeof(double) * n);
        rdotz1 = wdot<double>(n, w.data(), r, z.data());
        const double beta = it > 1 ? rdotz1 / rdotz2 : 0.0;
        for (long long i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
        op(p.data(), Ap.data());
        const double pAp = wdot<double>(n, w.data(), p.data(), Ap.data());
        alpha = rdotz1 / (pAp + 1e-300);
        double rdotr = 0;
        for (long long i = 0; i < n; ++i) {
          r[i] -= alpha * Ap[i];
          rdotr += r[i] * r[i] * w[i];
        }
        for (long long i = 0; i < n; ++i) x[i] += alpha * p[i];
        res = std::sqrt(rdotr / L.volume);
        if (std::isnan(res)) { status = 3; break; }
      } while (res > tol && it < maxit);
    for (long long i = 0; i < n; ++i) x[i] += x0[i];
    if (!status && it >= maxit && res > tol) status = 1;
    return it;
  }
};

} // namespace orc

using namespace orc;

extern "C" {

static BlockSpec make_spec(int nf, int stress, int poisson, long long loffset, const double *lam0, const double *lam1,
                           double l0, double l1)
{
  BlockSpec S;
  S.nf = nf;
  S.stress = stress != 0;
  S.poisson = poisson != 0;
  S.loffset = loffset;
  S.lam0 = lam0;
  S.lam1 = lam1;
  S.l0 = l0;
  S.l1 = l1;
  return S;
}

void orc_block_vgeo(void *h, double *out)
{
  std::vector<double> vg;
  vgeo_factors(((Elliptic *)h)->fine, vg);
  std::memcpy(out, vg.data(), vg.size() * sizeof(double));
}

void orc_block_ax(void *h, int nf, int stress, int poisson, long long loffset, const double *lam0, const double *lam1,
                  double l0, double l1, const double *q, double *Aq)
{
  const Level &L = ((Elliptic *)h)->fine;
  BlockSolver B(L, make_spec(nf, stress, poisson, loffset, lam0, lam1, l0, l1), false);
  B.ax(q, Aq);
}

void orc_block_diag(void *h, int nf, int poisson, long long loffset, const double *lam0, const double *lam1,
                    double l0, double l1, double *invDiag)
{
  const Level &L = ((Elliptic *)h)->fine;
  BlockSolver B(L, make_spec(nf, 0, poisson, loffset, lam0, lam1, l0, l1), true);
  std::memcpy(invDiag, B.invDiag.data(), B.invDiag.size() * sizeof(double));
}

// zero-normal frames of the first field's types EToB0 ([E][6]): sgeo [E][6][Nq^2][9] (n, t1, t2 on zero-normal
// faces, 0 elsewhere) and the mask [3][Nlocal]; returns 1 when some face is zero-normal
int orc_zero_normal(void *h, const int *EToB0, double *sgeo, double *mask)
{
  const Level &L = ((Elliptic *)h)->fine;
  ZeroNormal Z;
  build_zero_normal(L, EToB0, Z);
  if (!Z.active) return 0;
  std::memcpy(sgeo, Z.sgeo.data(), Z.sgeo.size() * sizeof(double));
  std::memcpy(mask, Z.mask.data(), Z.mask.size() * sizeof(double));
  return 1;
}

// applyZeroNormalMask with the frames of EToB0 on three fields U [3][Nlocal]
void orc_apply_zero_normal(void *h, const int *EToB0, double *U)
{
  const Level &L = ((Elliptic *)h)->fine;
  ZeroNormal Z;
  build_zero_normal(L, EToB0, Z);
  apply_zero_normal(Z, U);
}

// info: iterations, res0, res, status
void orc_block_solve(void *h, int nf, int stress, int poisson, long long loffset, const double *lam0,
                     const double *lam1, double l0, double l1, int jacobi, double tol, int relative, int maxit,
                     const int *EToBfields, double *r, double *x, double *info)
{
  const Level &L = ((Elliptic *)h)->fine;
  BlockSolver B(L, make_spec(nf, stress, poisson, loffset, lam0, lam1, l0, l1), jacobi != 0, EToBfields);
  double res0 = 0, res = 0;
  int status = 0;
  const int it = B.solve(r, x, tol, relative != 0, maxit, res0, res, status);
  info[0] = it;
  info[1] = res0;
  info[2] = res;
  info[3] = status;
}

} // extern "C"
