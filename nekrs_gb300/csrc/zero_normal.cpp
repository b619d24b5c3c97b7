// Zero-normal (symmetry) boundaries of any orientation for the three-field
// block solve: face type 2 among the first field's types.  At setup every node
// of an element that lies on one of the element's zero-normal faces becomes
// one entry: its E-vector index, the number of such faces of the element
// through it, the orthonormal frame (n, t1, t2) of its averaged normal and its
// mask (maskN, maskT1, maskT2).  The solve projects every entry's three field
// values on the frame (launch_zero_normal) before the Dirichlet mask and the
// gather-scatter, as ellipticApplyMask does (ellipticApplyMask.cpp:19-23,
// applyZeroNormalMask.okl).
//
// Setup follows the reference's construction:
//   face normals   surfaceGeometricFactorsHex3D.okl: faces t-, s-, r+, s+, r-,
//                  t+ take -grad t, -grad s, +grad r, +grad s, -grad r,
//                  +grad t, normalised;
//   node types     createEToBV.cpp: min over the faces through a node (types >
//                  0) across all its copies, none -> 0;
//   mask           initializeZeroNormalMask.okl: (0, 1, 1) at zero-normal
//                  nodes, (1, 1, 1) elsewhere;
//   normal frame   createZeroNormalMask (applyDirichlet.cpp:7-33): the
//                  zero-normal faces' normals summed per element in face
//                  order with a count, summed over the node's copies, averaged
//                  and normalised; t1 = (-ny, nx, 0) / |.| or (1, 0, 0) when
//                  |nz| ~ 1, t2 = n x t1 normalised (fixZeroNormalMask.okl).
// A node on k zero-normal faces of its element is projected k times, as the
// reference's face-by-face loop does.
#include "elliptic.hpp"

#include <cmath>

namespace nrsg {

namespace {

// volume node (i, j, k) of face node (a, b) of face f, nekRS face order t-, s-, r+, s+, r-, t+
int face_node(int nq, int f, int a, int b)
{
  int i = a, j = b, k = 0;
  if (f == 1) { i = a; j = 0; k = b; }
  else if (f == 2) { i = nq - 1; j = a; k = b; }
  else if (f == 3) { i = a; j = nq - 1; k = b; }
  else if (f == 4) { i = 0; j = a; k = b; }
  else if (f == 5) { i = a; j = b; k = nq - 1; }
  return i + nq * (j + nq * k);
}

// node coordinates of element e (trilinear map of its 8 vertices, one fused multiply-add per vertex)
void element_coords(const FieldLevel &L, long long e, std::vector<double> &x, std::vector<double> &y,
                    std::vector<double> &z)
{
  const int nq = L.Nq;
  x.assign((size_t)L.Np, 0.0);
  y.assign((size_t)L.Np, 0.0);
  z.assign((size_t)L.Np, 0.0);
  const double *v = L.VXh.data() + e * 24;
  for (int k = 0; k < nq; ++k)
    for (int j = 0; j < nq; ++j)
      for (int i = 0; i < nq; ++i) {
        const double hr[2] = {0.5 * (1 - L.z[i]), 0.5 * (1 + L.z[i])};
        const double hs[2] = {0.5 * (1 - L.z[j]), 0.5 * (1 + L.z[j])};
        const double ht[2] = {0.5 * (1 - L.z[k]), 0.5 * (1 + L.z[k])};
        double X = 0, Y = 0, Z = 0;
        for (int q = 0; q < 8; ++q) {
          const double wv = hr[q & 1] * hs[(q >> 1) & 1] * ht[(q >> 2) & 1];
          X = std::fma(wv, v[q * 3 + 0], X);
          Y = std::fma(wv, v[q * 3 + 1], Y);
          Z = std::fma(wv, v[q * 3 + 2], Z);
        }
        const int n = i + nq * (j + nq * k);
        x[n] = X;
        y[n] = Y;
        z[n] = Z;
      }
}

// unit outward normal of face f at volume node n from the element's node coordinates
void unit_normal(const FieldLevel &L, const std::vector<double> &xe, const std::vector<double> &ye,
                 const std::vector<double> &ze, int f, int n, double out[3])
{
  const int nq = L.Nq;
  const double *D = L.Dh.data();
  const int i = n % nq, j = (n / nq) % nq, k = n / (nq * nq);
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
  double g0, g1, g2; // gradient of the reference coordinate normal to the face
  if (f == 0 || f == 5) {
    g0 = minor2(yr, zs, zr, ys) * Ji, g1 = -minor2(xr, zs, zr, xs) * Ji, g2 = minor2(xr, ys, yr, xs) * Ji;
  } else if (f == 1 || f == 3) {
    g0 = -minor2(yr, zt, zr, yt) * Ji, g1 = minor2(xr, zt, zr, xt) * Ji, g2 = -minor2(xr, yt, yr, xt) * Ji;
  } else {
    g0 = cx * Ji, g1 = -cy * Ji, g2 = cz * Ji;
  }
  const double sgn = (f == 0 || f == 1 || f == 4) ? -1.0 : 1.0;
  const double nx = sgn * g0, ny = sgn * g1, nz = sgn * g2;
  const double invSJ = 1.0 / std::sqrt(nx * nx + ny * ny + nz * nz);
  out[0] = nx * invSJ;
  out[1] = ny * invSJ;
  out[2] = nz * invSJ;
}

} // namespace

void build_zero_normal(const FieldLevel &L, const int *EToB0, ZeroNormalPlan &P)
{
  P = ZeroNormalPlan();
  const int nq = L.Nq, nfp = nq * nq;
  const long long np = L.Np, nl = L.Nlocal;
  bool any = false;
  for (long long q = 0; q < L.E * 6 && !any; ++q) any = EToB0[q] == 2;
  if (!any) return;
  // node types
  const int none = 1 << 20;
  std::vector<int> type((size_t)nl, none);
  for (long long e = 0; e < L.E; ++e)
    for (int f = 0; f < 6; ++f) {
      const int bc = EToB0[6 * e + f];
      if (bc <= 0) continue;
      for (int q = 0; q < nfp; ++q) {
        int &t = type[(size_t)(e * np + face_node(nq, f, q % nq, q / nq))];
        t = std::min(t, bc);
      }
    }
  for (size_t g = 0; g + 1 < L.um.off.size(); ++g) {
    int t = none;
    for (int q = L.um.off[g]; q < L.um.off[g + 1]; ++q) t = std::min(t, type[(size_t)L.um.ids[q]]);
    for (int q = L.um.off[g]; q < L.um.off[g + 1]; ++q) type[(size_t)L.um.ids[q]] = t;
  }
  // summed normals and counts per node copy, then over the copies
  std::vector<double> sum((size_t)4 * nl, 0.0);
  std::vector<double> xe, ye, ze;
  for (long long e = 0; e < L.E; ++e) {
    bool has = false;
    for (int f = 0; f < 6; ++f) has = has || EToB0[6 * e + f] == 2;
    if (!has) continue;
    element_coords(L, e, xe, ye, ze);
    for (int f = 0; f < 6; ++f) {
      if (EToB0[6 * e + f] != 2) continue;
      for (int q = 0; q < nfp; ++q) {
        const int vn = face_node(nq, f, q % nq, q / nq);
        const size_t id = (size_t)(e * np + vn);
        double nv[3];
        unit_normal(L, xe, ye, ze, f, vn, nv);
        sum[id] += nv[0];
        sum[id + nl] += nv[1];
        sum[id + 2 * nl] += nv[2];
        sum[id + 3 * nl] += 1;
      }
    }
  }
  for (int c = 0; c < 4; ++c)
    for (size_t g = 0; g + 1 < L.um.off.size(); ++g) {
      double v = 0;
      for (int q = L.um.off[g]; q < L.um.off[g + 1]; ++q) v += sum[(size_t)L.um.ids[q] + c * nl];
      for (int q = L.um.off[g]; q < L.um.off[g + 1]; ++q) sum[(size_t)L.um.ids[q] + c * nl] = v;
    }
  // entries: the element's nodes on its zero-normal faces, in order of first appearance
  std::vector<int> reps((size_t)np);
  for (long long e = 0; e < L.E; ++e) {
    bool has = false;
    for (int f = 0; f < 6; ++f) has = has || EToB0[6 * e + f] == 2;
    if (!has) continue;
    std::fill(reps.begin(), reps.end(), 0);
    std::vector<int> order;
    for (int f = 0; f < 6; ++f) {
      if (EToB0[6 * e + f] != 2) continue;
      for (int q = 0; q < nfp; ++q) {
        const int vn = face_node(nq, f, q % nq, q / nq);
        if (reps[vn]++ == 0) order.push_back(vn);
      }
    }
    for (int vn : order) {
      const size_t id = (size_t)(e * np + vn);
      double vx = sum[id], vy = sum[id + nl], vz = sum[id + 2 * nl];
      const double invCount = 1.0 / sum[id + 3 * nl];
      vx *= invCount;
      vy *= invCount;
      vz *= invCount;
      const double invMag = 1.0 / std::sqrt(vx * vx + vy * vy + vz * vz);
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
      P.node.push_back((int)id);
      P.reps.push_back((unsigned char)reps[vn]);
      const double fr[9] = {nx, ny, nz, t1x, t1y, t1z, t2x, t2y, t2z};
      P.frame.insert(P.frame.end(), fr, fr + 9);
      const double mN = type[id] == 2 ? 0.0 : 1.0;
      P.mask.push_back(mN);
      P.mask.push_back(1.0);
      P.mask.push_back(1.0);
    }
  }
}

} // namespace nrsg
