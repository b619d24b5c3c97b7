// Block (vector) Helmholtz kernels, FP64: Nfields fields stored field after
// field (fieldOffset = Nlocal), coefficients either scalars or per-node
// arrays lambda0 / lambda1 (loffset 0: one array shared by the fields;
// loffset = Nlocal: one array per field).
//
// Reference (nekRS kernels/elliptic):
//   ellipticBlockPartialAxCoeffHex3D   per-field axhelm with coefficients
//   ellipticStressPartialAxCoeffHex3D  symmetric-gradient (stress) operator on
//                                      the volume factors vgeo, fields coupled
//   ellipticBlockBuildDiagonalHex3D    Jacobi diagonal per field
//   geometricFactorsHex3D              vgeo (rx..tz, J, JW, 1/JW)
//
// Layout on GB300: one CTA per element, the element's fields and the
// contraction intermediates in shared memory, threads looping over the nodes.
// These operators run in FP64, which GB300 executes at 1/64 of its FP32 rate:
// they are FP64-pipe bound, so the layout favours simplicity over the
// register-pencil scheme of the FP32 multigrid operator.

#include "nrsg_internal.hpp"

namespace nrsg {

namespace {
constexpr int kBlkThreads = 256;

__device__ __forceinline__ double coef(const double *a, double s, long long id, int f, long long loffset)
{
  return a ? a[id + f * loffset] : s;
}
} // namespace

template <int NQ>
__global__ void __launch_bounds__(kBlkThreads)
    vgeo_kernel(long long E, const double *__restrict__ VX, const double *__restrict__ gllz,
                const double *__restrict__ gllw, const double *__restrict__ D, double *__restrict__ vgeo)
{
  constexpr int NP = NQ * NQ * NQ;
  __shared__ double s_x[3][NP];
  __shared__ double s_D[NQ][NQ];
  __shared__ double s_v[24];
  __shared__ double s_z[NQ], s_w[NQ];
  const long long e = blockIdx.x;
  for (int t = threadIdx.x; t < NQ * NQ; t += blockDim.x) s_D[t / NQ][t % NQ] = D[t];
  if (threadIdx.x < 24) s_v[threadIdx.x] = VX[e * 24 + threadIdx.x];
  if (threadIdx.x < NQ) {
    s_z[threadIdx.x] = gllz[threadIdx.x];
    s_w[threadIdx.x] = gllw[threadIdx.x];
  }
  __syncthreads();
  for (int n = threadIdx.x; n < NP; n += blockDim.x) {
    const int i = n % NQ, j = (n / NQ) % NQ, k = n / (NQ * NQ);
    const double a[2] = {0.5 * (1 - s_z[i]), 0.5 * (1 + s_z[i])};
    const double b[2] = {0.5 * (1 - s_z[j]), 0.5 * (1 + s_z[j])};
    const double c[2] = {0.5 * (1 - s_z[k]), 0.5 * (1 + s_z[k])};
    double X[3] = {0, 0, 0};
    for (int v = 0; v < 8; ++v) {
      const double wv = a[v & 1] * b[(v >> 1) & 1] * c[v >> 2];
      for (int d = 0; d < 3; ++d) X[d] += wv * s_v[v * 3 + d];
    }
    for (int d = 0; d < 3; ++d) s_x[d][n] = X[d];
  }
  __syncthreads();
  double *g = vgeo + e * 12 * NP;
  for (int n = threadIdx.x; n < NP; n += blockDim.x) {
    const int i = n % NQ, j = (n / NQ) % NQ, k = n / (NQ * NQ);
    double dr[3] = {0, 0, 0}, ds[3] = {0, 0, 0}, dt[3] = {0, 0, 0};
    for (int m = 0; m < NQ; ++m)
      for (int d = 0; d < 3; ++d) {
        dr[d] += s_D[i][m] * s_x[d][m + NQ * (j + NQ * k)];
        ds[d] += s_D[j][m] * s_x[d][i + NQ * (m + NQ * k)];
        dt[d] += s_D[k][m] * s_x[d][i + NQ * (j + NQ * m)];
      }
    const double xr = dr[0], yr = dr[1], zr = dr[2], xs = ds[0], ys = ds[1], zs = ds[2], xt = dt[0], yt = dt[1],
                 zt = dt[2];
    const double J = xr * (ys * zt - zs * yt) - yr * (xs * zt - zs * xt) + zr * (xs * yt - ys * xt);
    const double Ji = 1.0 / J;
    const double JW = J * s_w[i] * s_w[j] * s_w[k];
    g[0 * NP + n] = (ys * zt - zs * yt) * Ji;
    g[1 * NP + n] = -(xs * zt - zs * xt) * Ji;
    g[2 * NP + n] = (xs * yt - ys * xt) * Ji;
    g[3 * NP + n] = -(yr * zt - zr * yt) * Ji;
    g[4 * NP + n] = (xr * zt - zr * xt) * Ji;
    g[5 * NP + n] = -(xr * yt - yr * xt) * Ji;
    g[6 * NP + n] = (yr * zs - zr * ys) * Ji;
    g[7 * NP + n] = -(xr * zs - zr * xs) * Ji;
    g[8 * NP + n] = (xr * ys - yr * xs) * Ji;
    g[9 * NP + n] = J;
    g[10 * NP + n] = JW;
    g[11 * NP + n] = 1.0 / JW;
  }
}

// ellipticBlockPartialAxCoeffHex3D: per field f,
//   G_f = lambda0_f G grad q_f,  A q_f = D^T G_f + GwJ lambda1_f q_f
template <int NQ>
__global__ void __launch_bounds__(kBlkThreads)
    block_ax_kernel(long long E, int nf, long long offset, long long loffset, const double *__restrict__ ggeo,
                    const double *__restrict__ D, const double *__restrict__ lam0, const double *__restrict__ lam1,
                    double l0, double l1, int poisson, const double *__restrict__ q, double *__restrict__ Aq)
{
  constexpr int NP = NQ * NQ * NQ;
  __shared__ double s_D[NQ][NQ];
  __shared__ double s_q[NP], s_Gr[NP], s_Gs[NP], s_Gt[NP];
  const long long e = blockIdx.x;
  for (int t = threadIdx.x; t < NQ * NQ; t += blockDim.x) s_D[t / NQ][t % NQ] = D[t];
  const double *g = ggeo + e * 7 * NP;
  for (int f = 0; f < nf; ++f) {
    __syncthreads();
    for (int n = threadIdx.x; n < NP; n += blockDim.x) s_q[n] = q[f * offset + e * NP + n];
    __syncthreads();
    for (int n = threadIdx.x; n < NP; n += blockDim.x) {
      const int i = n % NQ, j = (n / NQ) % NQ, k = n / (NQ * NQ);
      double qr = 0, qs = 0, qt = 0;
      for (int m = 0; m < NQ; ++m) {
        qr += s_D[i][m] * s_q[m + NQ * (j + NQ * k)];
        qs += s_D[j][m] * s_q[i + NQ * (m + NQ * k)];
        qt += s_D[k][m] * s_q[i + NQ * (j + NQ * m)];
      }
      const double G00 = g[0 * NP + n], G01 = g[1 * NP + n], G11 = g[2 * NP + n];
      const double G12 = g[3 * NP + n], G02 = g[4 * NP + n], G22 = g[5 * NP + n];
      const double lam = coef(lam0, l0, e * NP + n, f, loffset);
      s_Gr[n] = lam * (G00 * qr + G01 * qs + G02 * qt);
      s_Gs[n] = lam * (G01 * qr + G11 * qs + G12 * qt);
      s_Gt[n] = lam * (G02 * qr + G12 * qs + G22 * qt);
    }
    __syncthreads();
    for (int n = threadIdx.x; n < NP; n += blockDim.x) {
      const int i = n % NQ, j = (n / NQ) % NQ, k = n / (NQ * NQ);
      const double a0 = poisson ? 0.0 : g[6 * NP + n] * coef(lam1, l1, e * NP + n, f, loffset) * s_q[n];
      double ar = 0, as = 0, at = 0;
      for (int m = 0; m < NQ; ++m) ar += s_D[m][i] * s_Gr[m + NQ * (j + NQ * k)];
      for (int m = 0; m < NQ; ++m) as += s_D[m][j] * s_Gs[i + NQ * (m + NQ * k)];
      for (int m = 0; m < NQ; ++m) at += s_D[m][k] * s_Gt[i + NQ * (j + NQ * m)];
      Aq[f * offset + e * NP + n] = ar + as + at + a0;
    }
  }
}

// ellipticStressPartialAxCoeffHex3D: the three velocity components coupled
// through the symmetric gradient; shared memory holds U, V, W and the nine
// contracted stress components of the element (12 Np doubles, dynamic)
template <int NQ>
__global__ void __launch_bounds__(kBlkThreads)
    stress_ax_kernel(long long E, long long offset, long long loffset, const double *__restrict__ vgeo,
                     const double *__restrict__ D, const double *__restrict__ lam0, const double *__restrict__ lam1,
                     double l0, double l1, const double *__restrict__ q, double *__restrict__ Aq)
{
  constexpr int NP = NQ * NQ * NQ;
  extern __shared__ double s_dyn[];
  double *s_U = s_dyn, *s_V = s_U + NP, *s_W = s_V + NP;
  double *s_S = s_W + NP; // [9][NP]: SUr SUs SUt SVr SVs SVt SWr SWs SWt
  __shared__ double s_D[NQ][NQ];
  const long long e = blockIdx.x;
  for (int t = threadIdx.x; t < NQ * NQ; t += blockDim.x) s_D[t / NQ][t % NQ] = D[t];
  for (int n = threadIdx.x; n < NP; n += blockDim.x) {
    s_U[n] = q[e * NP + n];
    s_V[n] = q[offset + e * NP + n];
    s_W[n] = q[2 * offset + e * NP + n];
  }
  __syncthreads();
  const double *g = vgeo + e * 12 * NP;
  for (int n = threadIdx.x; n < NP; n += blockDim.x) {
    const int i = n % NQ, j = (n / NQ) % NQ, k = n / (NQ * NQ);
    double ur = 0, us = 0, ut = 0, vr = 0, vs = 0, vt = 0, wr = 0, ws = 0, wt = 0;
    for (int m = 0; m < NQ; ++m) {
      const double Dim = s_D[i][m], Djm = s_D[j][m], Dkm = s_D[k][m];
      const int ir = m + NQ * (j + NQ * k), is = i + NQ * (m + NQ * k), it = i + NQ * (j + NQ * m);
      ur += Dim * s_U[ir];
      us += Djm * s_U[is];
      ut += Dkm * s_U[it];
      vr += Dim * s_V[ir];
      vs += Djm * s_V[is];
      vt += Dkm * s_V[it];
      wr += Dim * s_W[ir];
      ws += Djm * s_W[is];
      wt += Dkm * s_W[it];
    }
    const double rx = g[0 * NP + n], ry = g[1 * NP + n], rz = g[2 * NP + n];
    const double sx = g[3 * NP + n], sy = g[4 * NP + n], sz = g[5 * NP + n];
    const double tx = g[6 * NP + n], ty = g[7 * NP + n], tz = g[8 * NP + n];
    const double JW = g[10 * NP + n];
    const long long id = e * NP + n;
    const double ul = coef(lam0, l0, id, 0, loffset), vl = coef(lam0, l0, id, 1, loffset),
                 wl = coef(lam0, l0, id, 2, loffset);
    const double dudx = rx * ur + sx * us + tx * ut, dudy = ry * ur + sy * us + ty * ut,
                 dudz = rz * ur + sz * us + tz * ut;
    const double dvdx = rx * vr + sx * vs + tx * vt, dvdy = ry * vr + sy * vs + ty * vt,
                 dvdz = rz * vr + sz * vs + tz * vt;
    const double dwdx = rx * wr + sx * ws + tx * wt, dwdy = ry * wr + sy * ws + ty * wt,
                 dwdz = rz * wr + sz * ws + tz * wt;
    const double s11 = ul * JW * (dudx + dudx), s12 = ul * JW * (dudy + dvdx), s13 = ul * JW * (dudz + dwdx);
    const double s21 = vl * JW * (dvdx + dudy), s22 = vl * JW * (dvdy + dvdy), s23 = vl * JW * (dvdz + dwdy);
    const double s31 = wl * JW * (dwdx + dudz), s32 = wl * JW * (dwdy + dvdz), s33 = wl * JW * (dwdz + dwdz);
    s_S[0 * NP + n] = rx * s11 + ry * s12 + rz * s13;
    s_S[1 * NP + n] = sx * s11 + sy * s12 + sz * s13;
    s_S[2 * NP + n] = tx * s11 + ty * s12 + tz * s13;
    s_S[3 * NP + n] = rx * s21 + ry * s22 + rz * s23;
    s_S[4 * NP + n] = sx * s21 + sy * s22 + sz * s23;
    s_S[5 * NP + n] = tx * s21 + ty * s22 + tz * s23;
    s_S[6 * NP + n] = rx * s31 + ry * s32 + rz * s33;
    s_S[7 * NP + n] = sx * s31 + sy * s32 + sz * s33;
    s_S[8 * NP + n] = tx * s31 + ty * s32 + tz * s33;
  }
  __syncthreads();
  for (int n = threadIdx.x; n < NP; n += blockDim.x) {
    const int i = n % NQ, j = (n / NQ) % NQ, k = n / (NQ * NQ);
    double au = 0, av = 0, aw = 0;
    for (int m = 0; m < NQ; ++m) {
      const double Dim = s_D[m][i], Djm = s_D[m][j], Dkm = s_D[m][k];
      const int ir = m + NQ * (j + NQ * k), is = i + NQ * (m + NQ * k), it = i + NQ * (j + NQ * m);
      au += Dim * s_S[0 * NP + ir];
      au += Djm * s_S[1 * NP + is];
      au += Dkm * s_S[2 * NP + it];
      av += Dim * s_S[3 * NP + ir];
      av += Djm * s_S[4 * NP + is];
      av += Dkm * s_S[5 * NP + it];
      aw += Dim * s_S[6 * NP + ir];
      aw += Djm * s_S[7 * NP + is];
      aw += Dkm * s_S[8 * NP + it];
    }
    const long long id = e * NP + n;
    const double JW = g[10 * NP + n];
    Aq[id] = au + coef(lam1, l1, id, 0, loffset) * JW * s_U[n];
    Aq[offset + id] = av + coef(lam1, l1, id, 1, loffset) * JW * s_V[n];
    Aq[2 * offset + id] = aw + coef(lam1, l1, id, 2, loffset) * JW * s_W[n];
  }
}

// ellipticBlockBuildDiagonalHex3D: diag(A_f) per element and field
template <int NQ>
__global__ void __launch_bounds__(kBlkThreads)
    block_diag_kernel(long long E, int nf, long long offset, long long loffset, const double *__restrict__ ggeo,
                      const double *__restrict__ D, const double *__restrict__ lam0, const double *__restrict__ lam1,
                      double l0, double l1, int poisson, double *__restrict__ diag)
{
  constexpr int NP = NQ * NQ * NQ;
  __shared__ double s_D[NQ][NQ];
  const long long e = blockIdx.x;
  for (int t = threadIdx.x; t < NQ * NQ; t += blockDim.x) s_D[t / NQ][t % NQ] = D[t];
  __syncthreads();
  const double *g = ggeo + e * 7 * NP;
  for (int f = 0; f < nf; ++f)
    for (int n = threadIdx.x; n < NP; n += blockDim.x) {
      const int i = n % NQ, j = (n / NQ) % NQ, k = n / (NQ * NQ);
      const long long id = e * NP + n;
      const double lam = coef(lam0, l0, id, f, loffset);
      double r = 0;
      r += 2.0 * g[1 * NP + n] * lam * s_D[i][i] * s_D[j][j];
      r += 2.0 * g[4 * NP + n] * lam * s_D[i][i] * s_D[k][k];
      r += 2.0 * g[3 * NP + n] * lam * s_D[j][j] * s_D[k][k];
      for (int m = 0; m < NQ; ++m) {
        const int a = m + NQ * (j + NQ * k), b = i + NQ * (m + NQ * k), c = i + NQ * (j + NQ * m);
        r += g[0 * NP + a] * coef(lam0, l0, e * NP + a, f, loffset) * s_D[m][i] * s_D[m][i];
        r += g[2 * NP + b] * coef(lam0, l0, e * NP + b, f, loffset) * s_D[m][j] * s_D[m][j];
        r += g[5 * NP + c] * coef(lam0, l0, e * NP + c, f, loffset) * s_D[m][k] * s_D[m][k];
      }
      if (!poisson) r += g[6 * NP + n] * coef(lam1, l1, id, f, loffset);
      diag[f * offset + id] = r;
    }
}

#define NRSG_DISPATCH_NQ_BLK(N, MACRO)                                                                       \
  switch (N) {                                                                                               \
  case 1: MACRO(2); break;                                                                                   \
  case 2: MACRO(3); break;                                                                                   \
  case 3: MACRO(4); break;                                                                                   \
  case 4: MACRO(5); break;                                                                                   \
  case 5: MACRO(6); break;                                                                                   \
  case 6: MACRO(7); break;                                                                                   \
  case 7: MACRO(8); break;                                                                                   \
  case 8: MACRO(9); break;                                                                                   \
  case 9: MACRO(10); break;                                                                                  \
  default: throw Error(NRSG_ERR_BAD_CONFIG, "polynomial order must be 1..9");                                \
  }

void launch_vgeo(int N, long long E, const double *VX, const double *gllz, const double *gllw, const double *D,
                 double *vgeo, cudaStream_t s)
{
  if (E <= 0) return;
#define NRSG_VG(NQ) vgeo_kernel<NQ><<<(unsigned)E, kBlkThreads, 0, s>>>(E, VX, gllz, gllw, D, vgeo)
  NRSG_DISPATCH_NQ_BLK(N, NRSG_VG)
#undef NRSG_VG
  NRSG_CHECK_LAUNCH();
}

void launch_block_ax(int N, long long E, int nf, long long offset, long long loffset, const double *ggeo,
                     const double *D, const double *lam0, const double *lam1, double l0, double l1, bool poisson,
                     const double *q, double *Aq, cudaStream_t s)
{
  if (E <= 0) return;
#define NRSG_BA(NQ)                                                                                          \
  block_ax_kernel<NQ><<<(unsigned)E, kBlkThreads, 0, s>>>(E, nf, offset, loffset, ggeo, D, lam0, lam1, l0, l1, \
                                                          poisson ? 1 : 0, q, Aq)
  NRSG_DISPATCH_NQ_BLK(N, NRSG_BA)
#undef NRSG_BA
  NRSG_CHECK_LAUNCH();
}

void launch_stress_ax(int N, long long E, long long offset, long long loffset, const double *vgeo, const double *D,
                      const double *lam0, const double *lam1, double l0, double l1, const double *q, double *Aq,
                      cudaStream_t s)
{
  if (E <= 0) return;
#define NRSG_SA(NQ)                                                                                          \
  {                                                                                                          \
    const size_t sm = (size_t)12 * NQ * NQ * NQ * sizeof(double);                                            \
    raise_dynamic_smem((const void *)stress_ax_kernel<NQ>, sm);                                              \
    stress_ax_kernel<NQ><<<(unsigned)E, kBlkThreads, sm, s>>>(E, offset, loffset, vgeo, D, lam0, lam1, l0, l1, q, \
                                                              Aq);                                           \
  }
  NRSG_DISPATCH_NQ_BLK(N, NRSG_SA)
#undef NRSG_SA
  NRSG_CHECK_LAUNCH();
}

void launch_block_diag(int N, long long E, int nf, long long offset, long long loffset, const double *ggeo,
                       const double *D, const double *lam0, const double *lam1, double l0, double l1, bool poisson,
                       double *diag, cudaStream_t s)
{
  if (E <= 0) return;
#define NRSG_BD(NQ)                                                                                          \
  block_diag_kernel<NQ><<<(unsigned)E, kBlkThreads, 0, s>>>(E, nf, offset, loffset, ggeo, D, lam0, lam1, l0, l1, \
                                                            poisson ? 1 : 0, diag)
  NRSG_DISPATCH_NQ_BLK(N, NRSG_BD)
#undef NRSG_BD
  NRSG_CHECK_LAUNCH();
}

} // namespace nrsg

namespace nrsg {

// zero-normal projection (applyZeroNormalMask.okl): per entry, reps times,
// R = (U.n) maskN, (U.t1) maskT1, (U.t2) maskT2 and U = R_n n + R_1 t1 + R_2 t2,
// every product and sum rounded separately in the reference kernel's order
__global__ void zero_normal_kernel(long long n, const int *__restrict__ node, const unsigned char *__restrict__ reps,
                                   const double *__restrict__ frame, const double *__restrict__ mask, long long offset,
                                   double *__restrict__ U)
{
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const long long id = node[t];
    const double *fr = frame + 9 * t, *mk = mask + 3 * t;
    double u = U[id], v = U[id + offset], w = U[id + 2 * offset];
    for (int r = 0; r < reps[t]; ++r) {
      const double Rn = __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(u, fr[0]), __dmul_rn(v, fr[1])), __dmul_rn(w, fr[2])),
                                  mk[0]);
      const double R1 = __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(u, fr[3]), __dmul_rn(v, fr[4])), __dmul_rn(w, fr[5])),
                                  mk[1]);
      const double R2 = __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(u, fr[6]), __dmul_rn(v, fr[7])), __dmul_rn(w, fr[8])),
                                  mk[2]);
      u = __dadd_rn(__dadd_rn(__dmul_rn(Rn, fr[0]), __dmul_rn(R1, fr[3])), __dmul_rn(R2, fr[6]));
      v = __dadd_rn(__dadd_rn(__dmul_rn(Rn, fr[1]), __dmul_rn(R1, fr[4])), __dmul_rn(R2, fr[7]));
      w = __dadd_rn(__dadd_rn(__dmul_rn(Rn, fr[2]), __dmul_rn(R1, fr[5])), __dmul_rn(R2, fr[8]));
    }
    U[id] = u;
    U[id + offset] = v;
    U[id + 2 * offset] = w;
  }
}

void launch_zero_normal(long long n, const int *node, const unsigned char *reps, const double *frame,
                        const double *mask, long long offset, double *U, cudaStream_t s)
{
  if (n <= 0) return;
  const long long blocks = (n + 255) / 256;
  zero_normal_kernel<<<(unsigned)(blocks < 4096 ? blocks : 4096), 256, 0, s>>>(n, node, reps, frame, mask, offset, U);
  NRSG_CHECK_LAUNCH();
}

} // namespace nrsg
