// axhelm kernels for sm_103a: A q = D^T G D q (+ GwJ lambda1 q) per hexahedral
// element, geometric factors either stored ([E][7][Np]) or rebuilt from the
// 8 trilinear vertices.
//
// Reference: kernels/elliptic/ellipticPartialAxCoeffHex3D.okl (v0 layout:
// an Nq x Nq thread plane per element sweeping k with a register pencil) and
// kernels/elliptic/ellipticPartialAxTrilinearHex3D.okl.
//
// Layout on GB300: EPB elements share a CTA (EPB * Nq^2 threads, >= 128),
// so that each k-plane load of a geometric factor is one coalesced 512 B
// (fp64, Nq = 8) transaction per element and D sits in shared memory once per
// CTA.  The fp64 kernel is bound by the FP64 pipe on GB300, not by HBM; the
// fp32 kernel (p-multigrid levels) is HBM bound.

#include "nrsg_internal.hpp"

namespace nrsg {

template <int NQ> struct AxShape {
  static constexpr int plane = NQ * NQ;
  static constexpr int epb = plane >= 128 ? 1 : (128 + plane - 1) / plane;
};

template <typename T, int NQ, bool POISSON>
__global__ void __launch_bounds__(NQ *NQ *AxShape<NQ>::epb)
    ax_stored_kernel(long long E, const T *__restrict__ ggeo, const T *__restrict__ D, T lambda0, T lambda1,
                     const T *__restrict__ q, T *__restrict__ Aq)
{
  constexpr int EPB = AxShape<NQ>::epb;
  constexpr int NP = NQ * NQ * NQ;
  __shared__ T s_D[NQ][NQ + 1];
  __shared__ T s_q[EPB][NQ][NQ];
  __shared__ T s_Gr[EPB][NQ][NQ];
  __shared__ T s_Gs[EPB][NQ][NQ];

  const int t = threadIdx.x;
  const int i = t % NQ, j = t / NQ;
  const int el = threadIdx.y;
  const long long e = (long long)blockIdx.x * EPB + el;
  const bool active = e < E;
  if (el == 0) s_D[j][i] = D[j * NQ + i];

  T r_q[NQ], r_Aq[NQ];
  const long long base = e * NP + t;
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    r_q[k] = active ? q[base + k * NQ * NQ] : T(0);
    r_Aq[k] = 0;
  }
  __syncthreads();

  const T *g = ggeo + e * 7 * NP + t;
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    T G00 = 0, G01 = 0, G11 = 0, G12 = 0, G02 = 0, G22 = 0, GWJ = 0;
    if (active) {
      const int o = k * NQ * NQ;
      G00 = __ldg(g + 0 * NP + o);
      G01 = __ldg(g + 1 * NP + o);
      G11 = __ldg(g + 2 * NP + o);
      G12 = __ldg(g + 3 * NP + o);
      G02 = __ldg(g + 4 * NP + o);
      G22 = __ldg(g + 5 * NP + o);
      if (!POISSON) GWJ = __ldg(g + 6 * NP + o);
    }
    s_q[el][j][i] = r_q[k];
    T qt = 0;
#pragma unroll
    for (int m = 0; m < NQ; ++m) qt += s_D[k][m] * r_q[m];
    __syncthreads();
    T qr = 0, qs = 0;
#pragma unroll
    for (int m = 0; m < NQ; ++m) {
      qr += s_D[i][m] * s_q[el][j][m];
      qs += s_D[j][m] * s_q[el][m][i];
    }
    s_Gr[el][j][i] = lambda0 * (G00 * qr + G01 * qs + G02 * qt);
    s_Gs[el][j][i] = lambda0 * (G01 * qr + G11 * qs + G12 * qt);
    const T Gt = lambda0 * (G02 * qr + G12 * qs + G22 * qt);
    T auk = POISSON ? T(0) : GWJ * lambda1 * r_q[k];
    __syncthreads();
#pragma unroll
    for (int m = 0; m < NQ; ++m) {
      auk += s_D[m][j] * s_Gs[el][m][i];
      r_Aq[m] += s_D[k][m] * Gt;
      auk += s_D[m][i] * s_Gr[el][j][m];
    }
    r_Aq[k] += auk;
    __syncthreads();
  }
  if (active) {
#pragma unroll
    for (int k = 0; k < NQ; ++k) Aq[base + k * NQ * NQ] = r_Aq[k];
  }
}

// Geometric factors of a trilinear hexahedron at GLL node (r,s,t) from its
// 8 vertices (CCW order 0:(-,-,-) 1:(+,-,-) 2:(+,+,-) 3:(-,+,-), 4-7 at t=+1).
template <typename T>
__device__ __forceinline__ void trilinear_G(const T *xe, const T *ye, const T *ze, T rn, T sn, T tn, T W, T &G00,
                                            T &G01, T &G02, T &G11, T &G12, T &G22, T &GWJ)
{
  const T e8 = T(0.125);
  const T am = (1 - tn) * (1 - sn), ap = (1 - tn) * (1 + sn), bm = (1 + tn) * (1 - sn), bp = (1 + tn) * (1 + sn);
  const T cm = (1 - tn) * (1 - rn), cp = (1 - tn) * (1 + rn), dm = (1 + tn) * (1 - rn), dp = (1 + tn) * (1 + rn);
  const T fm = (1 - rn) * (1 - sn), fp = (1 + rn) * (1 - sn), hp = (1 + rn) * (1 + sn), hm = (1 - rn) * (1 + sn);
#define NRSG_DR(X) (e8 * (am * (X[1] - X[0]) + ap * (X[2] - X[3]) + bm * (X[5] - X[4]) + bp * (X[6] - X[7])))
#define NRSG_DS(X) (e8 * (cm * (X[3] - X[0]) + cp * (X[2] - X[1]) + dm * (X[7] - X[4]) + dp * (X[6] - X[5])))
#define NRSG_DT(X) (e8 * (fm * (X[4] - X[0]) + fp * (X[5] - X[1]) + hp * (X[6] - X[2]) + hm * (X[7] - X[3])))
  const T xr = NRSG_DR(xe), xs = NRSG_DS(xe), xt = NRSG_DT(xe);
  const T yr = NRSG_DR(ye), ys = NRSG_DS(ye), yt = NRSG_DT(ye);
  const T zr = NRSG_DR(ze), zs = NRSG_DS(ze), zt = NRSG_DT(ze);
#undef NRSG_DR
#undef NRSG_DS
#undef NRSG_DT
  const T J = xr * (ys * zt - zs * yt) - yr * (xs * zt - zs * xt) + zr * (xs * yt - ys * xt);
  const T rx = (ys * zt - zs * yt), ry = -(xs * zt - zs * xt), rz = (xs * yt - ys * xt);
  const T sx = -(yr * zt - zr * yt), sy = (xr * zt - zr * xt), sz = -(xr * yt - yr * xt);
  const T tx = (yr * zs - zr * ys), ty = -(xr * zs - zr * xs), tz = (xr * ys - yr * xs);
  const T sc = W / J;
  G00 = sc * (rx * rx + ry * ry + rz * rz);
  G01 = sc * (rx * sx + ry * sy + rz * sz);
  G02 = sc * (rx * tx + ry * ty + rz * tz);
  G11 = sc * (sx * sx + sy * sy + sz * sz);
  G12 = sc * (sx * tx + sy * ty + sz * tz);
  G22 = sc * (tx * tx + ty * ty + tz * tz);
  GWJ = W * J;
}

template <typename T, int NQ, bool POISSON>
__global__ void __launch_bounds__(NQ *NQ *AxShape<NQ>::epb)
    ax_trilinear_kernel(long long E, const T *__restrict__ VX, const T *__restrict__ gllz,
                        const T *__restrict__ gllw, const T *__restrict__ D, T lambda0, T lambda1,
                        const T *__restrict__ q, T *__restrict__ Aq)
{
  constexpr int EPB = AxShape<NQ>::epb;
  constexpr int NP = NQ * NQ * NQ;
  __shared__ T s_D[NQ][NQ + 1];
  __shared__ T s_z[NQ], s_w[NQ];
  __shared__ T s_X[EPB][3][8];
  __shared__ T s_q[EPB][NQ][NQ];
  __shared__ T s_Gr[EPB][NQ][NQ];
  __shared__ T s_Gs[EPB][NQ][NQ];

  const int t = threadIdx.x;
  const int i = t % NQ, j = t / NQ;
  const int el = threadIdx.y;
  const long long e = (long long)blockIdx.x * EPB + el;
  const bool active = e < E;
  if (el == 0) {
    s_D[j][i] = D[j * NQ + i];
    if (j == 0) { s_z[i] = gllz[i]; s_w[i] = gllw[i]; }
  }
  for (int u = t; u < 24; u += NQ * NQ) {
    // input [e][8 hypercube][3] -> shared [3][8 CCW]
    const int v = u / 3, d = u % 3;
    const int ccw = (v & 2) ? (v ^ 1) : v; // hypercube 2<->3, 6<->7
    s_X[el][d][ccw] = active ? VX[e * 24 + u] : T(0);
  }
  T r_q[NQ], r_Aq[NQ];
  const long long base = e * NP + t;
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    r_q[k] = active ? q[base + k * NQ * NQ] : T(0);
    r_Aq[k] = 0;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    T G00, G01, G02, G11, G12, G22, GWJ;
    trilinear_G<T>(s_X[el][0], s_X[el][1], s_X[el][2], s_z[i], s_z[j], s_z[k], s_w[i] * s_w[j] * s_w[k], G00, G01,
                   G02, G11, G12, G22, GWJ);
    if (!active) { G00 = G01 = G02 = G11 = G12 = G22 = GWJ = 0; }
    s_q[el][j][i] = r_q[k];
    T qt = 0;
#pragma unroll
    for (int m = 0; m < NQ; ++m) qt += s_D[k][m] * r_q[m];
    __syncthreads();
    T qr = 0, qs = 0;
#pragma unroll
    for (int m = 0; m < NQ; ++m) {
      qr += s_D[i][m] * s_q[el][j][m];
      qs += s_D[j][m] * s_q[el][m][i];
    }
    s_Gr[el][j][i] = lambda0 * (G00 * qr + G01 * qs + G02 * qt);
    s_Gs[el][j][i] = lambda0 * (G01 * qr + G11 * qs + G12 * qt);
    const T Gt = lambda0 * (G02 * qr + G12 * qs + G22 * qt);
    T auk = POISSON ? T(0) : GWJ * lambda1 * r_q[k];
    __syncthreads();
#pragma unroll
    for (int m = 0; m < NQ; ++m) {
      auk += s_D[m][j] * s_Gs[el][m][i];
      r_Aq[m] += s_D[k][m] * Gt;
      auk += s_D[m][i] * s_Gr[el][j][m];
    }
    r_Aq[k] += auk;
    __syncthreads();
  }
  if (active) {
#pragma unroll
    for (int k = 0; k < NQ; ++k) Aq[base + k * NQ * NQ] = r_Aq[k];
  }
}

#define NRSG_DISPATCH_NQ(N, MACRO)                                                                         \
  switch (N) {                                                                                             \
  case 1: MACRO(2); break;                                                                                 \
  case 2: MACRO(3); break;                                                                                 \
  case 3: MACRO(4); break;                                                                                 \
  case 4: MACRO(5); break;                                                                                 \
  case 5: MACRO(6); break;                                                                                 \
  case 6: MACRO(7); break;                                                                                 \
  case 7: MACRO(8); break;                                                                                 \
  case 8: MACRO(9); break;                                                                                 \
  case 9: MACRO(10); break;                                                                                \
  default: throw Error(NRSG_ERR_BAD_CONFIG, "polynomial order must be 1..9");                              \
  }

template <typename T>
void launch_ax_stored(int N, long long E, const T *ggeo, const T *D, T lambda0, T lambda1, bool poisson, const T *q,
                      T *Aq, cudaStream_t s)
{
  if (E <= 0) return;
#define NRSG_AX(NQ)                                                                                        \
  {                                                                                                        \
    constexpr int EPB = AxShape<NQ>::epb;                                                                  \
    dim3 blk(NQ * NQ, EPB);                                                                                \
    const unsigned grid = (unsigned)((E + EPB - 1) / EPB);                                                 \
    if (poisson)                                                                                           \
      ax_stored_kernel<T, NQ, true><<<grid, blk, 0, s>>>(E, ggeo, D, lambda0, lambda1, q, Aq);             \
    else                                                                                                   \
      ax_stored_kernel<T, NQ, false><<<grid, blk, 0, s>>>(E, ggeo, D, lambda0, lambda1, q, Aq);            \
  }
  NRSG_DISPATCH_NQ(N, NRSG_AX)
#undef NRSG_AX
  NRSG_CHECK_LAUNCH();
}

template <typename T>
void launch_ax_trilinear(int N, long long E, const T *VX, const T *gllz, const T *gllw, const T *D, T lambda0,
                         T lambda1, bool poisson, const T *q, T *Aq, cudaStream_t s)
{
  if (E <= 0) return;
#define NRSG_AXT(NQ)                                                                                       \
  {                                                                                                        \
    constexpr int EPB = AxShape<NQ>::epb;                                                                  \
    dim3 blk(NQ * NQ, EPB);                                                                                \
    const unsigned grid = (unsigned)((E + EPB - 1) / EPB);                                                 \
    if (poisson)                                                                                           \
      ax_trilinear_kernel<T, NQ, true><<<grid, blk, 0, s>>>(E, VX, gllz, gllw, D, lambda0, lambda1, q, Aq); \
    else                                                                                                   \
      ax_trilinear_kernel<T, NQ, false><<<grid, blk, 0, s>>>(E, VX, gllz, gllw, D, lambda0, lambda1, q, Aq); \
  }
  NRSG_DISPATCH_NQ(N, NRSG_AXT)
#undef NRSG_AXT
  NRSG_CHECK_LAUNCH();
}

template void launch_ax_stored<double>(int, long long, const double *, const double *, double, double, bool,
                                       const double *, double *, cudaStream_t);
template void launch_ax_stored<float>(int, long long, const float *, const float *, float, float, bool, const float *,
                                      float *, cudaStream_t);
template void launch_ax_trilinear<double>(int, long long, const double *, const double *, const double *,
                                          const double *, double, double, bool, const double *, double *,
                                          cudaStream_t);
template void launch_ax_trilinear<float>(int, long long, const float *, const float *, const float *, const float *,
                                         float, float, bool, const float *, float *, cudaStream_t);

// ---------------------------------------------------------------------------
// diag(A_L) per node (ellipticBlockBuildDiagonalHex3D.okl:61-107), one field.
// ---------------------------------------------------------------------------
template <typename T, int NQ>
__global__ void build_diag_kernel(long long E, const T *__restrict__ ggeo, const T *__restrict__ D, T lambda0, T lambda1,
                                  bool poisson, T *__restrict__ diag)
{
  constexpr int NP = NQ * NQ * NQ;
  __shared__ T s_D[NQ][NQ];
  const long long e = blockIdx.x;
  for (int t = threadIdx.x; t < NQ * NQ; t += blockDim.x) s_D[t / NQ][t % NQ] = D[t];
  __syncthreads();
  const T *g = ggeo + e * 7 * NP;
  for (int n = threadIdx.x; n < NP; n += blockDim.x) {
    const int i = n % NQ, j = (n / NQ) % NQ, k = n / (NQ * NQ);
    T r = 0;
    r += T(2) * g[1 * NP + n] * lambda0 * s_D[i][i] * s_D[j][j];
    r += T(2) * g[4 * NP + n] * lambda0 * s_D[i][i] * s_D[k][k];
    r += T(2) * g[3 * NP + n] * lambda0 * s_D[j][j] * s_D[k][k];
    for (int m = 0; m < NQ; ++m) {
      r += g[0 * NP + m + NQ * (j + NQ * k)] * lambda0 * s_D[m][i] * s_D[m][i];
      r += g[2 * NP + i + NQ * (m + NQ * k)] * lambda0 * s_D[m][j] * s_D[m][j];
      r += g[5 * NP + i + NQ * (j + NQ * m)] * lambda0 * s_D[m][k] * s_D[m][k];
    }
    if (!poisson) r += g[6 * NP + n] * lambda1;
    diag[e * NP + n] = r;
  }
}

template <typename T>
void launch_build_diag(int N, long long E, const T *ggeo, const T *D, T lambda0, T lambda1, bool poisson, T *diag,
                       cudaStream_t s)
{
  if (E <= 0) return;
#define NRSG_DG(NQ) build_diag_kernel<T, NQ><<<(unsigned)E, 256, 0, s>>>(E, ggeo, D, lambda0, lambda1, poisson, diag)
  NRSG_DISPATCH_NQ(N, NRSG_DG)
#undef NRSG_DG
  NRSG_CHECK_LAUNCH();
}
template void launch_build_diag<double>(int, long long, const double *, const double *, double, double, bool, double *,
                                        cudaStream_t);
template void launch_build_diag<float>(int, long long, const float *, const float *, float, float, bool, float *,
                                       cudaStream_t);

// ---------------------------------------------------------------------------
// Geometric factors from trilinear vertices: node coordinates by trilinear
// blending, derivatives by D (geometricFactorsHex3D.okl:77-139), fp64.
// ---------------------------------------------------------------------------
template <int NQ>
__global__ void geofac_kernel(long long E, const double *__restrict__ VX, const double *__restrict__ gllz,
                              const double *__restrict__ gllw, const double *__restrict__ D, double *__restrict__ ggeo)
{
  constexpr int NP = NQ * NQ * NQ;
  __shared__ double s_x[3][NP];
  __shared__ double s_D[NQ][NQ];
  __shared__ double s_v[24];
  __shared__ double s_z[NQ], s_w[NQ];
  const long long e = blockIdx.x;
  for (int t = threadIdx.x; t < NQ * NQ; t += blockDim.x) s_D[t / NQ][t % NQ] = D[t];
  if (threadIdx.x < 24) s_v[threadIdx.x] = VX[e * 24 + threadIdx.x];
  if (threadIdx.x < NQ) { s_z[threadIdx.x] = gllz[threadIdx.x]; s_w[threadIdx.x] = gllw[threadIdx.x]; }
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
  double *g = ggeo + e * 7 * NP;
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
    const double rx = (ys * zt - zs * yt) * Ji, ry = -(xs * zt - zs * xt) * Ji, rz = (xs * yt - ys * xt) * Ji;
    const double sx = -(yr * zt - zr * yt) * Ji, sy = (xr * zt - zr * xt) * Ji, sz = -(xr * yt - yr * xt) * Ji;
    const double tx = (yr * zs - zr * ys) * Ji, ty = -(xr * zs - zr * xs) * Ji, tz = (xr * ys - yr * xs) * Ji;
    g[0 * NP + n] = JW * (rx * rx + ry * ry + rz * rz);
    g[1 * NP + n] = JW * (rx * sx + ry * sy + rz * sz);
    g[2 * NP + n] = JW * (sx * sx + sy * sy + sz * sz);
    g[3 * NP + n] = JW * (sx * tx + sy * ty + sz * tz);
    g[4 * NP + n] = JW * (rx * tx + ry * ty + rz * tz);
    g[5 * NP + n] = JW * (tx * tx + ty * ty + tz * tz);
    g[6 * NP + n] = JW;
  }
}

void launch_geofac(int N, long long E, const double *VX, const double *gllz, const double *gllw, const double *D,
                   double *ggeo, cudaStream_t s)
{
  if (E <= 0) return;
#define NRSG_GF(NQ) geofac_kernel<NQ><<<(unsigned)E, 256, 0, s>>>(E, VX, gllz, gllw, D, ggeo)
  NRSG_DISPATCH_NQ(N, NRSG_GF)
#undef NRSG_GF
  NRSG_CHECK_LAUNCH();
}

} // namespace nrsg
