// p-multigrid kernels (sm_103a): restriction / prolongation, Chebyshev
// updates, the fused FDM (Schwarz) local solve with direct neighbour-halo
// gather, the ASM overlap combine, and templated Jacobi-PCG kernels for the
// coarse level.
//
// Reference kernels (nekRS tree):
//   ellipticPreconCoarsenHex3D / ellipticPreconProlongateHex3D (kernels/elliptic/*.okl, *.c)
//   updateChebyshev.okl, updateFourthKindChebyshev.okl
//   preFDM / fusedFDM / postFDM (kernels/elliptic/*.okl, *.c)
//
// FDM on GB300: the reference scatters every element into an (N+3)^3
// extended array in HBM, gather-scatters the extended arrays to exchange
// the one-node overlap, solves, and (ASM) gather-scatters the extended result
// again.  Here one CTA per element builds the extended tile in shared memory
// straight from the element's own nodes plus a precomputed neighbour-halo map
// (src index of the neighbour node each halo point stands for), runs the six
// tensor contractions in shared memory, and writes only the element's own
// nodes (RAS) or its own nodes plus the 6 N_q^2 halo results (ASM).  The
// extended arrays never touch HBM.

#include "mg_kernels.hpp"

#include <cuda_fp16.h>

#include <type_traits>

namespace nrsg {

namespace {
constexpr int kT = 256;
inline unsigned grid_for(long long n)
{
  long long b = (n + kT - 1) / kT;
  if (b < 1) b = 1;
  const long long cap = 152LL * 16;
  return (unsigned)(b < cap ? b : cap);
}
#define MG_LOOP(i, n)                                                                                      \
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (n); i += (long long)gridDim.x * blockDim.x)
} // namespace

#define NRSG_DISPATCH_NQ_MG(N, MACRO)                                                                      \
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

// ---------------------------------------------------------------------------
// restriction qc = (R x R x R) qf, R[c][f]  (NQF fine points per direction)
// ---------------------------------------------------------------------------
template <typename T, int NQF>
__global__ void __launch_bounds__(NQF *NQF) coarsen_kernel(long long E, int NQC, const T *__restrict__ R,
                                                             const T *__restrict__ qf, T *__restrict__ qc)
{
  __shared__ T s_R[NQF][NQF];
  __shared__ T s_a[NQF][NQF][NQF]; // [c or k][j][i]
  __shared__ T s_b[NQF][NQF][NQF];
  const long long e = blockIdx.x;
  const int t = threadIdx.x, i = t % NQF, j = t / NQF;
  if (j < NQC) s_R[j][i] = R[j * NQF + i];
  const T *f = qf + e * NQF * NQF * NQF;
  T r[NQF];
#pragma unroll
  for (int k = 0; k < NQF; ++k) r[k] = f[i + NQF * (j + NQF * k)];
  __syncthreads();
  // along k (thread owns column (i,j))
  for (int c = 0; c < NQC; ++c) {
    T v = 0;
#pragma unroll
    for (int k = 0; k < NQF; ++k) v += s_R[c][k] * r[k];
    s_a[c][j][i] = v;
  }
  __syncthreads();
  // along j: thread (i, b) for b < NQC, all c
  if (j < NQC) {
    for (int c = 0; c < NQC; ++c) {
      T v = 0;
#pragma unroll
      for (int m = 0; m < NQF; ++m) v += s_R[j][m] * s_a[c][m][i];
      s_b[c][j][i] = v;
    }
  }
  __syncthreads();
  // along i: thread (a, b) for a, b < NQC
  if (i < NQC && j < NQC) {
    for (int c = 0; c < NQC; ++c) {
      T v = 0;
#pragma unroll
      for (int m = 0; m < NQF; ++m) v += s_R[i][m] * s_b[c][j][m];
      qc[e * NQC * NQC * NQC + i + NQC * (j + NQC * c)] = v;
    }
  }
}

// prolongation qf += (P x P x P) qc, P = R^T
template <typename T, int NQF>
__global__ void __launch_bounds__(NQF *NQF) prolong_kernel(long long E, int NQC, const T *__restrict__ R,
                                                             const T *__restrict__ qc, T *__restrict__ qf)
{
  __shared__ T s_R[NQF][NQF];
  __shared__ T s_c[NQF][NQF][NQF]; // coarse [c][b][a]
  __shared__ T s_a[NQF][NQF][NQF]; // [c][b][i]
  __shared__ T s_b[NQF][NQF][NQF]; // [c][j][i]
  const long long e = blockIdx.x;
  const int t = threadIdx.x, i = t % NQF, j = t / NQF;
  if (j < NQC) s_R[j][i] = R[j * NQF + i];
  const int npc = NQC * NQC * NQC;
  for (int q = t; q < npc; q += NQF * NQF) s_c[q / (NQC * NQC)][(q / NQC) % NQC][q % NQC] = qc[e * npc + q];
  __syncthreads();
  // along a -> i: thread (i, b)
  if (j < NQC)
    for (int c = 0; c < NQC; ++c) {
      T v = 0;
      for (int a = 0; a < NQC; ++a) v += s_R[a][i] * s_c[c][j][a];
      s_a[c][j][i] = v;
    }
  __syncthreads();
  // along b -> j: thread (i, j)
  for (int c = 0; c < NQC; ++c) {
    T v = 0;
    for (int b = 0; b < NQC; ++b) v += s_R[b][j] * s_a[c][b][i];
    s_b[c][j][i] = v;
  }
  __syncthreads();
  // along c -> k, accumulate
  T *f = qf + e * NQF * NQF * NQF;
#pragma unroll
  for (int k = 0; k < NQF; ++k) {
    T v = 0;
    for (int c = 0; c < NQC; ++c) v += s_R[c][k] * s_b[c][j][i];
    f[i + NQF * (j + NQF * k)] += v;
  }
}

template <typename T> void launch_coarsen(int Nf, int Nc, long long E, const T *R, const T *qf, T *qc, cudaStream_t s)
{
  if (E <= 0) return;
#define NRSG_CO(NQ) coarsen_kernel<T, NQ><<<(unsigned)E, NQ * NQ, 0, s>>>(E, Nc + 1, R, qf, qc)
  NRSG_DISPATCH_NQ_MG(Nf, NRSG_CO)
#undef NRSG_CO
  NRSG_CHECK_LAUNCH();
}
template <typename T> void launch_prolong(int Nf, int Nc, long long E, const T *R, const T *qc, T *qf, cudaStream_t s)
{
  if (E <= 0) return;
#define NRSG_PR(NQ) prolong_kernel<T, NQ><<<(unsigned)E, NQ * NQ, 0, s>>>(E, Nc + 1, R, qc, qf)
  NRSG_DISPATCH_NQ_MG(Nf, NRSG_PR)
#undef NRSG_PR
  NRSG_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// Chebyshev updates
// ---------------------------------------------------------------------------
template <typename T>
__global__ void cheby1_kernel(long long n, T dc, T rc, const T *__restrict__ SAd, T *__restrict__ d, T *__restrict__ r,
                              T *__restrict__ x)
{
  MG_LOOP(i, n)
  {
    const T xn = x[i], dn = d[i], rn = r[i], sa = SAd[i];
    const T r1 = rn - sa;
    x[i] = xn + dn;
    r[i] = r1;
    d[i] = dc * dn + rc * r1;
  }
}
// explicit roundings, shared with the fused gather-scatter updates
__device__ __forceinline__ float mg_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double mg_fma(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float mg_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mg_mul(double a, double b) { return __dmul_rn(a, b); }
// rout = rin - Ad (rin may be rout), x = fma(beta, d, x) (x = beta d when xzero)
template <typename T>
__global__ void cheby4_kernel(long long n, T beta, const T *__restrict__ Ad, const T *__restrict__ d, const T *rin,
                              T *rout, T *__restrict__ x, bool xzero)
{
  MG_LOOP(i, n)
  {
    x[i] = xzero ? mg_mul(beta, d[i]) : mg_fma(beta, d[i], x[i]);
    rout[i] = rin[i] - Ad[i];
  }
}
// 4th-kind Chebyshev, x update moved to where each direction is formed:
// d = c1 Su (first) or fma(c1, Su, c2 d), then x = beta d (xzero) or fma(beta, d, x)
template <typename T>
__global__ void cheby4_dx_kernel(long long n, T c1, const T *__restrict__ Su, T c2, T *__restrict__ d, T beta,
                                 T *__restrict__ x, bool first, bool xzero)
{
  MG_LOOP(i, n)
  {
    const T dn = first ? mg_mul(c1, Su[i]) : mg_fma(c1, Su[i], mg_mul(c2, d[i]));
    d[i] = dn;
    x[i] = xzero ? mg_mul(beta, dn) : mg_fma(beta, dn, x[i]);
  }
}
// rout = rin - Ad (rin may be rout)
template <typename T> __global__ void cheby4_res_kernel(long long n, const T *__restrict__ Ad, const T *rin, T *rout)
{
  MG_LOOP(i, n) rout[i] = rin[i] - Ad[i];
}
template <typename T>
void launch_cheby4_dx(long long n, T c1, const T *Su, T c2, T *d, T beta, T *x, bool first, bool xzero,
                      cudaStream_t s)
{
  cheby4_dx_kernel<T><<<grid_for(n), kT, 0, s>>>(n, c1, Su, c2, d, beta, x, first, xzero);
  NRSG_CHECK_LAUNCH();
}
template <typename T> void launch_cheby4_res(long long n, const T *Ad, const T *rin, T *rout, cudaStream_t s)
{
  cheby4_res_kernel<T><<<grid_for(n), kT, 0, s>>>(n, Ad, rin, rout);
  NRSG_CHECK_LAUNCH();
}

template <typename T>
void launch_cheby1_update(long long n, T dc, T rc, const T *SAd, T *d, T *r, T *x, cudaStream_t s)
{
  cheby1_kernel<T><<<grid_for(n), kT, 0, s>>>(n, dc, rc, SAd, d, r, x);
  NRSG_CHECK_LAUNCH();
}
template <typename T>
void launch_cheby4_update(long long n, T beta, const T *Ad, const T *d, const T *rin, T *rout, T *x, bool xzero,
                          cudaStream_t s)
{
  cheby4_kernel<T><<<grid_for(n), kT, 0, s>>>(n, beta, Ad, d, rin, rout, x, xzero);
  NRSG_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// fused FDM local solve.  Halo point h = (e*6 + f)*NQ^2 + a + NQ*b for face
// f in {x-, x+, y-, y+, z-, z+}; haloSrc[h] is the E-vector index of the
// neighbour node the halo point stands for (-1: none).
// S*_e[r + nl*c] = S(r, c) (column c = eigenvector c); invL[e][Npe].
// ---------------------------------------------------------------------------
template <int NQ> __device__ __forceinline__ int halo_ext_index(int f, int a, int b)
{
  constexpr int NL = NQ + 2;
  switch (f) {
  case 0: return 0 + NL * ((a + 1) + NL * (b + 1));
  case 1: return (NL - 1) + NL * ((a + 1) + NL * (b + 1));
  case 2: return (a + 1) + NL * (0 + NL * (b + 1));
  case 3: return (a + 1) + NL * ((NL - 1) + NL * (b + 1));
  case 4: return (a + 1) + NL * ((b + 1) + NL * 0);
  default: return (a + 1) + NL * ((b + 1) + NL * (NL - 1));
  }
}

template <int NQ> struct FdmShape {
  static constexpr int NL = NQ + 2;
  static constexpr int line = NL * NL;
  static constexpr int epb = line >= 256 ? 1 : 256 / line;
};

// EPB elements per CTA, (N+3)^2 threads per element (one line per thread and
// direction).  With RECIP the 1/(lx+ly+lz) scaling is rebuilt from the three
// 1-D eigenvalue sets (3 (N+3) values per element instead of (N+3)^3).
template <typename T, int NQ, bool RAS, bool RECIP>
__global__ void __launch_bounds__(FdmShape<NQ>::line *FdmShape<NQ>::epb)
    fdm_kernel(long long E, const T *__restrict__ u, const int *__restrict__ haloSrc, const T *__restrict__ Sx,
               const T *__restrict__ Sy, const T *__restrict__ Sz, const T *__restrict__ invL,
               const T *__restrict__ lam, const T *__restrict__ wts, T *__restrict__ Su, T *__restrict__ haloOut)
{
  constexpr int NL = NQ + 2, NPE = NL * NL * NL, NP = NQ * NQ * NQ, NF = NQ * NQ, LINE = NL * NL;
  constexpr int EPB = FdmShape<NQ>::epb;
  __shared__ T s_w[EPB][NPE];
  __shared__ T s_S[EPB][3][LINE];
  __shared__ T s_l[EPB][3][NL];
  const int t = threadIdx.x, el = threadIdx.y;
  const long long e = (long long)blockIdx.x * EPB + el;
  const bool active = e < E;
  const long long ee = active ? e : 0;
  for (int q = t; q < LINE; q += LINE) {
    s_S[el][0][q] = Sx[ee * LINE + q];
    s_S[el][1][q] = Sy[ee * LINE + q];
    s_S[el][2][q] = Sz[ee * LINE + q];
  }
  if (RECIP && t < 3 * NL) s_l[el][t / NL][t % NL] = lam[ee * 3 * NL + t];
  for (int q = t; q < NPE; q += LINE) s_w[el][q] = T(0);
  __syncthreads();
  const T *ue = u + ee * NP;
  for (int q = t; q < NP; q += LINE) {
    const int i = q % NQ, j = (q / NQ) % NQ, k = q / NF;
    s_w[el][(i + 1) + NL * ((j + 1) + NL * (k + 1))] = active ? ue[q] : T(0);
  }
  const int *hs = haloSrc + ee * 6 * NF;
  for (int q = t; q < 6 * NF; q += LINE) {
    const int f = q / NF, pp = q % NF;
    const int src = active ? hs[q] : -1;
    s_w[el][halo_ext_index<NQ>(f, pp % NQ, pp / NQ)] = src >= 0 ? u[src] : T(0);
  }
  __syncthreads();
  const int p = t % NL, q = t / NL;
  T line[NL];
  T *w = s_w[el];
  const T *SX = s_S[el][0], *SY = s_S[el][1], *SZ = s_S[el][2];
  // forward: S^T along x, y, z
#pragma unroll
  for (int l = 0; l < NL; ++l) line[l] = w[l + NL * (p + NL * q)];
#pragma unroll
  for (int i = 0; i < NL; ++i) {
    T v = 0;
#pragma unroll
    for (int l = 0; l < NL; ++l) v += SX[l + NL * i] * line[l];
    w[i + NL * (p + NL * q)] = v;
  }
  __syncthreads();
#pragma unroll
  for (int l = 0; l < NL; ++l) line[l] = w[p + NL * (l + NL * q)];
#pragma unroll
  for (int j = 0; j < NL; ++j) {
    T v = 0;
#pragma unroll
    for (int l = 0; l < NL; ++l) v += SY[l + NL * j] * line[l];
    w[p + NL * (j + NL * q)] = v;
  }
  __syncthreads();
#pragma unroll
  for (int l = 0; l < NL; ++l) line[l] = w[p + NL * (q + NL * l)];
  const T *iL = invL + ee * NPE;
#pragma unroll
  for (int k = 0; k < NL; ++k) {
    T v = 0;
#pragma unroll
    for (int l = 0; l < NL; ++l) v += SZ[l + NL * k] * line[l];
    T sc;
    if (RECIP) {
      const T d = s_l[el][0][p] + s_l[el][1][q] + s_l[el][2][k];
      sc = d > T(1e-5) ? T(1) / d : T(0);
    } else {
      sc = iL[p + NL * (q + NL * k)];
    }
    w[p + NL * (q + NL * k)] = v * sc;
  }
  __syncthreads();
  // backward: S along x, y, z
#pragma unroll
  for (int l = 0; l < NL; ++l) line[l] = w[l + NL * (p + NL * q)];
#pragma unroll
  for (int i = 0; i < NL; ++i) {
    T v = 0;
#pragma unroll
    for (int l = 0; l < NL; ++l) v += SX[i + NL * l] * line[l];
    w[i + NL * (p + NL * q)] = v;
  }
  __syncthreads();
#pragma unroll
  for (int l = 0; l < NL; ++l) line[l] = w[p + NL * (l + NL * q)];
#pragma unroll
  for (int j = 0; j < NL; ++j) {
    T v = 0;
#pragma unroll
    for (int l = 0; l < NL; ++l) v += SY[j + NL * l] * line[l];
    w[p + NL * (j + NL * q)] = v;
  }
  __syncthreads();
#pragma unroll
  for (int l = 0; l < NL; ++l) line[l] = w[p + NL * (q + NL * l)];
#pragma unroll
  for (int k = 0; k < NL; ++k) {
    T v = 0;
#pragma unroll
    for (int l = 0; l < NL; ++l) v += SZ[k + NL * l] * line[l];
    w[p + NL * (q + NL * k)] = v;
  }
  __syncthreads();
  if (!active) return;
  T *se = Su + e * NP;
  for (int qq = t; qq < NP; qq += LINE) {
    const int i = qq % NQ, j = (qq / NQ) % NQ, k = qq / NF;
    const T v = w[(i + 1) + NL * ((j + 1) + NL * (k + 1))];
    se[qq] = RAS ? v * wts[e * NP + qq] : v;
  }
  if (!RAS) {
    T *ho = haloOut + e * 6 * NF;
    for (int qq = t; qq < 6 * NF; qq += LINE) {
      const int f = qq / NF, pp = qq % NF;
      ho[qq] = w[halo_ext_index<NQ>(f, pp % NQ, pp / NQ)];
    }
  }
}

// ASM: add the neighbours' overlap results onto the nodes next to each face,
// face by face in the order x-, x+, y-, y+, z-, z+, then weight.
// haloPartner[h] is the halo index of the neighbour's halo point that maps
// onto the node next to face point h (-1: none).  One warp per element, the
// element's nodes in shared memory; every partner index and overlap value of
// the element is loaded before the first add.
constexpr int kAsmEpc = 8; // elements (warps) per CTA
template <typename T, int NQ>
__global__ void __launch_bounds__(32 * kAsmEpc)
    asm_combine_kernel(long long E, const int *__restrict__ haloPartner, const T *__restrict__ haloOut,
                       const T *__restrict__ wts, T *__restrict__ Su)
{
  constexpr int NP = NQ * NQ * NQ, NF = NQ * NQ, N = NQ - 1, PPF = (NF + 31) / 32;
  __shared__ T s_u[kAsmEpc][NP];
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  const long long e = (long long)blockIdx.x * kAsmEpc + wp;
  if (e >= E) return; // whole warp; warp-level synchronisation only
  T *su = s_u[wp];
  const int *hp = haloPartner + e * 6 * NF;
  constexpr int NPL = (NP + 31) / 32; // nodes per lane
  // every independent load first (own nodes, weights, partner indices), then the gathers
  T own[NPL], wt[NPL];
#pragma unroll
  for (int m = 0; m < NPL; ++m) {
    const int q = lane + 32 * m;
    own[m] = q < NP ? Su[e * NP + q] : T(0);
    wt[m] = q < NP ? __ldg(wts + e * NP + q) : T(0);
  }
  int hidx[6][PPF];
#pragma unroll
  for (int f = 0; f < 6; ++f)
#pragma unroll
    for (int m = 0; m < PPF; ++m) {
      const int p = lane + 32 * m;
      hidx[f][m] = p < NF ? __ldg(hp + f * NF + p) : -1;
    }
  T hval[6][PPF];
#pragma unroll
  for (int f = 0; f < 6; ++f)
#pragma unroll
    for (int m = 0; m < PPF; ++m) hval[f][m] = hidx[f][m] >= 0 ? __ldg(haloOut + hidx[f][m]) : T(0);
#pragma unroll
  for (int m = 0; m < NPL; ++m) {
    const int q = lane + 32 * m;
    if (q < NP) su[q] = own[m];
  }
  __syncwarp();
#pragma unroll
  for (int f = 0; f < 6; ++f) {
#pragma unroll
    for (int m = 0; m < PPF; ++m) {
      const int p = lane + 32 * m;
      if (p < NF && hidx[f][m] >= 0) {
        const int a = p % NQ, b = p / NQ;
        int n;
        switch (f) {
        case 0: n = 1 + NQ * (a + NQ * b); break;
        case 1: n = (N - 1) + NQ * (a + NQ * b); break;
        case 2: n = a + NQ * (1 + NQ * b); break;
        case 3: n = a + NQ * ((N - 1) + NQ * b); break;
        case 4: n = a + NQ * (b + NQ * 1); break;
        default: n = a + NQ * (b + NQ * (N - 1)); break;
        }
        su[n] += hval[f][m];
      }
    }
    __syncwarp();
  }
#pragma unroll
  for (int m = 0; m < NPL; ++m) {
    const int q = lane + 32 * m;
    if (q < NP) Su[e * NP + q] = su[q] * wt[m];
  }
}

// ---------------------------------------------------------------------------
// FP32 FDM for order 7 (NQ = 8, extended NL = 10): one warp per element.
// The generic kernel above gives every thread one line and reads each S entry
// from shared memory once per multiply-add, so it is bound by shared-memory
// wavefronts (about one per FMA).  Here each lane carries 4 lines (x
// direction) or a bundle of 4 adjacent x-lines (y and z directions), so each
// broadcast 128-bit load of an S row serves 4 lines, and the tile is laid out
// (x stride 1 padded to 12, y stride 12, z stride 140 = 12 mod 32) so that
// every 128-bit tile access of a warp is free of bank conflicts: in the y and
// z phases lanes 3b..3b+2 cover one 12-float row; in the x phase the lines of
// one 8-lane phase have distinct (y + z) mod 8 (kFdm8XLine).  Each output is
// the same sequence of FMAs as in the generic kernel (l = 0..9 in order).
// ---------------------------------------------------------------------------
namespace fdm8 {
constexpr int XS = 12, ZS = 140, WN = 10 * ZS; // tile strides; the z plane is padded to 140 floats
constexpr int SR = 12, SN = 3 * 10 * SR;       // S rows padded to 12 floats, 3 directions
constexpr int EPC = 4;                         // elements (warps) per CTA
} // namespace fdm8

// Tile offset of x-line r (0..3) of lane L (0..24), kFdm8XLine[r][L].  The
// 100 lines (y, z) are grouped by (y + z) mod 8 (class sizes 13, 14, 13, 12,
// 12, 12, 12, 12), each class ordered by y + z, then y; lanes 8p..8p+7 of
// step r take line 3r + p of classes 0..7 and lane 24 takes the four lines
// left over (class 0 #12, class 1 #12 and #13, class 2 #12).  Lines of one
// 8-lane phase then start in distinct 4-bank groups.
__device__ const short kFdm8XLine[4][32] = {
    {0, 140, 280, 420, 560, 700, 840, 980, 1120, 12, 152, 292, 432, 572, 712, 852,
     992, 1260, 24, 164, 304, 444, 584, 724, 1088, 0, 0, 0, 0, 0, 0, 0},
    {864, 1132, 1272, 36, 176, 316, 456, 596, 736, 1004, 1144, 1284, 48, 188, 328, 468,
     608, 876, 1016, 1156, 1296, 60, 200, 340, 1356, 0, 0, 0, 0, 0, 0, 0},
    {480, 748, 888, 1028, 1168, 1308, 72, 212, 352, 620, 760, 900, 1040, 1180, 1320, 84,
     224, 492, 632, 772, 912, 1052, 1192, 1332, 1228, 0, 0, 0, 0, 0, 0, 0},
    {96, 364, 504, 644, 784, 924, 1064, 1204, 1344, 236, 376, 516, 656, 796, 936, 1076,
     1216, 108, 248, 388, 528, 668, 808, 948, 1368, 0, 0, 0, 0, 0, 0, 0}};

__device__ __forceinline__ void fdm8_row(const float *S, float sv[10])
{
  const float4 a = *(const float4 *)S, b = *(const float4 *)(S + 4), c = *(const float4 *)(S + 8);
  sv[0] = a.x; sv[1] = a.y; sv[2] = a.z; sv[3] = a.w;
  sv[4] = b.x; sv[5] = b.y; sv[6] = b.z; sv[7] = b.w;
  sv[8] = c.x; sv[9] = c.y;
}

// out(i) = sum_l M[i][l] in(l) along x for the lane's 4 lines, in place
__device__ __forceinline__ void fdm8_x(float *w, const float *M, const int base[4], int lane)
{
  if (lane >= 25) return;
  float in[4][10], out[4][10];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const float4 a = *(const float4 *)(w + base[r]), b = *(const float4 *)(w + base[r] + 4);
    const float2 c = *(const float2 *)(w + base[r] + 8);
    in[r][0] = a.x; in[r][1] = a.y; in[r][2] = a.z; in[r][3] = a.w;
    in[r][4] = b.x; in[r][5] = b.y; in[r][6] = b.z; in[r][7] = b.w;
    in[r][8] = c.x; in[r][9] = c.y;
  }
#pragma unroll
  for (int i = 0; i < 10; ++i) {
    float sv[10];
    fdm8_row(M + fdm8::SR * i, sv);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      float v = 0.f;
#pragma unroll
      for (int l = 0; l < 10; ++l) v = fmaf(sv[l], in[r][l], v);
      out[r][i] = v;
    }
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    *(float4 *)(w + base[r]) = make_float4(out[r][0], out[r][1], out[r][2], out[r][3]);
    *(float4 *)(w + base[r] + 4) = make_float4(out[r][4], out[r][5], out[r][6], out[r][7]);
    *(float2 *)(w + base[r] + 8) = make_float2(out[r][8], out[r][9]);
  }
}

// the same along y (stride 12) or z (stride 140) for the lane's bundle of 4
// adjacent x-lines; with `lam`, the forward z pass scales by 1/(lx + ly + lz)
template <int STRIDE, bool SCALE>
__device__ __forceinline__ void fdm8_yz(float *w, const float *M, int off, int lane, const float *lam, int y)
{
  if (lane >= 30) return;
  float4 in[10];
#pragma unroll
  for (int l = 0; l < 10; ++l) in[l] = *(const float4 *)(w + off + STRIDE * l);
  const int x0 = 4 * (lane % 3);
#pragma unroll
  for (int j = 0; j < 10; ++j) {
    float sv[10];
    fdm8_row(M + fdm8::SR * j, sv);
    // paired FP32 FMAs (two round-to-nearest fmaf per instruction: the same results, half the issue slots)
    float2 va = make_float2(0.f, 0.f), vb = make_float2(0.f, 0.f);
#pragma unroll
    for (int l = 0; l < 10; ++l) {
      const float2 s2 = make_float2(sv[l], sv[l]);
      va = __ffma2_rn(s2, make_float2(in[l].x, in[l].y), va);
      vb = __ffma2_rn(s2, make_float2(in[l].z, in[l].w), vb);
    }
    float4 v = make_float4(va.x, va.y, vb.x, vb.y);
    if (SCALE) {
      float sc[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int x = x0 + c;
        const float d = x < 10 ? (lam[x] + lam[10 + y]) + lam[20 + j] : 0.f;
        sc[c] = d > 1e-5f ? __frcp_rn(d) : 0.f; // the correctly rounded 1/d, as 1.f / d
      }
      v.x *= sc[0];
      v.y *= sc[1];
      v.z *= sc[2];
      v.w *= sc[3];
    }
    *(float4 *)(w + off + STRIDE * j) = v;
  }
}

__device__ __forceinline__ int fdm8_ext(int f, int a, int b)
{
  using namespace fdm8;
  switch (f) {
  case 0: return 0 + XS * (a + 1) + ZS * (b + 1);
  case 1: return 9 + XS * (a + 1) + ZS * (b + 1);
  case 2: return (a + 1) + XS * 0 + ZS * (b + 1);
  case 3: return (a + 1) + XS * 9 + ZS * (b + 1);
  case 4: return (a + 1) + XS * (b + 1) + ZS * 0;
  default: return (a + 1) + XS * (b + 1) + ZS * 9;
  }
}

template <bool RAS>
__global__ void __launch_bounds__(32 * fdm8::EPC, 5)
    fdm8_kernel(long long E, const float *__restrict__ u, const int *__restrict__ haloSrc,
                const float *__restrict__ Sx, const float *__restrict__ Sy, const float *__restrict__ Sz,
                const float *__restrict__ lam, const float *__restrict__ wts, float *__restrict__ Su,
                float *__restrict__ haloOut)
{
  using namespace fdm8;
  constexpr int NP = 512, NF = 64;
  __shared__ __align__(16) float s_w[EPC][WN];
  __shared__ __align__(16) float s_F[EPC][SN]; // F[d][i][l] = S_d(l, i): forward rows
  __shared__ __align__(16) float s_B[EPC][SN]; // B[d][i][l] = S_d(i, l): backward rows
  __shared__ float s_lam[EPC][32];
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  const long long e = (long long)blockIdx.x * EPC + wp;
  if (e >= E) return; // whole warp; the kernel uses warp-level synchronisation only
  float *w = s_w[wp], *F = s_F[wp], *B = s_B[wp], *lm = s_lam[wp];
  // every global load of the element first, all independent (one round trip
  // for S, lambda, u and the halo indices, one more for the halo values)
  const float *Sd[3] = {Sx + e * 100, Sy + e * 100, Sz + e * 100};
  float sreg[3][4];
#pragma unroll
  for (int d = 0; d < 3; ++d)
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const int q = lane + 32 * m;
      sreg[d][m] = q < 100 ? __ldg(Sd[d] + q) : 0.f;
    }
  const float lmv = lane < 30 ? __ldg(lam + e * 30 + lane) : 0.f;
  const float4 *ue4 = (const float4 *)(u + e * NP);
  float4 uv[4];
#pragma unroll
  for (int m = 0; m < 4; ++m) uv[m] = __ldg(ue4 + lane + 32 * m);
  const int *hs = haloSrc + e * 6 * NF;
  int hsrc[12];
#pragma unroll
  for (int m = 0; m < 12; ++m) hsrc[m] = __ldg(hs + lane + 32 * m);
  float hv[12];
#pragma unroll
  for (int m = 0; m < 12; ++m) hv[m] = hsrc[m] >= 0 ? __ldg(u + hsrc[m]) : 0.f;
  // tile: zero, then own nodes and halo
  for (int q = lane; q < WN / 4; q += 32) ((float4 *)w)[q] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int d = 0; d < 3; ++d)
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const int q = lane + 32 * m;
      if (q < 100) {
        const int r = q % 10, c = q / 10; // S_d(r, c) = Sd[r + 10 c]
        F[(d * 10 + c) * SR + r] = sreg[d][m];
        B[(d * 10 + r) * SR + c] = sreg[d][m];
      }
    }
  for (int q = lane; q < 60; q += 32) { // row pads (columns 10, 11)
    const int row = q >> 1, col = 10 + (q & 1);
    F[row * SR + col] = 0.f;
    B[row * SR + col] = 0.f;
  }
  if (lane < 30) lm[lane] = lmv;
  __syncwarp();
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    const int q = lane + 32 * m;
    const int i = (4 * q) & 7, j = (q >> 1) & 7, k = q >> 4;
    float *dst = w + (i + 1) + XS * (j + 1) + ZS * (k + 1);
    dst[0] = uv[m].x;
    dst[1] = uv[m].y;
    dst[2] = uv[m].z;
    dst[3] = uv[m].w;
  }
#pragma unroll
  for (int m = 0; m < 12; ++m) {
    const int q = lane + 32 * m;
    const int f = q / NF, pp = q % NF;
    w[fdm8_ext(f, pp % 8, pp / 8)] = hv[m];
  }
  __syncwarp();
  int base[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) base[r] = kFdm8XLine[r][lane];
  const int offY = 4 * (lane % 3) + ZS * (lane / 3); // bundle (x quad, z) for the y pass
  const int offZ = 4 * (lane % 3) + XS * (lane / 3); // bundle (x quad, y) for the z pass
  fdm8_x(w, F, base, lane);
  __syncwarp();
  fdm8_yz<XS, false>(w, F + 10 * SR, offY, lane, lm, 0);
  __syncwarp();
  fdm8_yz<ZS, true>(w, F + 20 * SR, offZ, lane, lm, lane / 3);
  __syncwarp();
  fdm8_x(w, B, base, lane);
  __syncwarp();
  fdm8_yz<XS, false>(w, B + 10 * SR, offY, lane, lm, 0);
  __syncwarp();
  fdm8_yz<ZS, false>(w, B + 20 * SR, offZ, lane, lm, 0);
  __syncwarp();
  float *se = Su + e * NP;
  for (int q = lane; q < NP / 4; q += 32) {
    const int i = (4 * q) & 7, j = (q >> 1) & 7, k = q >> 4;
    const float *src = w + (i + 1) + XS * (j + 1) + ZS * (k + 1);
    float4 v = make_float4(src[0], src[1], src[2], src[3]);
    if (RAS) {
      const float4 wt = __ldg((const float4 *)(wts + e * NP) + q);
      v.x *= wt.x;
      v.y *= wt.y;
      v.z *= wt.z;
      v.w *= wt.w;
    }
    ((float4 *)se)[q] = v;
  }
  if (!RAS) {
    float *ho = haloOut + e * 6 * NF;
    for (int q = lane; q < 6 * NF; q += 32) {
      const int f = q / NF, pp = q % NF;
      ho[q] = w[fdm8_ext(f, pp % 8, pp / 8)];
    }
  }
}

// ---------------------------------------------------------------------------
// Order-7 RAS FDM in FP16 on the tensor cores, per-element max-abs scaling.
//
// One warp per element.  The (N+3)^3 = 10^3 extended tile lives in shared
// memory as FP16 "lines": line L = u + 10 v (the two coordinates other than
// the one contracted), its 10 entries along the contracted coordinate
// contiguous, padded to 16 (zeros) and strided by 24 halfs so that the B
// fragment loads are bank-conflict free.  Each of the six 1-D transforms
// (S^T along x, y, z, then S along x, y, z) is a 16x16 (padded 10x10)
// matrix times the 16 x 104 line block: 13 mma.sync.m16n8k16 (FP16 inputs,
// FP32 accumulation).  The output of a pass, row r (the new coordinate) of
// line L = u + 10 v, is stored for the next pass at line v + 10 r, entry u:
// the coordinates rotate (x, y, z) -> (y, z, x) every pass, so that every
// pass contracts over contiguous entries.  Scaling: the input tile is divided
// by max |u_ext| of the element, each direction's S by its max |S|, and each
// pass's FP32 result by its max before it is rounded to FP16 again; the scale
// factors multiply up in FP32 and are applied to the final FP32 result.  The
// z-forward pass multiplies by 1/(lx + ly + lz) (0 where <= 1e-5) in FP32.
// ---------------------------------------------------------------------------
namespace fdm8h {
constexpr int LS = 24;        // halfs per line (16 used)
constexpr int TN = 104 * LS;  // halfs per tile (104 lines: 13 blocks of 8)
constexpr int EPC = 4;        // elements (warps) per CTA
} // namespace fdm8h

__device__ __forceinline__ unsigned pack_h2(float lo, float hi)
{
  const __half2 h = __floats2half2_rn(lo, hi);
  return *reinterpret_cast<const unsigned *>(&h);
}

__device__ __forceinline__ void mma16816(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1)
{
  asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
               "{%0,%1,%2,%3};"
               : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
               : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ float warp_max(float v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// A fragment of the 16x16 matrix M[o][i] (o, i < 10; zero elsewhere) scaled by inv:
// forward (S^T) M[o][i] = S(i, o) = Sd[i + 10 o]; backward (S) M[o][i] = S(o, i) = Sd[o + 10 i]
__device__ __forceinline__ void fdm8h_afrag(const float *Sd, bool fwd, float inv, int g, int t, unsigned (&a)[4])
{
  auto m = [&](int o, int i) -> float {
    if (o >= 10 || i >= 10) return 0.f;
    return (fwd ? __ldg(Sd + i + 10 * o) : __ldg(Sd + o + 10 * i)) * inv;
  };
  a[0] = pack_h2(m(g, 2 * t), m(g, 2 * t + 1));
  a[1] = pack_h2(m(g + 8, 2 * t), m(g + 8, 2 * t + 1));
  a[2] = pack_h2(m(g, 2 * t + 8), m(g, 2 * t + 9));
  a[3] = pack_h2(m(g + 8, 2 * t + 8), m(g + 8, 2 * t + 9));
}

// fragment element q (0..3) of block nb: row r, line L
__device__ __forceinline__ void fdm8h_rl(int nb, int q, int g, int t, int &r, int &L)
{
  r = g + ((q & 2) ? 8 : 0);
  L = 8 * nb + 2 * t + (q & 1);
}

// 1/(lx + ly + lz) of mode (u, v, r) of the z-forward pass (0 where the sum is <= 1e-5)
__device__ __forceinline__ float fdm8h_invl(const float *lm, int uu, int vv, int r)
{
  const float den = (lm[uu] + lm[10 + vv]) + lm[20 + r];
  return den > 1e-5f ? __fdividef(1.f, den) : 0.f; // approximate: the value is rounded to FP16 next
}

// max |(A x tile_in) / (lx + ly + lz)| over the element (the z-forward pass's
// result, whose modes span many decades: it is scaled by its own maximum)
__device__ __forceinline__ float fdm8h_invl_max(const __half *tin, const unsigned (&a)[4], int g, int t,
                                                const float *lm)
{
  using namespace fdm8h;
  float mx = 0.f;
#pragma unroll
  for (int nb = 0; nb < 13; ++nb) {
    const __half *line = tin + (8 * nb + g) * LS + 2 * t;
    const unsigned b0 = *reinterpret_cast<const unsigned *>(line);
    const unsigned b1 = *reinterpret_cast<const unsigned *>(line + 8);
    float d[4] = {0.f, 0.f, 0.f, 0.f};
    mma16816(d, a, b0, b1);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int r, L;
      fdm8h_rl(nb, q, g, t, r, L);
      if (r < 10 && L < 100) mx = fmaxf(mx, fabsf(d[q] * fdm8h_invl(lm, L % 10, L / 10, r)));
    }
  }
  mx = warp_max(mx);
  return mx > 0.f ? mx : 1.f;
}

// One pass: D = A x tile_in, block by block (8 lines each); each result is
// multiplied by f (and, on the z-forward pass, by 1/(lx + ly + lz)) and stored
// rotated into tout: row r of line L = u + 10 v -> line v + 10 r, entry u.
template <bool INVL>
__device__ __forceinline__ void fdm8h_pass(const __half *tin, __half *tout, const unsigned (&a)[4], int g, int t,
                                           float f, const float *lm, const short *offs)
{
  using namespace fdm8h;
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int nb = 0; nb < 13; ++nb) {
    const __half *line = tin + (8 * nb + g) * LS + 2 * t;
    const unsigned b0 = *reinterpret_cast<const unsigned *>(line);
    const unsigned b1 = *reinterpret_cast<const unsigned *>(line + 8);
    float d[4] = {0.f, 0.f, 0.f, 0.f};
    mma16816(d, a, b0, b1);
    // d0, d1: row g, lines L and L + 1 (L even, so entries u and u + 1 of one
    // line of the next tile); d2, d3: row g + 8 (offset + 80 lines)
    const int off = offs[nb * 32 + lane];
    if (off >= 0) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        if (h == 0 || g < 2) {
          float v0 = d[2 * h] * f, v1 = d[2 * h + 1] * f;
          if (INVL) {
            const int L = 8 * nb + 2 * t, uu = L % 10, vv = L / 10, r = g + 8 * h;
            v0 *= fdm8h_invl(lm, uu, vv, r);
            v1 *= fdm8h_invl(lm, uu + 1, vv, r);
          }
          *reinterpret_cast<__half2 *>(tout + off + h * 80 * LS) = __floats2half2_rn(v0, v1);
        }
      }
    }
  }
}

__global__ void __launch_bounds__(32 * fdm8h::EPC)
    fdm8h_kernel(long long E, const float *__restrict__ u, const int *__restrict__ haloSrc,
                 const float *__restrict__ Sx, const float *__restrict__ Sy, const float *__restrict__ Sz,
                 const float *__restrict__ lam, const float *__restrict__ wts, float *__restrict__ Su)
{
  using namespace fdm8h;
  constexpr int NP = 512, NF = 64;
  __shared__ __align__(16) __half s_t[EPC][2][TN];
  __shared__ float s_lam[EPC][32];
  __shared__ short s_off[13 * 32]; // store offset of lane's row-g results of block nb, -1 past line 99
  for (int q = threadIdx.x; q < 13 * 32; q += blockDim.x) {
    const int nb = q / 32, ln = q % 32, L = 8 * nb + 2 * (ln & 3);
    s_off[q] = L < 100 ? (short)(((L / 10) + 10 * (ln >> 2)) * fdm8h::LS + L % 10) : (short)-1;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  __half *T0 = s_t[wp][0], *T1 = s_t[wp][1];
  float *lm = s_lam[wp];
  const long long e = (long long)blockIdx.x * EPC + wp;
  if (e >= E) return; // whole warp; warp-level synchronisation only
  // both tiles zero (16-byte stores): the K pads (entries 10..15), lines
  // 100..103 and the 104 points of the extended cube that neither own nodes
  // nor the halo cover stay zero; no pass writes the pads
  for (int q = lane; q < TN / 8; q += 32) {
    reinterpret_cast<uint4 *>(T0)[q] = make_uint4(0u, 0u, 0u, 0u);
    reinterpret_cast<uint4 *>(T1)[q] = make_uint4(0u, 0u, 0u, 0u);
  }
  // global loads first: own nodes, halo indices and values, lambda, S
  const float4 *ue4 = (const float4 *)(u + e * NP);
  float4 uv[4];
#pragma unroll
  for (int m = 0; m < 4; ++m) uv[m] = __ldg(ue4 + lane + 32 * m);
  const int *hs = haloSrc + e * 6 * NF;
  float hv[12];
#pragma unroll
  for (int m = 0; m < 12; ++m) {
    const int src = __ldg(hs + lane + 32 * m);
    hv[m] = src >= 0 ? __ldg(u + src) : 0.f;
  }
  const float lmv = lane < 30 ? __ldg(lam + e * 30 + lane) : 0.f;
  const float *Sxe = Sx + e * 100, *Sye = Sy + e * 100, *Sze = Sz + e * 100;
  float smx = 0.f, smy = 0.f, smz = 0.f;
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    const int q = lane + 32 * m;
    if (q < 100) {
      smx = fmaxf(smx, fabsf(__ldg(Sxe + q)));
      smy = fmaxf(smy, fabsf(__ldg(Sye + q)));
      smz = fmaxf(smz, fabsf(__ldg(Sze + q)));
    }
  }
  if (lane < 30) lm[lane] = lmv;
  // per-element scales: max |u_ext|, max |S_d|, max 1/(lx + ly + lz)
  float mx = 0.f;
#pragma unroll
  for (int m = 0; m < 4; ++m)
    mx = fmaxf(mx, fmaxf(fmaxf(fabsf(uv[m].x), fabsf(uv[m].y)), fmaxf(fabsf(uv[m].z), fabsf(uv[m].w))));
#pragma unroll
  for (int m = 0; m < 12; ++m) mx = fmaxf(mx, fabsf(hv[m]));
  mx = warp_max(mx);
  smx = warp_max(smx);
  smy = warp_max(smy);
  smz = warp_max(smz);
  if (!(mx > 0.f)) mx = 1.f;
  if (!(smx > 0.f)) smx = 1.f;
  if (!(smy > 0.f)) smy = 1.f;
  if (!(smz > 0.f)) smz = 1.f;
  const float inv = 1.f / mx;
  __syncwarp();
  // tile 0: line y + 10 z, entry x (extended coordinates 0..9; own nodes at 1..8)
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    const int q = lane + 32 * m;
    const int i = (4 * q) & 7, j = (q >> 1) & 7, k = q >> 4;
    __half *dst = T0 + ((j + 1) + 10 * (k + 1)) * LS + (i + 1);
    dst[0] = __float2half_rn(uv[m].x * inv);
    dst[1] = __float2half_rn(uv[m].y * inv);
    dst[2] = __float2half_rn(uv[m].z * inv);
    dst[3] = __float2half_rn(uv[m].w * inv);
  }
#pragma unroll
  for (int m = 0; m < 12; ++m) {
    const int q = lane + 32 * m;
    const int f = q / NF, pp = q % NF, a = pp % 8 + 1, b = pp / 8 + 1;
    int x, y, z;
    switch (f) {
    case 0: x = 0; y = a; z = b; break;
    case 1: x = 9; y = a; z = b; break;
    case 2: x = a; y = 0; z = b; break;
    case 3: x = a; y = 9; z = b; break;
    case 4: x = a; y = b; z = 0; break;
    default: x = a; y = b; z = 9; break;
    }
    T0[(y + 10 * z) * LS + x] = __float2half_rn(hv[m] * inv);
  }
  __syncwarp();
  // |S/max| <= 1 and |stored input| <= 1, so a pass result is at most 10 in
  // magnitude: stored passes are multiplied by 1/10, except the z-forward
  // pass, whose result times 1/(lx + ly + lz) is divided by its own maximum;
  // scale collects the true magnitude
  constexpr float kF = 0.1f;
  float scale = mx * (smx * smx) * (smy * smy) * (smz * smz) * 1e4f;
  unsigned a[4];
  fdm8h_afrag(Sxe, true, 1.f / smx, g, t, a);
  fdm8h_pass<false>(T0, T1, a, g, t, kF, lm, s_off);
  __syncwarp();
  fdm8h_afrag(Sye, true, 1.f / smy, g, t, a);
  fdm8h_pass<false>(T1, T0, a, g, t, kF, lm, s_off);
  __syncwarp();
  fdm8h_afrag(Sze, true, 1.f / smz, g, t, a);
  const float m2 = fdm8h_invl_max(T0, a, g, t, lm);
  scale *= m2;
  fdm8h_pass<true>(T0, T1, a, g, t, 1.f / m2, lm, s_off);
  __syncwarp();
  fdm8h_afrag(Sxe, false, 1.f / smx, g, t, a);
  fdm8h_pass<false>(T1, T0, a, g, t, kF, lm, s_off);
  __syncwarp();
  fdm8h_afrag(Sye, false, 1.f / smy, g, t, a);
  fdm8h_pass<false>(T0, T1, a, g, t, kF, lm, s_off);
  __syncwarp();
  // final pass (S_z) in FP32: rows r = z'', lines (x'', y''); own nodes at
  // 1..8, staged in T0 (not read by this pass) for coalesced stores
  fdm8h_afrag(Sze, false, 1.f / smz, g, t, a);
  float *stage = reinterpret_cast<float *>(T0);
#pragma unroll
  for (int nb = 0; nb < 13; ++nb) {
    const __half *line = T1 + (8 * nb + g) * LS + 2 * t;
    const unsigned b0 = *reinterpret_cast<const unsigned *>(line);
    const unsigned b1 = *reinterpret_cast<const unsigned *>(line + 8);
    float d[4] = {0.f, 0.f, 0.f, 0.f};
    mma16816(d, a, b0, b1);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int r, L;
      fdm8h_rl(nb, q, g, t, r, L);
      const int x = L % 10, y = L / 10;
      if (r >= 1 && r <= 8 && L < 100 && x >= 1 && x <= 8 && y >= 1 && y <= 8)
        stage[(x - 1) + 8 * (y - 1) + 64 * (r - 1)] = d[q] * scale;
    }
  }
  __syncwarp();
  float *se = Su + e * NP;
  for (int q = lane; q < NP / 4; q += 32) {
    float4 v = reinterpret_cast<const float4 *>(stage)[q];
    const float4 wt = __ldg((const float4 *)(wts + e * NP) + q);
    v.x *= wt.x;
    v.y *= wt.y;
    v.z *= wt.z;
    v.w *= wt.w;
    ((float4 *)se)[q] = v;
  }
}

// ---------------------------------------------------------------------------
// FDM (Schwarz local solve) on the tensor cores in TF32 (fdmPrecision = tf32).
// Each 1-D transform of the extended element is the product of the element's
// NX x NX eigenvector matrix (NX = N + 3) with its NX^2 lines, done as
// mma.sync m16n8k8 with TF32 inputs and FP32 accumulation: M = the NX output
// points (padded to 16), N = the lines in tiles of 8, K = the NX input points
// in steps of 8.  TF32 has FP16's 11-bit significand but FP32's exponent
// range, so, unlike the FP16 form, it needs no scaling.  One warp per element.
// The element lives in shared memory as lines of LS floats (line n, point k at
// n LS + k); every pass writes its result rotated, point (k; b, c) of the
// input becoming point b of line c + NX m of the output, so that the next
// direction is again the contiguous one and three passes restore the layout.
// With LS = 12 (= 4 mod 8) the 8 lines a fragment load touches start in
// distinct 4-bank groups, and the paired 64-bit result stores of a half-warp
// are free of bank conflicts.  Inputs of every pass are rounded to TF32
// (cvt.rna) when they are stored; the last pass keeps FP32.
// ---------------------------------------------------------------------------
namespace fdmtc {
constexpr int LS = 12;
constexpr int EPC = 4; // elements (warps) per CTA
template <int NQ> struct Shape {
  static constexpr int NX = NQ + 2, lines = NX * NX, nt = (lines + 7) / 8, ks = (NX + 7) / 8;
  static constexpr int buf = nt * 8 * LS; // floats per tile buffer (whole tiles of 8 lines)
  static_assert(NX % 2 == 0 && NX <= LS, "even extended size of at most 12 points");
};
} // namespace fdmtc

__device__ __forceinline__ uint32_t f2tf32(float x)
{
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float round_tf32(float x) { return __uint_as_float(f2tf32(x)); }

__device__ __forceinline__ void mma_tf32(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1)
{
  asm("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// A fragments (m16n8k8, row major) of one direction: forward M(i, l) = S(l, i), backward M(i, l) = S(i, l),
// S(r, c) = Sd[r + NX c]; a0..a3 = M(g, k), M(g + 8, k), M(g, k + 4), M(g + 8, k + 4) with k = 8 s + t
template <int NX, int KS>
__device__ __forceinline__ void fdmtc_afrag(const float *__restrict__ Sd, bool fwd, int g, int t, uint32_t A[KS][4])
{
#pragma unroll
  for (int s = 0; s < KS; ++s)
#pragma unroll
    for (int h = 0; h < 4; ++h) {
      const int row = g + 8 * (h & 1), col = 8 * s + t + 4 * (h >> 1);
      const float v = (row < NX && col < NX) ? __ldg(Sd + (fwd ? col + NX * row : row + NX * col)) : 0.f;
      A[s][h] = f2tf32(v);
    }
}

// one direction: out(m; line c + NX m, point b) = sum_k M(m, k) in(line b + NX c, point k).  MODE 0 rounds the
// result to TF32, MODE 1 first scales it by 1/(lxy[n] + lz[m]) (n = b + NX c), MODE 2 keeps FP32.
template <int NX, int KS, int NT, int MODE>
__device__ __forceinline__ void fdmtc_pass(const float *in, float *out, const uint32_t A[KS][4], int g, int t,
                                           const float *lxy, float lz0, float lz1)
{
  constexpr int LS = fdmtc::LS, LINES = NX * NX;
#pragma unroll
  for (int j = 0; j < NT; ++j) {
    const float *src = in + (8 * j + g) * LS;
    float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int s = 0; s < KS; ++s) {
      const int k0 = 8 * s + t, k1 = k0 + 4;
      uint32_t b0 = 0u, b1 = 0u;
      if (8 * s < NX) {
        const float v = src[k0]; // k0 < LS: inside the line; points past NX are taken as 0
        b0 = k0 < NX ? __float_as_uint(v) : 0u;
      }
      if (8 * s + 4 < NX) {
        const float v = src[k1];
        b1 = k1 < NX ? __float_as_uint(v) : 0u;
      }
      mma_tf32(c, A[s], b0, b1);
    }
    const int n0 = 8 * j + 2 * t; // this lane's result columns n0, n0 + 1 (same c: NX and n0 are even)
    if (n0 < LINES) {
      const int cc = n0 / NX, b = n0 - NX * cc;
      if (MODE == 1) {
        const float2 xy = *(const float2 *)(lxy + n0);
        const float d0 = xy.x + lz0, d1 = xy.y + lz0, d2 = xy.x + lz1, d3 = xy.y + lz1;
        c[0] *= d0 > 1e-5f ? __fdividef(1.f, d0) : 0.f;
        c[1] *= d1 > 1e-5f ? __fdividef(1.f, d1) : 0.f;
        c[2] *= d2 > 1e-5f ? __fdividef(1.f, d2) : 0.f;
        c[3] *= d3 > 1e-5f ? __fdividef(1.f, d3) : 0.f;
      }
      if (MODE != 2) {
#pragma unroll
        for (int h = 0; h < 4; ++h) c[h] = round_tf32(c[h]);
      }
      if (g < NX) *(float2 *)(out + (cc + NX * g) * LS + b) = make_float2(c[0], c[1]);
      if (g + 8 < NX) *(float2 *)(out + (cc + NX * (g + 8)) * LS + b) = make_float2(c[2], c[3]);
    }
  }
}

// extended-element point of halo node (a, b) of face f, in the lines-of-x layout
template <int NX> __device__ __forceinline__ int fdmtc_ext(int f, int a, int b)
{
  constexpr int LS = fdmtc::LS;
  int x, y, z;
  switch (f) {
  case 0: x = 0, y = a + 1, z = b + 1; break;
  case 1: x = NX - 1, y = a + 1, z = b + 1; break;
  case 2: x = a + 1, y = 0, z = b + 1; break;
  case 3: x = a + 1, y = NX - 1, z = b + 1; break;
  case 4: x = a + 1, y = b + 1, z = 0; break;
  default: x = a + 1, y = b + 1, z = NX - 1; break;
  }
  return (y + NX * z) * LS + x;
}

template <int NQ, bool RAS>
__global__ void __launch_bounds__(32 * fdmtc::EPC, 4)
    fdmtc_kernel(long long E, const float *__restrict__ u, const int *__restrict__ haloSrc,
                 const float *__restrict__ Sx, const float *__restrict__ Sy, const float *__restrict__ Sz,
                 const float *__restrict__ lam, const float *__restrict__ wts, float *__restrict__ Su,
                 float *__restrict__ haloOut)
{
  using Sh = fdmtc::Shape<NQ>;
  constexpr int NX = Sh::NX, KS = Sh::ks, NT = Sh::nt, LS = fdmtc::LS, BUF = Sh::buf;
  constexpr int NP = NQ * NQ * NQ, NF = NQ * NQ, LN = NX * NX;
  __shared__ __align__(16) float s_t[fdmtc::EPC][2][BUF];
  __shared__ __align__(16) float s_xy[fdmtc::EPC][(LN + 3) / 4 * 4];
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5, g = lane >> 2, t = lane & 3;
  const long long e = (long long)blockIdx.x * fdmtc::EPC + wp;
  if (e >= E) return; // whole warp; warp-level synchronisation only
  float *T0 = s_t[wp][0], *T1 = s_t[wp][1], *lxy = s_xy[wp];
  const float *le = lam + e * 3 * NX;
  // tile: zero (edges and corners of the extended element stay 0), own nodes, halo; lx + ly per line
  for (int q = lane; q < BUF / 4; q += 32) ((float4 *)T0)[q] = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int q = lane; q < LN; q += 32) lxy[q] = __ldg(le + q % NX) + __ldg(le + NX + q / NX);
  const float lz0 = g < NX ? __ldg(le + 2 * NX + g) : 0.f;
  const float lz1 = g + 8 < NX ? __ldg(le + 2 * NX + g + 8) : 0.f;
  __syncwarp();
  const float *ue = u + e * NP;
  for (int q = lane; q < NP; q += 32) {
    const int x = q % NQ, y = (q / NQ) % NQ, z = q / NF;
    T0[((y + 1) + NX * (z + 1)) * LS + (x + 1)] = round_tf32(__ldg(ue + q));
  }
  const int *hs = haloSrc + e * 6 * NF;
  for (int q = lane; q < 6 * NF; q += 32) {
    const int src = __ldg(hs + q);
    const int f = q / NF, pp = q % NF;
    T0[fdmtc_ext<NX>(f, pp % NQ, pp / NQ)] = src >= 0 ? round_tf32(__ldg(u + src)) : 0.f;
  }
  __syncwarp();
  const float *S3[3] = {Sx + e * LN, Sy + e * LN, Sz + e * LN};
  uint32_t A[KS][4];
  // forward S^T along x, y, z (scaling by 1/(lx + ly + lz) after z), then backward S along x, y, z
  fdmtc_afrag<NX, KS>(S3[0], true, g, t, A);
  fdmtc_pass<NX, KS, NT, 0>(T0, T1, A, g, t, lxy, lz0, lz1);
  __syncwarp();
  fdmtc_afrag<NX, KS>(S3[1], true, g, t, A);
  fdmtc_pass<NX, KS, NT, 0>(T1, T0, A, g, t, lxy, lz0, lz1);
  __syncwarp();
  fdmtc_afrag<NX, KS>(S3[2], true, g, t, A);
  fdmtc_pass<NX, KS, NT, 1>(T0, T1, A, g, t, lxy, lz0, lz1);
  __syncwarp();
  fdmtc_afrag<NX, KS>(S3[0], false, g, t, A);
  fdmtc_pass<NX, KS, NT, 0>(T1, T0, A, g, t, lxy, lz0, lz1);
  __syncwarp();
  fdmtc_afrag<NX, KS>(S3[1], false, g, t, A);
  fdmtc_pass<NX, KS, NT, 0>(T0, T1, A, g, t, lxy, lz0, lz1);
  __syncwarp();
  fdmtc_afrag<NX, KS>(S3[2], false, g, t, A);
  fdmtc_pass<NX, KS, NT, 2>(T1, T0, A, g, t, lxy, lz0, lz1);
  __syncwarp();
  float *se = Su + e * NP;
  for (int q = lane; q < NP; q += 32) {
    const int x = q % NQ, y = (q / NQ) % NQ, z = q / NF;
    float v = T0[((y + 1) + NX * (z + 1)) * LS + (x + 1)];
    if (RAS) v *= __ldg(wts + e * NP + q);
    se[q] = v;
  }
  if (!RAS) {
    float *ho = haloOut + e * 6 * NF;
    for (int q = lane; q < 6 * NF; q += 32) {
      const int f = q / NF, pp = q % NF;
      ho[q] = T0[fdmtc_ext<NX>(f, pp % NQ, pp / NQ)];
    }
  }
}

bool launch_fdm_tf32(int N, long long E, bool ras, const float *u, const int *haloSrc, const float *Sx,
                     const float *Sy, const float *Sz, const float *lam, const float *wts, float *Su, float *haloOut,
                     cudaStream_t s)
{
  if (E <= 0) return true;
  if (!lam) return false;
  const unsigned grid = (unsigned)((E + fdmtc::EPC - 1) / fdmtc::EPC);
  const unsigned blk = 32 * fdmtc::EPC;
#define NRSG_FDMTC(NQ)                                                                                     \
  if (ras)                                                                                                 \
    fdmtc_kernel<NQ, true><<<grid, blk, 0, s>>>(E, u, haloSrc, Sx, Sy, Sz, lam, wts, Su, haloOut);        \
  else                                                                                                     \
    fdmtc_kernel<NQ, false><<<grid, blk, 0, s>>>(E, u, haloSrc, Sx, Sy, Sz, lam, wts, Su, haloOut);
  switch (N) {
  case 3: NRSG_FDMTC(4) break;
  case 5: NRSG_FDMTC(6) break;
  case 7: NRSG_FDMTC(8) break;
  default: return false;
  }
#undef NRSG_FDMTC
  NRSG_CHECK_LAUNCH();
  return true;
}

bool launch_fdm8h(long long E, const float *u, const int *haloSrc, const float *Sx, const float *Sy, const float *Sz,
                  const float *lam, const float *wts, float *Su, cudaStream_t s)
{
  if (E <= 0) return true;
  if (!lam) return false;
  const unsigned grid = (unsigned)((E + fdm8h::EPC - 1) / fdm8h::EPC);
  fdm8h_kernel<<<grid, 32 * fdm8h::EPC, 0, s>>>(E, u, haloSrc, Sx, Sy, Sz, lam, wts, Su);
  NRSG_CHECK_LAUNCH();
  return true;
}

// ---------------------------------------------------------------------------
// Order-3 FP32 FDM (N + 3 = 6 points per direction, the 6^3 extended tile),
// RECIP form: the reference's preFDM / fusedFDM / postFDM at p_Nq = 4
// (kernels/elliptic/fusedFDM.okl, ellipticMultiGridSchwarz.cpp:1056-1156) in
// one launch, the halo read through haloSrc as in fdm_kernel.  Five elements per warp, six lanes per element (lanes 30 and
// 31 take part in the loads only).  Lane a of an element holds one 6 x 6
// plane of the tile in registers: the z-plane z = a for the forward x and y
// transforms, then the y-plane y = a for the forward z transform (scaled by
// 1/(lx + ly + lz)) and the backward x transform, then the x-plane x = a for
// the backward y and z transforms.  The planes pass through shared memory
// three times (warp synchronisation only, no CTA barrier), and each pass
// reads its 6 x 6 S once per lane (nine 16-byte loads) where the line-per-
// thread kernel reads one S entry per multiply-add: that kernel was bound
// by the shared-memory pipe (90% busy, 384 wavefronts per element).  Every
// output is the same sum in the same order as fdm_kernel<float, 4, RAS, true>
// (bit-identical).  Tile stride 228 floats: conflict-free 8-byte y-plane
// accesses, at most two-way conflicts on the z- and x-plane accesses.
// Requires u, S_x, S_y, S_z and wts 16-byte aligned.
// ---------------------------------------------------------------------------
namespace fdm4 {
constexpr int NL = 6, PL = 36, TS = 228; // points per direction, per plane; tile stride
constexpr int EPW = 5, WPC = 4;          // elements per warp, warps per CTA
constexpr int SSZ = 3 * PL;              // S_x, S_y, S_z of an element
} // namespace fdm4

template <bool RAS>
__global__ void __launch_bounds__(32 * fdm4::WPC)
    fdm4_kernel(long long E, const float *__restrict__ u, const int *__restrict__ haloSrc,
                const float *__restrict__ Sx, const float *__restrict__ Sy, const float *__restrict__ Sz,
                const float *__restrict__ lam, const float *__restrict__ wts, float *__restrict__ Su,
                float *__restrict__ haloOut, long long pfAhead)
{
  using namespace fdm4;
  constexpr int NP = 64, NF = 16, NH = 6 * NF;
  __shared__ __align__(16) float s_w[WPC][EPW * TS];
  __shared__ __align__(16) float s_S[WPC][EPW * SSZ];
  __shared__ float s_l[WPC][EPW * 18];
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  const long long e0 = ((long long)blockIdx.x * WPC + wp) * EPW;
  if (e0 >= E) return; // whole warp; the kernel uses warp-level synchronisation only
  const int ne = E - e0 < EPW ? (int)(E - e0) : EPW;
  float *W = s_w[wp], *SS = s_S[wp], *LL = s_l[wp];
  if (pfAhead > 0 && lane == 0 && e0 + pfAhead < E) {
    // the five elements of the warp one wave of CTAs later into L2: u, halo indices, S, weights
    // (contiguous), lambda by lines
    const long long en = e0 + pfAhead;
    const int nn = E - en < EPW ? (int)(E - en) : EPW;
    auto bulk = [](const void *p, unsigned bytes) {
      asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
    };
    bulk(u + en * NP, nn * NP * 4);
    bulk(haloSrc + en * NH, nn * NH * 4);
    bulk(Sx + en * PL, nn * PL * 4);
    bulk(Sy + en * PL, nn * PL * 4);
    bulk(Sz + en * PL, nn * PL * 4);
    if (RAS) bulk(wts + en * NP, nn * NP * 4);
    for (int c = 0; c < nn * 18; c += 32) asm volatile("prefetch.global.L2 [%0];" ::"l"(lam + en * 18 + c) : "memory");
  }
  // tile zero, S, lambda
  for (int q = lane; q < EPW * TS / 4; q += 32) ((float4 *)W)[q] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float4 *src = (const float4 *)((d == 0 ? Sx : d == 1 ? Sy : Sz) + e0 * PL);
    for (int q = lane; q < ne * 9; q += 32) *(float4 *)(SS + (q / 9) * SSZ + d * PL + 4 * (q % 9)) = __ldg(src + q);
  }
  for (int q = lane; q < ne * 18; q += 32) LL[q] = __ldg(lam + e0 * 18 + q);
  // halo indices, then own nodes and halo values
  constexpr int HM = (EPW * NH + 31) / 32;
  const int *hs = haloSrc + e0 * NH;
  int hsrc[HM];
#pragma unroll
  for (int m = 0; m < HM; ++m) {
    const int q = lane + 32 * m;
    hsrc[m] = q < ne * NH ? __ldg(hs + q) : -1;
  }
  float hv[HM];
#pragma unroll
  for (int m = 0; m < HM; ++m) hv[m] = hsrc[m] >= 0 ? __ldg(u + hsrc[m]) : 0.f;
  __syncwarp();
  const float4 *u4 = (const float4 *)(u + e0 * NP);
  for (int q = lane; q < ne * 16; q += 32) {
    const float4 v = __ldg(u4 + q);
    const int r = q % 16;
    float *dst = W + (q / 16) * TS + 1 + NL * (r % 4 + 1) + PL * (r / 4 + 1);
    dst[0] = v.x;
    dst[1] = v.y;
    dst[2] = v.z;
    dst[3] = v.w;
  }
#pragma unroll
  for (int m = 0; m < HM; ++m) {
    const int q = lane + 32 * m;
    if (q < ne * NH) {
      const int h = q % NH, f = h / NF, pp = h % NF;
      W[(q / NH) * TS + halo_ext_index<4>(f, pp % 4, pp / 4)] = hv[m];
    }
  }
  __syncwarp();
  const int ee = lane / 6, a = lane % 6;
  const bool act = lane < 30 && ee < ne;
  float *T = W + (act ? ee : 0) * TS;
  const float *S = SS + (act ? ee : 0) * SSZ, *L = LL + (act ? ee : 0) * 18;
  float P[PL], M[PL];
  auto loadS = [&](int d) {
#pragma unroll
    for (int m = 0; m < 9; ++m) {
      const float4 v = *(const float4 *)(S + d * PL + 4 * m);
      M[4 * m] = v.x, M[4 * m + 1] = v.y, M[4 * m + 2] = v.z, M[4 * m + 3] = v.w;
    }
  };
  if (act) {
    // z-plane z = a: P[x + 6 y]
#pragma unroll
    for (int m = 0; m < 9; ++m) {
      const float4 v = *(const float4 *)(T + PL * a + 4 * m);
      P[4 * m] = v.x, P[4 * m + 1] = v.y, P[4 * m + 2] = v.z, P[4 * m + 3] = v.w;
    }
    loadS(0); // forward x: out i of line y = sum_l S_x(l, i) P[l + 6 y]
#pragma unroll
    for (int y = 0; y < NL; ++y) {
      float o[NL];
#pragma unroll
      for (int i = 0; i < NL; ++i) {
        float v = 0;
#pragma unroll
        for (int l = 0; l < NL; ++l) v += M[l + NL * i] * P[l + NL * y];
        o[i] = v;
      }
#pragma unroll
      for (int i = 0; i < NL; ++i) P[i + NL * y] = o[i];
    }
    loadS(1); // forward y: out j of line x = sum_l S_y(l, j) P[x + 6 l]
#pragma unroll
    for (int x = 0; x < NL; ++x) {
      float o[NL];
#pragma unroll
      for (int j = 0; j < NL; ++j) {
        float v = 0;
#pragma unroll
        for (int l = 0; l < NL; ++l) v += M[l + NL * j] * P[x + NL * l];
        o[j] = v;
      }
#pragma unroll
      for (int j = 0; j < NL; ++j) P[x + NL * j] = o[j];
    }
#pragma unroll
    for (int m = 0; m < 9; ++m)
      *(float4 *)(T + PL * a + 4 * m) = make_float4(P[4 * m], P[4 * m + 1], P[4 * m + 2], P[4 * m + 3]);
  }
  __syncwarp();
  if (act) {
    // y-plane y = a: P[x + 6 z]
#pragma unroll
    for (int z = 0; z < NL; ++z)
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        const float2 v = *(const float2 *)(T + NL * a + PL * z + 2 * m);
        P[2 * m + NL * z] = v.x, P[2 * m + 1 + NL * z] = v.y;
      }
    loadS(2); // forward z, scaled: out k of line x = sum_l S_z(l, k) P[x + 6 l] / (lx[x] + ly[a] + lz[k])
#pragma unroll
    for (int x = 0; x < NL; ++x) {
      float o[NL];
#pragma unroll
      for (int k = 0; k < NL; ++k) {
        float v = 0;
#pragma unroll
        for (int l = 0; l < NL; ++l) v += M[l + NL * k] * P[x + NL * l];
        const float d = L[x] + L[NL + a] + L[2 * NL + k];
        const float sc = d > 1e-5f ? 1.f / d : 0.f;
        o[k] = v * sc;
      }
#pragma unroll
      for (int k = 0; k < NL; ++k) P[x + NL * k] = o[k];
    }
    loadS(0); // backward x: out i of line z = sum_l S_x(i, l) P[l + 6 z]
#pragma unroll
    for (int z = 0; z < NL; ++z) {
      float o[NL];
#pragma unroll
      for (int i = 0; i < NL; ++i) {
        float v = 0;
#pragma unroll
        for (int l = 0; l < NL; ++l) v += M[i + NL * l] * P[l + NL * z];
        o[i] = v;
      }
#pragma unroll
      for (int i = 0; i < NL; ++i) P[i + NL * z] = o[i];
    }
#pragma unroll
    for (int z = 0; z < NL; ++z)
#pragma unroll
      for (int m = 0; m < 3; ++m)
        *(float2 *)(T + NL * a + PL * z + 2 * m) = make_float2(P[2 * m + NL * z], P[2 * m + 1 + NL * z]);
  }
  __syncwarp();
  if (act) {
    // x-plane x = a: P[y + 6 z]
#pragma unroll
    for (int z = 0; z < NL; ++z)
#pragma unroll
      for (int y = 0; y < NL; ++y) P[y + NL * z] = T[a + NL * y + PL * z];
    loadS(1); // backward y: out j of line z = sum_l S_y(j, l) P[l + 6 z]
#pragma unroll
    for (int z = 0; z < NL; ++z) {
      float o[NL];
#pragma unroll
      for (int j = 0; j < NL; ++j) {
        float v = 0;
#pragma unroll
        for (int l = 0; l < NL; ++l) v += M[j + NL * l] * P[l + NL * z];
        o[j] = v;
      }
#pragma unroll
      for (int j = 0; j < NL; ++j) P[j + NL * z] = o[j];
    }
    loadS(2); // backward z: out k of line y = sum_l S_z(k, l) P[y + 6 l]
#pragma unroll
    for (int y = 0; y < NL; ++y) {
      float o[NL];
#pragma unroll
      for (int k = 0; k < NL; ++k) {
        float v = 0;
#pragma unroll
        for (int l = 0; l < NL; ++l) v += M[k + NL * l] * P[y + NL * l];
        o[k] = v;
      }
#pragma unroll
      for (int k = 0; k < NL; ++k) P[y + NL * k] = o[k];
    }
#pragma unroll
    for (int z = 0; z < NL; ++z)
#pragma unroll
      for (int y = 0; y < NL; ++y) T[a + NL * y + PL * z] = P[y + NL * z];
  }
  __syncwarp();
  // own nodes (RAS: weighted), ASM: the halo results as well
  float4 *su4 = (float4 *)(Su + e0 * NP);
  const float4 *wt4 = (const float4 *)(wts + e0 * NP);
  for (int q = lane; q < ne * 16; q += 32) {
    const int r = q % 16;
    const float *src = W + (q / 16) * TS + 1 + NL * (r % 4 + 1) + PL * (r / 4 + 1);
    float4 v = make_float4(src[0], src[1], src[2], src[3]);
    if (RAS) {
      const float4 wt = __ldg(wt4 + q);
      v.x *= wt.x;
      v.y *= wt.y;
      v.z *= wt.z;
      v.w *= wt.w;
    }
    su4[q] = v;
  }
  if (!RAS) {
    float *ho = haloOut + e0 * NH;
    for (int q = lane; q < ne * NH; q += 32) {
      const int h = q % NH, f = h / NF, pp = h % NF;
      ho[q] = W[(q / NH) * TS + halo_ext_index<4>(f, pp % 4, pp / 4)];
    }
  }
}

template <typename T>
void launch_fdm(int N, long long E, bool ras, const T *u, const int *haloSrc, const T *Sx, const T *Sy, const T *Sz,
                const T *invL, const T *lam, const T *wts, T *Su, T *haloOut, cudaStream_t s, bool generic)
{
  if (E <= 0) return;
  const bool recip = (lam != nullptr);
  if (std::is_same<T, float>::value && N == 3 && recip && !generic &&
      ((reinterpret_cast<uintptr_t>(u) | reinterpret_cast<uintptr_t>(Sx) | reinterpret_cast<uintptr_t>(Sy) |
        reinterpret_cast<uintptr_t>(Sz) | (ras ? reinterpret_cast<uintptr_t>(wts) : 0) |
        reinterpret_cast<uintptr_t>(Su)) &
       15) == 0) {
    constexpr long long per = fdm4::EPW * fdm4::WPC;
    const unsigned grid = (unsigned)((E + per - 1) / per);
    const float *uf = (const float *)u, *Sxf = (const float *)Sx, *Syf = (const float *)Sy, *Szf = (const float *)Sz;
    const float *lf = (const float *)lam, *wf = (const float *)wts;
    // prefetch distance: one wave of resident CTAs (two waves measured slower)
    long long ahead = 0;
    if ((reinterpret_cast<uintptr_t>(haloSrc) & 15) == 0) {
      static int slots[64] = {0};
      int dev = 0;
      NRSG_CUDA(cudaGetDevice(&dev));
      if (dev < 0 || dev >= 64) dev = 0;
      if (slots[dev] == 0) {
        int sms = 0, occ = 0;
        NRSG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        NRSG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fdm4_kernel<true>, 32 * fdm4::WPC, 0));
        slots[dev] = sms * std::max(occ, 1);
      }
      ahead = (long long)slots[dev] * per;
    }
    if (ras)
      fdm4_kernel<true><<<grid, 32 * fdm4::WPC, 0, s>>>(E, uf, haloSrc, Sxf, Syf, Szf, lf, wf, (float *)Su,
                                                         (float *)haloOut, ahead);
    else
      fdm4_kernel<false><<<grid, 32 * fdm4::WPC, 0, s>>>(E, uf, haloSrc, Sxf, Syf, Szf, lf, wf, (float *)Su,
                                                          (float *)haloOut, ahead);
    NRSG_CHECK_LAUNCH();
    return;
  }
  if (std::is_same<T, float>::value && N == 7 && recip && !generic) {
    const unsigned grid = (unsigned)((E + fdm8::EPC - 1) / fdm8::EPC);
    const float *uf = (const float *)u, *Sxf = (const float *)Sx, *Syf = (const float *)Sy, *Szf = (const float *)Sz;
    const float *lf = (const float *)lam, *wf = (const float *)wts;
    if (ras)
      fdm8_kernel<true><<<grid, 32 * fdm8::EPC, 0, s>>>(E, uf, haloSrc, Sxf, Syf, Szf, lf, wf, (float *)Su,
                                                         (float *)haloOut);
    else
      fdm8_kernel<false><<<grid, 32 * fdm8::EPC, 0, s>>>(E, uf, haloSrc, Sxf, Syf, Szf, lf, wf, (float *)Su,
                                                          (float *)haloOut);
    NRSG_CHECK_LAUNCH();
    return;
  }
#define NRSG_FDM(NQ)                                                                                       \
  {                                                                                                        \
    constexpr int EPB = FdmShape<NQ>::epb;                                                                 \
    const dim3 blk(FdmShape<NQ>::line, EPB);                                                               \
    const unsigned grid = (unsigned)((E + EPB - 1) / EPB);                                                 \
    if (ras && recip)                                                                                      \
      fdm_kernel<T, NQ, true, true><<<grid, blk, 0, s>>>(E, u, haloSrc, Sx, Sy, Sz, invL, lam, wts, Su, haloOut);   \
    else if (ras)                                                                                          \
      fdm_kernel<T, NQ, true, false><<<grid, blk, 0, s>>>(E, u, haloSrc, Sx, Sy, Sz, invL, lam, wts, Su, haloOut);  \
    else if (recip)                                                                                        \
      fdm_kernel<T, NQ, false, true><<<grid, blk, 0, s>>>(E, u, haloSrc, Sx, Sy, Sz, invL, lam, wts, Su, haloOut);  \
    else                                                                                                   \
      fdm_kernel<T, NQ, false, false><<<grid, blk, 0, s>>>(E, u, haloSrc, Sx, Sy, Sz, invL, lam, wts, Su, haloOut); \
  }
  NRSG_DISPATCH_NQ_MG(N, NRSG_FDM)
#undef NRSG_FDM
  NRSG_CHECK_LAUNCH();
}
template <typename T>
void launch_asm_combine(int N, long long E, const int *haloPartner, const T *haloOut, const T *wts, T *Su,
                        cudaStream_t s)
{
  if (E <= 0) return;
#define NRSG_ASMC(NQ)                                                                                      \
  asm_combine_kernel<T, NQ><<<(unsigned)((E + kAsmEpc - 1) / kAsmEpc), 32 * kAsmEpc, 0, s>>>(E, haloPartner,     \
                                                                                            haloOut, wts, Su)
  NRSG_DISPATCH_NQ_MG(N, NRSG_ASMC)
#undef NRSG_ASMC
  NRSG_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// seeded start vector for the Arnoldi lambda_max estimate: U[0,1) per index
// (splitmix64 of seed and the index)
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long smix64(unsigned long long x)
{
  x += 0x9E3779B97F4A7C15ull;
  unsigned long long z = x;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__global__ void random_fill_kernel(long long n, unsigned long long seed, double *v)
{
  MG_LOOP(i, n) v[i] = (double)(smix64(seed ^ smix64((unsigned long long)i)) >> 11) * (1.0 / 9007199254740992.0);
}
void launch_random_fill(long long n, unsigned long long seed, double *v, cudaStream_t s)
{
  random_fill_kernel<<<grid_for(n), kT, 0, s>>>(n, seed, v);
  NRSG_CHECK_LAUNCH();
}

#define NRSG_INST_MG(T)                                                                                    \
  template void launch_coarsen<T>(int, int, long long, const T *, const T *, T *, cudaStream_t);           \
  template void launch_prolong<T>(int, int, long long, const T *, const T *, T *, cudaStream_t);           \
  template void launch_cheby1_update<T>(long long, T, T, const T *, T *, T *, T *, cudaStream_t);          \
  template void launch_cheby4_dx<T>(long long, T, const T *, T, T *, T, T *, bool, bool, cudaStream_t);      \
  template void launch_cheby4_res<T>(long long, const T *, const T *, T *, cudaStream_t);                    \
  template void launch_cheby4_update<T>(long long, T, const T *, const T *, const T *, T *, T *, bool,       \
                                        cudaStream_t);                                                      \
  template void launch_fdm<T>(int, long long, bool, const T *, const int *, const T *, const T *, const T *, \
                              const T *, const T *, const T *, T *, T *, cudaStream_t, bool);              \
  template void launch_asm_combine<T>(int, long long, const int *, const T *, const T *, T *, cudaStream_t);
NRSG_INST_MG(double)
NRSG_INST_MG(float)

} // namespace nrsg
