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

// acc += a b.  FP64: one explicit fused multiply-add, so that the compiler's
// contraction choices cannot change the result (the oracle calls std::fma at
// the same places and the FP64 solve is bit-identical to it); FP32: the plain
// expression, contracted as before.
template <typename T> __device__ __forceinline__ void macc(T &acc, T a, T b) { acc += a * b; }
template <> __device__ __forceinline__ void macc<double>(double &acc, double a, double b) { acc = __fma_rn(a, b, acc); }
// lambda0 (Ga qr + Gb qs + Gc qt); FP64 as fma(Gc, qt, fma(Gb, qs, Ga qr)) with every rounding explicit
template <typename T> __device__ __forceinline__ T gflux(T l0, T Ga, T Gb, T Gc, T qr, T qs, T qt)
{
  return l0 * (Ga * qr + Gb * qs + Gc * qt);
}
template <>
__device__ __forceinline__ double gflux<double>(double l0, double Ga, double Gb, double Gc, double qr, double qs,
                                                double qt)
{
  return __dmul_rn(l0, __fma_rn(Gc, qt, __fma_rn(Gb, qs, __dmul_rn(Ga, qr))));
}
template <typename T> __device__ __forceinline__ T mul3(T a, T b, T c) { return a * b * c; }
template <> __device__ __forceinline__ double mul3<double>(double a, double b, double c)
{
  return __dmul_rn(__dmul_rn(a, b), c);
}

template <int NQ> struct AxShape {
  static constexpr int plane = NQ * NQ;
  static constexpr int epb = plane >= 128 ? 1 : (128 + plane - 1) / plane;
};

// FP32 order 7: at most 80 registers so that 6 CTAs (24 warps) fit per SM
// (measured 2.7% faster at E=48^3 than the unbounded 100-register build)
// EPB elements per CTA (default: enough for 128 threads); the arithmetic of an element does not depend on it
template <typename T, int NQ, bool POISSON, int EPB = AxShape<NQ>::epb>
__global__ void __launch_bounds__(NQ *NQ *EPB, (sizeof(T) == 4 && NQ == 8 && EPB == AxShape<NQ>::epb) ? 6 : 1)
    ax_stored_kernel(long long E, const T *__restrict__ ggeo, const T *__restrict__ D, T lambda0, T lambda1,
                     const T *__restrict__ q, T *__restrict__ Aq)
{
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
  // FP32 (HBM-bound): issue every plane's geometric-factor loads up front so
  // that enough bytes are in flight per SM; FP64 (FP64-pipe bound) loads per
  // plane to keep register pressure down.
  constexpr bool PRELOAD = (sizeof(T) == 4);
  constexpr int NG = POISSON ? 6 : 7;
  T gpre[PRELOAD ? NG * NQ : 1];
  if (PRELOAD) {
#pragma unroll
    for (int k = 0; k < NQ; ++k)
#pragma unroll
      for (int c = 0; c < NG; ++c) gpre[c * NQ + k] = active ? __ldg(g + c * NP + k * NQ * NQ) : T(0);
  }
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    T G00 = 0, G01 = 0, G11 = 0, G12 = 0, G02 = 0, G22 = 0, GWJ = 0;
    if (PRELOAD) {
      G00 = gpre[0 * NQ + k];
      G01 = gpre[1 * NQ + k];
      G11 = gpre[2 * NQ + k];
      G12 = gpre[3 * NQ + k];
      G02 = gpre[4 * NQ + k];
      G22 = gpre[5 * NQ + k];
      if (!POISSON) GWJ = gpre[(NG - 1) * NQ + k];
    } else if (active) {
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
    for (int m = 0; m < NQ; ++m) macc(qt, s_D[k][m], r_q[m]);
    __syncthreads();
    T qr = 0, qs = 0;
#pragma unroll
    for (int m = 0; m < NQ; ++m) {
      macc(qr, s_D[i][m], s_q[el][j][m]);
      macc(qs, s_D[j][m], s_q[el][m][i]);
    }
    s_Gr[el][j][i] = gflux(lambda0, G00, G01, G02, qr, qs, qt);
    s_Gs[el][j][i] = gflux(lambda0, G01, G11, G12, qr, qs, qt);
    const T Gt = gflux(lambda0, G02, G12, G22, qr, qs, qt);
    T auk = POISSON ? T(0) : mul3(GWJ, lambda1, r_q[k]);
    __syncthreads();
#pragma unroll
    for (int m = 0; m < NQ; ++m) {
      macc(auk, s_D[m][j], s_Gs[el][m][i]);
      macc(r_Aq[m], s_D[k][m], Gt);
      macc(auk, s_D[m][i], s_Gr[el][j][m]);
    }
    r_Aq[k] += auk;
    __syncthreads();
  }
  if (active) {
#pragma unroll
    for (int k = 0; k < NQ; ++k) Aq[base + k * NQ * NQ] = r_Aq[k];
  }
}

// ---------------------------------------------------------------------------
// FP32 order-7 axhelm with vector shared-memory traffic.  Same thread layout,
// register pencils and arithmetic as ax_stored_kernel<float, 8, POISSON>
// (bit-identical results), but every operand row a thread contracts against
// is read as two 16-byte loads: D and its transpose are both kept, and each
// plane of q and of G_s is stored twice (row-major and transposed) so that the
// column sums read rows too.  Row strides: 8 floats for the planes written
// row-major (conflict-free 32-thread stores, 4 distinct rows per read), 12
// floats for the transposed planes and D (8 distinct rows per read land on
// disjoint bank quads).  This cuts the shared-memory wavefronts per node and
// plane from about 75 to about 25, which is what bounds the plain kernel.
// ---------------------------------------------------------------------------
template <bool POISSON>
__global__ void __launch_bounds__(128, 5)
    ax8v_kernel(long long E, const float *__restrict__ ggeo, const float *__restrict__ D, float lambda0,
                float lambda1, const float *__restrict__ q, float *__restrict__ Aq)
{
  constexpr int NQ = 8, NP = 512, EPB = 2, RT = 12;
  __shared__ __align__(16) float s_D[NQ][RT];   // D[a][b] at [a][b]
  __shared__ __align__(16) float s_DT[NQ][RT];  // D[a][b] at [b][a]
  __shared__ __align__(16) float s_q[EPB][NQ][NQ];
  __shared__ __align__(16) float s_qT[EPB][NQ][RT];
  __shared__ __align__(16) float s_Gr[EPB][NQ][NQ];
  __shared__ __align__(16) float s_GsT[EPB][NQ][RT];

  const int t = threadIdx.x;
  const int i = t % NQ, j = t / NQ;
  const int el = threadIdx.y;
  const long long e = (long long)blockIdx.x * EPB + el;
  const bool active = e < E;
  if (el == 0) {
    const float d = D[j * NQ + i];
    s_D[j][i] = d;
    s_DT[i][j] = d;
  }
  float r_q[NQ], r_Aq[NQ];
  const long long base = e * NP + t;
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    r_q[k] = active ? q[base + k * NQ * NQ] : 0.f;
    r_Aq[k] = 0;
  }
  constexpr int NG = POISSON ? 6 : 7;
  const float *g = ggeo + e * 7 * NP + t;
  float gpre[NG * NQ];
#pragma unroll
  for (int k = 0; k < NQ; ++k)
#pragma unroll
    for (int c = 0; c < NG; ++c) gpre[c * NQ + k] = active ? __ldg(g + c * NP + k * NQ * NQ) : 0.f;
  __syncthreads();

  auto row8 = [](const float *p, float (&v)[NQ]) {
    const float4 a = *reinterpret_cast<const float4 *>(p);
    const float4 b = *reinterpret_cast<const float4 *>(p + 4);
    v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w, v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w;
  };
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    const float G00 = gpre[0 * NQ + k], G01 = gpre[1 * NQ + k], G11 = gpre[2 * NQ + k];
    const float G12 = gpre[3 * NQ + k], G02 = gpre[4 * NQ + k], G22 = gpre[5 * NQ + k];
    const float GWJ = POISSON ? 0.f : gpre[(NG - 1) * NQ + k];
    s_q[el][j][i] = r_q[k];
    s_qT[el][i][j] = r_q[k];
    float Dk[NQ];
    row8(&s_D[k][0], Dk);
    float qt = 0;
#pragma unroll
    for (int m = 0; m < NQ; ++m) qt += Dk[m] * r_q[m];
    __syncthreads();
    float Di[NQ], Dj[NQ], qrow[NQ], qcol[NQ];
    row8(&s_D[i][0], Di);
    row8(&s_D[j][0], Dj);
    row8(&s_q[el][j][0], qrow);
    row8(&s_qT[el][i][0], qcol);
    float qr = 0, qs = 0;
#pragma unroll
    for (int m = 0; m < NQ; ++m) {
      qr += Di[m] * qrow[m];
      qs += Dj[m] * qcol[m];
    }
    s_Gr[el][j][i] = lambda0 * (G00 * qr + G01 * qs + G02 * qt);
    s_GsT[el][i][j] = lambda0 * (G01 * qr + G11 * qs + G12 * qt);
    const float Gt = lambda0 * (G02 * qr + G12 * qs + G22 * qt);
    float auk = POISSON ? 0.f : GWJ * lambda1 * r_q[k];
    __syncthreads();
    float DTi[NQ], DTj[NQ], gsc[NQ], grr[NQ];
    row8(&s_DT[j][0], DTj);
    row8(&s_DT[i][0], DTi);
    row8(&s_GsT[el][i][0], gsc);
    row8(&s_Gr[el][j][0], grr);
#pragma unroll
    for (int m = 0; m < NQ; ++m) {
      auk += DTj[m] * gsc[m];
      r_Aq[m] += Dk[m] * Gt;
      auk += DTi[m] * grr[m];
    }
    r_Aq[k] += auk;
    __syncthreads();
  }
  if (active) {
#pragma unroll
    for (int k = 0; k < NQ; ++k) Aq[base + k * NQ * NQ] = r_Aq[k];
  }
}

// ---------------------------------------------------------------------------
// FP32 order-7 axhelm with D out of shared memory.  Same arithmetic as
// ax8v_kernel (bit-identical), but a 16-byte shared load costs four
// wavefronts per warp whatever its address pattern, so ax8v still moves
// about 76 wavefronts per warp and plane through the shared pipe.  Here the
// broadcast row D[k][*] is read from constant memory (uniform, compile-time
// offsets: no shared traffic) and the rows D[i][*], D[j][*] and columns
// D[*][i], D[*][j] each thread contracts against are held in 32 registers for
// the whole element, leaving only the q and G planes in shared memory.
// ---------------------------------------------------------------------------
__constant__ float c_D8[64];

// LAM1: lambda0 == 1 (Poisson, the headline), whose multiplies are exact and skipped.
// PF: persistent CTAs walking the element pairs with a stride of the grid; before a pair is
// computed one thread asks L2 for the next pair of this CTA (cp.async.bulk.prefetch.L2: q and the
// geometric factors of two elements, two contiguous ranges), so the DRAM reads of the next pair
// overlap the contractions of this one instead of every resident CTA waiting on DRAM at the same
// time.  Without PF the grid has one CTA per pair and the loop runs once.  pf: the two ranges are
// 16-byte aligned (the bulk prefetch's requirement); when not, nothing is prefetched.
template <bool POISSON, bool LAM1, bool PF>
__global__ void __launch_bounds__(128, 4)
    ax8c_kernel(long long E, const float *__restrict__ ggeo, float lambda0, float lambda1,
                const float *__restrict__ q, float *__restrict__ Aq, bool pf)
{
  constexpr int NQ = 8, NP = 512, EPB = 2, RT = 12;
  __shared__ __align__(16) float s_q[EPB][NQ][NQ];
  __shared__ __align__(16) float s_qT[EPB][NQ][RT];
  __shared__ __align__(16) float s_Gr[EPB][NQ][NQ];
  __shared__ __align__(16) float s_GsT[EPB][NQ][RT];

  const int t = threadIdx.x;
  const int i = t % NQ, j = t / NQ;
  const int el = threadIdx.y;
  float Di[NQ], Dj[NQ], DTi[NQ], DTj[NQ];
#pragma unroll
  for (int m = 0; m < NQ; ++m) {
    Di[m] = c_D8[i * NQ + m];
    Dj[m] = c_D8[j * NQ + m];
    DTi[m] = c_D8[m * NQ + i];
    DTj[m] = c_D8[m * NQ + j];
  }
  constexpr int NG = POISSON ? 6 : 7;
  const long long npairs = (E + EPB - 1) / EPB;
  // one element pair: the whole computation (a lambda, so the single-pass form compiles to straight-line code)
  auto pair = [&](const long long pr) {
    if (PF && pf && t == 0 && el == 0 && pr + gridDim.x < npairs) {
      // the factors this kernel reads (six for Poisson: the seventh, GWJ, is skipped) and q
      const long long en = (pr + gridDim.x) * EPB;
      const int cnt = E - en < EPB ? (int)(E - en) : EPB;
      for (int c = 0; c < cnt; ++c)
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(ggeo + (en + c) * 7 * NP),
                     "r"((unsigned)(NG * NP * sizeof(float)))
                     : "memory");
      asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(q + en * NP),
                   "r"((unsigned)(cnt * NP * sizeof(float)))
                   : "memory");
    }
    const long long e = pr * EPB + el;
    const bool active = e < E;
    float r_q[NQ], r_Aq[NQ];
    const long long base = e * NP + t;
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      r_q[k] = active ? q[base + k * NQ * NQ] : 0.f;
      r_Aq[k] = 0;
    }
    const float *g = ggeo + e * 7 * NP + t;
    float gpre[NG * NQ];
#pragma unroll
    for (int k = 0; k < NQ; ++k)
#pragma unroll
      for (int c = 0; c < NG; ++c) gpre[c * NQ + k] = active ? __ldg(g + c * NP + k * NQ * NQ) : 0.f;

    auto row8 = [](const float *p, float (&v)[NQ]) {
      const float4 a = *reinterpret_cast<const float4 *>(p);
      const float4 b = *reinterpret_cast<const float4 *>(p + 4);
      v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w, v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w;
    };
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      const float G00 = gpre[0 * NQ + k], G01 = gpre[1 * NQ + k], G11 = gpre[2 * NQ + k];
      const float G12 = gpre[3 * NQ + k], G02 = gpre[4 * NQ + k], G22 = gpre[5 * NQ + k];
      const float GWJ = POISSON ? 0.f : gpre[(NG - 1) * NQ + k];
      s_q[el][j][i] = r_q[k];
      s_qT[el][i][j] = r_q[k];
      float qt = 0;
#pragma unroll
      for (int m = 0; m < NQ; ++m) qt += c_D8[k * NQ + m] * r_q[m];
      __syncthreads();
      float qrow[NQ], qcol[NQ];
      row8(&s_q[el][j][0], qrow);
      row8(&s_qT[el][i][0], qcol);
      float qr = 0, qs = 0;
#pragma unroll
      for (int m = 0; m < NQ; ++m) {
        qr += Di[m] * qrow[m];
        qs += Dj[m] * qcol[m];
      }
      const float gr = G00 * qr + G01 * qs + G02 * qt;
      const float gs = G01 * qr + G11 * qs + G12 * qt;
      const float gt = G02 * qr + G12 * qs + G22 * qt;
      s_Gr[el][j][i] = LAM1 ? gr : lambda0 * gr;
      s_GsT[el][i][j] = LAM1 ? gs : lambda0 * gs;
      const float Gt = LAM1 ? gt : lambda0 * gt;
      float auk = POISSON ? 0.f : GWJ * lambda1 * r_q[k];
      __syncthreads();
      float gsc[NQ], grr[NQ];
      row8(&s_GsT[el][i][0], gsc);
      row8(&s_Gr[el][j][0], grr);
      // A q update of the 8 planes: independent accumulators, two round-to-nearest fmaf per paired instruction
      const float2 gt2 = make_float2(Gt, Gt);
#pragma unroll
      for (int m = 0; m < NQ; m += 2) {
        const float2 r = __ffma2_rn(make_float2(c_D8[k * NQ + m], c_D8[k * NQ + m + 1]), gt2,
                                    make_float2(r_Aq[m], r_Aq[m + 1]));
        r_Aq[m] = r.x;
        r_Aq[m + 1] = r.y;
      }
#pragma unroll
      for (int m = 0; m < NQ; ++m) {
        auk += DTj[m] * gsc[m];
        auk += DTi[m] * grr[m];
      }
      r_Aq[k] += auk;
      __syncthreads();
    }
    if (active) {
#pragma unroll
      for (int k = 0; k < NQ; ++k) Aq[base + k * NQ * NQ] = r_Aq[k];
    }
  };
  if constexpr (PF) {
    for (long long pr = blockIdx.x; pr < npairs; pr += gridDim.x) pair(pr);
  } else {
    pair(blockIdx.x);
  }
}

template <bool PF>
static void ax8c_launch(unsigned grid, long long E, const float *ggeo, float lambda0, float lambda1, bool poisson,
                        const float *q, float *Aq, bool pf, cudaStream_t s)
{
  const bool one = lambda0 == 1.f;
  if (poisson && one)
    ax8c_kernel<true, true, PF><<<grid, dim3(64, 2), 0, s>>>(E, ggeo, lambda0, lambda1, q, Aq, pf);
  else if (poisson)
    ax8c_kernel<true, false, PF><<<grid, dim3(64, 2), 0, s>>>(E, ggeo, lambda0, lambda1, q, Aq, pf);
  else if (one)
    ax8c_kernel<false, true, PF><<<grid, dim3(64, 2), 0, s>>>(E, ggeo, lambda0, lambda1, q, Aq, pf);
  else
    ax8c_kernel<false, false, PF><<<grid, dim3(64, 2), 0, s>>>(E, ggeo, lambda0, lambda1, q, Aq, pf);
}

bool launch_ax_const(int N, long long E, const float *ggeo, const float *D, float lambda0, float lambda1,
                     bool poisson, const float *q, float *Aq, cudaStream_t s, bool prefetch)
{
  if (N != 7 || E <= 0) return false;
  // D (64 floats, device memory) into the constant bank, ordered on the stream
  NRSG_CUDA(cudaMemcpyToSymbolAsync(c_D8, D, sizeof(float) * 64, 0, cudaMemcpyDeviceToDevice, s));
  const long long npairs = (E + 1) / 2;
  if (!prefetch) {
    ax8c_launch<false>((unsigned)npairs, E, ggeo, lambda0, lambda1, poisson, q, Aq, false, s);
  } else {
    // persistent: every resident CTA slot of the device (4 per SM at 128 registers a thread)
    static int slots[64] = {0};
    int dev = 0;
    NRSG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return false;
    if (slots[dev] == 0) {
      int sms = 0, per = 0;
      NRSG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
      NRSG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, ax8c_kernel<true, true, true>, 128, 0));
      slots[dev] = sms * std::max(per, 1);
    }
    const unsigned grid = (unsigned)std::min<long long>(npairs, slots[dev]);
    const bool aligned = ((reinterpret_cast<uintptr_t>(ggeo) | reinterpret_cast<uintptr_t>(q)) & 15) == 0;
    ax8c_launch<true>(grid, E, ggeo, lambda0, lambda1, poisson, q, Aq, aligned, s);
  }
  NRSG_CHECK_LAUNCH();
  return true;
}

// ---------------------------------------------------------------------------
// FP32 order-7 axhelm through a bulk-copy pipeline (sm_90+ cp.async.bulk into
// shared memory, completion counted on an mbarrier).  Persistent CTAs walk
// chunks of kPipeEps consecutive elements; while the chunk in one stage is
// computed, the next chunk's geometric factors (one contiguous slab of 6 or 7
// x 2 KB per element) and q (one slab for the chunk) stream into the other
// stage, so every SM keeps HBM requests in flight through the compute phases
// that leave the plain kernel's loads bursty.  The arithmetic is that of
// ax_stored_kernel<float, 8, POISSON> operation for operation (bit-identical
// results); only where the operands come from differs.
// ---------------------------------------------------------------------------
constexpr int kPipeEps = 3;    // elements per stage (3 x 64 threads)
constexpr int kPipeStages = 2;
constexpr unsigned kPipeSpinLimit = 1u << 22;
__device__ unsigned g_ax_pipe_err = 0;

__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long *bar, unsigned bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity)
{
  unsigned ok;
  asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
               "selp.u32 %0, 1, 0, p;\n\t}"
               : "=r"(ok)
               : "r"(smem_addr(bar)), "r"(parity)
               : "memory");
  return ok != 0;
}
// global -> shared bulk copy (16-byte aligned addresses, size a multiple of 16)
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *bar)
{
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

template <bool POISSON> constexpr int pipe_factors() { return POISSON ? 6 : 7; }
template <bool POISSON> constexpr size_t pipe_smem_bytes()
{
  return (size_t)kPipeStages * kPipeEps * (pipe_factors<POISSON>() + 1) * 512 * sizeof(float);
}

template <bool POISSON>
__global__ void __launch_bounds__(64 * kPipeEps, 2)
    ax_pipe_kernel(long long E, const float *__restrict__ ggeo, const float *__restrict__ D, float lambda0,
                   float lambda1, const float *__restrict__ q, float *__restrict__ Aq)
{
  constexpr int NQ = 8, NP = 512, NG = pipe_factors<POISSON>();
  extern __shared__ __align__(128) unsigned char pipe_smem[];
  float *sg = reinterpret_cast<float *>(pipe_smem);           // [stage][element][factor][NP]
  float *sq = sg + (size_t)kPipeStages * kPipeEps * NG * NP;  // [stage][element][NP]
  __shared__ float s_D[NQ][NQ + 1];
  __shared__ float s_q[kPipeEps][NQ][NQ];
  __shared__ float s_Gr[kPipeEps][NQ][NQ];
  __shared__ float s_Gs[kPipeEps][NQ][NQ];
  __shared__ __align__(8) unsigned long long bar[kPipeStages];

  const int tid = threadIdx.x;
  const int el = tid / 64, t = tid % 64, i = t % NQ, j = t / NQ;
  const long long nchunk = (E + kPipeEps - 1) / kPipeEps;
  if (tid < 64) s_D[j][i] = D[j * NQ + i];
  if (tid == 0) {
    for (int st = 0; st < kPipeStages; ++st) mbar_init(&bar[st], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  auto issue = [&](long long c, int st) {
    const long long e0 = c * kPipeEps;
    const int ne = (int)(E - e0 < kPipeEps ? E - e0 : kPipeEps);
    mbar_arrive_expect_tx(&bar[st], (unsigned)(ne * (NG + 1) * NP * sizeof(float)));
    for (int x = 0; x < ne; ++x)
      bulk_copy_g2s(sg + ((size_t)st * kPipeEps + x) * NG * NP, ggeo + (e0 + x) * 7 * NP, NG * NP * sizeof(float),
                    &bar[st]);
    bulk_copy_g2s(sq + (size_t)st * kPipeEps * NP, q + e0 * NP, ne * NP * sizeof(float), &bar[st]);
  };
  if (tid == 0)
    for (int st = 0; st < kPipeStages; ++st) {
      const long long c = blockIdx.x + (long long)st * gridDim.x;
      if (c < nchunk) issue(c, st);
    }

  int it = 0;
  for (long long c = blockIdx.x; c < nchunk; c += gridDim.x, ++it) {
    const int st = it % kPipeStages;
    const unsigned parity = (it / kPipeStages) & 1;
    unsigned spins = 0;
    bool late = false;
    while (!mbar_try_wait(&bar[st], parity))
      if (++spins > kPipeSpinLimit) {
        late = true;
        break;
      }
    if (__syncthreads_or(late)) {
      // a copy did not land within the limit: flag it, give the other stage's
      // copies a bounded wait, and leave (the host reads the flag after the solve)
      if (tid == 0) {
        atomicExch(&g_ax_pipe_err, 1u);
        for (int k = 1; k < kPipeStages; ++k) {
          const long long c2 = c + (long long)k * gridDim.x;
          if (c2 >= nchunk) break;
          const int s2 = (it + k) % kPipeStages;
          unsigned n2 = 0;
          while (!mbar_try_wait(&bar[s2], ((it + k) / kPipeStages) & 1) && ++n2 < kPipeSpinLimit) {
          }
        }
      }
      return;
    }
    const long long e = c * kPipeEps + el;
    const bool active = e < E;
    const float *gs = sg + ((size_t)st * kPipeEps + el) * NG * NP + t;
    const float *qs = sq + ((size_t)st * kPipeEps + el) * NP;
    float r_q[NQ], r_Aq[NQ];
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      r_q[k] = active ? qs[k * NQ * NQ + t] : 0.f;
      r_Aq[k] = 0;
    }
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      const int o = k * NQ * NQ;
      float G00 = 0, G01 = 0, G11 = 0, G12 = 0, G02 = 0, G22 = 0, GWJ = 0;
      if (active) {
        G00 = gs[0 * NP + o];
        G01 = gs[1 * NP + o];
        G11 = gs[2 * NP + o];
        G12 = gs[3 * NP + o];
        G02 = gs[4 * NP + o];
        G22 = gs[5 * NP + o];
        if (!POISSON) GWJ = gs[6 * NP + o];
      }
      s_q[el][j][i] = r_q[k];
      float qt = 0;
#pragma unroll
      for (int m = 0; m < NQ; ++m) qt += s_D[k][m] * r_q[m];
      __syncthreads();
      float qr = 0, qsd = 0;
#pragma unroll
      for (int m = 0; m < NQ; ++m) {
        qr += s_D[i][m] * s_q[el][j][m];
        qsd += s_D[j][m] * s_q[el][m][i];
      }
      s_Gr[el][j][i] = lambda0 * (G00 * qr + G01 * qsd + G02 * qt);
      s_Gs[el][j][i] = lambda0 * (G01 * qr + G11 * qsd + G12 * qt);
      const float Gt = lambda0 * (G02 * qr + G12 * qsd + G22 * qt);
      float auk = POISSON ? 0.f : GWJ * lambda1 * r_q[k];
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
      for (int k = 0; k < NQ; ++k) Aq[e * NP + k * NQ * NQ + t] = r_Aq[k];
    }
    // every thread has read this stage (the last __syncthreads of the plane
    // loop): refill it with the chunk kPipeStages grid-strides ahead
    if (tid == 0) {
      const long long cn = c + (long long)kPipeStages * gridDim.x;
      if (cn < nchunk) issue(cn, st);
    }
  }
}

bool launch_ax_pipe(int N, long long E, const float *ggeo, const float *D, float lambda0, float lambda1, bool poisson,
                    const float *q, float *Aq, cudaStream_t s)
{
  if (N != 7 || E <= 0) return false;
  if (((uintptr_t)ggeo | (uintptr_t)q) & 15) return false; // bulk copies need 16-byte aligned sources
  int dev = 0;
  NRSG_CUDA(cudaGetDevice(&dev));
  static int smsOf[64] = {0}; // SM count per device, looked up once
  int sms = smsOf[dev & 63];
  if (!sms) {
    NRSG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    smsOf[dev & 63] = sms;
  }
  const long long nchunk = (E + kPipeEps - 1) / kPipeEps;
  const unsigned grid = (unsigned)std::min<long long>(nchunk, 2LL * sms);
  if (poisson) {
    raise_dynamic_smem((const void *)ax_pipe_kernel<true>, pipe_smem_bytes<true>());
    ax_pipe_kernel<true><<<grid, 64 * kPipeEps, pipe_smem_bytes<true>(), s>>>(E, ggeo, D, lambda0, lambda1, q, Aq);
  } else {
    raise_dynamic_smem((const void *)ax_pipe_kernel<false>, pipe_smem_bytes<false>());
    ax_pipe_kernel<false><<<grid, 64 * kPipeEps, pipe_smem_bytes<false>(), s>>>(E, ggeo, D, lambda0, lambda1, q, Aq);
  }
  NRSG_CHECK_LAUNCH();
  return true;
}

unsigned ax_pipe_error(cudaStream_t s)
{
  unsigned h = 0, zero = 0;
  NRSG_CUDA(cudaMemcpyFromSymbolAsync(&h, g_ax_pipe_err, sizeof(h), 0, cudaMemcpyDeviceToHost, s));
  NRSG_CUDA(cudaStreamSynchronize(s));
  if (h) NRSG_CUDA(cudaMemcpyToSymbolAsync(g_ax_pipe_err, &zero, sizeof(zero), 0, cudaMemcpyHostToDevice, s));
  return h;
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
// FP64: the same factors with every rounding explicit (the oracle performs these operations in this order)
template <>
__device__ __forceinline__ void trilinear_G<double>(const double *xe, const double *ye, const double *ze, double rn,
                                                    double sn, double tn, double W, double &G00, double &G01,
                                                    double &G02, double &G11, double &G12, double &G22, double &GWJ)
{
  const double am = __dmul_rn(1 - tn, 1 - sn), ap = __dmul_rn(1 - tn, 1 + sn), bm = __dmul_rn(1 + tn, 1 - sn),
               bp = __dmul_rn(1 + tn, 1 + sn);
  const double cm = __dmul_rn(1 - tn, 1 - rn), cp = __dmul_rn(1 - tn, 1 + rn), dm = __dmul_rn(1 + tn, 1 - rn),
               dp = __dmul_rn(1 + tn, 1 + rn);
  const double fm = __dmul_rn(1 - rn, 1 - sn), fp = __dmul_rn(1 + rn, 1 - sn), hp = __dmul_rn(1 + rn, 1 + sn),
               hm = __dmul_rn(1 - rn, 1 + sn);
  // 0.125 (a0 d0 + a1 d1 + a2 d2 + a3 d3) as 0.125 fma(a3, d3, fma(a2, d2, fma(a1, d1, a0 d0)))
  auto comb = [](double a0, double d0, double a1, double d1, double a2, double d2, double a3, double d3) {
    return __dmul_rn(0.125, __fma_rn(a3, d3, __fma_rn(a2, d2, __fma_rn(a1, d1, __dmul_rn(a0, d0)))));
  };
  auto dr = [&](const double *X) { return comb(am, X[1] - X[0], ap, X[2] - X[3], bm, X[5] - X[4], bp, X[6] - X[7]); };
  auto ds = [&](const double *X) { return comb(cm, X[3] - X[0], cp, X[2] - X[1], dm, X[7] - X[4], dp, X[6] - X[5]); };
  auto dt = [&](const double *X) { return comb(fm, X[4] - X[0], fp, X[5] - X[1], hp, X[6] - X[2], hm, X[7] - X[3]); };
  const double xr = dr(xe), xs = ds(xe), xt = dt(xe);
  const double yr = dr(ye), ys = ds(ye), yt = dt(ye);
  const double zr = dr(ze), zs = ds(ze), zt = dt(ze);
  auto minor2 = [](double a, double b, double c, double d) { return __fma_rn(a, b, -__dmul_rn(c, d)); };
  const double rx = minor2(ys, zt, zs, yt), ry = -minor2(xs, zt, zs, xt), rz = minor2(xs, yt, ys, xt);
  const double sx = -minor2(yr, zt, zr, yt), sy = minor2(xr, zt, zr, xt), sz = -minor2(xr, yt, yr, xt);
  const double tx = minor2(yr, zs, zr, ys), ty = -minor2(xr, zs, zr, xs), tz = minor2(xr, ys, yr, xs);
  const double J = __fma_rn(zr, rz, __fma_rn(yr, ry, __dmul_rn(xr, rx)));
  const double sc = W / J;
  auto dot3 = [](double a0, double b0, double a1, double b1, double a2, double b2) {
    return __fma_rn(a2, b2, __fma_rn(a1, b1, __dmul_rn(a0, b0)));
  };
  G00 = __dmul_rn(sc, dot3(rx, rx, ry, ry, rz, rz));
  G01 = __dmul_rn(sc, dot3(rx, sx, ry, sy, rz, sz));
  G02 = __dmul_rn(sc, dot3(rx, tx, ry, ty, rz, tz));
  G11 = __dmul_rn(sc, dot3(sx, sx, sy, sy, sz, sz));
  G12 = __dmul_rn(sc, dot3(sx, tx, sy, ty, sz, tz));
  G22 = __dmul_rn(sc, dot3(tx, tx, ty, ty, tz, tz));
  GWJ = __dmul_rn(W, J);
}

template <typename T, int NQ, bool POISSON>
__global__ void __launch_bounds__(NQ *NQ *AxShape<NQ>::epb)
    ax_trilinear_kernel(long long E, const T *__restrict__ VX, const T *__restrict__ gllz,
                        const T *__restrict__ gllw, const T *__restrict__ D, T l0rs, T l0t, T lambda1,
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
    for (int m = 0; m < NQ; ++m) macc(qt, s_D[k][m], r_q[m]);
    __syncthreads();
    T qr = 0, qs = 0;
#pragma unroll
    for (int m = 0; m < NQ; ++m) {
      macc(qr, s_D[i][m], s_q[el][j][m]);
      macc(qs, s_D[j][m], s_q[el][m][i]);
    }
    // the reference scales the t-flux by lambda0 only (ellipticPartialAxTrilinearHex3D.okl:154-157);
    // l0rs = lambda0 scales all three (option trilinearLambda0 = all), l0rs = 1 is the reference
    s_Gr[el][j][i] = gflux(l0rs, G00, G01, G02, qr, qs, qt);
    s_Gs[el][j][i] = gflux(l0rs, G01, G11, G12, qr, qs, qt);
    const T Gt = gflux(l0t, G02, G12, G22, qr, qs, qt);
    T auk = POISSON ? T(0) : mul3(GWJ, lambda1, r_q[k]);
    __syncthreads();
#pragma unroll
    for (int m = 0; m < NQ; ++m) {
      macc(auk, s_D[m][j], s_Gs[el][m][i]);
      macc(r_Aq[m], s_D[k][m], Gt);
      macc(auk, s_D[m][i], s_Gr[el][j][m]);
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
  if constexpr (std::is_same<T, float>::value) {
    if (N == 7) {
      const unsigned grid = (unsigned)((E + 1) / 2);
      if (poisson)
        ax8v_kernel<true><<<grid, dim3(64, 2), 0, s>>>(E, ggeo, D, lambda0, lambda1, q, Aq);
      else
        ax8v_kernel<false><<<grid, dim3(64, 2), 0, s>>>(E, ggeo, D, lambda0, lambda1, q, Aq);
      NRSG_CHECK_LAUNCH();
      return;
    }
  }
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

// One named FP32 axhelm variant (the multigrid autotuner's candidates; all give the same bits):
// kAxVec   the default dispatch (order 7: the 16-byte shared-memory row-load kernel; else the plain kernel)
// kAxPlain the plain kernel at its default elements per CTA
// kAxEpb2  the plain kernel at twice the elements per CTA
// kAxPipe  the bulk-copy pipelined kernel (order 7 Poisson only)
// kAxConst D in constant memory and registers (order 7 only)
// kAxConstPf the same kernel as persistent CTAs prefetching their next element pair into L2
// Returns false where the variant does not apply.
bool launch_ax_f32_variant(int variant, int N, long long E, const float *ggeo, const float *D, float lambda0,
                           float lambda1, bool poisson, const float *q, float *Aq, cudaStream_t s)
{
  if (E <= 0) return true;
  switch (variant) {
  case kAxVec: launch_ax_stored<float>(N, E, ggeo, D, lambda0, lambda1, poisson, q, Aq, s); return true;
  case kAxPipe: return launch_ax_pipe(N, E, ggeo, D, lambda0, lambda1, poisson, q, Aq, s);
  case kAxConst: return launch_ax_const(N, E, ggeo, D, lambda0, lambda1, poisson, q, Aq, s);
  case kAxConstPf: return launch_ax_const(N, E, ggeo, D, lambda0, lambda1, poisson, q, Aq, s, true);
  case kAxPlain:
  case kAxEpb2: break;
  default: return false;
  }
  const bool two = variant == kAxEpb2;
#define NRSG_AXV(NQ)                                                                                       \
  {                                                                                                        \
    constexpr int B1 = AxShape<NQ>::epb, B2 = 2 * AxShape<NQ>::epb;                                        \
    if (two) {                                                                                             \
      const unsigned grid = (unsigned)((E + B2 - 1) / B2);                                                 \
      if (poisson)                                                                                         \
        ax_stored_kernel<float, NQ, true, B2><<<grid, dim3(NQ * NQ, B2), 0, s>>>(E, ggeo, D, lambda0, lambda1, q, Aq); \
      else                                                                                                 \
        ax_stored_kernel<float, NQ, false, B2><<<grid, dim3(NQ * NQ, B2), 0, s>>>(E, ggeo, D, lambda0, lambda1, q, Aq); \
    } else {                                                                                               \
      const unsigned grid = (unsigned)((E + B1 - 1) / B1);                                                 \
      if (poisson)                                                                                         \
        ax_stored_kernel<float, NQ, true, B1><<<grid, dim3(NQ * NQ, B1), 0, s>>>(E, ggeo, D, lambda0, lambda1, q, Aq); \
      else                                                                                                 \
        ax_stored_kernel<float, NQ, false, B1><<<grid, dim3(NQ * NQ, B1), 0, s>>>(E, ggeo, D, lambda0, lambda1, q, Aq); \
    }                                                                                                      \
  }
  NRSG_DISPATCH_NQ(N, NRSG_AXV)
#undef NRSG_AXV
  NRSG_CHECK_LAUNCH();
  return true;
}

template <typename T>
void launch_ax_trilinear(int N, long long E, const T *VX, const T *gllz, const T *gllw, const T *D, T lambda0,
                         T lambda1, bool poisson, const T *q, T *Aq, cudaStream_t s, bool lambda0All)
{
  if (E <= 0) return;
  const T l0rs = lambda0All ? lambda0 : T(1), l0t = lambda0;
#define NRSG_AXT(NQ)                                                                                       \
  {                                                                                                        \
    constexpr int EPB = AxShape<NQ>::epb;                                                                  \
    dim3 blk(NQ * NQ, EPB);                                                                                \
    const unsigned grid = (unsigned)((E + EPB - 1) / EPB);                                                 \
    if (poisson)                                                                                           \
      ax_trilinear_kernel<T, NQ, true><<<grid, blk, 0, s>>>(E, VX, gllz, gllw, D, l0rs, l0t, lambda1, q, Aq); \
    else                                                                                                   \
      ax_trilinear_kernel<T, NQ, false><<<grid, blk, 0, s>>>(E, VX, gllz, gllw, D, l0rs, l0t, lambda1, q, Aq); \
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
                                          cudaStream_t, bool);
template void launch_ax_trilinear<float>(int, long long, const float *, const float *, const float *, const float *,
                                         float, float, bool, const float *, float *, cudaStream_t, bool);

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
    if constexpr (sizeof(T) == 8) {
      // FP64: r = fma(((2 g) l0) Da, Db, r) etc., every rounding explicit (mirrored by the oracle)
      auto cross = [&](double g0, double Da, double Db) {
        r = __fma_rn(__dmul_rn(__dmul_rn(__dmul_rn(2.0, g0), lambda0), Da), Db, r);
      };
      auto line = [&](double g0, double Dm) { r = __fma_rn(__dmul_rn(__dmul_rn(g0, lambda0), Dm), Dm, r); };
      cross(g[1 * NP + n], s_D[i][i], s_D[j][j]);
      cross(g[4 * NP + n], s_D[i][i], s_D[k][k]);
      cross(g[3 * NP + n], s_D[j][j], s_D[k][k]);
      for (int m = 0; m < NQ; ++m) {
        line(g[0 * NP + m + NQ * (j + NQ * k)], s_D[m][i]);
        line(g[2 * NP + i + NQ * (m + NQ * k)], s_D[m][j]);
        line(g[5 * NP + i + NQ * (j + NQ * m)], s_D[m][k]);
      }
      if (!poisson) r = __fma_rn(g[6 * NP + n], lambda1, r);
    } else {
      r += T(2) * g[1 * NP + n] * lambda0 * s_D[i][i] * s_D[j][j];
      r += T(2) * g[4 * NP + n] * lambda0 * s_D[i][i] * s_D[k][k];
      r += T(2) * g[3 * NP + n] * lambda0 * s_D[j][j] * s_D[k][k];
      for (int m = 0; m < NQ; ++m) {
        r += g[0 * NP + m + NQ * (j + NQ * k)] * lambda0 * s_D[m][i] * s_D[m][i];
        r += g[2 * NP + i + NQ * (m + NQ * k)] * lambda0 * s_D[m][j] * s_D[m][j];
        r += g[5 * NP + i + NQ * (j + NQ * m)] * lambda0 * s_D[m][k] * s_D[m][k];
      }
      if (!poisson) r += g[6 * NP + n] * lambda1;
    }
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
      const double wv = __dmul_rn(__dmul_rn(a[v & 1], b[(v >> 1) & 1]), c[v >> 2]);
      for (int d = 0; d < 3; ++d) X[d] = __fma_rn(wv, s_v[v * 3 + d], X[d]);
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
        dr[d] = __fma_rn(s_D[i][m], s_x[d][m + NQ * (j + NQ * k)], dr[d]);
        ds[d] = __fma_rn(s_D[j][m], s_x[d][i + NQ * (m + NQ * k)], ds[d]);
        dt[d] = __fma_rn(s_D[k][m], s_x[d][i + NQ * (j + NQ * m)], dt[d]);
      }
    const double xr = dr[0], yr = dr[1], zr = dr[2], xs = ds[0], ys = ds[1], zs = ds[2], xt = dt[0], yt = dt[1],
                 zt = dt[2];
    // 2x2 minors a b - c d as fma(a, b, -(c d)); every rounding explicit (mirrored by the oracle)
    auto minor2 = [](double a, double b, double c, double d) { return __fma_rn(a, b, -__dmul_rn(c, d)); };
    const double cx = minor2(ys, zt, zs, yt), cy = minor2(xs, zt, zs, xt), cz = minor2(xs, yt, ys, xt);
    const double J = __fma_rn(zr, cz, __fma_rn(-yr, cy, __dmul_rn(xr, cx)));
    const double Ji = 1.0 / J;
    const double JW = __dmul_rn(__dmul_rn(__dmul_rn(J, s_w[i]), s_w[j]), s_w[k]);
    const double rx = __dmul_rn(cx, Ji), ry = __dmul_rn(-cy, Ji), rz = __dmul_rn(cz, Ji);
    const double sx = __dmul_rn(-minor2(yr, zt, zr, yt), Ji), sy = __dmul_rn(minor2(xr, zt, zr, xt), Ji),
                 sz = __dmul_rn(-minor2(xr, yt, yr, xt), Ji);
    const double tx = __dmul_rn(minor2(yr, zs, zr, ys), Ji), ty = __dmul_rn(-minor2(xr, zs, zr, xs), Ji),
                 tz = __dmul_rn(minor2(xr, ys, yr, xs), Ji);
    auto dot3 = [](double a0, double b0, double a1, double b1, double a2, double b2) {
      return __fma_rn(a2, b2, __fma_rn(a1, b1, __dmul_rn(a0, b0)));
    };
    g[0 * NP + n] = __dmul_rn(JW, dot3(rx, rx, ry, ry, rz, rz));
    g[1 * NP + n] = __dmul_rn(JW, dot3(rx, sx, ry, sy, rz, sz));
    g[2 * NP + n] = __dmul_rn(JW, dot3(sx, sx, sy, sy, sz, sz));
    g[3 * NP + n] = __dmul_rn(JW, dot3(sx, tx, sy, ty, sz, tz));
    g[4 * NP + n] = __dmul_rn(JW, dot3(rx, tx, ry, ty, rz, tz));
    g[5 * NP + n] = __dmul_rn(JW, dot3(tx, tx, ty, ty, tz, tz));
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

namespace nrsg {

// ===========================================================================
// FP64-accurate axhelm in FP32-pair arithmetic (for the FP64 outer operator).
//
// GB300 executes FP32 at 64x the FP64 rate.  This kernel computes the same
// A q as ax_stored_kernel<double> with every value carried as an unevaluated
// sum hi + lo of two floats (about 48 significant bits): products are formed
// exactly with fmaf (TwoProduct), sums are accumulated with Knuth's TwoSum
// and the rounding errors are carried in a second float.  D and the geometric
// factors are split once at setup; q is split on load (integer bit
// operations, no FP64 instructions) and A q is returned as the double hi + lo
// (one FP64 add).  Accuracy is about 2^-47 relative per term (FP64: 2^-53),
// i.e. ~1e-14 on the operator; see the parity tests for the measured error.
// ===========================================================================
namespace {
struct F2 {
  float s, t; // running sum (s) and carried error (t)
};
__device__ __forceinline__ void acc_prod(F2 &a, float xh, float xl, float yh, float yl)
{
  const float p = xh * yh;
  float e = fmaf(xh, yh, -p);
  e = fmaf(xh, yl, e);
  e = fmaf(xl, yh, e);
  const float u = a.s + p;
  const float bb = u - a.s;
  const float err = (a.s - (u - bb)) + (p - bb);
  a.s = u;
  a.t += err + e;
}
__device__ __forceinline__ void norm2(F2 a, float &hi, float &lo)
{
  hi = a.s + a.t;
  lo = a.t - (hi - a.s);
}
// x = hi + lo from the bits of x, without FP64 instructions (the FP64 pipe is
// 1/64 of the FP32 rate): hi = x with its mantissa truncated to 23 bits, lo =
// the 29 bits below, rounded to 24 bits (I2F) and scaled by 2^(e - 52).
// Together about 2^-47 relative.  |x| < 2^-126 flushes to 0; for
// |x| < 2^-74 lo (below the normal float range) flushes to 0.
__device__ __forceinline__ void split_d(double x, float &hi, float &lo)
{
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned w1 = (unsigned)(b >> 32), w0 = (unsigned)b;
  const int ex = (int)((w1 >> 20) & 0x7FF);
  const unsigned sign = w1 & 0x80000000u;
  if (ex < 897 || ex > 1150) { // zero, subnormal, below/above the float range
    hi = 0.f;
    lo = 0.f;
    return;
  }
  hi = __uint_as_float(sign | ((unsigned)(ex - 896) << 23) | ((w1 & 0xFFFFFu) << 3) | (w0 >> 29));
  const float r = __uint2float_rn(w0 & 0x1FFFFFFFu);
  lo = ex >= 949 ? __uint_as_float(sign | __float_as_uint(r * __uint_as_float((unsigned)(ex - 1075 + 127) << 23))) : 0.f;
}
// the double of a float from its bits (normal floats; zero and subnormals give 0)
__device__ __forceinline__ double widen(float f)
{
  const unsigned u = __float_as_uint(f);
  const unsigned ef = (u >> 23) & 0xFFu;
  if (ef == 0u) return 0.0;
  const unsigned long long b = ((unsigned long long)(u & 0x80000000u) << 32) |
                               ((unsigned long long)(ef + 896u) << 52) | ((unsigned long long)(u & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)b);
}
} // namespace

template <int NQ, bool POISSON>
__global__ void __launch_bounds__(NQ *NQ *AxShape<NQ>::epb)
    ax_fp32x2_kernel(long long E, const float2 *__restrict__ ggeo, const float2 *__restrict__ D, float2 lam0,
                     float2 lam1, const double *__restrict__ q, double *__restrict__ Aq)
{
  constexpr int EPB = AxShape<NQ>::epb;
  constexpr int NP = NQ * NQ * NQ;
  __shared__ float s_Dh[NQ][NQ + 1], s_Dl[NQ][NQ + 1];
  __shared__ float s_qh[EPB][NQ][NQ], s_ql[EPB][NQ][NQ];
  __shared__ float s_Grh[EPB][NQ][NQ], s_Grl[EPB][NQ][NQ];
  __shared__ float s_Gsh[EPB][NQ][NQ], s_Gsl[EPB][NQ][NQ];

  const int t = threadIdx.x;
  const int i = t % NQ, j = t / NQ;
  const int el = threadIdx.y;
  const long long e = (long long)blockIdx.x * EPB + el;
  const bool active = e < E;
  if (el == 0) {
    const float2 d = D[j * NQ + i];
    s_Dh[j][i] = d.x;
    s_Dl[j][i] = d.y;
  }
  float qh[NQ], ql[NQ];
  F2 aq[NQ];
  const long long base = e * NP + t;
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    split_d(active ? q[base + k * NQ * NQ] : 0.0, qh[k], ql[k]);
    aq[k].s = 0.f;
    aq[k].t = 0.f;
  }
  __syncthreads();
  const float2 *g = ggeo + e * 7 * NP + t;
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    float2 G00 = {0, 0}, G01 = {0, 0}, G11 = {0, 0}, G12 = {0, 0}, G02 = {0, 0}, G22 = {0, 0}, GWJ = {0, 0};
    if (active) {
      const int o = k * NQ * NQ;
      G00 = g[0 * NP + o];
      G01 = g[1 * NP + o];
      G11 = g[2 * NP + o];
      G12 = g[3 * NP + o];
      G02 = g[4 * NP + o];
      G22 = g[5 * NP + o];
      if (!POISSON) GWJ = g[6 * NP + o];
    }
    s_qh[el][j][i] = qh[k];
    s_ql[el][j][i] = ql[k];
    F2 at = {0.f, 0.f};
#pragma unroll
    for (int m = 0; m < NQ; ++m) acc_prod(at, s_Dh[k][m], s_Dl[k][m], qh[m], ql[m]);
    __syncthreads();
    F2 ar = {0.f, 0.f}, as = {0.f, 0.f};
#pragma unroll
    for (int m = 0; m < NQ; ++m) {
      acc_prod(ar, s_Dh[i][m], s_Dl[i][m], s_qh[el][j][m], s_ql[el][j][m]);
      acc_prod(as, s_Dh[j][m], s_Dl[j][m], s_qh[el][m][i], s_ql[el][m][i]);
    }
    float rh, rl, sh, sl, th, tl;
    norm2(ar, rh, rl);
    norm2(as, sh, sl);
    norm2(at, th, tl);
    F2 gr = {0.f, 0.f}, gs = {0.f, 0.f}, gt = {0.f, 0.f};
    acc_prod(gr, G00.x, G00.y, rh, rl);
    acc_prod(gr, G01.x, G01.y, sh, sl);
    acc_prod(gr, G02.x, G02.y, th, tl);
    acc_prod(gs, G01.x, G01.y, rh, rl);
    acc_prod(gs, G11.x, G11.y, sh, sl);
    acc_prod(gs, G12.x, G12.y, th, tl);
    acc_prod(gt, G02.x, G02.y, rh, rl);
    acc_prod(gt, G12.x, G12.y, sh, sl);
    acc_prod(gt, G22.x, G22.y, th, tl);
    float grh, grl, gsh, gsl, gth, gtl;
    norm2(gr, grh, grl);
    norm2(gs, gsh, gsl);
    norm2(gt, gth, gtl);
    if (lam0.x != 1.f || lam0.y != 0.f) {
      F2 a = {0.f, 0.f}, b = {0.f, 0.f}, c = {0.f, 0.f};
      acc_prod(a, lam0.x, lam0.y, grh, grl);
      acc_prod(b, lam0.x, lam0.y, gsh, gsl);
      acc_prod(c, lam0.x, lam0.y, gth, gtl);
      norm2(a, grh, grl);
      norm2(b, gsh, gsl);
      norm2(c, gth, gtl);
    }
    s_Grh[el][j][i] = grh;
    s_Grl[el][j][i] = grl;
    s_Gsh[el][j][i] = gsh;
    s_Gsl[el][j][i] = gsl;
    F2 auk = {0.f, 0.f};
    if (!POISSON) {
      F2 w = {0.f, 0.f};
      acc_prod(w, GWJ.x, GWJ.y, lam1.x, lam1.y);
      float wh, wl;
      norm2(w, wh, wl);
      acc_prod(auk, wh, wl, qh[k], ql[k]);
    }
    __syncthreads();
#pragma unroll
    for (int m = 0; m < NQ; ++m) {
      acc_prod(auk, s_Dh[m][j], s_Dl[m][j], s_Gsh[el][m][i], s_Gsl[el][m][i]);
      acc_prod(aq[m], s_Dh[k][m], s_Dl[k][m], gth, gtl);
      acc_prod(auk, s_Dh[m][i], s_Dl[m][i], s_Grh[el][j][m], s_Grl[el][j][m]);
    }
    float uh, ul;
    norm2(auk, uh, ul);
    acc_prod(aq[k], uh, ul, 1.f, 0.f);
    __syncthreads();
  }
  if (active) {
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      float h, l;
      norm2(aq[k], h, l);
      Aq[base + k * NQ * NQ] = widen(h) + widen(l);
    }
  }
}

void launch_ax_fp32x2(int N, long long E, const float2 *ggeo, const float2 *D, double lambda0, double lambda1,
                      bool poisson, const double *q, double *Aq, cudaStream_t s)
{
  if (E <= 0) return;
  float2 l0, l1;
  l0.x = (float)lambda0;
  l0.y = (float)(lambda0 - (double)l0.x);
  l1.x = (float)lambda1;
  l1.y = (float)(lambda1 - (double)l1.x);
#define NRSG_AXD(NQ)                                                                                       \
  {                                                                                                        \
    constexpr int EPB = AxShape<NQ>::epb;                                                                  \
    dim3 blk(NQ * NQ, EPB);                                                                                \
    const unsigned grid = (unsigned)((E + EPB - 1) / EPB);                                                 \
    if (poisson)                                                                                           \
      ax_fp32x2_kernel<NQ, true><<<grid, blk, 0, s>>>(E, ggeo, D, l0, l1, q, Aq);                          \
    else                                                                                                   \
      ax_fp32x2_kernel<NQ, false><<<grid, blk, 0, s>>>(E, ggeo, D, l0, l1, q, Aq);                         \
  }
  NRSG_DISPATCH_NQ(N, NRSG_AXD)
#undef NRSG_AXD
  NRSG_CHECK_LAUNCH();
}

// split doubles into (hi, lo) float pairs
__global__ void split_pairs_kernel(long long n, const double *__restrict__ x, float2 *__restrict__ y)
{
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float h, l;
    split_d(x[i], h, l);
    y[i] = make_float2(h, l);
  }
}
void launch_split_pairs(long long n, const double *x, float2 *y, cudaStream_t s)
{
  if (n <= 0) return;
  long long b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  split_pairs_kernel<<<(unsigned)b, 256, 0, s>>>(n, x, y);
  NRSG_CHECK_LAUNCH();
}

} // namespace nrsg
