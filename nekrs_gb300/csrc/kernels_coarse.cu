// Coarse-level Jacobi-PCG on the assembled operator as one persistent
// cooperative kernel (sm_103a).
//
// The coarsest pMG level (order 1 in the configurations here) is solved by
// Jacobi-preconditioned CG to a relative tolerance (1e-4 by default), the
// build's stand-in for the reference's AMG coarse solve (coarseLevel_t::solve,
// src/solvers/elliptic/MG/coarseLevel.cpp:182-222).  Like the reference, the
// solve works on the assembled matrix of the level operator over the unmasked
// unique nodes (ellipticBuildFEMHex3D, src/solvers/elliptic/MG/
// ellipticBuildFEM.cpp:73-230).  That removes the gather-scatter, the mask
// and the E-vector redundancy (8 copies per node of an order-1 hexahedral
// mesh) from every iteration.
//
// The solve is a distributed SpMV inside one launch.  Rows are split into
// contiguous blocks, one per CTA (one CTA per SM).  Everything a CTA owns
// stays in shared memory for the whole solve: its rows of x, r, p, A p, z and
// 1/diag, the list of other blocks' rows it reads (its halo) and, when it
// fits, its block of the matrix in ELL form with local 16-bit column indices
// (own rows first, then the halo).  Per iteration a CTA reads only the halo
// values of z from L2 and writes only its own z back.  A p is carried by the
// recurrence A p_new = A z + beta A p_old, so z is the only vector that
// crosses CTAs.  One iteration is two phases separated by grid barriers:
//   A  halo of z into shared memory; w = A z; p = z + beta p;
//      Ap = w + beta Ap; partial (p, Ap)
//   B  x += alpha p, r -= alpha Ap, z = invDiag r; partials (r, r), (r, z)
// Per-thread products and warp sums run in the solve's precision (FP32 in
// the mixed and FP32 multigrid; FP64 pipes are a small fraction of the FP32
// ones on this part); sums across warps and CTAs are FP64 (FP32 in the
// pipelined FP32 variant).  Thread 0 forms
// the scalars (alpha, beta, the convergence test) and shares them through
// shared memory.
// The grid barrier is one arrival counter per launch: each CTA adds 1 with a
// release, then waits with acquire loads until the counter reaches its next
// multiple of the grid size, then fences.  Every wait is bounded: on timeout
// the kernel records an error flag and every CTA returns.  Values other CTAs
// wrote during the launch (z, the solution, the partial sums) are read with
// ld.global.cg from L2: an SM's L1 is not coherent with other SMs' stores.
// Dot products are deterministic: each CTA writes a partial and every CTA
// sums all partials in the same fixed order.

#include "mg_kernels.hpp"

#include <algorithm>
#include <mutex>

namespace nrsg {

namespace {
constexpr int kCT = 1024;              // most threads per CTA (one CTA per SM; a row block of fewer rows uses fewer)
constexpr int kMinRowsPerCta = 128;
constexpr long long kOneCtaRows = 4096; // 10 FP32 row vectors = 160 KB of shared memory
constexpr int kMaxCluster = 8;          // portable thread-block cluster size

struct CoarseState {
  unsigned arrive;
  int err;
  int iters;
  int pad;
  double res0, res;
};

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p)
{
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void red_release_add_u32(unsigned *p, unsigned v)
{
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

template <typename T> __device__ __forceinline__ T wsum(T v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// CTA sums of one or two per-thread values (warp sums in T, then FP64 across
// warps in warp 0); thread 0 stores them to dst0 / dst1.  `sh` holds 64 doubles.
template <typename T> __device__ __forceinline__ void cta_partial(T a, double *sh, double *dst0)
{
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  a = wsum(a);
  if (lane == 0) sh[wid] = (double)a;
  __syncthreads();
  if (wid == 0) {
    const double x = wsum(lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0);
    if (lane == 0) *dst0 = x;
  }
}
template <typename T> __device__ __forceinline__ void cta_partial2(T a, T b, double *sh, double *dst0, double *dst1)
{
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  a = wsum(a);
  b = wsum(b);
  if (lane == 0) {
    sh[wid] = (double)a;
    sh[32 + wid] = (double)b;
  }
  __syncthreads();
  if (wid == 0) {
    const bool in = lane < (int)(blockDim.x >> 5);
    const double x = wsum(in ? sh[lane] : 0.0), y = wsum(in ? sh[32 + lane] : 0.0);
    if (lane == 0) {
      *dst0 = x;
      *dst1 = y;
    }
  }
}

// Three CTA sums entirely in T (the pipelined variant; FP32 sums are enough
// for a solve to 1e-4 and avoid the slow FP64 pipe), fixed order.  `sh`
// holds 96 values of T.
template <typename T>
__device__ __forceinline__ void cta_partial3(T a, T b, T c, T *sh, T *dst0, T *dst1, T *dst2)
{
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  a = wsum(a);
  b = wsum(b);
  c = wsum(c);
  if (lane == 0) {
    sh[wid] = a;
    sh[32 + wid] = b;
    sh[64 + wid] = c;
  }
  __syncthreads();
  if (wid == 0) {
    const bool in = lane < (int)(blockDim.x >> 5);
    const T x = wsum(in ? sh[lane] : T(0)), y = wsum(in ? sh[32 + lane] : T(0)), z = wsum(in ? sh[64 + lane] : T(0));
    if (lane == 0) {
      *dst0 = x;
      *dst1 = y;
      *dst2 = z;
    }
  }
}

// Sum of the per-CTA partials of one slot, in warp 0 (valid in its lanes).
// The first 160 partials are loaded at once (one L2 round trip for grids of
// up to 160 CTAs), then added in a fixed order.
__device__ __forceinline__ double grid_sum(const double *part)
{
  const int G = (int)gridDim.x;
  double v[5];
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    const int b = threadIdx.x + 32 * j;
    v[j] = b < G ? __ldcg(part + b) : 0.0;
  }
  double s = (v[0] + v[1]) + (v[2] + v[3]) + v[4];
  for (int b = threadIdx.x + 160; b < G; b += 32) s += __ldcg(part + b);
  return wsum(s);
}

// Sums of three consecutive slots of per-CTA partials, in warp 0: every load
// is issued before the first add.
template <typename T> __device__ __forceinline__ void grid_sum3(const T *part, T &s0, T &s1, T &s2)
{
  const int G = (int)gridDim.x;
  T v[3][5];
#pragma unroll
  for (int q = 0; q < 3; ++q)
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      const int b = threadIdx.x + 32 * j;
      v[q][j] = b < G ? __ldcg(part + q * G + b) : T(0);
    }
  T t[3];
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    t[q] = (v[q][0] + v[q][1]) + (v[q][2] + v[q][3]) + v[q][4];
    for (int b = threadIdx.x + 160; b < G; b += 32) t[q] += __ldcg(part + q * G + b);
  }
  s0 = wsum(t[0]);
  s1 = wsum(t[1]);
  s2 = wsum(t[2]);
}

// Grid barrier number `nb` (1, 2, ...).  Returns false in every thread of the
// CTA if the wait timed out (more than spinLimit polls) or another CTA
// reported an error.  `extra` arrivals are added to the target: 0 in
// ordinary use; a nonzero value makes the target unreachable, which is how
// the test of the bounded wait makes every wait run out.
__device__ __forceinline__ bool grid_barrier(CoarseState *st, unsigned nb, long long spinLimit, unsigned extra,
                                             int cluster)
{
  if (cluster) {
    // the grid is one thread-block cluster, co-scheduled by the hardware: its
    // barrier (release / acquire at cluster scope, global memory included)
    // never spins and cannot be left waiting
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
    return true;
  }
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    red_release_add_u32(&st->arrive, 1u);
    const unsigned target = nb * gridDim.x + extra;
    int ok = 1;
    long long spins = 0;
    while ((int)(ld_acquire_u32(&st->arrive) - target) < 0) {
      ++spins;
      if ((spins & 63) == 0) {
        if (*(volatile int *)&st->err) { ok = 0; break; }
        if (spins > spinLimit) {
          atomicExch(&st->err, 1);
          ok = 0;
          break;
        }
      }
      if (spins > 2048) __nanosleep(64);
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

template <typename T> __device__ __forceinline__ T fma_t(T a, T b, T c);
template <> __device__ __forceinline__ float fma_t<float>(float a, float b, float c) { return __fmaf_rn(a, b, c); }
template <> __device__ __forceinline__ double fma_t<double>(double a, double b, double c) { return __fma_rn(a, b, c); }

__host__ __device__ __forceinline__ size_t align16(size_t b) { return (b + 15) & ~size_t(15); }

// dynamic shared memory: z (own rows, then halo), x, r, p, Ap, 1/diag of the
// own rows, the halo row list; then the matrix block when it is kept there
template <typename T> __host__ __device__ __forceinline__ size_t vec_bytes(int chunk, int maxHalo)
{
  return align16(sizeof(T) * (6 * (size_t)chunk + maxHalo) + sizeof(int) * (size_t)maxHalo);
}
// pipelined variant: m (own rows, then halo), x, r, u, w, z, q, s, p, 1/diag, the halo list
template <typename T> __host__ __device__ __forceinline__ size_t vec_bytes_pipe(int chunk, int maxHalo)
{
  return align16(sizeof(T) * (10 * (size_t)chunk + maxHalo) + sizeof(int) * (size_t)maxHalo);
}
template <typename T> __host__ __device__ __forceinline__ size_t mat_bytes(int chunk, int width)
{
  return align16((size_t)width * chunk * (sizeof(T) + sizeof(unsigned short)));
}
} // namespace

template <typename T> struct CoarseArgs {
  long long nrow, nE;
  int width, chunk, maxHalo, matInSmem;
  const unsigned short *lcol; // [grid][width][chunk]
  const T *val;               // [grid][width][chunk]
  const int *haloOff, *haloIds;
  const T *invDiag;           // [nrow]
  const int *rep;             // [nrow] an E-vector node of each row
  const int *rowOf;           // [nE] row of each E-vector node, -1 where masked
  const T *b;                 // E-vector right-hand side (continuous, masked)
  T *xE;                      // E-vector solution
  T *x, *z;                   // [nrow]: the solution rows (for the scatter), z (for the halos)
  T *z2;                      // [nrow]: second exchange buffer (pipelined variant)
  double *partials;           // [3][gridDim] (pipelined: [2][3][gridDim])
  CoarseState *st;
  double tol;                 // relative
  int maxit;
  unsigned barrierExtra;      // added to every grid barrier's target (0; nonzero only to test the bounded wait)
  int cluster;                // the grid is one cluster: hardware cluster barrier in place of the counter
  long long spinLimit;        // polls before a grid barrier wait gives up
};

template <typename T> __global__ void __launch_bounds__(kCT, 1) coarse_pcg_kernel(CoarseArgs<T> a)
{
  __shared__ double sh[64];
  __shared__ T s_alpha, s_beta;
  __shared__ int s_cont;
  extern __shared__ __align__(16) unsigned char dsm[];
  const int chunk = a.chunk, W = a.width, mh = a.maxHalo;
  const long long start = (long long)blockIdx.x * chunk;
  const int cnt = (int)min((long long)chunk, a.nrow - start);
  const int h0 = __ldg(a.haloOff + blockIdx.x), nh = __ldg(a.haloOff + blockIdx.x + 1) - h0;
  T *zs = (T *)dsm; // [chunk + maxHalo]: own z, then the halo
  T *xs = zs + chunk + mh, *rs = xs + chunk, *ps = rs + chunk, *aps = ps + chunk, *ids = aps + chunk;
  int *hs = (int *)(ids + chunk);
  const T *V;
  const unsigned short *Lc;
  {
    const size_t off = (size_t)blockIdx.x * W * chunk;
    if (a.matInSmem) {
      T *sv = (T *)(dsm + vec_bytes<T>(chunk, mh));
      unsigned short *sl = (unsigned short *)(sv + (size_t)W * chunk);
      for (int i = threadIdx.x; i < W * chunk; i += blockDim.x) {
        sv[i] = __ldg(a.val + off + i);
        sl[i] = __ldg(a.lcol + off + i);
      }
      V = sv;
      Lc = sl;
    } else {
      V = a.val + off;
      Lc = a.lcol + off;
    }
  }
  for (int i = threadIdx.x; i < nh; i += blockDim.x) hs[i] = __ldg(a.haloIds + h0 + i);
  T *zg = a.z + start;
  T rr = T(0), rz = T(0);
  for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
    const T ru = __ldg(a.b + __ldg(a.rep + start + t));
    const T iv = __ldg(a.invDiag + start + t);
    const T zu = iv * ru;
    xs[t] = T(0);
    ps[t] = T(0);
    aps[t] = T(0);
    rs[t] = ru;
    ids[t] = iv;
    zs[t] = zu;
    zg[t] = zu;
    rr = fma_t<T>(ru, ru, rr);
    rz = fma_t<T>(ru, zu, rz);
  }
  cta_partial2<T>(rr, rz, sh, a.partials + blockIdx.x, a.partials + gridDim.x + blockIdx.x);
  if (!grid_barrier(a.st, 1, a.spinLimit, a.barrierExtra, a.cluster)) return;
  unsigned nb = 1;
  // scalars, kept by thread 0 of each CTA (identical in every CTA)
  double r0 = 0, rn = 0, tol = 0, rdotz = 0;
  int it = 0;
  if (threadIdx.x < 32) {
    const double srr = grid_sum(a.partials), srz = grid_sum(a.partials + gridDim.x);
    if (threadIdx.x == 0) {
      r0 = sqrt(srr);
      rn = r0;
      rdotz = srz;
      tol = a.tol * r0;
      s_beta = T(0);
      s_cont = (rn > tol && a.maxit > 0 && r0 > 0) ? 1 : 0;
    }
  }
  __syncthreads();
  while (s_cont) {
    const T beta = s_beta;
    // A: halo of z, then w = A z, p, Ap, (p, Ap)
#pragma unroll 4
    for (int i = threadIdx.x; i < nh; i += blockDim.x) zs[chunk + i] = __ldcg(a.z + hs[i]);
    __syncthreads();
    T pap = T(0);
    for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
      T w = T(0);
#pragma unroll 9
      for (int k = 0; k < W; ++k) w = fma_t<T>(V[k * chunk + t], zs[Lc[k * chunk + t]], w);
      const T pu = fma_t<T>(beta, ps[t], zs[t]);
      const T apu = fma_t<T>(beta, aps[t], w);
      ps[t] = pu;
      aps[t] = apu;
      pap = fma_t<T>(pu, apu, pap);
    }
    cta_partial<T>(pap, sh, a.partials + 2 * gridDim.x + blockIdx.x);
    if (!grid_barrier(a.st, ++nb, a.spinLimit, a.barrierExtra, a.cluster)) return;
    if (threadIdx.x < 32) {
      const double spap = grid_sum(a.partials + 2 * gridDim.x);
      if (threadIdx.x == 0) s_alpha = (T)(rdotz / (spap + 1e-300));
    }
    __syncthreads();
    const T alpha = s_alpha;
    // B: x += alpha p, r -= alpha Ap, z = invDiag r, (r, r), (r, z)
    rr = T(0);
    rz = T(0);
    for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
      xs[t] = fma_t<T>(alpha, ps[t], xs[t]);
      const T ru = fma_t<T>(-alpha, aps[t], rs[t]);
      rs[t] = ru;
      const T zu = ids[t] * ru;
      zs[t] = zu;
      zg[t] = zu;
      rr = fma_t<T>(ru, ru, rr);
      rz = fma_t<T>(ru, zu, rz);
    }
    cta_partial2<T>(rr, rz, sh, a.partials + blockIdx.x, a.partials + gridDim.x + blockIdx.x);
    if (!grid_barrier(a.st, ++nb, a.spinLimit, a.barrierExtra, a.cluster)) return;
    if (threadIdx.x < 32) {
      const double srr = grid_sum(a.partials);
      const double srz = grid_sum(a.partials + gridDim.x);
      if (threadIdx.x == 0) {
        ++it;
        rn = sqrt(srr);
        const double rdotz_old = rdotz;
        rdotz = srz;
        s_beta = (T)(rdotz / rdotz_old);
        s_cont = (rn > tol && it < a.maxit) ? 1 : 0;
      }
    }
    __syncthreads();
  }
  // E-vector solution: every copy of a row takes its value, masked nodes 0
  for (int t = threadIdx.x; t < cnt; t += blockDim.x) a.x[start + t] = xs[t];
  if (!grid_barrier(a.st, ++nb, a.spinLimit, a.barrierExtra, a.cluster)) return;
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x, nth = (long long)gridDim.x * blockDim.x;
  for (long long i = tid; i < a.nE; i += nth) {
    const int u = __ldg(a.rowOf + i);
    a.xE[i] = u >= 0 ? __ldcg(a.x + u) : T(0);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.st->iters = it;
    a.st->res0 = r0;
    a.st->res = rn;
  }
}

// Pipelined Jacobi-PCG (Ghysels and Vanroose, "Hiding global synchronization
// latency in the preconditioned conjugate gradient algorithm", Parallel
// Computing 40 (2014), Alg. 4) in the same row-block layout: the dot products
// (r,u), (w,u), (r,r) of an iteration and the exchange of m = M^-1 w complete
// at one grid barrier, and the SpMV n = A m and all vector updates follow
// without another; one barrier per iteration instead of two.  Mathematically
// the same iterates as PCG; the convergence test reads ||r_i|| before the
// update that would produce r_{i+1}, so the iteration count is PCG's.  The
// published m and the partial sums alternate between two buffers by iteration
// parity: a CTA rewrites a buffer only after passing a barrier that every
// reader of its previous contents has reached.
template <typename T> __global__ void __launch_bounds__(kCT, 1) coarse_ppcg_kernel(CoarseArgs<T> a)
{
  __shared__ T sh[96];
  __shared__ T s_alpha, s_beta;
  __shared__ int s_cont;
  extern __shared__ __align__(16) unsigned char dsm[];
  const int chunk = a.chunk, W = a.width, mh = a.maxHalo;
  const long long start = (long long)blockIdx.x * chunk;
  const int cnt = (int)min((long long)chunk, a.nrow - start);
  const int h0 = __ldg(a.haloOff + blockIdx.x), nh = __ldg(a.haloOff + blockIdx.x + 1) - h0;
  T *ms = (T *)dsm; // [chunk + maxHalo]: m (own rows, then halo)
  T *xs = ms + chunk + mh, *rs = xs + chunk, *us = rs + chunk, *wv = us + chunk, *zv = wv + chunk;
  T *qv = zv + chunk, *sv = qv + chunk, *pv = sv + chunk, *ids = pv + chunk;
  int *hs = (int *)(ids + chunk);
  const T *V;
  const unsigned short *Lc;
  {
    const size_t off = (size_t)blockIdx.x * W * chunk;
    if (a.matInSmem) {
      T *svm = (T *)(dsm + vec_bytes_pipe<T>(chunk, mh));
      unsigned short *sl = (unsigned short *)(svm + (size_t)W * chunk);
      for (int i = threadIdx.x; i < W * chunk; i += blockDim.x) {
        svm[i] = __ldg(a.val + off + i);
        sl[i] = __ldg(a.lcol + off + i);
      }
      V = svm;
      Lc = sl;
    } else {
      V = a.val + off;
      Lc = a.lcol + off;
    }
  }
  for (int i = threadIdx.x; i < nh; i += blockDim.x) hs[i] = __ldg(a.haloIds + h0 + i);
  // exchange buffers: u0 goes through a.z, m_i through a.z2 (i even) / a.z (i odd)
  // r0 = b, u0 = M^-1 r0 (published for the halos), x0 = 0
  for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
    const T ru = __ldg(a.b + __ldg(a.rep + start + t));
    const T iv = __ldg(a.invDiag + start + t);
    const T uu = iv * ru;
    xs[t] = T(0);
    rs[t] = ru;
    us[t] = uu;
    ids[t] = iv;
    zv[t] = T(0);
    qv[t] = T(0);
    sv[t] = T(0);
    pv[t] = T(0);
    ms[t] = uu;
    a.z[start + t] = uu;
  }
  if (!grid_barrier(a.st, 1, a.spinLimit, a.barrierExtra, a.cluster)) return;
  unsigned nb = 1;
  // w0 = A u0
#pragma unroll 4
  for (int i = threadIdx.x; i < nh; i += blockDim.x) ms[chunk + i] = __ldcg(a.z + hs[i]);
  __syncthreads();
  for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
    T w = T(0);
#pragma unroll 9
    for (int k = 0; k < W; ++k) w = fma_t<T>(V[k * chunk + t], ms[Lc[k * chunk + t]], w);
    wv[t] = w;
  }
  // scalars, kept by thread 0 of each CTA (identical in every CTA)
  double r0 = 0, rn = 0, tol = 0, gamma_old = 1, alpha_old = 1;
  int it = 0;
  for (int i = 0;; ++i) {
    T *mg = (i & 1) ? a.z : a.z2;
    T *part = (T *)a.partials + (size_t)(i & 1) * 3 * gridDim.x; // partials in T
    __syncthreads(); // the previous SpMV has read ms
    // phase 1: partial (r,u), (w,u), (r,r); m = M^-1 w, published
    T g = T(0), d = T(0), rr = T(0);
    for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
      const T ru = rs[t], uu = us[t], ww = wv[t];
      g = fma_t<T>(ru, uu, g);
      d = fma_t<T>(ww, uu, d);
      rr = fma_t<T>(ru, ru, rr);
      const T mm = ids[t] * ww;
      ms[t] = mm;
      mg[start + t] = mm;
    }
    cta_partial3<T>(g, d, rr, sh, part + blockIdx.x, part + gridDim.x + blockIdx.x, part + 2 * gridDim.x + blockIdx.x);
    if (!grid_barrier(a.st, ++nb, a.spinLimit, a.barrierExtra, a.cluster)) return;
    if (threadIdx.x < 32) {
      T sgT, sdT, srrT;
      grid_sum3<T>(part, sgT, sdT, srrT);
      const double sg = (double)sgT, sd = (double)sdT, srr = (double)srrT;
      if (threadIdx.x == 0) {
        // scalars in the solve's precision T (FP32 here: no FP64 divide or sqrt)
        rn = (double)sqrt((T)srr);
        if (i == 0) {
          r0 = rn;
          tol = a.tol * r0;
        }
        const int cont = (rn > tol && it < a.maxit && r0 > 0) ? 1 : 0;
        if (cont) {
          const T g = (T)sg, dd = (T)sd;
          const T beta = (i == 0) ? T(0) : g / (T)gamma_old;
          const T alpha = (i == 0) ? g / dd : g / (dd - beta * g / (T)alpha_old);
          gamma_old = sg;
          alpha_old = (double)alpha;
          s_alpha = alpha;
          s_beta = beta;
          ++it;
        }
        s_cont = cont;
      }
    }
    __syncthreads();
    if (!s_cont) break;
    const T alpha = s_alpha, beta = s_beta;
    // phase 2: n = A m; recurrences
#pragma unroll 4
    for (int q = threadIdx.x; q < nh; q += blockDim.x) ms[chunk + q] = __ldcg(mg + hs[q]);
    __syncthreads();
    for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
      T nn = T(0);
#pragma unroll 9
      for (int k = 0; k < W; ++k) nn = fma_t<T>(V[k * chunk + t], ms[Lc[k * chunk + t]], nn);
      const T z1 = fma_t<T>(beta, zv[t], nn);
      const T q1 = fma_t<T>(beta, qv[t], ms[t]);
      const T s1 = fma_t<T>(beta, sv[t], wv[t]);
      const T p1 = fma_t<T>(beta, pv[t], us[t]);
      zv[t] = z1;
      qv[t] = q1;
      sv[t] = s1;
      pv[t] = p1;
      xs[t] = fma_t<T>(alpha, p1, xs[t]);
      rs[t] = fma_t<T>(-alpha, s1, rs[t]);
      us[t] = fma_t<T>(-alpha, q1, us[t]);
      wv[t] = fma_t<T>(-alpha, z1, wv[t]);
    }
  }
  // E-vector solution: every copy of a row takes its value, masked nodes 0
  for (int t = threadIdx.x; t < cnt; t += blockDim.x) a.x[start + t] = xs[t];
  if (!grid_barrier(a.st, ++nb, a.spinLimit, a.barrierExtra, a.cluster)) return;
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x, nth = (long long)gridDim.x * blockDim.x;
  for (long long i = tid; i < a.nE; i += nth) {
    const int u = __ldg(a.rowOf + i);
    a.xE[i] = u >= 0 ? __ldcg(a.x + u) : T(0);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.st->iters = it;
    a.st->res0 = r0;
    a.st->res = rn;
  }
}

// The dynamic shared-memory limit is an attribute of the kernel function, not
// of a launch, and every solver in the process shares the function: raise it
// to the largest size any solver on the device has needed, never lower it.
void raise_dynamic_smem(const void *kfn, size_t bytes)
{
  static std::mutex m;
  static std::vector<std::pair<std::pair<int, const void *>, size_t>> set;
  int dev = 0;
  NRSG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(m);
  for (auto &e : set)
    if (e.first.first == dev && e.first.second == kfn) {
      if (bytes > e.second) {
        NRSG_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
        e.second = bytes;
      }
      return;
    }
  NRSG_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  set.push_back({{dev, kfn}, bytes});
}

// Host: partition the rows over one CTA per SM, build each CTA's ELL block
// (local columns: own rows 0..chunk-1, halo rows chunk..), its halo list and
// the shared-memory plan.
template <typename T>
void coarse_matrix_setup(long long n, const long long *rowPtr, const long long *col, const double *val, long long nE,
                         const long long *rowOfNode, const int *rep, CoarseMatrix<T> &M, bool noCluster)
{
  int dev = 0, sms = 0, optin = 0;
  NRSG_CUDA(cudaGetDevice(&dev));
  NRSG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  NRSG_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  if (nE >= (1LL << 31) || n >= (1LL << 31)) throw Error(NRSG_ERR_BAD_CONFIG, "coarse level too large for 32-bit indices");
  int width = 1;
  for (long long r = 0; r < n; ++r) width = std::max(width, (int)(rowPtr[r + 1] - rowPtr[r]));
  long long grid = std::min<long long>(sms, std::max<long long>(1, (n + kMinRowsPerCta - 1) / kMinRowsPerCta));
  // a level whose row vectors fit one CTA's shared memory is solved by one CTA: no grid barrier ever
  // waits, so it is an ordinary launch (no cooperative launch, no ordering against other solvers);
  // one that fits kMaxCluster such CTAs runs as one thread-block cluster (hardware barrier, co-scheduled,
  // again an ordinary launch), when the device can hold such a cluster
  M.cluster = 0;
  if (n <= kOneCtaRows) {
    grid = 1;
  } else if (!noCluster && n <= kMaxCluster * kOneCtaRows) {
    grid = (n + kOneCtaRows - 1) / kOneCtaRows;
    M.cluster = 1;
  }
  const long long chunk = std::max<long long>(1, (n + grid - 1) / grid);
  grid = std::max<long long>(1, (n + chunk - 1) / chunk);
  if (M.cluster) M.cluster = (int)grid;
  std::vector<int> haloOff(grid + 1, 0), haloIds;
  std::vector<unsigned short> lcol((size_t)grid * width * chunk, 0);
  std::vector<T> v((size_t)grid * width * chunk, T(0));
  std::vector<long long> loc(n > 0 ? n : 1, -1);
  int maxHalo = 0;
  for (long long b = 0; b < grid; ++b) {
    const long long s0 = b * chunk, s1 = std::min(n, s0 + chunk);
    std::vector<long long> halo;
    for (long long r = s0; r < s1; ++r)
      for (long long q = rowPtr[r]; q < rowPtr[r + 1]; ++q)
        if (col[q] < s0 || col[q] >= s1) halo.push_back(col[q]);
    std::sort(halo.begin(), halo.end());
    halo.erase(std::unique(halo.begin(), halo.end()), halo.end());
    if (chunk + (long long)halo.size() > 65535)
      throw Error(NRSG_ERR_BAD_CONFIG, "coarse level: row block and halo exceed 16-bit local indices");
    for (size_t h = 0; h < halo.size(); ++h) loc[halo[h]] = chunk + (long long)h;
    const size_t base = (size_t)b * width * chunk;
    for (long long r = s0; r < s1; ++r) {
      const long long t = r - s0, len = rowPtr[r + 1] - rowPtr[r];
      for (int k = 0; k < width; ++k) {
        const size_t at = base + (size_t)k * chunk + t;
        if (k < len) {
          const long long c = col[rowPtr[r] + k];
          lcol[at] = (unsigned short)((c >= s0 && c < s1) ? c - s0 : loc[c]);
          v[at] = (T)val[rowPtr[r] + k];
        } else {
          lcol[at] = (unsigned short)t; // padding: zero entry on the row itself
        }
      }
    }
    for (long long c : halo) haloIds.push_back((int)c);
    haloOff[b + 1] = (int)haloIds.size();
    maxHalo = std::max(maxHalo, (int)halo.size());
  }
  std::vector<T> invD(n > 0 ? n : 1, T(0));
  for (long long r = 0; r < n; ++r)
    for (long long q = rowPtr[r]; q < rowPtr[r + 1]; ++q)
      if (col[q] == r && val[q] != 0.0) invD[r] = (T)(1.0 / val[q]);
  std::vector<int> rowOf(nE);
  for (long long i = 0; i < nE; ++i) rowOf[i] = (int)rowOfNode[i];
  // shared memory: the row vectors and the halo list always; the matrix block when it fits
  // FP32 solves use the pipelined variant (one barrier per iteration); FP64
  // keeps the two-barrier PCG, the same recurrences as the host-driven loop
  M.pipelined = sizeof(T) == 4;
  const void *kfn = M.pipelined ? (const void *)coarse_ppcg_kernel<T> : (const void *)coarse_pcg_kernel<T>;
  const size_t vBytes = M.pipelined ? vec_bytes_pipe<T>((int)chunk, maxHalo) : vec_bytes<T>((int)chunk, maxHalo);
  const size_t mBytes = mat_bytes<T>((int)chunk, width);
  const size_t limit = (size_t)optin > 2048 ? (size_t)optin - 2048 : 0; // static shared memory of the kernel
  if (vBytes > limit && M.cluster) // the cluster's row blocks and halos do not fit: many smaller blocks instead
    return coarse_matrix_setup<T>(n, rowPtr, col, val, nE, rowOfNode, rep, M, true);
  if (vBytes > limit) throw Error(NRSG_ERR_BAD_CONFIG, "coarse level: row block too large for shared memory");
  M.matInSmem = vBytes + mBytes <= limit;
  M.smem = vBytes + (M.matInSmem ? mBytes : 0);
  raise_dynamic_smem(kfn, M.smem);
  int perSM = 0;
  NRSG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kfn, std::min<long long>(kCT, std::max<long long>(32, (chunk + 31) / 32 * 32)), M.smem));
  if (perSM < 1) throw Error(NRSG_ERR_CUDA, "coarse solver: kernel cannot be resident");
  if (M.cluster) {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = (unsigned)grid;
    attr.val.clusterDim.y = 1;
    attr.val.clusterDim.z = 1;
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)std::min<long long>(kCT, std::max<long long>(32, (chunk + 31) / 32 * 32)));
    cfg.dynamicSmemBytes = M.smem;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, kfn, &cfg) != cudaSuccess || clusters < 1) {
      (void)cudaGetLastError();
      M.cluster = 0; // not schedulable as one cluster: the cooperative launch of the same row blocks
    }
  }
  M.threads = (int)std::min<long long>(kCT, std::max<long long>(32, (chunk + 31) / 32 * 32));
  M.nrow = n;
  M.nE = nE;
  M.width = width;
  M.grid = (int)grid;
  M.chunk = (int)chunk;
  M.maxHalo = maxHalo;
  M.nnz = n > 0 ? rowPtr[n] : 0;
  M.lcol.upload(lcol);
  M.val.upload(v);
  M.haloOff.upload(haloOff);
  if (haloIds.empty()) haloIds.push_back(0);
  M.haloIds.upload(haloIds);
  M.invDiag.upload(invD);
  std::vector<int> repv(rep, rep + n);
  if (repv.empty()) repv.push_back(0);
  M.rep.upload(repv);
  M.rowOf.upload(rowOf);
}

// Persistent coarse kernels of all solvers in the process are ordered on the
// device (each waits for the previous one, whatever its stream): every one
// occupies a CTA on every SM, and solvers on different streams (batched and
// served solves) must not have two such grids in flight at once.
namespace {
struct CoarseGate {
  std::mutex m;
  cudaEvent_t ev[64] = {};
};
CoarseGate &coarse_gate()
{
  static CoarseGate g;
  return g;
}
} // namespace

template <typename T>
int coarse_pcg_persistent(const CoarseMatrix<T> &A, const T *b, T *xE, T *x, T *z, T *z2, double *partials,
                          void *state, int gridMax, double tol, int maxit, cudaStream_t s, long long spinLimit,
                          unsigned barrierExtra)
{
  if (A.grid > gridMax) throw Error(NRSG_ERR_CUDA, "coarse solver: partial-sum buffer too small");
  int dev = 0;
  NRSG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) throw Error(NRSG_ERR_CUDA, "coarse solver: device index out of range");
  // a cluster-sized level runs as one cluster (no cross-solver ordering); the test knob barrierExtra
  // needs the counting barrier, so it takes the cooperative launch
  const bool useCluster = A.cluster > 0 && barrierExtra == 0;
  const bool cooperative = A.grid > 1 && !useCluster;
  CoarseGate &gate = coarse_gate();
  std::unique_lock<std::mutex> lock(gate.m, std::defer_lock);
  if (cooperative) {
    lock.lock();
    if (!gate.ev[dev]) NRSG_CUDA(cudaEventCreateWithFlags(&gate.ev[dev], cudaEventDisableTiming));
    NRSG_CUDA(cudaStreamWaitEvent(s, gate.ev[dev], 0));
  }
  // the arrival counter starts at zero for every launch; the error flag is kept (sticky for the
  // outer solve, cleared by coarse_state_clear when the solve begins)
  NRSG_CUDA(cudaMemsetAsync(state, 0, sizeof(unsigned), s));
  CoarseArgs<T> a;
  a.nrow = A.nrow;
  a.nE = A.nE;
  a.width = A.width;
  a.chunk = A.chunk;
  a.maxHalo = A.maxHalo;
  a.matInSmem = A.matInSmem ? 1 : 0;
  a.lcol = A.lcol.p;
  a.val = A.val.p;
  a.haloOff = A.haloOff.p;
  a.haloIds = A.haloIds.p;
  a.invDiag = A.invDiag.p;
  a.rep = A.rep.p;
  a.rowOf = A.rowOf.p;
  a.b = b;
  a.xE = xE;
  a.x = x;
  a.z = z;
  a.z2 = z2;
  a.partials = partials;
  a.st = (CoarseState *)state;
  a.tol = tol;
  a.maxit = maxit;
  a.barrierExtra = barrierExtra;
  a.spinLimit = spinLimit;
  a.cluster = 0;
  void *args[] = {&a};
  const void *kfn = A.pipelined ? (const void *)coarse_ppcg_kernel<T> : (const void *)coarse_pcg_kernel<T>;
  if (useCluster) {
    a.cluster = 1;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = (unsigned)A.grid;
    attr.val.clusterDim.y = 1;
    attr.val.clusterDim.z = 1;
    cfg.gridDim = dim3(A.grid);
    cfg.blockDim = dim3(A.threads);
    cfg.dynamicSmemBytes = A.smem;
    cfg.stream = s;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    NRSG_CUDA(cudaLaunchKernelExC(&cfg, kfn, args));
    count_launch();
  } else if (cooperative) {
    NRSG_CUDA(cudaLaunchCooperativeKernel(kfn, dim3(A.grid), dim3(A.threads), args, A.smem, s));
    count_launch();
    NRSG_CUDA(cudaEventRecord(gate.ev[dev], s));
  } else {
    NRSG_CUDA(cudaLaunchKernel(kfn, dim3(1), dim3(A.threads), args, A.smem, s));
    count_launch();
  }
  return A.grid;
}

size_t coarse_state_bytes() { return sizeof(CoarseState); }
void coarse_state_clear(void *state, cudaStream_t s) { NRSG_CUDA(cudaMemsetAsync(state, 0, sizeof(CoarseState), s)); }
int coarse_state_read(const void *state_host, int *iters, double *res0, double *res)
{
  const CoarseState *st = (const CoarseState *)state_host;
  if (iters) *iters = st->iters;
  if (res0) *res0 = st->res0;
  if (res) *res = st->res;
  return st->err;
}

template void coarse_matrix_setup<double>(long long, const long long *, const long long *, const double *, long long,
                                          const long long *, const int *, CoarseMatrix<double> &, bool);
template void coarse_matrix_setup<float>(long long, const long long *, const long long *, const double *, long long,
                                         const long long *, const int *, CoarseMatrix<float> &, bool);
template int coarse_pcg_persistent<double>(const CoarseMatrix<double> &, const double *, double *, double *, double *,
                                           double *, double *, void *, int, double, int, cudaStream_t, long long,
                                           unsigned);
template int coarse_pcg_persistent<float>(const CoarseMatrix<float> &, const float *, float *, float *, float *,
                                          float *, double *, void *, int, double, int, cudaStream_t, long long,
                                          unsigned);

} // namespace nrsg
