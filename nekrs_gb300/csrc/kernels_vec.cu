// Gather-scatter, mask, BLAS-1 and fused Krylov vector kernels (sm_103a).
//
// Reference kernels (nekRS tree):
//   gatherScatterMany_*Add   3rd_party/gslib/ogs/okl/gatherScatterMany.okl
//   mask                     kernels/core/mask.okl:27-35
//   weightedInnerProdMany    kernels/linAlg/weightedInnerProdMany.okl:27-105
//   ellipticBlockUpdatePCG   kernels/elliptic/ellipticBlockUpdatePCG.okl:26-111
//   axpbyMany, axmyzMany, adyMany, fill, copyDfloatToPfloat (kernels/linAlg, kernels/core)
//
// Reductions are one launch each and are bit-reproducible: every FP64 sum
// is formed in one fixed order that depends only on n, and the oracle's
// wsum() performs the same operations in the same order:
//   term      each entry contributes through one fused multiply-add,
//             s = fma(x_i, y_i, s), with the factors defined per kernel (a
//             weighted inner product: x_i = w_i a_i rounded, y_i = b_i);
//   chunk c   entries [1024 c, 1024 c + 1024): lane l of the warp accumulates
//             entries 1024 c + l + 32 j, j = 0..31 ascending, from 0 (entries
//             past n are skipped); the 32 lane sums are added by the tree
//             s[l] += s[l + o], o = 16, 8, 4, 2, 1;
//   result    the chunk sums added by the blocked pairwise tree
//             ((P0 + P1) + (P2 + P3)) + ..., zero-padded to a power of two.
// The reference forms w (a b) per entry, adds 256-entry blocks by a tree and
// the block sums one after another on the host (weightedInnerProdMany.okl:
// 27-105, linAlg.cpp:986-1035).  On GB300 the FP64 pipe issues one warp
// instruction per ~16 clocks per SM, so that order (about 3.5 FP64
// operations per entry) is FP64-bound at a third of the HBM rate; this one
// takes about 2.2 per entry and runs at the memory bound.  Each warp owns an
// aligned, power-of-two run of chunks and merges its chunk sums by the
// blocked tree on a small stack; the CTA that finishes last (atomic ticket)
// adds the warp sums, still by the same tree, and stores the result on the
// device.  Krylov scalars (alpha, beta) are formed on the device by the
// kernels that consume them, so there is no host round trip.
//
// FP64 element-wise arithmetic on the plain solve path uses explicit
// roundings (__fma_rn / __dmul_rn / __dadd_rn) so that the compiler's
// contraction choices cannot change results; the oracle calls std::fma at the
// same places.

#include "nrsg_internal.hpp"

namespace nrsg {

namespace {
constexpr int kThreads = kRedThreads;
constexpr int kWarps = kThreads / 32;
constexpr int kChunk = 1024;   // entries per chunk: 32 lanes x 32 entries
constexpr int kStack = 24;     // depth of the per-warp merge stack (runs of up to 2^23 chunks)

__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }

// Sum of chunk c in lane 0.  F: void operator()(long long i, double &x, double &y) const gives
// the factors of entry i < n (and performs the entry's side effects).
template <typename F> __device__ __forceinline__ double chunk_sum(long long c, long long n, const F &f)
{
  const long long i0 = c * kChunk + (threadIdx.x & 31);
  double s = 0.0;
  if ((c + 1) * kChunk <= n) {
#pragma unroll 8
    for (int j = 0; j < 32; ++j) {
      double x, y;
      f(i0 + 32 * j, x, y);
      s = __fma_rn(x, y, s);
    }
  } else {
    for (int j = 0; j < 32; ++j) {
      const long long i = i0 + 32 * j;
      if (i < n) {
        double x, y;
        f(i, x, y);
        s = __fma_rn(x, y, s);
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s = dadd(s, __shfl_down_sync(0xffffffffu, s, o));
  return s;
}

// Work split of one reduction: W warp runs of `len` chunks each (both powers
// of two, W <= kRedSegments), CTAs = ceil(W / 8).
struct RedSplit {
  long long len;
  int warps, ctas;
};
inline RedSplit red_split(long long n)
{
  const long long nc = (n + kChunk - 1) / kChunk;
  long long M = 1;
  while (M < nc) M <<= 1;
  const long long W = M < kRedSegments ? M : kRedSegments;
  RedSplit r;
  r.len = M / W;
  r.warps = (int)W;
  r.ctas = (int)((W + kWarps - 1) / kWarps);
  return r;
}

// The sum of warp run `wid` (chunks [wid*len, (wid+1)*len)) by the blocked
// tree, merged on a per-warp stack in shared memory (lane 0 writes it); the
// result is returned to every lane.
template <typename F>
__device__ __forceinline__ double run_sum(long long wid, long long len, long long n, const F &f)
{
  __shared__ double s_stk[kWarps][kStack];
  double *stk = s_stk[threadIdx.x >> 5];
  const bool lane0 = (threadIdx.x & 31) == 0;
  int sp = 0;
  for (long long q = 0; q < len; ++q) {
    double v = chunk_sum(wid * len + q, n, f);
    for (long long k = q + 1; (k & 1) == 0; k >>= 1) v = dadd(stk[--sp], v);
    if (lane0) stk[sp] = v;
    ++sp;
    __syncwarp();
  }
  return stk[0];
}

// Blocked tree over row[0, W) (zero past W, W <= 8192) by the whole CTA; the
// result is valid in thread 0.
__device__ __forceinline__ double final_tree(const double *row, int W)
{
  __shared__ double sh[kThreads];
  const int t = threadIdx.x;
  const volatile double *vr = row;
  double st[6];
  int sp = 0;
#pragma unroll
  for (int j = 0; j < 32; ++j) {
    const int idx = 32 * t + j;
    double v = idx < W ? vr[idx] : 0.0;
#pragma unroll
    for (int k = j + 1; (k & 1) == 0; k >>= 1) v = dadd(st[--sp], v);
    st[sp++] = v;
  }
  sh[t] = st[0];
  __syncthreads();
#pragma unroll
  for (int o = 1; o < kThreads; o <<= 1) {
    if ((t & (2 * o - 1)) == 0) sh[t] = dadd(sh[t], sh[t + o]);
    __syncthreads();
  }
  const double r = sh[0];
  __syncthreads();
  return r;
}

// Store this warp's run sum (lane 0), then take the CTA's ticket; true in
// every thread of the CTA that finished last.
__device__ __forceinline__ bool store_run_and_ticket(bool storing, double v, double *row, long long wid,
                                                     unsigned *counter)
{
  if (storing && (threadIdx.x & 31) == 0) {
    row[wid] = v;
    __threadfence();
  }
  __shared__ bool s_last;
  __syncthreads();
  if (threadIdx.x == 0) s_last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  return true;
}

// One-vector reduction body shared by the kernels below: run sums, ticket,
// final tree into *out; returns true in the thread that stored *out.
template <typename F>
__device__ __forceinline__ bool reduce1(long long n, long long len, int W, const F &f, double *row, unsigned *counter,
                                        double *out)
{
  const long long wid = (long long)blockIdx.x * kWarps + (threadIdx.x >> 5);
  double v = 0;
  if (wid < W) v = run_sum(wid, len, n, f);
  if (!store_run_and_ticket(wid < W, v, row, wid, counter)) return false;
  const double r = final_tree(row, W);
  if (threadIdx.x == 0) {
    *out = r;
    *counter = 0; // ready for the next launch on this slot
  }
  return threadIdx.x == 0;
}

#define NRSG_GRID_LOOP_VEC(i, n)                                                                           \
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (n); i += (long long)gridDim.x * blockDim.x)
inline unsigned vec_grid(long long n)
{
  long long b = (n + kThreads - 1) / kThreads;
  if (b < 1) b = 1;
  const long long cap = 152LL * 16;
  return (unsigned)(b < cap ? b : cap);
}
} // namespace

// ---------------------------------------------------------------------------
// gather-scatter (ogs add) over groups with >= 2 members
// ---------------------------------------------------------------------------
template <typename T>
__global__ void gs_kernel(long long ng, const int *__restrict__ off, const int *__restrict__ ids, T *__restrict__ q)
{
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < ng; g += (long long)gridDim.x * blockDim.x) {
    const int s = off[g], e = off[g + 1];
    T v = 0;
    for (int m = s; m < e; ++m) v += q[ids[m]];
    for (int m = s; m < e; ++m) q[ids[m]] = v;
  }
}
template <typename T> void launch_gs(long long ng, const int *off, const int *ids, T *q, cudaStream_t s)
{
  if (ng <= 0) return;
  gs_kernel<T><<<vec_grid(ng), kThreads, 0, s>>>(ng, off, ids, q);
  NRSG_CHECK_LAUNCH();
}
template void launch_gs<double>(long long, const int *, const int *, double *, cudaStream_t);
template void launch_gs<float>(long long, const int *, const int *, float *, cudaStream_t);

// gather-scatter by plan (pairs, then the other groups), then optionally the
// mask, in one launch; each group sums its members in member order.  Groups
// share no node, so a thread loads the members of several groups before it
// stores into any: four pairs (or two larger groups of up to eight members,
// larger ones member by member) per pass keep that many independent loads in
// flight, where one group at a time waits on its index load, then on its
// value loads, before the next group starts.
// 4 CTAs of 256 threads per SM for FP32 (64 registers), 3 for FP64 (no spills)
template <typename T>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 3) gs_mask_kernel(GsPlan P, long long nmask, T *__restrict__ q)
{
  constexpr int UP = 4, UR = 2, MR = 8;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  for (long long t = t0; t < P.npairs; t += UP * stride) {
    int2 pr[UP];
#pragma unroll
    for (int u = 0; u < UP; ++u) {
      const long long k = t + u * stride;
      pr[u] = k < P.npairs ? __ldg(P.pairs + k) : make_int2(-1, -1);
    }
    T a[UP], b[UP];
#pragma unroll
    for (int u = 0; u < UP; ++u) {
      a[u] = pr[u].x >= 0 ? q[pr[u].x] : T(0);
      b[u] = pr[u].x >= 0 ? q[pr[u].y] : T(0);
    }
#pragma unroll
    for (int u = 0; u < UP; ++u)
      if (pr[u].x >= 0) {
        const T v = a[u] + b[u];
        q[pr[u].x] = v;
        q[pr[u].y] = v;
      }
  }
  for (long long t = t0; t < P.nrest; t += UR * stride) {
    int s0[UR], m[UR];
#pragma unroll
    for (int u = 0; u < UR; ++u) {
      const long long g = t + u * stride;
      s0[u] = g < P.nrest ? __ldg(P.restOff + g) : 0;
      m[u] = g < P.nrest ? __ldg(P.restOff + g + 1) - s0[u] : 0;
    }
    int id[UR][MR];
    T val[UR][MR];
#pragma unroll
    for (int u = 0; u < UR; ++u)
#pragma unroll
      for (int c = 0; c < MR; ++c) id[u][c] = c < m[u] ? __ldg(P.restIds + s0[u] + c) : 0;
#pragma unroll
    for (int u = 0; u < UR; ++u)
#pragma unroll
      for (int c = 0; c < MR; ++c) val[u][c] = c < m[u] ? q[id[u][c]] : T(0);
#pragma unroll
    for (int u = 0; u < UR; ++u) {
      T v = 0;
      if (m[u] <= MR) {
#pragma unroll
        for (int c = 0; c < MR; ++c)
          if (c < m[u]) v += val[u][c];
#pragma unroll
        for (int c = 0; c < MR; ++c)
          if (c < m[u]) q[id[u][c]] = v;
      } else {
        for (int c = 0; c < m[u]; ++c) v += q[__ldg(P.restIds + s0[u] + c)];
        for (int c = 0; c < m[u]; ++c) q[__ldg(P.restIds + s0[u] + c)] = v;
      }
    }
  }
  for (long long t = t0; t < nmask; t += UP * stride) {
    int id[UP];
#pragma unroll
    for (int u = 0; u < UP; ++u) {
      const long long k = t + u * stride;
      id[u] = k < nmask ? __ldg(P.mask + k) : -1;
    }
#pragma unroll
    for (int u = 0; u < UP; ++u)
      if (id[u] >= 0) q[id[u]] = T(0);
  }
}
template <typename T> void launch_gs_mask(const GsPlan &P, T *q, bool mask, cudaStream_t s)
{
  const long long nm = mask ? P.nmask : 0, n = P.npairs + P.nrest + nm;
  if (n <= 0) return;
  gs_mask_kernel<T><<<vec_grid(n), kThreads, 0, s>>>(P, nm, q);
  NRSG_CHECK_LAUNCH();
}
template void launch_gs_mask<double>(const GsPlan &, double *, bool, cudaStream_t);

__global__ void accumulate_kernel(long long n, int m, const double *__restrict__ alpha, const double *__restrict__ X,
                                  double *__restrict__ y)
{
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double v = dmul(alpha[0], X[i]);
    for (int k = 1; k < m; ++k) v = __fma_rn(alpha[k], X[(size_t)k * n + i], v);
    y[i] = v;
  }
}
void launch_accumulate(long long n, int m, const double *alpha, const double *X, double *y, cudaStream_t s)
{
  if (n <= 0 || m <= 0) return;
  accumulate_kernel<<<vec_grid(n), kThreads, 0, s>>>(n, m, alpha, X, y);
  NRSG_CHECK_LAUNCH();
}
__global__ void multi_scaled_sub_kernel(long long n, int m, const double *__restrict__ alpha, double *__restrict__ X)
{
  double *xm = X + (size_t)(m - 1) * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double v = xm[i];
    for (int k = 0; k < m - 1; ++k) v = __fma_rn(-alpha[k], X[(size_t)k * n + i], v);
    xm[i] = v;
  }
}
void launch_multi_scaled_sub(long long n, int m, const double *alpha, double *X, cudaStream_t s)
{
  if (n <= 0 || m <= 1) return;
  multi_scaled_sub_kernel<<<vec_grid(n), kThreads, 0, s>>>(n, m, alpha, X);
  NRSG_CHECK_LAUNCH();
}
// q -= (T)(sum / denom) with the sum already reduced on the device (ellipticZeroMean; the
// projection of a singular coarse right-hand side)
template <typename T>
__global__ void sub_mean_kernel(long long n, const double *__restrict__ sum, double denom, T *__restrict__ q)
{
  const T mean = (T)(sum[0] / denom);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    q[i] -= mean;
}
template <typename T> void launch_sub_mean(long long n, const double *sum, double denom, T *q, cudaStream_t s)
{
  if (n <= 0) return;
  sub_mean_kernel<T><<<vec_grid(n), kThreads, 0, s>>>(n, sum, denom, q);
  NRSG_CHECK_LAUNCH();
}
template void launch_sub_mean<double>(long long, const double *, double, double *, cudaStream_t);
template void launch_sub_mean<float>(long long, const double *, double, float *, cudaStream_t);
__global__ void scale_inplace_kernel(long long n, double a, double *x)
{
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    x[i] *= a;
}
void launch_scale_inplace(long long n, double a, double *x, cudaStream_t s)
{
  if (n <= 0) return;
  scale_inplace_kernel<<<vec_grid(n), kThreads, 0, s>>>(n, a, x);
  NRSG_CHECK_LAUNCH();
}
template void launch_gs_mask<float>(const GsPlan &, float *, bool, cudaStream_t);

// q[i] = a hash of (seed, i) mapped to [-1, 1) (a reproducible test vector)
__global__ void hash_fill_kernel(long long n, unsigned long long seed, float *q)
{
  NRSG_GRID_LOOP_VEC(i, n)
  {
    unsigned long long h = (unsigned long long)i * 0x9E3779B97F4A7C15ull + seed;
    h ^= h >> 31;
    h *= 0xBF58476D1CE4E5B9ull;
    h ^= h >> 29;
    q[i] = (float)((double)(h >> 11) * (1.0 / 4503599627370496.0) - 1.0);
  }
}
void launch_hash_fill(long long n, unsigned long long seed, float *q, cudaStream_t s)
{
  if (n <= 0) return;
  hash_fill_kernel<<<vec_grid(n), kThreads, 0, s>>>(n, seed, q);
  NRSG_CHECK_LAUNCH();
}
// counter += number of i with a[i], b[i] of different bits
__global__ void count_mismatch_kernel(long long n, const float *__restrict__ a, const float *__restrict__ b,
                                      unsigned *counter)
{
  unsigned c = 0;
  NRSG_GRID_LOOP_VEC(i, n) c += (__float_as_uint(a[i]) != __float_as_uint(b[i])) ? 1u : 0u;
  if (c) atomicAdd(counter, c);
}
void launch_count_mismatch(long long n, const float *a, const float *b, unsigned *counter, cudaStream_t s)
{
  if (n <= 0) return;
  count_mismatch_kernel<<<vec_grid(n), kThreads, 0, s>>>(n, a, b, counter);
  NRSG_CHECK_LAUNCH();
}

template <typename T> __global__ void mask_kernel(long long n, const int *__restrict__ ids, T *__restrict__ q)
{
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < n; m += (long long)gridDim.x * blockDim.x)
    q[ids[m]] = T(0);
}
template <typename T> void launch_mask(long long n, const int *ids, T *q, cudaStream_t s)
{
  if (n <= 0) return;
  mask_kernel<T><<<vec_grid(n), kThreads, 0, s>>>(n, ids, q);
  NRSG_CHECK_LAUNCH();
}
template void launch_mask<double>(long long, const int *, double *, cudaStream_t);
template void launch_mask<float>(long long, const int *, float *, cudaStream_t);

// ---------------------------------------------------------------------------
// weighted inner product
// ---------------------------------------------------------------------------
// Launch geometry of a reduction over n entries and the Reduce row of `slot`.
#define NRSG_RED_ARGS(n, red, slot)                                                                         \
  const RedSplit sp_ = red_split(n);                                                                      \
  double *row_ = red.row(slot);                                                                          \
  unsigned *cnt_ = red.counters + (slot)

template <typename T>
__global__ void __launch_bounds__(kThreads)
    wdot_kernel(long long n, long long len, int W, const T *__restrict__ w, const T *__restrict__ a,
                const T *__restrict__ b, double *row, unsigned *counter, double *out)
{
  reduce1(
      n, len, W,
      [&](long long i, double &x, double &y) {
        const double av = (double)a[i];
        y = b ? (double)b[i] : av;
        x = w ? dmul((double)w[i], av) : av;
      },
      row, counter, out);
}
template <typename T>
void launch_wdot(long long n, const T *w, const T *a, const T *b, double *out, Reduce &red, int slot, cudaStream_t s)
{
  NRSG_RED_ARGS(n, red, slot);
  wdot_kernel<T><<<sp_.ctas, kThreads, 0, s>>>(n, sp_.len, sp_.warps, w, a, b, row_, cnt_, out);
  NRSG_CHECK_LAUNCH();
}
template void launch_wdot<double>(long long, const double *, const double *, const double *, double *, Reduce &, int,
                                  cudaStream_t);
template void launch_wdot<float>(long long, const float *, const float *, const float *, double *, Reduce &, int,
                                 cudaStream_t);

// ---------------------------------------------------------------------------
// BLAS-1
// ---------------------------------------------------------------------------
#define NRSG_GRID_LOOP(i, n)                                                                               \
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (n); i += (long long)gridDim.x * blockDim.x)

template <typename T> __global__ void fill_kernel(long long n, T v, T *x) { NRSG_GRID_LOOP(i, n) x[i] = v; }
template <typename T> __global__ void axpby_kernel(long long n, T a, const T *__restrict__ x, T b, T *__restrict__ y)
{
  NRSG_GRID_LOOP(i, n) y[i] = a * x[i] + b * y[i];
}
// FP64: y = fma(a, x, b*y)
template <> __global__ void axpby_kernel<double>(long long n, double a, const double *__restrict__ x, double b,
                                                 double *__restrict__ y)
{
  NRSG_GRID_LOOP(i, n) y[i] = __fma_rn(a, x[i], dmul(b, y[i]));
}
// FP32: y = fma(a, x, b*y), the same explicit rounding
template <> __global__ void axpby_kernel<float>(long long n, float a, const float *__restrict__ x, float b,
                                                float *__restrict__ y)
{
  NRSG_GRID_LOOP(i, n) y[i] = __fmaf_rn(a, x[i], __fmul_rn(b, y[i]));
}
template <typename T> __global__ void axmy_kernel(long long n, const T *__restrict__ w, T *__restrict__ x)
{
  NRSG_GRID_LOOP(i, n) x[i] = w[i] * x[i];
}
template <typename T> __global__ void axmyz_kernel(long long n, const T *__restrict__ a, const T *__restrict__ b, T *z)
{
  NRSG_GRID_LOOP(i, n) z[i] = a[i] * b[i];
}
template <typename T> __global__ void recip_kernel(long long n, T *x) { NRSG_GRID_LOOP(i, n) x[i] = T(1) / x[i]; }
template <typename Ti, typename To> __global__ void cast_kernel(long long n, const Ti *__restrict__ x, To *__restrict__ y)
{
  NRSG_GRID_LOOP(i, n) y[i] = (To)x[i];
}

template <typename T> void launch_fill(long long n, T v, T *x, cudaStream_t s)
{
  if (n <= 0) return;
  fill_kernel<T><<<vec_grid(n), kThreads, 0, s>>>(n, v, x);
  NRSG_CHECK_LAUNCH();
}
template <typename T> void launch_axpby(long long n, T a, const T *x, T b, T *y, cudaStream_t s)
{
  if (n <= 0) return;
  axpby_kernel<T><<<vec_grid(n), kThreads, 0, s>>>(n, a, x, b, y);
  NRSG_CHECK_LAUNCH();
}
template <typename T> void launch_axmy(long long n, const T *w, T *x, cudaStream_t s)
{
  if (n <= 0) return;
  axmy_kernel<T><<<vec_grid(n), kThreads, 0, s>>>(n, w, x);
  NRSG_CHECK_LAUNCH();
}
template <typename T> void launch_axmyz(long long n, const T *a, const T *b, T *z, cudaStream_t s)
{
  if (n <= 0) return;
  axmyz_kernel<T><<<vec_grid(n), kThreads, 0, s>>>(n, a, b, z);
  NRSG_CHECK_LAUNCH();
}
template <typename T> void launch_recip(long long n, T *x, cudaStream_t s)
{
  if (n <= 0) return;
  recip_kernel<T><<<vec_grid(n), kThreads, 0, s>>>(n, x);
  NRSG_CHECK_LAUNCH();
}
template <typename Ti, typename To> void launch_copy_cast(long long n, const Ti *x, To *y, cudaStream_t s)
{
  if (n <= 0) return;
  cast_kernel<Ti, To><<<vec_grid(n), kThreads, 0, s>>>(n, x, y);
  NRSG_CHECK_LAUNCH();
}
#define NRSG_INST_BLAS(T)                                                                                  \
  template void launch_fill<T>(long long, T, T *, cudaStream_t);                                           \
  template void launch_axpby<T>(long long, T, const T *, T, T *, cudaStream_t);                            \
  template void launch_axmy<T>(long long, const T *, T *, cudaStream_t);                                   \
  template void launch_axmyz<T>(long long, const T *, const T *, T *, cudaStream_t);                       \
  template void launch_recip<T>(long long, T *, cudaStream_t);
NRSG_INST_BLAS(double)
NRSG_INST_BLAS(float)
template void launch_copy_cast<double, float>(long long, const double *, float *, cudaStream_t);
template void launch_copy_cast<float, double>(long long, const float *, double *, cudaStream_t);
template void launch_copy_cast<double, double>(long long, const double *, double *, cudaStream_t);
template void launch_copy_cast<float, float>(long long, const float *, float *, cudaStream_t);

// ---------------------------------------------------------------------------
// PCG kernels with device-resident scalars
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads)
    jacobi_rdotz_kernel(long long n, long long len, int W, const double *__restrict__ w,
                        const double *__restrict__ invDiag, const double *__restrict__ r, double *__restrict__ z,
                        PcgScalars *sc, double *row, unsigned *counter)
{
  __shared__ double s_old;
  if (threadIdx.x == 0) s_old = sc->rdotz;
  // every block reads rdotz before the last block overwrites it: the last
  // block only finishes after all tickets are taken, i.e. after every block
  // passed this point.
  __syncthreads();
  const bool last = reduce1(
      n, len, W,
      [&](long long i, double &x, double &y) {
        const double ri = r[i];
        const double zi = dmul(ri, invDiag[i]);
        z[i] = zi;
        x = dmul(w[i], ri);
        y = zi;
      },
      row, counter, &sc->rdotz);
  if (last) sc->rdotz_old = s_old;
}
void launch_jacobi_rdotz(long long n, const double *w, const double *invDiag, const double *r, double *z,
                         PcgScalars *sc, Reduce &red, int slot, cudaStream_t s)
{
  NRSG_RED_ARGS(n, red, slot);
  jacobi_rdotz_kernel<<<sp_.ctas, kThreads, 0, s>>>(n, sp_.len, sp_.warps, w, invDiag, r, z, sc, row_, cnt_);
  NRSG_CHECK_LAUNCH();
}

// p = z + beta p as fma(beta, p, z)
__global__ void update_p_kernel(long long n, const double *__restrict__ z, double *__restrict__ p, const PcgScalars *sc,
                                bool first, bool flexible)
{
  double beta = 0;
  if (!first) beta = flexible ? -sc->alpha * sc->zAp / sc->rdotz_old : sc->rdotz / sc->rdotz_old;
  NRSG_GRID_LOOP(i, n) p[i] = __fma_rn(beta, p[i], z[i]);
}
void launch_update_p(long long n, const double *z, double *p, const PcgScalars *sc, bool first, bool flexible,
                     cudaStream_t s)
{
  update_p_kernel<<<vec_grid(n), kThreads, 0, s>>>(n, z, p, sc, first, flexible);
  NRSG_CHECK_LAUNCH();
}

// r = fma(-alpha, Ap, r), x = fma(alpha, p, x), term w (r r)
__global__ void __launch_bounds__(kThreads)
    update_xr_kernel(long long n, long long len, int W, const double *__restrict__ w, const double *__restrict__ p,
                     const double *__restrict__ Ap, double *__restrict__ x, double *__restrict__ r, PcgScalars *sc,
                     double *row, unsigned *counter)
{
  const double alpha = sc->rdotz / (sc->pAp + 1e-300);
  const bool last = reduce1(
      n, len, W,
      [&](long long i, double &fx, double &fy) {
        const double ri = __fma_rn(-alpha, Ap[i], r[i]);
        r[i] = ri;
        x[i] = __fma_rn(alpha, p[i], x[i]);
        fx = dmul(w[i], ri);
        fy = ri;
      },
      row, counter, &sc->rdotr);
  if (last) sc->alpha = alpha;
}
void launch_update_xr(long long n, const double *w, const double *p, const double *Ap, double *x, double *r,
                      PcgScalars *sc, Reduce &red, int slot, cudaStream_t s)
{
  NRSG_RED_ARGS(n, red, slot);
  update_xr_kernel<<<sp_.ctas, kThreads, 0, s>>>(n, sp_.len, sp_.warps, w, p, Ap, x, r, sc, row_, cnt_);
  NRSG_CHECK_LAUNCH();
}

__global__ void __launch_bounds__(kThreads)
    update_pcg_alpha_kernel(long long n, long long len, int W, const double *__restrict__ w,
                            const double *__restrict__ p, const double *__restrict__ Ap, double alpha,
                            double *__restrict__ x, double *__restrict__ r, double *row, unsigned *counter,
                            double *out)
{
  reduce1(
      n, len, W,
      [&](long long i, double &fx, double &fy) {
        const double ri = __fma_rn(-alpha, Ap[i], r[i]);
        r[i] = ri;
        x[i] = __fma_rn(alpha, p[i], x[i]);
        fx = dmul(w[i], ri);
        fy = ri;
      },
      row, counter, out);
}
void launch_update_pcg_alpha(long long n, const double *w, const double *p, const double *Ap, double alpha, double *x,
                             double *r, double *rdotr, Reduce &red, int slot, cudaStream_t s)
{
  NRSG_RED_ARGS(n, red, slot);
  update_pcg_alpha_kernel<<<sp_.ctas, kThreads, 0, s>>>(n, sp_.len, sp_.warps, w, p, Ap, alpha, x, r, row_, cnt_,
                                                        rdotr);
  NRSG_CHECK_LAUNCH();
}

__global__ void scalar_move_kernel(double *dst, const double *src, double *save_old)
{
  if (save_old) *save_old = *dst;
  *dst = *src;
}
void launch_scalar_move(double *dst, const double *src, double *save_old, cudaStream_t s)
{
  scalar_move_kernel<<<1, 1, 0, s>>>(dst, src, save_old);
  NRSG_CHECK_LAUNCH();
}

} // namespace nrsg

// ===========================================================================
// (F)GMRES kernels: weighted multi-dot (weightedInnerProdMulti.okl), fused
// Gram-Schmidt + norm (gramSchmidtOrthogonalization.okl), solution update
// (updatePGMRESSolution.okl) and fused residual + norm
// (fusedResidualAndNorm.okl).  V is stored as nvec contiguous E-vectors.
// ===========================================================================
#include "elliptic.hpp"

namespace nrsg {
namespace {
constexpr int kMultiVec = 8;
}

// One pass over x and w for up to kMultiVec vectors: entry factors (w x, V_k),
// w x rounded once and shared by the vectors; every vector's sum follows the
// one-vector order exactly.
__global__ void __launch_bounds__(kThreads)
    multi_wdot_kernel(long long n, long long len, int W, const double *__restrict__ w, const double *__restrict__ V,
                      int nvec, const double *__restrict__ x, double *rows, long long stride, unsigned *counter,
                      double *out)
{
  __shared__ double s_stk[kWarps][kMultiVec][kStack];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long wid = (long long)blockIdx.x * kWarps + warp;
  if (wid < W) {
    int sp = 0;
    for (long long q = 0; q < len; ++q) {
      const long long c = wid * len + q;
      const long long i0 = c * kChunk + lane;
      double v[kMultiVec];
#pragma unroll
      for (int k = 0; k < kMultiVec; ++k) v[k] = 0.0;
      for (int j = 0; j < 32; ++j) {
        const long long i = i0 + 32 * j;
        if (i < n) {
          const double wx = dmul(w[i], x[i]);
#pragma unroll
          for (int k = 0; k < kMultiVec; ++k)
            if (k < nvec) v[k] = __fma_rn(wx, V[(size_t)k * n + i], v[k]);
        }
      }
#pragma unroll
      for (int k = 0; k < kMultiVec; ++k) {
        if (k >= nvec) break;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] = dadd(v[k], __shfl_down_sync(0xffffffffu, v[k], o));
      }
      for (long long kk = q + 1; (kk & 1) == 0; kk >>= 1) {
        --sp;
#pragma unroll
        for (int k = 0; k < kMultiVec; ++k)
          if (k < nvec) v[k] = dadd(s_stk[warp][k][sp], v[k]);
      }
      if (lane == 0) {
#pragma unroll
        for (int k = 0; k < kMultiVec; ++k)
          if (k < nvec) s_stk[warp][k][sp] = v[k];
      }
      ++sp;
      __syncwarp();
    }
    if (lane == 0) {
      for (int k = 0; k < nvec; ++k) rows[(size_t)k * stride + wid] = s_stk[warp][k][0];
      __threadfence();
    }
  }
  __shared__ bool s_last;
  __syncthreads();
  if (threadIdx.x == 0) s_last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  for (int k = 0; k < nvec; ++k) {
    const double r = final_tree(rows + (size_t)k * stride, W);
    if (threadIdx.x == 0) out[k] = r;
  }
  if (threadIdx.x == 0) *counter = 0;
}

void launch_multi_wdot(long long n, const double *w, const double *V, int nvec, const double *x, double *out,
                       Reduce &red, int slot, cudaStream_t s)
{
  // chunks of kMultiVec vectors; each chunk uses kMultiVec consecutive rows starting at `slot`
  if (slot + kMultiVec > red.slots) throw Error(NRSG_ERR_INVALID, "multi-dot needs 8 reduction rows");
  const RedSplit sp = red_split(n);
  for (int k0 = 0; k0 < nvec; k0 += kMultiVec) {
    const int m = (nvec - k0) < kMultiVec ? (nvec - k0) : kMultiVec;
    multi_wdot_kernel<<<sp.ctas, kThreads, 0, s>>>(n, sp.len, sp.warps, w, V + (size_t)k0 * n, m, x, red.row(slot),
                                                  red.stride, red.counters + slot, out + k0);
    NRSG_CHECK_LAUNCH();
  }
}

// x -= sum_k y_k V_k (fma in k order), nrm2 = (x, x)_w
__global__ void __launch_bounds__(kThreads)
    gram_schmidt_kernel(long long n, long long len, int W, const double *__restrict__ w,
                        const double *__restrict__ V, int nvec, const double *__restrict__ y, double *__restrict__ x,
                        double *row, unsigned *counter, double *nrm2)
{
  __shared__ double s_y[64];
  for (int k = threadIdx.x; k < nvec; k += kThreads) s_y[k] = y[k];
  __syncthreads();
  reduce1(
      n, len, W,
      [&](long long i, double &fx, double &fy) {
        double v = x[i];
        for (int k = 0; k < nvec; ++k) v = __fma_rn(-s_y[k], V[(size_t)k * n + i], v);
        x[i] = v;
        fx = dmul(w[i], v);
        fy = v;
      },
      row, counter, nrm2);
}
void launch_gram_schmidt(long long n, const double *w, const double *V, int nvec, const double *y, double *x,
                         double *nrm2, Reduce &red, int slot, cudaStream_t s)
{
  if (nvec > 64) throw Error(NRSG_ERR_BAD_CONFIG, "GMRES restart length above 64");
  NRSG_RED_ARGS(n, red, slot);
  gram_schmidt_kernel<<<sp_.ctas, kThreads, 0, s>>>(n, sp_.len, sp_.warps, w, V, nvec, y, x, row_, cnt_, nrm2);
  NRSG_CHECK_LAUNCH();
}

// x += sum_k y_k V_k (fma in k order)
__global__ void gmres_update_kernel(long long n, const double *__restrict__ V, int nvec, const double *__restrict__ y,
                                    double *__restrict__ x)
{
  __shared__ double s_y[64];
  for (int k = threadIdx.x; k < nvec; k += blockDim.x) s_y[k] = y[k];
  __syncthreads();
  NRSG_GRID_LOOP(i, n)
  {
    double v = x[i];
    for (int k = 0; k < nvec; ++k) v = __fma_rn(s_y[k], V[(size_t)k * n + i], v);
    x[i] = v;
  }
}
void launch_gmres_update(long long n, const double *V, int nvec, const double *y, double *x, cudaStream_t s)
{
  gmres_update_kernel<<<vec_grid(n), kThreads, 0, s>>>(n, V, nvec, y, x);
  NRSG_CHECK_LAUNCH();
}

// r = b - Ax, nrm2 = (r, r)_w
__global__ void __launch_bounds__(kThreads)
    residual_norm_kernel(long long n, long long len, int W, const double *__restrict__ w,
                         const double *__restrict__ b, const double *__restrict__ Ax, double *__restrict__ r,
                         double *row, unsigned *counter, double *nrm2)
{
  reduce1(
      n, len, W,
      [&](long long i, double &fx, double &fy) {
        const double v = dadd(b[i], -Ax[i]);
        r[i] = v;
        fx = dmul(w[i], v);
        fy = v;
      },
      row, counter, nrm2);
}
void launch_residual_norm(long long n, const double *w, const double *b, const double *Ax, double *r, double *nrm2,
                          Reduce &red, int slot, cudaStream_t s)
{
  NRSG_RED_ARGS(n, red, slot);
  residual_norm_kernel<<<sp_.ctas, kThreads, 0, s>>>(n, sp_.len, sp_.warps, w, b, Ax, r, row_, cnt_, nrm2);
  NRSG_CHECK_LAUNCH();
}

template <typename T> __global__ void scale_copy_kernel(long long n, T a, const T *__restrict__ x, T *__restrict__ y)
{
  NRSG_GRID_LOOP(i, n) y[i] = a * x[i];
}
template <typename T> void launch_scale_copy(long long n, T a, const T *x, T *y, cudaStream_t s)
{
  if (n <= 0) return;
  scale_copy_kernel<T><<<vec_grid(n), kThreads, 0, s>>>(n, a, x, y);
  NRSG_CHECK_LAUNCH();
}
template void launch_scale_copy<double>(long long, double, const double *, double *, cudaStream_t);
template void launch_scale_copy<float>(long long, float, const float *, float *, cudaStream_t);

} // namespace nrsg

// ===========================================================================
// Jacobi-PCG kernels in precision T with double scalars (coarse-level solve)
// ===========================================================================
#include "mg_kernels.hpp"

namespace nrsg {

template <typename T>
__global__ void __launch_bounds__(kThreads)
    pcgT_rdotz_kernel(long long n, long long len, int W, const T *__restrict__ w, const T *__restrict__ invDiag,
                      const T *__restrict__ r, T *__restrict__ z, PcgScalars *sc, double *row, unsigned *counter)
{
  __shared__ double s_old;
  if (threadIdx.x == 0) s_old = sc->rdotz;
  __syncthreads();
  const bool last = reduce1(
      n, len, W,
      [&](long long i, double &fx, double &fy) {
        const T ri = r[i];
        const T zi = invDiag[i] * ri;
        z[i] = zi;
        fx = dmul((double)w[i], (double)ri);
        fy = (double)zi;
      },
      row, counter, &sc->rdotz);
  if (last) sc->rdotz_old = s_old;
}
template <typename T>
__global__ void pcgT_p_kernel(long long n, const T *__restrict__ z, T *__restrict__ p, const PcgScalars *sc, bool first)
{
  const T beta = first ? T(0) : (T)(sc->rdotz / sc->rdotz_old);
  NRSG_GRID_LOOP(i, n) p[i] = z[i] + beta * p[i];
}
template <typename T>
__global__ void __launch_bounds__(kThreads)
    pcgT_xr_kernel(long long n, long long len, int W, const T *__restrict__ w, const T *__restrict__ p,
                   const T *__restrict__ Ap, T *__restrict__ x, T *__restrict__ r, PcgScalars *sc, double *row,
                   unsigned *counter)
{
  const T alpha = (T)(sc->rdotz / (sc->pAp + 1e-300));
  reduce1(
      n, len, W,
      [&](long long i, double &fx, double &fy) {
        x[i] += alpha * p[i];
        const T ri = r[i] - alpha * Ap[i];
        r[i] = ri;
        fx = dmul((double)w[i], (double)ri);
        fy = (double)ri;
      },
      row, counter, &sc->rdotr);
}

template <typename T>
void launch_pcg_rdotz(long long n, const T *w, const T *invDiag, const T *r, T *z, PcgScalars *sc, Reduce &red, int slot,
                      cudaStream_t s)
{
  NRSG_RED_ARGS(n, red, slot);
  pcgT_rdotz_kernel<T><<<sp_.ctas, kThreads, 0, s>>>(n, sp_.len, sp_.warps, w, invDiag, r, z, sc, row_, cnt_);
  NRSG_CHECK_LAUNCH();
}
template <typename T> void launch_pcg_p(long long n, const T *z, T *p, const PcgScalars *sc, bool first, cudaStream_t s)
{
  pcgT_p_kernel<T><<<vec_grid(n), kThreads, 0, s>>>(n, z, p, sc, first);
  NRSG_CHECK_LAUNCH();
}
template <typename T>
void launch_pcg_xr(long long n, const T *w, const T *p, const T *Ap, T *x, T *r, PcgScalars *sc, Reduce &red, int slot,
                   cudaStream_t s)
{
  NRSG_RED_ARGS(n, red, slot);
  pcgT_xr_kernel<T><<<sp_.ctas, kThreads, 0, s>>>(n, sp_.len, sp_.warps, w, p, Ap, x, r, sc, row_, cnt_);
  NRSG_CHECK_LAUNCH();
}
#define NRSG_INST_PCGT(T)                                                                                  \
  template void launch_pcg_rdotz<T>(long long, const T *, const T *, const T *, T *, PcgScalars *, Reduce &, int, \
                                    cudaStream_t);                                                         \
  template void launch_pcg_p<T>(long long, const T *, T *, const PcgScalars *, bool, cudaStream_t);        \
  template void launch_pcg_xr<T>(long long, const T *, const T *, const T *, T *, T *, PcgScalars *, Reduce &, int, \
                                 cudaStream_t);
NRSG_INST_PCGT(double)
NRSG_INST_PCGT(float)

} // namespace nrsg
