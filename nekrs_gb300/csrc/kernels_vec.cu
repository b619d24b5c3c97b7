// Gather-scatter, mask, BLAS-1 and fused Krylov vector kernels (sm_103a).
//
// Reference kernels (nekRS tree):
//   gatherScatterMany_*Add   3rd_party/gslib/ogs/okl/gatherScatterMany.okl
//   mask                     kernels/core/mask.okl:27-35
//   weightedInnerProdMany    kernels/linAlg/weightedInnerProdMany.okl:27-105
//   ellipticBlockUpdatePCG   kernels/elliptic/ellipticBlockUpdatePCG.okl:26-111
//   axpbyMany, axmyzMany, adyMany, fill, copyDfloatToPfloat (kernels/linAlg, kernels/core)
//
// Reductions are one launch each: every CTA writes its partial sum, the last
// CTA to finish (atomic ticket) adds the partials in index order and stores
// the result on the device.  The partial layout and the order of every sum
// are fixed, so results are bit-reproducible run to run.  There is no host
// round trip: Krylov scalars (alpha, beta) are formed on the device by the
// kernels that consume them.

#include "nrsg_internal.hpp"

namespace nrsg {

namespace {
constexpr int kThreads = kRedThreads;

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Block sum (fixed order), result valid in thread 0.
__device__ __forceinline__ double block_sum(double v)
{
  __shared__ double s_w[kThreads / 32];
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) s_w[wid] = v;
  __syncthreads();
  double r = 0;
  if (wid == 0) {
    r = (lane < kThreads / 32) ? s_w[lane] : 0.0;
    r = warp_sum(r);
  }
  __syncthreads();
  return r;
}

// Write this block's partial; the last block reduces all partials into *out.
// Returns true in the thread that stored *out.
__device__ __forceinline__ bool finish_reduction(double partial, double *partials, unsigned *counter, double *out)
{
  __shared__ bool s_last;
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = partial;
    __threadfence();
    const unsigned ticket = atomicAdd(counter, 1u);
    s_last = (ticket == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  double v = 0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += kThreads) v += ((volatile double *)partials)[b];
  v = block_sum(v);
  if (threadIdx.x == 0) {
    *out = v;
    *counter = 0; // ready for the next launch on this slot
  }
  return threadIdx.x == 0;
}

inline unsigned red_grid(long long n)
{
  long long b = (n + kThreads - 1) / kThreads;
  if (b < 1) b = 1;
  return (unsigned)(b < kRedBlocks ? b : kRedBlocks);
}
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
// mask, in one launch; each group sums its members in member order
template <typename T> __global__ void gs_mask_kernel(GsPlan P, long long nmask, T *__restrict__ q)
{
  const long long n1 = P.npairs, n2 = n1 + P.nrest, n3 = n2 + nmask;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n3; t += (long long)gridDim.x * blockDim.x) {
    if (t < n1) {
      const int2 pr = __ldg(P.pairs + t);
      const T v = q[pr.x] + q[pr.y];
      q[pr.x] = v;
      q[pr.y] = v;
    } else if (t < n2) {
      const long long g = t - n1;
      const int s = __ldg(P.restOff + g), e = __ldg(P.restOff + g + 1);
      T v = 0;
      for (int m = s; m < e; ++m) v += q[__ldg(P.restIds + m)];
      for (int m = s; m < e; ++m) q[__ldg(P.restIds + m)] = v;
    } else {
      q[__ldg(P.mask + (t - n2))] = T(0);
    }
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
    double v = alpha[0] * X[i];
    for (int k = 1; k < m; ++k) v += alpha[k] * X[(size_t)k * n + i];
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
    for (int k = 0; k < m - 1; ++k) v = -alpha[k] * X[(size_t)k * n + i] + v;
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
template <typename T>
__global__ void wdot_kernel(long long n, const T *__restrict__ w, const T *__restrict__ a, const T *__restrict__ b,
                            double *partials, unsigned *counter, double *out)
{
  double acc = 0;
  for (long long i = blockIdx.x * (long long)kThreads + threadIdx.x; i < n; i += (long long)gridDim.x * kThreads) {
    const double av = (double)a[i];
    const double bv = b ? (double)b[i] : av;
    const double wv = w ? (double)w[i] : 1.0;
    acc += wv * av * bv;
  }
  finish_reduction(block_sum(acc), partials, counter, out);
}
template <typename T>
void launch_wdot(long long n, const T *w, const T *a, const T *b, double *out, Reduce &red, int slot, cudaStream_t s)
{
  wdot_kernel<T><<<red_grid(n), kThreads, 0, s>>>(n, w, a, b, red.partials + (size_t)slot * kRedBlocks,
                                                   red.counters + slot, out);
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
__global__ void jacobi_rdotz_kernel(long long n, const double *__restrict__ w, const double *__restrict__ invDiag,
                                    const double *__restrict__ r, double *__restrict__ z, PcgScalars *sc,
                                    double *partials, unsigned *counter)
{
  double acc = 0;
  for (long long i = blockIdx.x * (long long)kThreads + threadIdx.x; i < n; i += (long long)gridDim.x * kThreads) {
    const double ri = r[i];
    const double zi = ri * invDiag[i];
    z[i] = zi;
    acc += w[i] * ri * zi;
  }
  __shared__ double s_old;
  if (threadIdx.x == 0) s_old = sc->rdotz;
  // every block reads rdotz before the last block overwrites it: the last
  // block only finishes after all tickets are taken, i.e. after every block
  // passed this point.
  __syncthreads();
  if (finish_reduction(block_sum(acc), partials, counter, &sc->rdotz)) sc->rdotz_old = s_old;
}
void launch_jacobi_rdotz(long long n, const double *w, const double *invDiag, const double *r, double *z,
                         PcgScalars *sc, Reduce &red, int slot, cudaStream_t s)
{
  jacobi_rdotz_kernel<<<red_grid(n), kThreads, 0, s>>>(n, w, invDiag, r, z, sc, red.partials + (size_t)slot * kRedBlocks,
                                                       red.counters + slot);
  NRSG_CHECK_LAUNCH();
}

__global__ void update_p_kernel(long long n, const double *__restrict__ z, double *__restrict__ p, const PcgScalars *sc,
                                bool first, bool flexible)
{
  double beta = 0;
  if (!first) beta = flexible ? -sc->alpha * sc->zAp / sc->rdotz_old : sc->rdotz / sc->rdotz_old;
  NRSG_GRID_LOOP(i, n) p[i] = z[i] + beta * p[i];
}
void launch_update_p(long long n, const double *z, double *p, const PcgScalars *sc, bool first, bool flexible,
                     cudaStream_t s)
{
  update_p_kernel<<<vec_grid(n), kThreads, 0, s>>>(n, z, p, sc, first, flexible);
  NRSG_CHECK_LAUNCH();
}

__global__ void update_xr_kernel(long long n, const double *__restrict__ w, const double *__restrict__ p,
                                 const double *__restrict__ Ap, double *__restrict__ x, double *__restrict__ r,
                                 PcgScalars *sc, double *partials, unsigned *counter)
{
  const double alpha = sc->rdotz / (sc->pAp + 1e-300);
  double acc = 0;
  for (long long i = blockIdx.x * (long long)kThreads + threadIdx.x; i < n; i += (long long)gridDim.x * kThreads) {
    double ri = r[i];
    ri -= alpha * Ap[i];
    r[i] = ri;
    acc += ri * ri * w[i];
    x[i] += alpha * p[i];
  }
  if (finish_reduction(block_sum(acc), partials, counter, &sc->rdotr)) sc->alpha = alpha;
}
void launch_update_xr(long long n, const double *w, const double *p, const double *Ap, double *x, double *r,
                      PcgScalars *sc, Reduce &red, int slot, cudaStream_t s)
{
  update_xr_kernel<<<red_grid(n), kThreads, 0, s>>>(n, w, p, Ap, x, r, sc, red.partials + (size_t)slot * kRedBlocks,
                                                    red.counters + slot);
  NRSG_CHECK_LAUNCH();
}

__global__ void update_pcg_alpha_kernel(long long n, const double *__restrict__ w, const double *__restrict__ p,
                                        const double *__restrict__ Ap, double alpha, double *__restrict__ x,
                                        double *__restrict__ r, double *partials, unsigned *counter, double *out)
{
  double acc = 0;
  for (long long i = blockIdx.x * (long long)kThreads + threadIdx.x; i < n; i += (long long)gridDim.x * kThreads) {
    double ri = r[i];
    ri -= alpha * Ap[i];
    r[i] = ri;
    acc += ri * ri * w[i];
    x[i] += alpha * p[i];
  }
  finish_reduction(block_sum(acc), partials, counter, out);
}
void launch_update_pcg_alpha(long long n, const double *w, const double *p, const double *Ap, double alpha, double *x,
                             double *r, double *rdotr, Reduce &red, int slot, cudaStream_t s)
{
  update_pcg_alpha_kernel<<<red_grid(n), kThreads, 0, s>>>(n, w, p, Ap, alpha, x, r,
                                                           red.partials + (size_t)slot * kRedBlocks,
                                                           red.counters + slot, rdotr);
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

__global__ void multi_wdot_kernel(long long n, const double *__restrict__ w, const double *__restrict__ V, int nvec,
                                  const double *__restrict__ x, double *partials, unsigned *counter, double *out)
{
  double acc[kMultiVec];
#pragma unroll
  for (int k = 0; k < kMultiVec; ++k) acc[k] = 0;
  for (long long i = blockIdx.x * (long long)kThreads + threadIdx.x; i < n; i += (long long)gridDim.x * kThreads) {
    const double wx = w[i] * x[i];
#pragma unroll
    for (int k = 0; k < kMultiVec; ++k)
      if (k < nvec) acc[k] += wx * V[(size_t)k * n + i];
  }
  __shared__ bool s_last;
#pragma unroll
  for (int k = 0; k < kMultiVec; ++k) {
    if (k >= nvec) break;
    const double v = block_sum(acc[k]);
    if (threadIdx.x == 0) partials[(size_t)k * kRedBlocks + blockIdx.x] = v;
  }
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  for (int k = 0; k < nvec; ++k) {
    double v = 0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += kThreads) v += ((volatile double *)partials)[(size_t)k * kRedBlocks + b];
    v = block_sum(v);
    if (threadIdx.x == 0) out[k] = v;
  }
  if (threadIdx.x == 0) *counter = 0;
}

void launch_multi_wdot(long long n, const double *w, const double *V, int nvec, const double *x, double *out,
                       Reduce &red, int slot, cudaStream_t s)
{
  // chunks of kMultiVec vectors; each chunk uses kMultiVec consecutive partial rows of `slot`
  for (int k0 = 0; k0 < nvec; k0 += kMultiVec) {
    const int m = (nvec - k0) < kMultiVec ? (nvec - k0) : kMultiVec;
    multi_wdot_kernel<<<red_grid(n), kThreads, 0, s>>>(n, w, V + (size_t)k0 * n, m, x,
                                                      red.partials + (size_t)slot * kRedBlocks, red.counters + slot,
                                                      out + k0);
    NRSG_CHECK_LAUNCH();
  }
}

__global__ void gram_schmidt_kernel(long long n, const double *__restrict__ w, const double *__restrict__ V, int nvec,
                                    const double *__restrict__ y, double *__restrict__ x, double *partials,
                                    unsigned *counter, double *nrm2)
{
  __shared__ double s_y[64];
  for (int k = threadIdx.x; k < nvec; k += kThreads) s_y[k] = y[k];
  __syncthreads();
  double acc = 0;
  for (long long i = blockIdx.x * (long long)kThreads + threadIdx.x; i < n; i += (long long)gridDim.x * kThreads) {
    double v = x[i];
    for (int k = 0; k < nvec; ++k) v -= s_y[k] * V[(size_t)k * n + i];
    x[i] = v;
    acc += w[i] * v * v;
  }
  finish_reduction(block_sum(acc), partials, counter, nrm2);
}
void launch_gram_schmidt(long long n, const double *w, const double *V, int nvec, const double *y, double *x,
                         double *nrm2, Reduce &red, int slot, cudaStream_t s)
{
  if (nvec > 64) throw Error(NRSG_ERR_BAD_CONFIG, "GMRES restart length above 64");
  gram_schmidt_kernel<<<red_grid(n), kThreads, 0, s>>>(n, w, V, nvec, y, x, red.partials + (size_t)slot * kRedBlocks,
                                                       red.counters + slot, nrm2);
  NRSG_CHECK_LAUNCH();
}

__global__ void gmres_update_kernel(long long n, const double *__restrict__ V, int nvec, const double *__restrict__ y,
                                    double *__restrict__ x)
{
  __shared__ double s_y[64];
  for (int k = threadIdx.x; k < nvec; k += blockDim.x) s_y[k] = y[k];
  __syncthreads();
  NRSG_GRID_LOOP(i, n)
  {
    double v = x[i];
    for (int k = 0; k < nvec; ++k) v += s_y[k] * V[(size_t)k * n + i];
    x[i] = v;
  }
}
void launch_gmres_update(long long n, const double *V, int nvec, const double *y, double *x, cudaStream_t s)
{
  gmres_update_kernel<<<vec_grid(n), kThreads, 0, s>>>(n, V, nvec, y, x);
  NRSG_CHECK_LAUNCH();
}

__global__ void residual_norm_kernel(long long n, const double *__restrict__ w, const double *__restrict__ b,
                                     const double *__restrict__ Ax, double *__restrict__ r, double *partials,
                                     unsigned *counter, double *nrm2)
{
  double acc = 0;
  for (long long i = blockIdx.x * (long long)kThreads + threadIdx.x; i < n; i += (long long)gridDim.x * kThreads) {
    const double v = b[i] - Ax[i];
    r[i] = v;
    acc += w[i] * v * v;
  }
  finish_reduction(block_sum(acc), partials, counter, nrm2);
}
void launch_residual_norm(long long n, const double *w, const double *b, const double *Ax, double *r, double *nrm2,
                          Reduce &red, int slot, cudaStream_t s)
{
  residual_norm_kernel<<<red_grid(n), kThreads, 0, s>>>(n, w, b, Ax, r, red.partials + (size_t)slot * kRedBlocks,
                                                        red.counters + slot, nrm2);
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
__global__ void pcgT_rdotz_kernel(long long n, const T *__restrict__ w, const T *__restrict__ invDiag,
                                  const T *__restrict__ r, T *__restrict__ z, PcgScalars *sc, double *partials,
                                  unsigned *counter)
{
  double acc = 0;
  for (long long i = blockIdx.x * (long long)kThreads + threadIdx.x; i < n; i += (long long)gridDim.x * kThreads) {
    const T ri = r[i];
    const T zi = invDiag[i] * ri;
    z[i] = zi;
    acc += (double)w[i] * (double)ri * (double)zi;
  }
  __shared__ double s_old;
  if (threadIdx.x == 0) s_old = sc->rdotz;
  __syncthreads();
  if (finish_reduction(block_sum(acc), partials, counter, &sc->rdotz)) sc->rdotz_old = s_old;
}
template <typename T>
__global__ void pcgT_p_kernel(long long n, const T *__restrict__ z, T *__restrict__ p, const PcgScalars *sc, bool first)
{
  const T beta = first ? T(0) : (T)(sc->rdotz / sc->rdotz_old);
  NRSG_GRID_LOOP(i, n) p[i] = z[i] + beta * p[i];
}
template <typename T>
__global__ void pcgT_xr_kernel(long long n, const T *__restrict__ w, const T *__restrict__ p, const T *__restrict__ Ap,
                               T *__restrict__ x, T *__restrict__ r, PcgScalars *sc, double *partials,
                               unsigned *counter)
{
  const T alpha = (T)(sc->rdotz / (sc->pAp + 1e-300));
  double acc = 0;
  for (long long i = blockIdx.x * (long long)kThreads + threadIdx.x; i < n; i += (long long)gridDim.x * kThreads) {
    x[i] += alpha * p[i];
    const T ri = r[i] - alpha * Ap[i];
    r[i] = ri;
    acc += (double)w[i] * (double)ri * (double)ri;
  }
  finish_reduction(block_sum(acc), partials, counter, &sc->rdotr);
}

template <typename T>
void launch_pcg_rdotz(long long n, const T *w, const T *invDiag, const T *r, T *z, PcgScalars *sc, Reduce &red, int slot,
                      cudaStream_t s)
{
  pcgT_rdotz_kernel<T><<<red_grid(n), kThreads, 0, s>>>(n, w, invDiag, r, z, sc, red.partials + (size_t)slot * kRedBlocks,
                                                        red.counters + slot);
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
  pcgT_xr_kernel<T><<<red_grid(n), kThreads, 0, s>>>(n, w, p, Ap, x, r, sc, red.partials + (size_t)slot * kRedBlocks,
                                                     red.counters + slot);
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
