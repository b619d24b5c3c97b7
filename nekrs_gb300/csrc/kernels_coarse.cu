// Coarse-level Jacobi-PCG as one persistent cooperative kernel (sm_103a).
//
// The coarsest pMG level (order 1 in the configurations here) is solved by
// Jacobi-preconditioned CG to a relative tolerance (1e-4 by default), the
// build's stand-in for the reference's AMG coarse solve (coarseLevel_t::solve,
// src/solvers/elliptic/MG/coarseLevel.cpp:182-222).  That solve takes on the
// order of a hundred iterations on a few hundred thousand nodes: launch- and
// latency-bound as separate kernels with a host convergence test per
// iteration.  Here every iteration runs inside one kernel whose CTAs are all
// co-resident (cooperative launch): element-parallel p = z + beta p and
// A p (order-1 hexahedra, one thread per element), then mask + gather-
// scatter, then the fused update x += alpha p, r -= alpha A p, z = invDiag r
// with both dot products.  Grid-wide dependencies use a generation barrier
// whose waits are bounded: on timeout the kernel records an error and every
// CTA returns.  Dot products are deterministic: each CTA writes a partial,
// every CTA sums all partials in index order after the barrier.  The whole
// working set (about 40 B per node) stays in the 129 MB L2.

#include "mg_kernels.hpp"

namespace nrsg {

namespace {
constexpr int kCT = 256;              // threads per CTA
constexpr long long kSpinLimit = 1LL << 22;

struct CoarseState {
  unsigned count;
  unsigned gen;
  int err;
  int iters;
  double res0, res;
};

__device__ __forceinline__ double cwarp(double v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double cblock(double v, double *sh)
{
  v = cwarp(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double r = 0;
  if (wid == 0) r = cwarp(lane < kCT / 32 ? sh[lane] : 0.0);
  __syncthreads();
  return r; // valid in thread 0
}

// Grid barrier with bounded waiting.  Returns false (in every thread) if the
// wait timed out or another CTA reported an error.
__device__ bool grid_barrier(CoarseState *st)
{
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned *vgen = &st->gen;
    volatile int *verr = &st->err;
    const unsigned g = *vgen;
    __threadfence();
    const unsigned arrived = atomicAdd(&st->count, 1u);
    int ok = 1;
    if (arrived == gridDim.x - 1) {
      st->count = 0;
      __threadfence();
      atomicAdd(&st->gen, 1u);
    } else {
      long long spins = 0;
      while (*vgen == g) {
        if (*verr) { ok = 0; break; }
        if (++spins > kSpinLimit) {
          atomicExch(&st->err, 1);
          ok = 0;
          break;
        }
        if (spins > 256) __nanosleep(32);
      }
    }
    __threadfence();
    if (*verr) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// sum of the per-CTA partials of `nslot` quantities (identical in every CTA)
__device__ void grid_sums(const double *partials, int nslot, double *out, double *sh)
{
  for (int q = 0; q < nslot; ++q) {
    double v = 0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += kCT) v += ((volatile const double *)partials)[q * gridDim.x + b];
    v = cblock(v, sh);
    if (threadIdx.x == 0) sh[32 + q] = v;
    __syncthreads();
    out[q] = sh[32 + q];
    __syncthreads();
  }
}

// A q on one order-1 hexahedron (D = [[-1/2, 1/2], [-1/2, 1/2]])
template <typename T>
__device__ __forceinline__ void ax_n1(const T *__restrict__ g, T lam0, T lam1, bool poisson, const T q[8], T out[8])
{
  T Gr[8], Gs[8], Gt[8];
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    const int i = n & 1, j = (n >> 1) & 1, k = n >> 2;
    const T qr = T(0.5) * (q[1 + 2 * j + 4 * k] - q[0 + 2 * j + 4 * k]);
    const T qs = T(0.5) * (q[i + 2 + 4 * k] - q[i + 0 + 4 * k]);
    const T qt = T(0.5) * (q[i + 2 * j + 4] - q[i + 2 * j + 0]);
    const T G00 = g[0 * 8 + n], G01 = g[1 * 8 + n], G11 = g[2 * 8 + n];
    const T G12 = g[3 * 8 + n], G02 = g[4 * 8 + n], G22 = g[5 * 8 + n];
    Gr[n] = lam0 * (G00 * qr + G01 * qs + G02 * qt);
    Gs[n] = lam0 * (G01 * qr + G11 * qs + G12 * qt);
    Gt[n] = lam0 * (G02 * qr + G12 * qs + G22 * qt);
  }
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    const int i = n & 1, j = (n >> 1) & 1, k = n >> 2;
    const T si = i ? T(0.5) : T(-0.5), sj = j ? T(0.5) : T(-0.5), sk = k ? T(0.5) : T(-0.5);
    T v = si * (Gr[0 + 2 * j + 4 * k] + Gr[1 + 2 * j + 4 * k]) + sj * (Gs[i + 0 + 4 * k] + Gs[i + 2 + 4 * k]) +
          sk * (Gt[i + 2 * j + 0] + Gt[i + 2 * j + 4]);
    if (!poisson) v += g[6 * 8 + n] * lam1 * q[n];
    out[n] = v;
  }
}
} // namespace

template <typename T> struct CoarseArgs {
  long long E;
  const T *ggeo;
  T lam0, lam1;
  bool poisson;
  long long ngroups;
  const int *gsOff, *gsIds;
  long long nmask;
  const int *mask;
  const T *invDiag, *w, *b;
  const unsigned char *gathered; // 1 where the node belongs to a gather group
  T *x, *r, *p, *z, *Ap;
  double *partials; // [3][gridDim]
  CoarseState *st;
  double tol;       // relative
  int maxit;
};

template <typename T> __global__ void __launch_bounds__(kCT) coarse_pcg_kernel(CoarseArgs<T> a)
{
  __shared__ double sh[64];
  const long long n = a.E * 8;
  const long long tid = blockIdx.x * (long long)kCT + threadIdx.x;
  const long long nth = (long long)gridDim.x * kCT;
  double sums[2];
  // x = 0, p = 0, r = b, z = invDiag r; partials: (r,r)_w and (r,z)_w
  double rr = 0, rz = 0;
  for (long long i = tid; i < n; i += nth) {
    const T ri = a.b[i];
    const T zi = a.invDiag[i] * ri;
    a.x[i] = T(0);
    a.p[i] = T(0);
    a.r[i] = ri;
    a.z[i] = zi;
    rr += (double)a.w[i] * (double)ri * (double)ri;
    rz += (double)a.w[i] * (double)ri * (double)zi;
  }
  rr = cblock(rr, sh);
  rz = cblock(rz, sh);
  if (threadIdx.x == 0) {
    a.partials[0 * gridDim.x + blockIdx.x] = rr;
    a.partials[1 * gridDim.x + blockIdx.x] = rz;
  }
  if (!grid_barrier(a.st)) return;
  grid_sums(a.partials, 2, sums, sh);
  const double r0 = sqrt(sums[0]);
  double rdotz = sums[1], rdotz_old = 0;
  double rn = r0;
  const double tol = a.tol * r0;
  int it = 0;
  while (rn > tol && it < a.maxit && r0 > 0) {
    ++it;
    const T beta = (it == 1) ? T(0) : (T)(rdotz / rdotz_old);
    // A: p = z + beta p and A p, one element per thread; (p, Ap)_w over nodes outside gather groups
    double pap = 0;
    for (long long e = tid; e < a.E; e += nth) {
      T q[8], out[8];
#pragma unroll
      for (int m = 0; m < 8; ++m) {
        const T v = a.z[e * 8 + m] + beta * a.p[e * 8 + m];
        a.p[e * 8 + m] = v;
        q[m] = v;
      }
      ax_n1<T>(a.ggeo + e * 56, a.lam0, a.lam1, a.poisson, q, out);
#pragma unroll
      for (int m = 0; m < 8; ++m) {
        a.Ap[e * 8 + m] = out[m];
        if (!a.gathered[e * 8 + m]) pap += (double)a.w[e * 8 + m] * (double)q[m] * (double)out[m];
      }
    }
    if (!grid_barrier(a.st)) return;
    // B: mask and gather-scatter (disjoint node sets); (p, Ap)_w over the gathered nodes
    for (long long m = tid; m < a.nmask; m += nth) a.Ap[a.mask[m]] = T(0);
    for (long long g = tid; g < a.ngroups; g += nth) {
      const int s0 = a.gsOff[g], t0 = a.gsOff[g + 1];
      T v = 0;
      for (int q = s0; q < t0; ++q) v += a.Ap[a.gsIds[q]];
      for (int q = s0; q < t0; ++q) {
        const int id = a.gsIds[q];
        a.Ap[id] = v;
        pap += (double)a.w[id] * (double)a.p[id] * (double)v;
      }
    }
    pap = cblock(pap, sh);
    if (threadIdx.x == 0) a.partials[2 * gridDim.x + blockIdx.x] = pap;
    if (!grid_barrier(a.st)) return;
    grid_sums(a.partials + 2 * gridDim.x, 1, sums, sh);
    const T alpha = (T)(rdotz / (sums[0] + 1e-300));
    // D: x += alpha p, r -= alpha Ap, z = invDiag r, partial (r,r)_w, (r,z)_w
    rr = 0;
    rz = 0;
    for (long long i = tid; i < n; i += nth) {
      a.x[i] += alpha * a.p[i];
      const T ri = a.r[i] - alpha * a.Ap[i];
      a.r[i] = ri;
      const T zi = a.invDiag[i] * ri;
      a.z[i] = zi;
      rr += (double)a.w[i] * (double)ri * (double)ri;
      rz += (double)a.w[i] * (double)ri * (double)zi;
    }
    rr = cblock(rr, sh);
    rz = cblock(rz, sh);
    if (threadIdx.x == 0) {
      a.partials[0 * gridDim.x + blockIdx.x] = rr;
      a.partials[1 * gridDim.x + blockIdx.x] = rz;
    }
    if (!grid_barrier(a.st)) return;
    grid_sums(a.partials, 2, sums, sh);
    rn = sqrt(sums[0]);
    rdotz_old = rdotz;
    rdotz = sums[1];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.st->iters = it;
    a.st->res0 = r0;
    a.st->res = rn;
  }
}

template <typename T> struct CoarseSolverImpl;

// Host side: grid sizing, scratch, launch.
template <typename T>
int coarse_pcg_persistent(long long E, const T *ggeo, T lam0, T lam1, bool poisson, long long ngroups,
                          const int *gsOff, const int *gsIds, long long nmask, const int *mask, const T *invDiag,
                          const T *w, const unsigned char *gathered, const T *b, T *x, T *r, T *p, T *z, T *Ap,
                          double *partials, void *state, int gridMax, double tol, int maxit, cudaStream_t s)
{
  int dev = 0, sms = 0, perSM = 0;
  NRSG_CUDA(cudaGetDevice(&dev));
  NRSG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  NRSG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, coarse_pcg_kernel<T>, kCT, 0));
  int grid = sms * (perSM < 1 ? perSM : 1);
  const long long need = (E * 8 + kCT - 1) / kCT;
  if (grid > need) grid = (int)(need > 0 ? need : 1);
  if (grid > gridMax) grid = gridMax;
  if (grid < 1) throw Error(NRSG_ERR_CUDA, "coarse solver: no co-resident CTAs");
  NRSG_CUDA(cudaMemsetAsync(state, 0, sizeof(CoarseState), s));
  CoarseArgs<T> a;
  a.E = E;
  a.ggeo = ggeo;
  a.lam0 = lam0;
  a.lam1 = lam1;
  a.poisson = poisson;
  a.ngroups = ngroups;
  a.gsOff = gsOff;
  a.gsIds = gsIds;
  a.nmask = nmask;
  a.mask = mask;
  a.invDiag = invDiag;
  a.w = w;
  a.gathered = gathered;
  a.b = b;
  a.x = x;
  a.r = r;
  a.p = p;
  a.z = z;
  a.Ap = Ap;
  a.partials = partials;
  a.st = (CoarseState *)state;
  a.tol = tol;
  a.maxit = maxit;
  void *args[] = {&a};
  NRSG_CUDA(cudaLaunchCooperativeKernel((const void *)coarse_pcg_kernel<T>, dim3(grid), dim3(kCT), args, 0, s));
  count_launch();
  return grid;
}

size_t coarse_state_bytes() { return sizeof(CoarseState); }
int coarse_state_read(const void *state_host, int *iters, double *res0, double *res)
{
  const CoarseState *st = (const CoarseState *)state_host;
  if (iters) *iters = st->iters;
  if (res0) *res0 = st->res0;
  if (res) *res = st->res;
  return st->err;
}

template int coarse_pcg_persistent<double>(long long, const double *, double, double, bool, long long, const int *,
                                           const int *, long long, const int *, const double *, const double *,
                                           const unsigned char *, const double *, double *, double *, double *,
                                           double *, double *, double *, void *, int, double, int, cudaStream_t);
template int coarse_pcg_persistent<float>(long long, const float *, float, float, bool, long long, const int *,
                                          const int *, long long, const int *, const float *, const float *,
                                          const unsigned char *, const float *, float *, float *, float *, float *,
                                          float *, double *, void *, int, double, int, cudaStream_t);

} // namespace nrsg
