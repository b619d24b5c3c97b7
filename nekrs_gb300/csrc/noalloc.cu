// Allocation-free variant of the weighted inner product.
//
// Some callers cannot call cudaMalloc: an application whose device memory is
// owned and budgeted by another allocator (a framework's caching allocator,
// a fixed arena set up at start-up), or a latency-critical loop that must not
// take the implicit device synchronisation of an allocation.  For them
// nrsg_weighted_inner_prod_f64_noalloc computes the same sum as
// nrsg_weighted_inner_prod_f64 (which keeps cudaMalloc'ed partial sums per
// device) with its scratch in a fixed array of this library instead.
//
// Scratch: kNoAllocSlots = 8192 partial sums plus a completion counter in one
// file-scope __device__ array (64 KiB + 256 B per GPU that loads the
// library, held until the process exits).  One CTA covers 8192 entries, so
// n is limited to 8192 * 8192 = 67,108,864 entries; larger n is rejected with
// NRSG_ERR_INVALID before anything is launched.
//
// Set-up: the first call on a device looks up the device address of the
// array (cudaGetSymbolAddress) with that device current and caches it; make
// that first call before capturing any stream work.  Every call shares the
// one array and therefore the calls must not overlap on the GPU: two calls
// running at the same time (different streams, or different host threads on
// one device) race on the partial sums and the counter.  The counter is
// cleared on the caller's stream before each launch; the partial sums are
// fully rewritten by every call.

#include "nrsg_internal.hpp"

#include <mutex>

namespace nrsg {
namespace {

constexpr int kNoAllocSlots = 8192;
constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocPerThread = 32;
constexpr long long kNoAllocChunk = (long long)kNoAllocThreads * kNoAllocPerThread; // entries per CTA
constexpr long long kNoAllocMaxN = kNoAllocChunk * kNoAllocSlots;                    // 67,108,864
constexpr int kNoAllocWords = kNoAllocSlots + 32; // partial sums, then the counter (own 256 B line)

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocWords];

__device__ __forceinline__ double na_warp_sum(double v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double na_block_sum(double v)
{
  __shared__ double s_w[kNoAllocThreads / 32];
  v = na_warp_sum(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) s_w[wid] = v;
  __syncthreads();
  double r = 0;
  if (wid == 0) r = na_warp_sum(lane < kNoAllocThreads / 32 ? s_w[lane] : 0.0);
  __syncthreads();
  return r;
}

// one CTA per chunk of kNoAllocChunk entries; the last CTA to finish adds the
// partial sums in index order (deterministic) and stores the result
__global__ void __launch_bounds__(kNoAllocThreads)
    wdot_noalloc_kernel(long long n, const double *__restrict__ w, const double *__restrict__ a,
                        const double *__restrict__ b, double *scratch, double *out)
{
  const long long begin = (long long)blockIdx.x * kNoAllocChunk;
  const long long end = begin + kNoAllocChunk < n ? begin + kNoAllocChunk : n;
  double acc = 0;
  for (long long i = begin + threadIdx.x; i < end; i += kNoAllocThreads) {
    const double av = a[i];
    acc += (w ? w[i] : 1.0) * av * (b ? b[i] : av);
  }
  acc = na_block_sum(acc);
  unsigned *counter = reinterpret_cast<unsigned *>(scratch + kNoAllocSlots);
  __shared__ bool s_last;
  if (threadIdx.x == 0) {
    scratch[blockIdx.x] = acc;
    __threadfence();
    s_last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  double v = 0;
  for (int q = threadIdx.x; q < (int)gridDim.x; q += kNoAllocThreads) v += ((volatile double *)scratch)[q];
  v = na_block_sum(v);
  if (threadIdx.x == 0) {
    *out = v;
    *counter = 0u;
  }
}

std::mutex g_noalloc_mutex;
double *g_noalloc_ptr[64] = {nullptr};

// device address of the scratch array for the current device (looked up once)
double *noalloc_scratch()
{
  int dev = -1;
  NRSG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) throw Error(NRSG_ERR_INVALID, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    double *ptr = nullptr;
    const cudaError_t err = cudaGetSymbolAddress((void **)&ptr, g_noalloc_scratch);
    if (err != cudaSuccess || !ptr)
      throw Error(NRSG_ERR_CUDA, std::string("cudaGetSymbolAddress(no-alloc scratch): ") + cudaGetErrorString(err));
    g_noalloc_ptr[dev] = ptr;
  }
  return g_noalloc_ptr[dev];
}

} // namespace
} // namespace nrsg

extern "C" int nrsg_weighted_inner_prod_f64_noalloc(long long n, const double *d_w, const double *d_a,
                                                    const double *d_b, double *d_out, void *stream)
{
  using nrsg::kNoAllocChunk;
  using nrsg::kNoAllocMaxN;
  if (!d_a || !d_out || n < 1) {
    nrsg::set_last_error("weighted_inner_prod_f64_noalloc: null buffer or n < 1");
    return NRSG_ERR_INVALID;
  }
  if (n > kNoAllocMaxN) {
    nrsg::set_last_error("weighted_inner_prod_f64_noalloc: n = " + std::to_string(n) +
                         " exceeds the fixed scratch limit of " + std::to_string(kNoAllocMaxN) + " entries");
    return NRSG_ERR_INVALID;
  }
  try {
    double *scratch = nrsg::noalloc_scratch();
    cudaStream_t s = (cudaStream_t)stream;
    NRSG_CUDA(cudaMemsetAsync(scratch + nrsg::kNoAllocSlots, 0, sizeof(unsigned), s));
    const unsigned grid = (unsigned)((n + kNoAllocChunk - 1) / kNoAllocChunk);
    nrsg::wdot_noalloc_kernel<<<grid, nrsg::kNoAllocThreads, 0, s>>>(n, d_w, d_a, d_b, scratch, d_out);
    NRSG_CHECK_LAUNCH();
    return NRSG_OK;
  } catch (const nrsg::Error &e) {
    nrsg::set_last_error(e.what());
    return e.code;
  }
}
