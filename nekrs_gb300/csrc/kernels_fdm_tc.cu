// Order-7 RAS FDM (the Schwarz local solve of the finest multigrid level) on
// the 5th-generation tensor cores: tcgen05.mma kind::tf32, operands in shared
// memory, accumulator in tensor memory.
//
// One element per pass of a CTA of 128 threads.  A 1-D transform along one
// direction is D = A B^T with
//   A (128 x 16, K-major): row = one of the element's 100 lines of the
//     extended 10^3 element (rows 100..127 unused), column = the 10 points
//     of the line (columns 10..15 zero);
//   B (16 x 16, K-major): row i = output point, column l = input point:
//     S^T for the forward transforms, S for the backward ones (rows and
//     columns 10..15 zero);
//   D (128 x 16 FP32) in tensor memory: TMEM lane = line, column = output.
// Two MMAs (K = 8 each) per transform.  Thread t owns TMEM lane t, reads its
// line's 10 outputs with tcgen05.ld and writes them rotated into the other A
// tile (point b of line b + 10 c becomes point b of line c + 10 m for output
// m), so that the next direction is again the K dimension; three transforms
// restore the layout.  The forward z result is scaled by 1/(lx + ly + lz)
// from the three 1-D eigenvalue sets; the last backward transform goes from
// tensor memory straight to the element's own nodes (times the RAS weight).
//
// Shared tiles use the no-swizzle K-major canonical layout: core matrices of
// 8 rows x 16 bytes (4 TF32 values); B's are 128 bytes apart along K and 512
// along the rows, A's 160 and 608 (fewer bank conflicts in the rotated
// stores).  Inputs of every transform are rounded to TF32
// (cvt.rna) when they are stored; accumulation is FP32.
//
// Persistent CTAs walk the elements (grid = SMs x resident CTAs).  The only
// wait is on the MMA-completion mbarrier; it gives up after a set number of
// polls, records an error flag the host reads after the solve, and the CTA
// frees its tensor memory and leaves.
#include "mg_kernels.hpp"
#include "nrsg_internal.hpp"

#include <cuda_runtime.h>

#include <cstdint>

namespace nrsg {

namespace fdmtc5 {
constexpr int kThreads = 128;                  // = TMEM lanes = A rows
// A tile: 16 groups of 8 rows, 608 bytes apart; 4 core matrices per group along K, 160 bytes apart (the
// spacing that keeps the rotated result stores of a warp at most 2-way bank-conflicted)
constexpr unsigned kALbo = 160, kASbo = 608;
constexpr int kTileFloats = 16 * kASbo / 4;    // 9728 bytes
constexpr int kBFloats = 16 * 16;              // one B matrix (1 KB)
constexpr unsigned kTmemCols = 32;             // smallest allocation; D uses 16
constexpr unsigned kSpinLimit = 1u << 24;      // polls of the MMA-completion barrier
// instruction descriptor, kind::tf32: D FP32 (bits 4-5 = 1), A and B TF32 (bits 7-9, 10-12 = 2), both
// K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28
constexpr unsigned kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((16u >> 3) << 17) | ((128u >> 4) << 24);
} // namespace fdmtc5

__device__ unsigned g_fdm_tc_err = 0;

namespace {

__device__ __forceinline__ unsigned sm_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

// float index of (row r, column k) in a no-swizzle K-major tile of 16 TF32 columns: core matrices of 8 rows
// x 16 bytes, LBO bytes apart along K and SBO bytes apart along the rows (B: 128 / 512, A: kALbo / kASbo)
__device__ __forceinline__ int tcf(int r, int k) { return (r >> 3) * 128 + (k >> 2) * 32 + (r & 7) * 4 + (k & 3); }
__device__ __forceinline__ int taf(int r, int k)
{
  return (r >> 3) * (int)(fdmtc5::kASbo / 4) + (k >> 2) * (int)(fdmtc5::kALbo / 4) + (r & 7) * 4 + (k & 3);
}

// shared-memory matrix descriptor: start >> 4 (bits 0-13), leading (K) byte offset >> 4 (bits 16-29),
// stride (row-group) byte offset >> 4 (bits 32-45), version 1 (bits 46-47), no swizzle (bits 61-63 = 0)
__device__ __forceinline__ unsigned long long tile_desc(unsigned addr, unsigned lbo, unsigned sbo)
{
  return (unsigned long long)((addr & 0x3FFFFu) >> 4) | ((unsigned long long)(lbo >> 4) << 16) |
         ((unsigned long long)(sbo >> 4) << 32) | (1ull << 46);
}

__device__ __forceinline__ float to_tf32(float x)
{
  unsigned r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

__device__ __forceinline__ void umma_tf32(unsigned dtmem, unsigned long long ad, unsigned long long bd, int acc)
{
  asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
               "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
               "l"(ad), "l"(bd), "r"(fdmtc5::kIdesc), "r"(acc)
               : "memory");
}

__device__ __forceinline__ void umma_commit(unsigned long long *bar)
{
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(sm_addr(bar))
               : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ bool bar_try_wait(unsigned long long *bar, unsigned parity)
{
  unsigned ok;
  asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
               "selp.u32 %0, 1, 0, p;\n\t}"
               : "=r"(ok)
               : "r"(sm_addr(bar)), "r"(parity)
               : "memory");
  return ok != 0;
}

// this thread's TMEM lane, columns 0..15 (load and its completion in one asm block)
__device__ __forceinline__ void tmem_ld16(unsigned taddr, float v[16])
{
  unsigned r[16];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
               "[%16];\n\ttcgen05.wait::ld.sync.aligned;"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                 "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                 "=r"(r[15])
               : "r"(taddr)
               : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// extended-element point (x, y, z) of halo node (a, b) of face f
__device__ __forceinline__ void halo_xyz(int f, int a, int b, int &x, int &y, int &z)
{
  switch (f) {
  case 0: x = 0, y = a + 1, z = b + 1; break;
  case 1: x = 9, y = a + 1, z = b + 1; break;
  case 2: x = a + 1, y = 0, z = b + 1; break;
  case 3: x = a + 1, y = 9, z = b + 1; break;
  case 4: x = a + 1, y = b + 1, z = 0; break;
  default: x = a + 1, y = b + 1, z = 9; break;
  }
}

// the 104 edge and corner points of the extended element (two or three coordinates in {0, 9})
__device__ __forceinline__ void edge_xyz(int t, int &x, int &y, int &z)
{
  if (t < 96) {
    const int edge = t >> 3, s = (t & 7) + 1, p = 9 * (edge & 1), q = 9 * ((edge >> 1) & 1);
    switch (edge >> 2) {
    case 0: x = s, y = p, z = q; break;
    case 1: x = p, y = s, z = q; break;
    default: x = p, y = q, z = s; break;
    }
  } else {
    const int c = t - 96;
    x = 9 * (c & 1), y = 9 * ((c >> 1) & 1), z = 9 * (c >> 2);
  }
}

} // namespace

// next element's operands, brought in while the current one is transformed: u, S and the halo
// indices by bulk copy (16-byte aligned slabs), the halo values and the eigenvalues by 4-byte cp.async
struct FdmTcStage {
  float u[512];
  float S[300];
  int hidx[384];
  float hval[384];
  float lam[32];
};

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *bar)
{
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   sm_addr(dst)),
               "l"(src), "r"(bytes), "r"(sm_addr(bar))
               : "memory");
}
__device__ __forceinline__ void cp_async4(void *dst, const void *src)
{
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sm_addr(dst)), "l"(src) : "memory");
}

__global__ void __launch_bounds__(fdmtc5::kThreads, 8)
    fdm_tc_kernel(long long E, const float *__restrict__ u, const int *__restrict__ haloSrc,
                  const float *__restrict__ Sx, const float *__restrict__ Sy, const float *__restrict__ Sz,
                  const float *__restrict__ lam, const float *__restrict__ wts, float *__restrict__ Su)
{
  using namespace fdmtc5;
  constexpr int NX = 10, NP = 512, NF = 64, LN = 100;
  // one A tile: an MMA has read all of it when its completion is signalled, so each transform's result
  // is written over its own input
  __shared__ __align__(1024) float sA[kTileFloats];
  __shared__ __align__(1024) float sB[6][kBFloats]; // forward x, y, z; backward x, y, z
  __shared__ __align__(16) FdmTcStage stage;
  __shared__ __align__(16) float s_wts[NP];
  __shared__ float s_lxy[LN], s_lz[16];
  __shared__ __align__(8) unsigned long long bar, ldbar;
  __shared__ unsigned s_tmem;
  const int tid = threadIdx.x, warp = tid >> 5;

  for (int q = tid; q < kTileFloats / 4; q += kThreads) ((float4 *)sA)[q] = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int q = tid; q < 6 * kBFloats / 4; q += kThreads) ((float4 *)sB)[q] = make_float4(0.f, 0.f, 0.f, 0.f);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sm_addr(&s_tmem)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sm_addr(&bar)), "r"(1) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sm_addr(&ldbar)), "r"(1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const unsigned tmem = s_tmem;
  const unsigned tlane = tmem + ((unsigned)(warp * 32) << 16); // this warp's TMEM sub-partition
  const unsigned aAddr = sm_addr(sA), bAddr = sm_addr(sB[0]);
  const int bq = tid % NX, cq = tid / NX; // this thread's line tid = bq + NX cq (tid < 100)
  // where this thread's 10 results go in the rotated tile (row cq + 10 i, column bq), two 16-bit offsets
  // per register
  unsigned roff[5];
#pragma unroll
  for (int h = 0; h < 5; ++h)
    roff[h] = (unsigned)taf(cq + NX * (2 * h), bq) | ((unsigned)taf(cq + NX * (2 * h + 1), bq) << 16);
  unsigned phase = 0, ldphase = 0;
  bool late = false, mmaInFlight = false;

  // thread 0: bulk copies of element en's u, S and halo indices into the stage (en < E) and of element
  // ew's RAS weights (ew >= 0), all counted on ldbar
  auto issue = [&](long long en, long long ew) {
    const unsigned bytes = (en < E ? (NP + 3 * LN + 6 * NF) * 4u : 0u) + (ew >= 0 ? NP * 4u : 0u);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sm_addr(&ldbar)), "r"(bytes)
                 : "memory");
    if (en < E) {
      bulk_g2s(stage.u, u + en * NP, NP * 4, &ldbar);
      bulk_g2s(stage.S, Sx + en * LN, LN * 4, &ldbar);
      bulk_g2s(stage.S + LN, Sy + en * LN, LN * 4, &ldbar);
      bulk_g2s(stage.S + 2 * LN, Sz + en * LN, LN * 4, &ldbar);
      bulk_g2s(stage.hidx, haloSrc + en * 6 * NF, 6 * NF * 4, &ldbar);
    }
    if (ew >= 0) bulk_g2s(s_wts, wts + ew * NP, NP * 4, &ldbar);
  };
  // all threads: bounded wait for the current ldbar phase
  auto wait_ld = [&]() -> bool {
    unsigned spins = 0;
    bool mine = false;
    while (!bar_try_wait(&ldbar, ldphase))
      if (++spins > kSpinLimit) {
        mine = true;
        break;
      }
    if (__syncthreads_or(mine)) return true;
    ldphase ^= 1u;
    return false;
  };
  // all threads: halo values and eigenvalues of element en (its halo indices are in the stage)
  auto gather = [&](long long en) {
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      const int q = tid + kThreads * m, src = stage.hidx[q];
      if (src >= 0)
        cp_async4(&stage.hval[q], u + src);
      else
        stage.hval[q] = 0.f;
    }
    if (tid < 3 * NX) cp_async4(&stage.lam[tid], lam + en * 3 * NX + tid);
    asm volatile("cp.async.commit_group;" ::: "memory");
  };

  long long e = blockIdx.x;
  if (tid == 0) issue(e, -1);
  late = wait_ld();
  if (!late) gather(e);

  for (; e < E && !late; e += gridDim.x) {
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncthreads();
    // ---- element e from the stage: A in the lines-of-x layout (line y + 10 z, point x), B, lambdas
    {
      const float4 uv = ((const float4 *)stage.u)[tid];
      const int x = (4 * tid) & 7, y = (tid >> 1) & 7, z = tid >> 4;
      const int line = (y + 1) + NX * (z + 1);
      sA[taf(line, x + 1)] = to_tf32(uv.x);
      sA[taf(line, x + 2)] = to_tf32(uv.y);
      sA[taf(line, x + 3)] = to_tf32(uv.z);
      sA[taf(line, x + 4)] = to_tf32(uv.w);
    }
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      const int q = tid + kThreads * m;
      int x, y, z;
      halo_xyz(q / NF, (q % NF) % 8, (q % NF) / 8, x, y, z);
      sA[taf(y + NX * z, x)] = to_tf32(stage.hval[q]);
    }
    if (tid < 104) {
      int x, y, z;
      edge_xyz(tid, x, y, z);
      sA[taf(y + NX * z, x)] = 0.f;
    }
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      const int q = tid + kThreads * m;
      if (q < 3 * LN) {
        const int d = q / LN, rc = q % LN, r = rc % NX, c = rc / NX; // S_d(r, c) = Sd[r + 10 c]
        const float sv = to_tf32(stage.S[q]);
        sB[d][tcf(c, r)] = sv;     // forward: B(i, l) = S(l, i)
        sB[3 + d][tcf(r, c)] = sv; // backward: B(i, l) = S(i, l)
      }
    }
    if (tid < LN) s_lxy[tid] = stage.lam[tid % NX] + stage.lam[NX + tid / NX];
    if (tid < NX) s_lz[tid] = stage.lam[2 * NX + tid];
    fence_async_smem();
    __syncthreads();
    const long long en = e + gridDim.x;
    if (tid == 0) issue(en, e);

    // ---- six transforms: forward x, y, z (scaled), backward x, y, z
#pragma unroll 1
    for (int p = 0; p < 6; ++p) {
      if (tid == 0) {
        fence_after();
#pragma unroll
        for (int s = 0; s < 2; ++s)
          umma_tf32(tmem, tile_desc(aAddr + s * 2 * kALbo, kALbo, kASbo),
                    tile_desc(bAddr + p * kBFloats * 4 + s * 256, 128, 512), s);
        umma_commit(&bar);
        mmaInFlight = true;
      }
      if (p == 1) {
        // the next element's slabs and this element's weights have had one transform's time to land
        if (wait_ld()) {
          late = true;
          break;
        }
        if (en < E) gather(en);
      }
      // warp 0 watches the MMA-completion barrier; the other warps wait at the CTA barrier
      bool mine = false;
      if (warp == 0) {
        unsigned spins = 0;
        while (!bar_try_wait(&bar, phase))
          if (++spins > kSpinLimit) {
            mine = true;
            break;
          }
      }
      if (__syncthreads_or(mine)) {
        late = true;
        break;
      }
      phase ^= 1u;
      mmaInFlight = false;
      fence_after();
      float v[16];
      tmem_ld16(tlane, v);
      if (tid < LN) {
        if (p == 2) {
          const float sxy = s_lxy[tid];
#pragma unroll
          for (int i = 0; i < NX; ++i) {
            const float d = sxy + s_lz[i];
            v[i] *= d > 1e-5f ? __fdividef(1.f, d) : 0.f;
          }
        }
        if (p < 5) {
#pragma unroll
          for (int i = 0; i < NX; ++i) sA[(roff[i >> 1] >> (16 * (i & 1))) & 0xFFFFu] = to_tf32(v[i]);
        } else if (bq >= 1 && bq <= 8 && cq >= 1 && cq <= 8) {
          // line x + 10 y of the last transform: own nodes (x, y, z) for z = 1..8
          const int base = (bq - 1) + 8 * (cq - 1);
          float *se = Su + e * NP + base;
#pragma unroll
          for (int z = 1; z <= 8; ++z) se[64 * (z - 1)] = v[z] * s_wts[base + 64 * (z - 1)];
        }
      }
      fence_before();
      fence_async_smem();
      __syncthreads();
    }
  }
  asm volatile("cp.async.wait_all;" ::: "memory");
  if (late) {
    // a wait ran out: flag it, give the MMA and the bulk copies in flight one more bounded wait each,
    // free the tensor memory and leave
    if (tid == 0) {
      atomicExch(&g_fdm_tc_err, 1u);
      for (unsigned k = 0; mmaInFlight && k < kSpinLimit && !bar_try_wait(&bar, phase); ++k) {
      }
      // every issue() is followed by exactly one wait of ldbar, so an unfinished phase is the last one
      for (unsigned k = 0; k < kSpinLimit && !bar_try_wait(&ldbar, ldphase); ++k) {
      }
    }
    fence_before();
  }
  __syncthreads();
  if (warp == 0) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
  }
}

bool launch_fdm_tc(long long E, const float *u, const int *haloSrc, const float *Sx, const float *Sy, const float *Sz,
                   const float *lam, const float *wts, float *Su, cudaStream_t s)
{
  if (E <= 0) return true;
  if (!lam) return false;
  // the bulk copies take 16-byte aligned slabs
  for (const void *p : {(const void *)u, (const void *)haloSrc, (const void *)Sx, (const void *)Sy,
                        (const void *)Sz, (const void *)wts})
    if (reinterpret_cast<uintptr_t>(p) % 16) return false;
  static int resident = 0, sms = 0;
  if (!resident) {
    // resident CTAs per SM from the kernel's registers and shared memory (the occupancy query counts a
    // kernel that allocates tensor memory as one CTA per SM); tensor memory caps it at 512 / 32 = 16
    int dev = 0, smemSM = 0, regsSM = 0;
    NRSG_CUDA(cudaGetDevice(&dev));
    NRSG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    NRSG_CUDA(cudaDeviceGetAttribute(&smemSM, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    NRSG_CUDA(cudaDeviceGetAttribute(&regsSM, cudaDevAttrMaxRegistersPerMultiprocessor, dev));
    cudaFuncAttributes fa{};
    NRSG_CUDA(cudaFuncGetAttributes(&fa, fdm_tc_kernel));
    const int regs = ((fa.numRegs + 7) / 8) * 8 * fdmtc5::kThreads;
    const int byRegs = regs > 0 ? regsSM / regs : 16;
    const int bySmem = smemSM / ((int)fa.sharedSizeBytes + 1024);
    int r = byRegs < bySmem ? byRegs : bySmem;
    if (r > 16) r = 16;
    if (r < 1) r = 1;
    resident = r;
  }
  const long long want = (long long)sms * resident;
  const unsigned grid = (unsigned)(E < want ? E : want);
  fdm_tc_kernel<<<grid, fdmtc5::kThreads, 0, s>>>(E, u, haloSrc, Sx, Sy, Sz, lam, wts, Su);
  NRSG_CHECK_LAUNCH();
  return true;
}

unsigned fdm_tc_error(cudaStream_t s)
{
  unsigned h = 0;
  NRSG_CUDA(cudaMemcpyFromSymbolAsync(&h, g_fdm_tc_err, sizeof(h), 0, cudaMemcpyDeviceToHost, s));
  NRSG_CUDA(cudaStreamSynchronize(s));
  const unsigned zero = 0;
  if (h) NRSG_CUDA(cudaMemcpyToSymbolAsync(g_fdm_tc_err, &zero, sizeof(zero), 0, cudaMemcpyHostToDevice, s));
  return h;
}

} // namespace nrsg
