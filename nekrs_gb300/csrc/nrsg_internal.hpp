// Internal declarations of the nekrs_gb300 library (host + device).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/nekrs_gb300.h"

namespace nrsg {

struct Error : public std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

void set_last_error(const std::string &msg);

#define NRSG_CUDA(call)                                                                                    \
  do {                                                                                                     \
    cudaError_t err__ = (call);                                                                            \
    if (err__ != cudaSuccess)                                                                              \
      throw ::nrsg::Error(err__ == cudaErrorMemoryAllocation ? NRSG_ERR_OOM : NRSG_ERR_CUDA,             \
                          std::string(#call) + ": " + cudaGetErrorString(err__));                        \
  } while (0)

// Every launcher ends with NRSG_CHECK_LAUNCH(), which also counts the launch.
void count_launch();
// while a tally is set on this thread, count_launch() adds to it instead of
// the process counter (kernels recorded into a CUDA graph are not launched)
void set_launch_tally(long long *tally);
void add_launches(long long n);
#define NRSG_CHECK_LAUNCH()                                                                                \
  do {                                                                                                     \
    ::nrsg::count_launch();                                                                                \
    NRSG_CUDA(cudaGetLastError());                                                                         \
  } while (0)

// Owning device buffer.
template <typename T> struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  explicit DevBuf(size_t count) { alloc(count); }
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  DevBuf(DevBuf &&o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DevBuf &operator=(DevBuf &&o) noexcept
  {
    if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
    return *this;
  }
  ~DevBuf() { release(); }
  void alloc(size_t count)
  {
    release();
    if (count == 0) return;
    NRSG_CUDA(cudaMalloc((void **)&p, count * sizeof(T)));
    n = count;
  }
  void release()
  {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void upload(const T *h, size_t count)
  {
    alloc(count);
    if (count) NRSG_CUDA(cudaMemcpy(p, h, count * sizeof(T), cudaMemcpyHostToDevice));
  }
  void upload(const std::vector<T> &v) { upload(v.data(), v.size()); }
  std::vector<T> download() const
  {
    std::vector<T> h(n);
    if (n) NRSG_CUDA(cudaMemcpy(h.data(), p, n * sizeof(T), cudaMemcpyDeviceToHost));
    return h;
  }
  size_t bytes() const { return n * sizeof(T); }
};

// ----------------------------------------------------------------------------
// Options: the .par [PRESSURE]-section keys that reach the elliptic solve.
// ----------------------------------------------------------------------------
struct Options {
  std::string solver = "pcg";   // pcg | pfcg | pgmres | pfgmres
  int nVector = 15;
  double tol = 1e-8;
  bool relative = true;
  int maxIter = 500;
  std::string precon = "jacobi"; // none | jacobi | multigrid
  std::string smoother = "cheby+jac";
  int chebyDegree = 2;
  double minEigFactor = 0.1, maxEigFactor = 1.1;
  std::string schedule;
  std::string coarse = "jpcg";
  bool galerkin = false;            // coarseGridDiscretization = FEM+Galerkin: B^T A_fine B on the order-1 level
  bool semfem = false;              // coarseGridDiscretization = SEMFEM: linear tetrahedra on the coarse GLL grid
  double coarseTol = 1e-4;
  int coarseMaxIter = 200;
  bool coarsePersistent = true;     // order-1 coarse Jacobi-PCG as one cooperative kernel
  long long coarseSpinLimit = 1LL << 22; // polls before a grid-barrier wait of that kernel gives up
  int coarseBarrierExtra = 0;       // arrivals added to every barrier target: nonzero only to test the bounded wait
  bool graphs = true;               // CUDA graphs of the steady-state PCG iteration (non-legacy streams)
  bool axPipeline = false;          // FP32 order-7 levels: bulk-copy pipelined axhelm
  bool axConst = false;             // FP32 order-7 levels: axhelm with D in constant memory / registers
  std::string axKernel = "auto";    // FP32 level axhelm: auto (timed at setup) | vec | plain | epb2 | pipe | const | constpf
  int nfields = 1;                  // block solver: fields at fieldOffset = Nlocal ("solver = pcg+block" -> 3)
  bool stress = false;              // stressFormulation: symmetric-gradient operator (nfields = 3)
  int projection = 0;               // initialGuess: 0 none, 1 projection (classic), 2 projectionAconj
  int projVecs = 8;                 // residualProjectionVectors
  int projStart = 5;                // residualProjectionStart
  std::string mgPrecision = "fp64"; // fp64 | fp32 | mixed
  bool fdmFp16 = false;             // fdmPrecision = fp16: order-7 RAS FDM transforms in FP16 on the tensor cores
  bool fdmTf32 = false;              // fdmPrecision = tf32: FDM transforms in TF32 on the tensor cores (orders 3, 5, 7)
  bool fdmTcgen05 = true;            // fdmMma = tcgen05 | sync: the TF32 order-7 RAS FDM on tcgen05.mma or mma.sync
  bool fdmGeneric = false;           // fdmKernel = auto | generic: the FP32 FDM's specialised order-3 / order-7
                                     // kernels, or the line-per-thread kernel for every order
  int amgIterations = 1;             // V-cycles per coarse solve with coarseSolver = amg (BOOMERAMG ITERATIONS)
  std::string axPrecision = "fp64"; // fine-level operator: fp64 | fp32x2 (FP64-accurate FP32-pair arithmetic)
  bool poisson = true;
  double lambda0 = 1.0, lambda1 = 0.0;
  bool trilinear = false;
  bool trilinearLambda0All = false; // trilinearLambda0 = all: lambda0 scales every flux (reference: the t-flux only)
  unsigned long long seed = 0x5eed;
};
Options parse_options(const char *text);

// ----------------------------------------------------------------------------
// Host-side setup (setup.cpp)
// ----------------------------------------------------------------------------
void gll_nodes(int N, std::vector<double> &z, std::vector<double> &w);
void diff_matrix(const std::vector<double> &z, std::vector<double> &D);
void lagrange_interp(const std::vector<double> &zin, const std::vector<double> &zout, std::vector<double> &I);
void nek_global_ids(int N, long long E, const long long *EToV, std::vector<long long> &ids);
struct GatherMap {
  std::vector<int> off, ids;          // all groups (CSR), reference order
  std::vector<int> devOff, devIds;    // groups with >= 2 members only (what the kernel visits)
  std::vector<double> invDegree;
};
void build_gather(const std::vector<long long> &ids, GatherMap &gm);
void dirichlet_nodes(int N, long long E, const int *EToB, const GatherMap &unmasked, std::vector<int> &maskIds);
void trilinear_nodes(int N, long long E, const double *VX, const std::vector<double> &z1, std::vector<double> &x,
                     std::vector<double> &y, std::vector<double> &zz);

// ----------------------------------------------------------------------------
// Device kernels (launchers)
// ----------------------------------------------------------------------------
constexpr int kRedThreads = 256;
constexpr int kRedSegments = 4096; // warp runs per reduction: doubles per Reduce row
struct Reduce {              // scratch for deterministic one-launch reductions
  double *partials = nullptr; // [slots][stride] warp-run sums
  unsigned *counters = nullptr;
  int slots = 0;
  long long stride = kRedSegments;
  double *row(int slot) const { return partials + (size_t)slot * stride; }
};

template <typename T>
void launch_ax_stored(int N, long long E, const T *ggeo, const T *D, T lambda0, T lambda1, bool poisson, const T *q,
                      T *Aq, cudaStream_t s);
// lambda0 scales the t-flux only, as the reference's trilinear kernel does; lambda0All: all three fluxes
template <typename T>
void launch_ax_trilinear(int N, long long E, const T *VX, const T *gllz, const T *gllw, const T *D, T lambda0,
                         T lambda1, bool poisson, const T *q, T *Aq, cudaStream_t s, bool lambda0All = false);
template <typename T> void launch_gs(long long ngroups, const int *off, const int *ids, T *q, cudaStream_t s);
// Gather-scatter plan of one level: the groups of exactly two members as
// index pairs (most of them: face-interior nodes), the other groups (>= 3
// members) as CSR, and the Dirichlet mask ids.  Masked nodes belong to no
// group, so one launch applies both.
struct GsPlan {
  long long npairs = 0, nrest = 0, nmask = 0;
  const int2 *pairs = nullptr;
  const int *restOff = nullptr, *restIds = nullptr;
  const int *mask = nullptr;
};
template <typename T> void launch_gs_mask(const GsPlan &P, T *q, bool mask, cudaStream_t s);
// solution projection (accumulate.okl, multiScaledAddwOffset.okl): y = sum_k alpha_k X_k (k < m), and
// X_{m-1} -= sum_{k < m-1} alpha_k X_k; X holds m vectors of n; alpha on the device
void launch_accumulate(long long n, int m, const double *alpha, const double *X, double *y, cudaStream_t s);
void launch_multi_scaled_sub(long long n, int m, const double *alpha, double *X, cudaStream_t s);
void launch_scale_inplace(long long n, double a, double *x, cudaStream_t s);
template <typename T> void launch_sub_mean(long long n, const double *sum, double denom, T *q, cudaStream_t s);
// block (vector) Helmholtz, kernels_block.cu
void launch_vgeo(int N, long long E, const double *VX, const double *gllz, const double *gllw, const double *D,
                 double *vgeo, cudaStream_t s);
void launch_block_ax(int N, long long E, int nf, long long offset, long long loffset, const double *ggeo,
                     const double *D, const double *lam0, const double *lam1, double l0, double l1, bool poisson,
                     const double *q, double *Aq, cudaStream_t s);
void launch_stress_ax(int N, long long E, long long offset, long long loffset, const double *vgeo, const double *D,
                      const double *lam0, const double *lam1, double l0, double l1, const double *q, double *Aq,
                      cudaStream_t s);
// zero-normal projection of three fields at offset `offset` on the n entries (U = (U.n) maskN n + (U.t1) maskT1 t1
// + (U.t2) maskT2 t2, reps times per entry)
void launch_zero_normal(long long n, const int *node, const unsigned char *reps, const double *frame,
                        const double *mask, long long offset, double *U, cudaStream_t s);
void launch_block_diag(int N, long long E, int nf, long long offset, long long loffset, const double *ggeo,
                       const double *D, const double *lam0, const double *lam1, double l0, double l1, bool poisson,
                       double *diag, cudaStream_t s);
// Raise (never lower) a kernel function's dynamic shared-memory limit on the current device.
void raise_dynamic_smem(const void *kfn, size_t bytes);
// FP32 order-7 Poisson axhelm through the bulk-copy pipeline (false: not applicable, caller
// launches the plain kernel); its wait-limit flag is read and cleared by ax_pipe_error.
bool launch_ax_pipe(int N, long long E, const float *ggeo, const float *D, float lambda0, float lambda1, bool poisson,
                    const float *q, float *Aq, cudaStream_t s);
unsigned ax_pipe_error(cudaStream_t s);
// FP32 order-7 Poisson / Helmholtz axhelm with D in constant memory and registers (false: not
// applicable).  D is copied into one constant bank per launch: concurrent launches must pass the same D.
// prefetch: persistent CTAs that prefetch their next element pair into L2 (same results).
bool launch_ax_const(int N, long long E, const float *ggeo, const float *D, float lambda0, float lambda1,
                     bool poisson, const float *q, float *Aq, cudaStream_t s, bool prefetch = false);
template <typename T> void launch_mask(long long n, const int *ids, T *q, cudaStream_t s);
// FP32 axhelm variants the multigrid autotuner chooses between (identical results)
enum AxVariant { kAxVec = 0, kAxPlain = 1, kAxEpb2 = 2, kAxPipe = 3, kAxConst = 4, kAxConstPf = 5, kAxVariants = 6 };
bool launch_ax_f32_variant(int variant, int N, long long E, const float *ggeo, const float *D, float lambda0,
                           float lambda1, bool poisson, const float *q, float *Aq, cudaStream_t s);
// autotuner helpers: a reproducible [-1, 1) test vector; count entries whose bits differ
void launch_hash_fill(long long n, unsigned long long seed, float *q, cudaStream_t s);
void launch_count_mismatch(long long n, const float *a, const float *b, unsigned *counter, cudaStream_t s);
template <typename T>
void launch_build_diag(int N, long long E, const T *ggeo, const T *D, T lambda0, T lambda1, bool poisson, T *diag,
                       cudaStream_t s);
// FP64-accurate Ax in FP32-pair arithmetic: ggeo/D as (hi, lo) float pairs, q and Aq FP64
void launch_ax_fp32x2(int N, long long E, const float2 *ggeo, const float2 *D, double lambda0, double lambda1,
                      bool poisson, const double *q, double *Aq, cudaStream_t s);
void launch_split_pairs(long long n, const double *x, float2 *y, cudaStream_t s);
void launch_geofac(int N, long long E, const double *VX, const double *gllz, const double *gllw, const double *D,
                   double *ggeo, cudaStream_t s);

// reductions: out = sum w*a*b (w may be null -> 1; b may be null -> a)
template <typename T>
void launch_wdot(long long n, const T *w, const T *a, const T *b, double *out, Reduce &red, int slot, cudaStream_t s);

// vector ops
template <typename T> void launch_fill(long long n, T v, T *x, cudaStream_t s);
template <typename T> void launch_axpby(long long n, T a, const T *x, T b, T *y, cudaStream_t s); // y = a x + b y
template <typename T> void launch_axmy(long long n, const T *w, T *x, cudaStream_t s);             // x = w .* x
template <typename T> void launch_axmyz(long long n, const T *a, const T *b, T *z, cudaStream_t s);   // z = a .* b
template <typename T> void launch_recip(long long n, T *x, cudaStream_t s);                           // x = 1/x
template <typename T> void launch_scale_copy(long long n, T a, const T *x, T *y, cudaStream_t s);     // y = a x
template <typename Ti, typename To> void launch_copy_cast(long long n, const Ti *x, To *y, cudaStream_t s);

// PCG device scalars
struct PcgScalars {
  double rdotz, rdotz_old, pAp, rdotr, zAp, alpha, beta, pad;
};
// z = invDiag .* r; scal.rdotz = (r,z)_w   (rdotz_old <- rdotz first)
void launch_jacobi_rdotz(long long n, const double *w, const double *invDiag, const double *r, double *z,
                         PcgScalars *sc, Reduce &red, int slot, cudaStream_t s);
// p = z + beta p, beta from scalars (first => 0; flexible => -alpha zAp / rdotz_old)
void launch_update_p(long long n, const double *z, double *p, const PcgScalars *sc, bool first, bool flexible,
                     cudaStream_t s);
// alpha = rdotz/(pAp+1e-300); r -= alpha Ap; x += alpha p; rdotr = (r,r)_w
void launch_update_xr(long long n, const double *w, const double *p, const double *Ap, double *x, double *r,
                      PcgScalars *sc, Reduce &red, int slot, cudaStream_t s);
// store a reduction result into a scalar field: dst = src (device), optionally save old
void launch_scalar_move(double *dst, const double *src, double *save_old, cudaStream_t s);
// fused update with explicit alpha (kernel-level entry point)
void launch_update_pcg_alpha(long long n, const double *w, const double *p, const double *Ap, double alpha, double *x,
                             double *r, double *rdotr, Reduce &red, int slot, cudaStream_t s);

} // namespace nrsg
