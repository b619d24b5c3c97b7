// Device V-cycle of the algebraic multigrid coarse solve (hierarchy built on
// the host by amg.cpp).  One V-cycle from x = 0:
//   down, level l:  x_l = w D^-1 b_l;  r_l = b_l - A_l x_l;  b_{l+1} = R_l r_l
//   coarsest:       x_c = A_c^-1 b_c (dense inverse)
//   up, level l:    x_l += P_l x_{l+1};  xo_l = x_l + w D^-1 (b_l - A_l x_l)
// with w = 2 / (1.3 lmax) (Chebyshev of degree 1 on [0.3 lmax, lmax]).  Every
// sparse product is a CSR row walk by a group of lanes with a fixed shuffle
// reduction, so results do not depend on scheduling.
#include "amg.hpp"

namespace nrsg {

namespace {

constexpr int kAmgThreads = 256;

inline unsigned amg_grid(long long work)
{
  long long b = (work + kAmgThreads - 1) / kAmgThreads;
  if (b < 1) b = 1;
  return (unsigned)b;
}

enum AmgMode { kPlain = 0, kResid = 1, kAdd = 2, kSmooth = 3 };

// TPR lanes per row; MODE: out = A x (plain), b - A x (resid), out + A x (add),
// x + wdinv (b - A x) (smooth)
template <typename T, int TPR, int MODE>
__global__ void amg_spmv_kernel(int n, const int *__restrict__ rp, const int *__restrict__ ci,
                                const T *__restrict__ v, const T *__restrict__ x, const T *__restrict__ b,
                                const T *__restrict__ wdinv, T *__restrict__ out)
{
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long row = tid / TPR;
  const int lane = (int)(tid % TPR);
  const bool active = row < n; // every lane reaches the full-warp shuffle
  T s = 0;
  if (active)
    for (int q = rp[row] + lane; q < rp[row + 1]; q += TPR) s += v[q] * x[ci[q]];
#pragma unroll
  for (int o = TPR / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, TPR);
  if (!active || lane != 0) return;
  if (MODE == kPlain) out[row] = s;
  else if (MODE == kResid) out[row] = b[row] - s;
  else if (MODE == kAdd) out[row] += s;
  else out[row] = x[row] + wdinv[row] * (b[row] - s);
}

template <typename T, int MODE>
void spmv(int n, int nnz, const int *rp, const int *ci, const T *v, const T *x, const T *b, const T *wdinv, T *out,
          cudaStream_t s)
{
  if (n <= 0) return;
  const double avg = n ? (double)nnz / n : 0;
  // a group of TPR lanes per row (TPR divides 32; lanes past the last row take part in the shuffles only)
  if (avg > 12) {
    amg_spmv_kernel<T, 8, MODE><<<amg_grid((long long)n * 8), kAmgThreads, 0, s>>>(n, rp, ci, v, x, b, wdinv, out);
  } else if (avg > 3) {
    amg_spmv_kernel<T, 4, MODE><<<amg_grid((long long)n * 4), kAmgThreads, 0, s>>>(n, rp, ci, v, x, b, wdinv, out);
  } else {
    amg_spmv_kernel<T, 1, MODE><<<amg_grid((long long)n), kAmgThreads, 0, s>>>(n, rp, ci, v, x, b, wdinv, out);
  }
  NRSG_CHECK_LAUNCH();
}

template <typename T> __global__ void amg_scale_kernel(int n, const T *__restrict__ w, const T *__restrict__ b, T *x)
{
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) x[i] = w[i] * b[i];
}

template <typename T>
__global__ void amg_dense_kernel(int n, const T *__restrict__ inv, const T *__restrict__ b, T *__restrict__ x)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  T s = 0;
  for (int j = 0; j < n; ++j) s += inv[(size_t)i * n + j] * b[j];
  x[i] = s;
}

template <typename T> __global__ void amg_add_kernel(int n, const T *__restrict__ e, T *__restrict__ x)
{
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) x[i] += e[i];
}

template <typename T> __global__ void rows_gather_kernel(long long n, const int *rep, const T *ev, T *rows)
{
  const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (r < n) rows[r] = ev[rep[r]];
}
template <typename T> __global__ void rows_scatter_kernel(long long n, const int *rowOf, const T *rows, T *ev)
{
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) {
    const int r = rowOf[i];
    ev[i] = r >= 0 ? rows[r] : T(0);
  }
}

template <typename T> void upload_cast(DevBuf<T> &d, const std::vector<double> &h)
{
  std::vector<T> t(h.begin(), h.end());
  d.upload(t);
}

} // namespace

template <typename T> void amg_upload(const AmgHierarchy &H, AmgDevice<T> &D)
{
  D = AmgDevice<T>();
  D.lv.resize(H.levels.size());
  for (size_t l = 0; l < H.levels.size(); ++l) {
    const AmgLevelHost &h = H.levels[l];
    AmgDevLevel<T> &d = D.lv[l];
    d.n = h.A.n;
    d.nc = h.P.m;
    d.arp.upload(h.A.rp);
    d.aci.upload(h.A.ci);
    upload_cast(d.av, h.A.v);
    d.prp.upload(h.P.rp);
    d.pci.upload(h.P.ci);
    upload_cast(d.pv, h.P.v);
    d.rrp.upload(h.R.rp);
    d.rci.upload(h.R.ci);
    upload_cast(d.rv, h.R.v);
    const double w = 2.0 / (1.3 * h.lmax);
    std::vector<double> wd(h.dinv.size());
    for (size_t i = 0; i < wd.size(); ++i) wd[i] = w * h.dinv[i];
    upload_cast(d.wdinv, wd);
    d.b.alloc(std::max(d.n, 1));
    d.x.alloc(std::max(d.n, 1));
    d.xo.alloc(std::max(d.n, 1));
    d.r.alloc(std::max(d.n, 1));
  }
  D.nc = H.coarse.n;
  upload_cast(D.inv, H.coarseInv);
  D.bc.alloc(std::max(D.nc, 1));
  D.xc.alloc(std::max(D.nc, 1));
}

template <typename T> const T *amg_vcycle(AmgDevice<T> &D, const T *b0, cudaStream_t s)
{
  const int L = (int)D.lv.size();
  const T *b = b0;
  for (int l = 0; l < L; ++l) {
    AmgDevLevel<T> &d = D.lv[l];
    if (l > 0) b = d.b.p;
    amg_scale_kernel<T><<<amg_grid(d.n), kAmgThreads, 0, s>>>(d.n, d.wdinv.p, b, d.x.p);
    NRSG_CHECK_LAUNCH();
    spmv<T, kResid>(d.n, (int)d.aci.n, d.arp.p, d.aci.p, d.av.p, d.x.p, b, nullptr, d.r.p, s);
    T *bn = (l + 1 < L) ? D.lv[l + 1].b.p : D.bc.p;
    spmv<T, kPlain>(d.nc, (int)d.rci.n, d.rrp.p, d.rci.p, d.rv.p, d.r.p, nullptr, nullptr, bn, s);
  }
  if (D.nc > 0) {
    if (L == 0) {
      NRSG_CUDA(cudaMemcpyAsync(D.bc.p, b0, sizeof(T) * D.nc, cudaMemcpyDeviceToDevice, s));
    }
    amg_dense_kernel<T><<<(D.nc + 127) / 128, 128, 0, s>>>(D.nc, D.inv.p, D.bc.p, D.xc.p);
    NRSG_CHECK_LAUNCH();
  }
  const T *xcoarse = D.xc.p;
  for (int l = L - 1; l >= 0; --l) {
    AmgDevLevel<T> &d = D.lv[l];
    const T *bl = (l == 0) ? b0 : d.b.p;
    spmv<T, kAdd>(d.n, (int)d.pci.n, d.prp.p, d.pci.p, d.pv.p, xcoarse, nullptr, nullptr, d.x.p, s);
    spmv<T, kSmooth>(d.n, (int)d.aci.n, d.arp.p, d.aci.p, d.av.p, d.x.p, bl, d.wdinv.p, d.xo.p, s);
    xcoarse = d.xo.p;
  }
  return xcoarse;
}

// further V-cycles as a stationary iteration: x += V(b - A_0 x), (cycles - 1) times
template <typename T> void amg_more_cycles(AmgDevice<T> &D, const T *b, T *x, T *r, int cycles, cudaStream_t s)
{
  const bool lv0 = !D.lv.empty();
  const int n = lv0 ? D.lv[0].n : D.nc;
  for (int c = 1; c < cycles; ++c) {
    if (lv0) {
      const AmgDevLevel<T> &d = D.lv[0];
      spmv<T, kResid>(d.n, (int)d.aci.n, d.arp.p, d.aci.p, d.av.p, x, b, nullptr, r, s);
    } else {
      return; // the dense coarsest solve is exact: a further cycle changes nothing
    }
    const T *e = amg_vcycle<T>(D, r, s);
    amg_add_kernel<T><<<amg_grid(n), kAmgThreads, 0, s>>>(n, e, x);
    NRSG_CHECK_LAUNCH();
  }
}

template <typename Ti, typename To>
__global__ void rows_gather_cast_kernel(long long n, const int *rep, const Ti *ev, To *rows)
{
  const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (r < n) rows[r] = (To)ev[rep[r]];
}
template <typename Ti, typename To>
__global__ void rows_scatter_cast_kernel(long long n, const int *rowOf, const Ti *rows, To *ev)
{
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) {
    const int r = rowOf[i];
    ev[i] = r >= 0 ? (To)rows[r] : To(0);
  }
}
void launch_rows_gather_f64_f32(long long nrow, const int *rep, const double *ev, float *rows, cudaStream_t s)
{
  if (nrow <= 0) return;
  rows_gather_cast_kernel<double, float><<<amg_grid(nrow), kAmgThreads, 0, s>>>(nrow, rep, ev, rows);
  NRSG_CHECK_LAUNCH();
}
void launch_rows_scatter_f32_f64(long long n, const int *rowOf, const float *rows, double *ev, cudaStream_t s)
{
  if (n <= 0) return;
  rows_scatter_cast_kernel<float, double><<<amg_grid(n), kAmgThreads, 0, s>>>(n, rowOf, rows, ev);
  NRSG_CHECK_LAUNCH();
}

template <typename T> void launch_rows_gather(long long nrow, const int *rep, const T *ev, T *rows, cudaStream_t s)
{
  if (nrow <= 0) return;
  rows_gather_kernel<T><<<amg_grid(nrow), kAmgThreads, 0, s>>>(nrow, rep, ev, rows);
  NRSG_CHECK_LAUNCH();
}
template <typename T> void launch_rows_scatter(long long n, const int *rowOf, const T *rows, T *ev, cudaStream_t s)
{
  if (n <= 0) return;
  rows_scatter_kernel<T><<<amg_grid(n), kAmgThreads, 0, s>>>(n, rowOf, rows, ev);
  NRSG_CHECK_LAUNCH();
}

#define NRSG_AMG_INST(T)                                                                                     \
  template void amg_upload<T>(const AmgHierarchy &, AmgDevice<T> &);                                         \
  template const T *amg_vcycle<T>(AmgDevice<T> &, const T *, cudaStream_t);                                  \
  template void amg_more_cycles<T>(AmgDevice<T> &, const T *, T *, T *, int, cudaStream_t);                  \
  template void launch_rows_gather<T>(long long, const int *, const T *, T *, cudaStream_t);                 \
  template void launch_rows_scatter<T>(long long, const int *, const T *, T *, cudaStream_t);
NRSG_AMG_INST(float)
NRSG_AMG_INST(double)
#undef NRSG_AMG_INST

} // namespace nrsg
