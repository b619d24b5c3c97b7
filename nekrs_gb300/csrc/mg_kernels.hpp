// Launchers of the p-multigrid kernels (kernels_mg.cu, kernels_vec.cu).
#pragma once

#include "nrsg_internal.hpp"

namespace nrsg {

template <typename T> void launch_coarsen(int Nf, int Nc, long long E, const T *R, const T *qf, T *qc, cudaStream_t s);
template <typename T> void launch_prolong(int Nf, int Nc, long long E, const T *R, const T *qc, T *qf, cudaStream_t s);
template <typename T>
void launch_cheby1_update(long long n, T dc, T rc, const T *SAd, T *d, T *r, T *x, cudaStream_t s);
template <typename T>
void launch_cheby4_update(long long n, T beta, const T *Ad, const T *d, const T *rin, T *rout, T *x, bool xzero,
                          cudaStream_t s);
// 4th-kind Chebyshev with the x update where each direction is formed: d = c1 Su (first) or c1 Su + c2 d,
// x = beta d (xzero) or x + beta d; and the residual update rout = rin - Ad
template <typename T>
void launch_cheby4_dx(long long n, T c1, const T *Su, T c2, T *d, T beta, T *x, bool first, bool xzero,
                      cudaStream_t s);
template <typename T> void launch_cheby4_res(long long n, const T *Ad, const T *rin, T *rout, cudaStream_t s);
// generic: the line-per-thread kernel even where a specialised one applies (FP32 orders 3 and 7)
template <typename T>
void launch_fdm(int N, long long E, bool ras, const T *u, const int *haloSrc, const T *Sx, const T *Sy, const T *Sz,
                const T *invL, const T *lam, const T *wts, T *Su, T *haloOut, cudaStream_t s, bool generic = false);
// order-7 RAS FDM in FP16 on the tensor cores (per-element max-abs scaling); false if not applicable
bool launch_fdm8h(long long E, const float *u, const int *haloSrc, const float *Sx, const float *Sy, const float *Sz,
                  const float *lam, const float *wts, float *Su, cudaStream_t s);
// the FDM in TF32 on the tensor cores (orders 3, 5, 7; RAS or ASM; needs the 1-D eigenvalues); false when
// the level is not covered
bool launch_fdm_tf32(int N, long long E, bool ras, const float *u, const int *haloSrc, const float *Sx,
                     const float *Sy, const float *Sz, const float *lam, const float *wts, float *Su, float *haloOut,
                     cudaStream_t s);
// the order-7 RAS FDM in TF32 on the 5th-generation tensor cores (tcgen05.mma, accumulator in tensor
// memory); false when not applicable.  fdm_tc_error reads and clears its bounded-wait error flag.
bool launch_fdm_tc(long long E, const float *u, const int *haloSrc, const float *Sx, const float *Sy, const float *Sz,
                   const float *lam, const float *wts, float *Su, cudaStream_t s);
unsigned fdm_tc_error(cudaStream_t s);
template <typename T>
void launch_asm_combine(int N, long long E, const int *haloPartner, const T *haloOut, const T *wts, T *Su,
                        cudaStream_t s);
void launch_random_fill(long long n, unsigned long long seed, double *v, cudaStream_t s);

// Jacobi-PCG in precision T with double scalars (coarse-level solve)
template <typename T>
void launch_pcg_rdotz(long long n, const T *w, const T *invDiag, const T *r, T *z, PcgScalars *sc, Reduce &red, int slot,
                      cudaStream_t s);
template <typename T> void launch_pcg_p(long long n, const T *z, T *p, const PcgScalars *sc, bool first, cudaStream_t s);
template <typename T>
void launch_pcg_xr(long long n, const T *w, const T *p, const T *Ap, T *x, T *r, PcgScalars *sc, Reduce &red, int slot,
                   cudaStream_t s);

// assembled level operator on the device, partitioned into one row block per
// CTA (kernels_coarse.cu)
template <typename T> struct CoarseMatrix {
  long long nrow = 0, nE = 0, nnz = 0;
  int width = 0, grid = 0, chunk = 0, maxHalo = 0;
  int threads = 1024;            // threads per CTA: the row block rounded up to a warp, at most 1024
  bool matInSmem = false;
  bool pipelined = false;        // one-barrier pipelined PCG (FP32)
  int cluster = 0;               // > 0: the grid is one thread-block cluster of this many CTAs (hardware barrier)
  size_t smem = 0;               // dynamic shared memory per CTA
  DevBuf<unsigned short> lcol;   // [grid][width][chunk] local column: own row, or chunk + halo slot
  DevBuf<T> val;                 // [grid][width][chunk], padding 0
  DevBuf<int> haloOff, haloIds;  // per CTA: rows of other blocks it reads
  DevBuf<T> invDiag;             // [nrow]
  DevBuf<int> rep;               // [nrow] an E-vector node of each row
  DevBuf<int> rowOf;             // [nE] row of each E-vector node, -1 where masked
};
// noCluster: the many-CTA cooperative layout even where one thread-block cluster would hold the level
template <typename T>
void coarse_matrix_setup(long long n, const long long *rowPtr, const long long *col, const double *val, long long nE,
                         const long long *rowOfNode, const int *rep, CoarseMatrix<T> &M, bool noCluster = false);

// persistent cooperative Jacobi-PCG on the assembled coarse operator: b and xE
// are E-vectors, x, z and z2 row vectors (solution rows, two exchange
// buffers); returns the grid size used.  `state` holds coarse_state_bytes()
// bytes, `partials` 6 * gridMax doubles.
// Every grid-barrier wait gives up after spinLimit polls and sets the state's
// error flag; barrierExtra (0 in use) is added to every barrier's target.
template <typename T>
int coarse_pcg_persistent(const CoarseMatrix<T> &A, const T *b, T *xE, T *x, T *z, T *z2, double *partials,
                          void *state, int gridMax, double tol, int maxit, cudaStream_t s,
                          long long spinLimit = 1LL << 22, unsigned barrierExtra = 0);
size_t coarse_state_bytes();
// zero the whole state, error flag included (once per outer solve)
void coarse_state_clear(void *state, cudaStream_t s);
// decode a host copy of the state; returns the error flag (0 = ok)
int coarse_state_read(const void *state_host, int *iters, double *res0, double *res);

} // namespace nrsg
