// Classical algebraic multigrid for the coarsest p-multigrid level: host setup
// (amg.cpp) and the device V-cycle (kernels_amg.cu).
#pragma once

#include "nrsg_internal.hpp"

#include <vector>

namespace nrsg {

struct AmgCsr {
  int n = 0, m = 0; // rows, columns
  std::vector<int> rp, ci;
  std::vector<double> v;
};

struct AmgParams {
  double theta = 0.25; // strength threshold
  int pmax = 4;        // interpolation entries kept per row
  int maxCoarse = 50;  // rows at which the dense coarsest solve takes over
  int maxLevels = 25;
};

struct AmgLevelHost {
  AmgCsr A, P, R;            // operator, interpolation to this level from the next, restriction
  std::vector<double> dinv;  // 1 / a_ii
  double lmax = 0;           // largest eigenvalue of D^-1 A
};

struct AmgHierarchy {
  std::vector<AmgLevelHost> levels; // every level but the coarsest
  AmgCsr coarse;
  std::vector<double> coarseInv;    // dense inverse of the coarsest operator (row major)
  bool invertible = false;
};

void amg_build(long long n, const long long *rowPtr, const long long *col, const double *val, AmgHierarchy &H,
               const AmgParams &prm = AmgParams());

// device copy in precision T and one V-cycle (x = 0 on entry) on row vectors
template <typename T> struct AmgDevLevel {
  int n = 0, nc = 0;
  DevBuf<int> arp, aci, prp, pci, rrp, rci;
  DevBuf<T> av, pv, rv, wdinv, b, x, xo, r;
};
template <typename T> struct AmgDevice {
  std::vector<AmgDevLevel<T>> lv;
  int nc = 0;
  DevBuf<T> inv, bc, xc;
};
template <typename T> void amg_upload(const AmgHierarchy &H, AmgDevice<T> &D);
// b and x: level-0 row vectors (may be D.lv[0].b / the returned pointer); returns the buffer holding x
template <typename T> const T *amg_vcycle(AmgDevice<T> &D, const T *b, cudaStream_t s);
// cycles - 1 further V-cycles on x (level-0 rows; r: scratch of the same size)
template <typename T> void amg_more_cycles(AmgDevice<T> &D, const T *b, T *x, T *r, int cycles, cudaStream_t s);
// E-vector <-> rows of the assembled operator: rows[r] = ev[rep[r]]; ev[i] = rowOf[i] >= 0 ? rows[rowOf[i]] : 0
template <typename T> void launch_rows_gather(long long nrow, const int *rep, const T *ev, T *rows, cudaStream_t s);
template <typename T>
void launch_rows_scatter(long long n, const int *rowOf, const T *rows, T *ev, cudaStream_t s);

// FP64 E-vector -> FP32 rows and back (the SEMFEM preconditioner's pfloat solve)
void launch_rows_gather_f64_f32(long long nrow, const int *rep, const double *ev, float *rows, cudaStream_t s);
void launch_rows_scatter_f32_f64(long long n, const int *rowOf, const float *rows, double *ev, cudaStream_t s);

} // namespace nrsg
