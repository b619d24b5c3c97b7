// ORACLE — test infrastructure only (see oracle_mesh.cpp header).
#pragma once
#include "oracle.hpp"

#include <cmath>
#include <memory>
#include <vector>

namespace orc {

// Mesh data of one polynomial order (a pMG level or the fine mesh).
struct Level {
  int N = 0, Nq = 0, Np = 0;
  long long E = 0, Nlocal = 0;
  std::vector<double> z, w, D;            // GLL nodes/weights, D[i*Nq+m] = l_m'(z_i)
  std::vector<double> x, y, zc;           // node coordinates
  std::vector<double> ggeo;               // [e][7][Np]
  std::vector<long long> ids, maskedIds;  // global ids (0 = not gathered)
  std::vector<int> gsOff, gsIds;          // masked gather groups (CSR)
  std::vector<double> invDegree;
  std::vector<int> maskIds;
  double volume = 0;
  std::vector<double> VX;                 // [e][8 hypercube][3]
  std::vector<int> EToB;
  std::vector<long long> EToV;
};

void build_level(Level &L, int N, long long E, const double *VX, const long long *EToV, const int *EToB);

template <typename T>
void ax_stored(const Level &L, const T *ggeo, const T *D, T lambda0, T lambda1, bool poisson, const T *q, T *Aq);
void ax_trilinear(const Level &L, double lambda0, double lambda1, bool poisson, bool lambda0All, const double *q,
                  double *Aq);
template <typename T>
void build_diag(const Level &L, const T *ggeo, const T *D, T lambda0, T lambda1, bool poisson, T *diag);
template <typename T> void gs_add(const Level &L, T *q);
template <typename T> void apply_mask(const Level &L, T *q);
template <typename T> T wdot(long long n, const T *w, const T *a, const T *b);
void ax_stored_dev(const Level &L, const double *ggeo, const double *D, double lambda0, double lambda1, bool poisson,
                   const double *q, double *Aq);

// Sum over i < n in the device library's reduction order: entry i
// contributes s = fma(x_i, y_i, s), f(i, x, y) giving the factors.  Chunk c
// = entries [1024 c, 1024 c + 1024); lane l (0..31) accumulates entries
// 1024 c + l + 32 j for j ascending from s = 0 (entries past n skipped); the
// 32 lane sums are added by the tree s[l] += s[l + o], o = 16, 8, 4, 2, 1;
// the chunk sums by the blocked pairwise tree ((P0 + P1) + (P2 + P3)) + ...,
// zero-padded to a power of two.
template <typename F> double wsum(long long n, const F &f)
{
  const long long nc = (n + 1023) / 1024;
  if (nc <= 0) return 0.0;
  long long M = 1;
  while (M < nc) M <<= 1;
  std::vector<double> P((size_t)M, 0.0);
#pragma omp parallel for schedule(static)
  for (long long c = 0; c < nc; ++c) {
    double s[32];
    for (int l = 0; l < 32; ++l) {
      double acc = 0.0;
      for (int j = 0; j < 32; ++j) {
        const long long i = c * 1024 + l + 32 * j;
        if (i < n) {
          double x, y;
          f(i, x, y);
          acc = std::fma(x, y, acc);
        }
      }
      s[l] = acc;
    }
    for (int o = 16; o >= 1; o >>= 1)
      for (int l = 0; l < o; ++l) s[l] = s[l] + s[l + o];
    P[(size_t)c] = s[0];
  }
  for (long long len = M; len > 1; len >>= 1)
    for (long long x = 0; x < len / 2; ++x) P[(size_t)x] = P[(size_t)(2 * x)] + P[(size_t)(2 * x + 1)];
  return P[0];
}

void assemble_fem(const Level &L, double lambda0, double lambda1, bool poisson, std::vector<long long> &rowPtr,
                  std::vector<long long> &cols, std::vector<double> &vals);
void assemble_semfem(const Level &L, double lambda0, std::vector<long long> &rowPtr, std::vector<long long> &cols,
                     std::vector<double> &vals);
void assemble_galerkin(const Level &F, const Level &C, double lambda0, double lambda1, bool poisson,
                       std::vector<long long> &rowPtr, std::vector<long long> &cols, std::vector<double> &vals);

struct MG; // multigrid state (oracle_mg.cpp)

struct Elliptic {
  Options o;
  Level fine;
  std::vector<double> invDiag;            // Jacobi preconditioner
  std::shared_ptr<MG> mg;
  std::vector<double> history;            // residual norm per iteration
  bool allNeumann = false;                // Poisson with no Dirichlet face: constant null space
  void zero_mean(double *q) const;
  int status = 0;                         // 0 ok, 1 max-iterations, 3 NaN

  void setup(int N, long long E, const double *VX, const long long *EToV, const int *EToB, const std::string &opt);
  void ax(const double *q, double *Aq) const;      // FP64 operator in the device's operation order
  void ax_ref(const double *q, double *Aq) const;  // the reference serial kernel's operation order
  void op(const double *q, double *Aq) const;
  void precond(const double *r, double *z);
  double norm(const double *r) const;
  int pcg(double *r, double *x, double tol, int maxit, double &rnorm);
  int pgmres(double *r, double *x, double tol, int maxit, double &rnorm);
  int solve(double *r, double *x, double &res0, double &res);
  // solution projection state (ellipticSolutionProjection.cpp)
  std::vector<double> projXX, projBB, projXbar;
  int projM = 0, projStep = 0;
  void proj_pre(double *r);
  void proj_post(double *x);
  void proj_update_space();
};

void mg_setup(Elliptic &el);
void mg_apply(Elliptic &el, const double *r, double *z);
std::vector<double> mg_info(const Elliptic &el, const std::string &what);
void mg_level_smooth_schwarz(Elliptic &el, int level, const double *u, double *Su);
long long mg_level_size(Elliptic &el, int level);
std::vector<double> mg_level_array(Elliptic &el, int level, const std::string &name);
double hessenberg_rho_public(int n, const double *Hcol);
void mg_level_transfer(Elliptic &el, int level, bool restrict_, const double *in, double *out);

} // namespace orc
