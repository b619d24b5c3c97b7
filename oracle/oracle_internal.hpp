// ORACLE — test infrastructure only (see oracle_mesh.cpp header).
#pragma once
#include "oracle.hpp"

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
void ax_trilinear(const Level &L, double lambda0, double lambda1, bool poisson, const double *q, double *Aq);
template <typename T>
void build_diag(const Level &L, const T *ggeo, const T *D, T lambda0, T lambda1, bool poisson, T *diag);
template <typename T> void gs_add(const Level &L, T *q);
template <typename T> void apply_mask(const Level &L, T *q);
template <typename T> T wdot(long long n, const T *w, const T *a, const T *b);

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
  void ax(const double *q, double *Aq) const;
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
