// ORACLE — test infrastructure only (see oracle_mesh.cpp header).
#pragma once
#include <array>
#include <string>
#include <vector>

namespace orc {

void gll(int N, double *z, double *w);
void dmatrix(int N, const double *z, double *D);
void interp_matrix(int nin, const double *zin, int nout, const double *zout, double *I);
void kershaw_map(double epsy, double epsz, double x, double y, double z, double &xx, double &yy, double &zz);
void box_mesh(int nx, int ny, int nz, double eps, double *VX, long long *EToV, int *EToB, int allDirichlet);
void trilinear_coords(int N, long long E, const double *VX, const double *z1, double *x, double *y, double *z);
void geometric_factors(int N, long long E, const double *D, const double *w, const double *x, const double *y,
                       const double *z, double *ggeo, double *J);
void global_ids(int N, long long E, const long long *EToV, long long *ids);
void ogs_setup(long long Nlocal, const long long *ids, std::vector<int> &offsets, std::vector<int> &gids,
               std::vector<double> &invDegree);
void dirichlet_mask(int N, long long E, const int *EToB, const std::vector<int> &offsets, const std::vector<int> &gids,
                    std::vector<int> &maskIds);

// Parsed solver options (subset of the .par [PRESSURE] keys that reach the path)
struct Options {
  std::string solver = "pcg";            // pcg | pfcg | pgmres | pfgmres
  int nVector = 15;                      // (F)GMRES restart length
  double tol = 1e-8;
  bool relative = true;
  int maxIter = 500;
  std::string precon = "jacobi";         // none | jacobi | multigrid
  std::string smoother = "cheby+jac";    // cheby|fourthcheby|fourthoptcheby + jac|asm|ras
  int chebyDegree = 2;
  double minEigFactor = 0.1, maxEigFactor = 1.1;
  std::string schedule;                  // pMGSchedule
  std::string coarse = "jpcg";           // jpcg (on-device Jacobi-PCG) | smooth
  double coarseTol = 1e-4;
  int coarseMaxIter = 200;
  bool galerkin = false;                 // coarseGridDiscretization = FEM+Galerkin
  bool semfem = false;                   // coarseGridDiscretization = SEMFEM
  std::string mgPrecision = "fp64";      // fp64 | fp32
  bool poisson = true;
  double lambda0 = 1.0, lambda1 = 0.0;
  bool trilinear = false;                // ELEMENT MAP = TRILINEAR
  bool trilinearLambda0All = false;      // lambda0 on every flux (the reference: the t-flux only)
  unsigned long long seed = 0x5eed;      // Arnoldi start vector seed
  int projection = 0;                    // INITIAL GUESS: 0 none, 1 PROJECTION (classic), 2 PROJECTION-ACONJ
  int projVecs = 8;                      // RESIDUAL PROJECTION VECTORS
  int projStart = 5;                     // RESIDUAL PROJECTION START
};
Options parse_options(const std::string &text);

} // namespace orc
