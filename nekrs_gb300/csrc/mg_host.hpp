// Host-side p-multigrid setup helpers (mg_setup.cpp).
#pragma once

#include "elliptic.hpp"

#include <map>
#include <vector>

namespace nrsg {

struct MGPlan {
  std::vector<int> orders;     // down-leg polynomial orders, finest first
  std::map<int, int> down, up; // Chebyshev degree per order (-1 / absent: default)
  int base = 0;                // 0 Jacobi, 1 ASM, 2 RAS
  int kind = 0;                // 0 1st-kind, 1 4th-kind, 2 optimal 4th-kind Chebyshev
};
MGPlan plan_levels(const Options &o, int N);
const std::vector<double> &opt4_betas(int degree);

struct FdmLengths {
  std::vector<double> left, mid, right; // [E][3] (x, y, z)
};
FdmLengths fdm_lengths(const FieldLevel &fine, const GatherMap &unmaskedFine);
void fdm_1d_operator(const FieldLevel &L, int lbc, int rbc, double ll, double lm, double lr, std::vector<double> &S,
                     std::vector<double> &lam);
void fdm_halo_maps(const FieldLevel &L, std::vector<int> &haloSrc, std::vector<int> &haloPartner,
                   std::vector<double> &wts);
double hessenberg_spectral_radius(int n, const std::vector<double> &Hcol);

// assembled level operator on the unmasked unique nodes (CSR, columns ascending)
struct CsrMatrix {
  long long nrow = 0;
  std::vector<long long> rowPtr, col, rowOfNode; // rowOfNode: E-vector node -> row, -1 where masked
  std::vector<double> val;
};
void assemble_level(int N, long long E, const std::vector<double> &Dh, const double *ggeo, double lam0, double lam1,
                    bool poisson, const GatherMap &gm, CsrMatrix &A);
void assemble_rows(int np, long long E, const std::vector<double> &Ae, const GatherMap &gm, CsrMatrix &A);
void semfem_assemble(int N, long long E, const double *x, const double *y, const double *z, const GatherMap &gm,
                     const std::vector<int> &maskIds, double lam0, CsrMatrix &A);
void galerkin_element_matrices(int Nf, long long E, const std::vector<double> &Dh, const std::vector<double> &z,
                               const double *ggeo, double lam0, double lam1, bool poisson, std::vector<double> &Ae);

} // namespace nrsg
