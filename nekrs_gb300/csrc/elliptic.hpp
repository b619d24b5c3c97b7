// Solver state of one elliptic problem (the elliptic_t counterpart).
#pragma once

#include "amg.hpp"
#include "nrsg_internal.hpp"

#include <memory>
#include <string>
#include <vector>

namespace nrsg {

// Mesh data of one polynomial order on the device (fine level or pMG level).
struct FieldLevel {
  int N = 0, Nq = 0, Np = 0;
  long long E = 0, Nlocal = 0;
  std::vector<double> z, w, Dh;
  std::vector<long long> ids, maskedIds;
  GatherMap gm;  // masked (the solver's gather-scatter)
  GatherMap um;  // unmasked (mesh->ogs)
  std::vector<int> maskIds;
  std::vector<double> VXh;
  std::vector<int> EToBh;
  std::vector<long long> EToVh;
  double volume = 0;
  long long ngroups = 0;
  DevBuf<double> d_ggeo64, d_D64, d_z64, d_w64, d_VX64, d_invDegree64;
  DevBuf<float> d_ggeo32, d_D32, d_z32, d_w32, d_VX32, d_invDegree32;
  DevBuf<int> d_gsOff, d_gsIds, d_mask;
  DevBuf<int2> d_gsPairs;                // gather-scatter plan (pairs + other groups + mask)
  DevBuf<int> d_gsRestOff, d_gsRestIds;
  GsPlan gsPlan;

  void build(int N, long long E, const double *VX, const long long *EToV, const int *EToB, const double *h_ggeo,
             cudaStream_t s);
  void make_fp32(cudaStream_t s);
};

// Mask and gather-scatter of one field of a block solve whose boundary types
// differ from the level's (elliptic->EToB holds Nfields sections in the
// reference, ellipticSetup.cpp:190-199): its own Dirichlet nodes and the
// gather groups of its unmasked nodes.
struct FieldMaskPlan {
  std::vector<int> maskIds;
  GatherMap gm;
  DevBuf<int> gsOff, gsIds, mask, restOff, restIds;
  DevBuf<int2> pairs;
  GsPlan plan;
  long long ngroups = 0;
};
void build_mask_plan(const FieldLevel &L, const int *EToB, FieldMaskPlan &P);

// zero-normal (symmetry) boundaries of any orientation, face type 2 of the first field (three fields):
// one entry per node of an element on the element's zero-normal faces
struct ZeroNormalPlan {
  std::vector<int> node;           // E-vector index
  std::vector<unsigned char> reps; // zero-normal faces of the element through the node
  std::vector<double> frame;       // n, t1, t2 per entry
  std::vector<double> mask;        // maskN, maskT1, maskT2 per entry
};
void build_zero_normal(const FieldLevel &L, const int *EToB0, ZeroNormalPlan &P);

struct MGState;   // p-multigrid hierarchy (mg.cu)
struct MGDeleter {
  void operator()(MGState *m) const;
};

struct Elliptic {
  static constexpr int kRedSlots = 8;
  Options opt;
  cudaStream_t stream = nullptr;
  bool ownStream = false;
  FieldLevel fine;

  // Krylov workspace (elliptic.h:240-262 slices)
  DevBuf<double> p, z, Ap, x0, invDiag;
  DevBuf<float2> ggeoPairs, DPairs;     // axPrecision = fp32x2
  DevBuf<double> io_r, io_x;            // staging for the host-buffer solve
  DevBuf<PcgScalars> d_scal;
  PcgScalars *h_scal = nullptr;          // pinned
  DevBuf<double> red_partials;
  DevBuf<unsigned> red_counters;
  Reduce red;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;

  // GMRES workspace
  DevBuf<double> gV, gZ, gW, gB, gY;
  double *h_y = nullptr;                  // pinned: y[0..nr] + nw

  // Block (vector) solve: nfields fields at fieldOffset = Nlocal, weights
  // invDegree repeated per field; optional per-node coefficients
  // (elliptic->o_lambda0 / o_lambda1 with loffset); stress form on vgeo.
  DevBuf<double> wBlock, lam0, lam1, vgeo;
  bool coef = false;
  long long loffset = 0;
  long long nT() const { return fine.Nlocal * opt.nfields; }
  const double *wT() const { return opt.nfields > 1 ? wBlock.p : fine.d_invDegree64.p; }
  bool block_mode() const { return opt.nfields > 1 || coef || opt.stress; }
  void gs_mask_fields(double *v);
  std::vector<FieldMaskPlan> fieldPlans; // empty: every field uses the level's mask
  // preconditioner = semfem: algebraic multigrid on the low-order (linear tetrahedra) operator of the fine
  // level's GLL nodes (SEMFEMSolver.cpp), in FP32
  std::unique_ptr<AmgDevice<float>> semfem;
  DevBuf<int> sfRep, sfRowOf;
  DevBuf<float> sfRows;
  long long sfNrow = 0;
  std::vector<double> sfInfo; // rows and nonzeros per level
  void semfem_setup();
  DevBuf<int> znNode;                    // zero-normal entries (empty: none)
  DevBuf<unsigned char> znReps;
  DevBuf<double> znFrame, znMask;
  void set_field_bcs(const int *h_EToB);
  // null space of the all-Neumann Poisson operator (ellipticSetup.cpp:187-205):
  // remove the E-vector mean from r, z and x (ellipticZeroMean)
  bool allNeumann = false;
  DevBuf<double> ones, d_sum;
  void zero_mean(double *q);
  void build_jacobi();
  void set_coefficients(const double *d_lambda0, const double *d_lambda1, long long loff);

  std::unique_ptr<MGState, MGDeleter> mg;
  std::vector<double> history;
  int status = NRSG_OK;
  int lastIters = 0;
  long long deviceBytes = 0; // device memory the handle took at creation (admission estimate for serving)

  Elliptic(const nrsg_mesh_desc *mesh, const char *options);
  ~Elliptic();

  void ax(const double *q, double *Aq);
  void op(const double *q, double *Aq);
  void precondition(const double *r, double *z);
  double read_scalar(const double *d_src);
  void gmres_setup();
  int pgmres(double *r, double *x, double tol, int maxit, double &rnorm);
  int solve(double *r, double *x, nrsg_solve_info *info);

  // Resumable solve (PCG / flexible PCG): begin() queues the initial residual,
  // advance() consumes each residual norm once its copy has landed and queues
  // the next iteration; with block = false it never waits on the device.
  // solve() is begin() + advance(block = true).  GMRES runs inside begin().
  struct StepState {
    int phase = 0; // 0 idle, 1 res0 in flight, 2 iteration in flight, 3 final update in flight, 4 done
    double *r = nullptr, *x = nullptr;
    double res0 = 0, tol = 0, res = 0;
    int it = 0;
    nrsg_solve_info info{};
  } st;
  cudaEvent_t evRead = nullptr;
  void begin(double *r, double *x);
  bool advance(bool block, nrsg_solve_info *info);
  void pcg_issue_iteration();
  void issue_iteration_kernels(bool first);
  void finish_issue();

  // CUDA graphs of the steady-state PCG iteration (iterations 2, 3, ...),
  // split at the persistent coarse solve, which stays an ordinary launch
  // (ordered against every other solver's, see kernels_coarse.cu).  Used on
  // non-legacy streams; rebuilt when the solve's r / x change.
  struct GraphSeg {
    cudaGraphExec_t exec = nullptr;
    bool coarse = false;
    long long kernels = 0;
  };
  std::vector<GraphSeg> iterGraph;
  double *graphR = nullptr, *graphX = nullptr;
  bool capturing = false, graphsFailed = false;
  long long capTally = 0;
  bool graphs_usable();
  void build_iteration_graph();
  void end_segment();
  void capture_split();
  void graph_release();
  void mg_coarse_launch();
  bool mg_graph_capturable();

  // Solution projection for the initial guess (SolutionProjection,
  // ellipticSolutionProjection.cpp): a basis of up to projVecs previous
  // solutions, A-orthonormal (A-conjugate form) or with their A-images
  // (classic form); pre() runs on the device without host reads, post()
  // reads the Gram-Schmidt coefficients for its dependence test.
  DevBuf<double> projXX, projBB, projXbar, projAlpha;
  int projM = 0, projStep = 0;
  void proj_pre(double *r);
  void proj_post(double *x);
  void proj_update_space();

  void mg_setup();
  void mg_apply(const double *r, double *z);
  void mg_release();
  int mg_error();
  void mg_clear_error(); // clears the coarse kernel's sticky error flag (solve begin)
  std::vector<double> mg_get(const std::string &name);
  long long mg_level_size(int level);
  void mg_schwarz(int level, const double *u, double *Su);
  void mg_fdm(int level, const void *u, void *Su);
};

// GMRES kernels (kernels_vec.cu)
void launch_multi_wdot(long long n, const double *w, const double *V, int nvec, const double *x, double *out,
                       Reduce &red, int slot, cudaStream_t s);
void launch_gram_schmidt(long long n, const double *w, const double *V, int nvec, const double *y, double *x,
                         double *nrm2, Reduce &red, int slot, cudaStream_t s);
void launch_gmres_update(long long n, const double *V, int nvec, const double *y, double *x, cudaStream_t s);
void launch_residual_norm(long long n, const double *w, const double *b, const double *Ax, double *r, double *nrm2,
                          Reduce &red, int slot, cudaStream_t s);

} // namespace nrsg
