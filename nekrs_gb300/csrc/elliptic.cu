// Elliptic solver driver and C ABI.
//
// Mirrors (nekRS tree):
//   ellipticSolveSetup   src/solvers/elliptic/ellipticSetup.cpp:116-327
//   ellipticSolve        src/solvers/elliptic/ellipticSolve.cpp:32-190
//   ellipticOperator     src/solvers/elliptic/ellipticOperator.cpp:117-172
//   pcg (+ flexible)     src/solvers/elliptic/linearSolver/PCG.cpp:86-203
//   pgmres (+ flexible)  src/solvers/elliptic/linearSolver/PGMRES.cpp:111-340
//   Jacobi               src/solvers/elliptic/ellipticUpdateJacobi.cpp:32-89
//
// GB300 design: one CUDA stream per solver; Krylov scalars stay on the
// device (alpha/beta are formed by the kernels that use them) and the only
// host synchronisation per PCG iteration is an 8-byte read of the residual
// norm for the convergence test.

#include "amg.hpp"
#include "elliptic.hpp"
#include "mg_host.hpp"

#include <chrono>
#include <cmath>
#include <cstring>
#include <atomic>
#include <mutex>

namespace nrsg {

static thread_local std::string g_last_error;
void set_last_error(const std::string &msg) { g_last_error = msg; }
static std::atomic<long long> g_launches{0};
static thread_local long long *t_tally = nullptr;
void count_launch()
{
  if (t_tally)
    ++*t_tally;
  else
    g_launches.fetch_add(1, std::memory_order_relaxed);
}
void set_launch_tally(long long *tally) { t_tally = tally; }
void add_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

// ---------------------------------------------------------------------------
// Level setup
// ---------------------------------------------------------------------------
void FieldLevel::build(int N_, long long E_, const double *VX, const long long *EToV, const int *EToB,
                       const double *h_ggeo, cudaStream_t s)
{
  N = N_;
  Nq = N + 1;
  Np = Nq * Nq * Nq;
  E = E_;
  Nlocal = E * Np;
  gll_nodes(N, z, w);
  diff_matrix(z, Dh);
  d_D64.upload(Dh);
  d_z64.upload(z);
  d_w64.upload(w);
  d_VX64.upload(VX, (size_t)E * 24);
  // geometric factors: caller-provided or computed on the device
  d_ggeo64.alloc((size_t)7 * Nlocal);
  if (h_ggeo) {
    NRSG_CUDA(cudaMemcpy(d_ggeo64.p, h_ggeo, sizeof(double) * 7 * Nlocal, cudaMemcpyHostToDevice));
  } else {
    launch_geofac(N, E, d_VX64.p, d_z64.p, d_w64.p, d_D64.p, d_ggeo64.p, s);
  }
  // numbering, gather maps, mask
  nek_global_ids(N, E, EToV, ids);
  build_gather(ids, um);
  dirichlet_nodes(N, E, EToB, um, maskIds);
  maskedIds = ids;
  for (int m : maskIds) maskedIds[m] = 0;
  build_gather(maskedIds, gm);
  d_gsOff.upload(gm.devOff);
  d_gsIds.upload(gm.devIds);
  d_mask.upload(maskIds);
  d_invDegree64.upload(gm.invDegree);
  ngroups = (long long)gm.devOff.size() - 1;
  {
    std::vector<int2> pairs;
    std::vector<int> roff(1, 0), rids;
    for (long long g = 0; g < ngroups; ++g) {
      const int s0 = gm.devOff[g], s1 = gm.devOff[g + 1];
      if (s1 - s0 == 2) {
        pairs.push_back(make_int2(gm.devIds[s0], gm.devIds[s0 + 1]));
      } else {
        rids.insert(rids.end(), gm.devIds.begin() + s0, gm.devIds.begin() + s1);
        roff.push_back((int)rids.size());
      }
    }
    d_gsPairs.upload(pairs);
    d_gsRestOff.upload(roff);
    d_gsRestIds.upload(rids);
    gsPlan.npairs = (long long)pairs.size();
    gsPlan.nrest = (long long)roff.size() - 1;
    gsPlan.nmask = (long long)maskIds.size();
    gsPlan.pairs = d_gsPairs.p;
    gsPlan.restOff = d_gsRestOff.p;
    gsPlan.restIds = d_gsRestIds.p;
    gsPlan.mask = d_mask.p;
  }
  // volume = sum of JW over the E-vector (meshSetup.cpp:444)
  std::vector<double> gg = d_ggeo64.download();
  volume = 0;
  for (long long e = 0; e < E; ++e)
    for (int n = 0; n < Np; ++n) volume += gg[(size_t)e * 7 * Np + 6 * Np + n];
  VXh.assign(VX, VX + E * 24);
  EToBh.assign(EToB, EToB + E * 6);
  EToVh.assign(EToV, EToV + E * 8);
}

void FieldLevel::make_fp32(cudaStream_t s)
{
  if (d_ggeo32.p) return;
  d_ggeo32.alloc(d_ggeo64.n);
  launch_copy_cast<double, float>((long long)d_ggeo64.n, d_ggeo64.p, d_ggeo32.p, s);
  std::vector<float> D32(Dh.begin(), Dh.end()), z32(z.begin(), z.end()), w32(w.begin(), w.end()), v32(VXh.begin(), VXh.end());
  d_D32.upload(D32);
  d_z32.upload(z32);
  d_w32.upload(w32);
  d_VX32.upload(v32);
  std::vector<float> inv32(gm.invDegree.begin(), gm.invDegree.end());
  d_invDegree32.upload(inv32);
}

// ---------------------------------------------------------------------------
// Elliptic
// ---------------------------------------------------------------------------
Elliptic::Elliptic(const nrsg_mesh_desc *m, const char *options)
{
  if (!m || !m->h_VX || !m->h_EToV || !m->h_EToB) throw Error(NRSG_ERR_INVALID, "mesh description incomplete");
  if (m->N < 1 || m->N > 9) throw Error(NRSG_ERR_BAD_CONFIG, "polynomial order must be 1..9");
  if (m->Nelements < 1) throw Error(NRSG_ERR_BAD_CONFIG, "Nelements must be positive");
  if ((long long)m->Nelements * (m->N + 1) * (m->N + 1) * (m->N + 1) >= (1LL << 31))
    throw Error(NRSG_ERR_BAD_CONFIG, "E*Np must stay below 2^31 (32-bit node indices)");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) throw Error(NRSG_ERR_NO_DEVICE, "no CUDA device");
  opt = parse_options(options);
  NRSG_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  ownStream = true;
  fine.build(m->N, m->Nelements, m->h_VX, m->h_EToV, m->h_EToB, m->h_ggeo, stream);
  if (opt.nfields < 1 || opt.nfields > 3) throw Error(NRSG_ERR_BAD_CONFIG, "nFields must be 1..3");
  if (opt.stress && opt.nfields != 3) throw Error(NRSG_ERR_BAD_CONFIG, "stressFormulation needs the 3-field block solver");
  if (block_mode() && (opt.precon == "multigrid" || opt.axPrecision == "fp32x2" || opt.trilinear))
    throw Error(NRSG_ERR_BAD_CONFIG, "the block solver takes preconditioner = jacobi or none and stored FP64 geometry");
  const long long n = nT();
  // all-Neumann Poisson problem: no face is Dirichlet (ellipticSetup.cpp:187-205)
  if (opt.poisson && opt.nfields == 1) {
    allNeumann = true;
    for (int bc : fine.EToBh)
      if (bc > 0 && bc != NRSG_BC_NEUMANN) { allNeumann = false; break; }
    if (allNeumann) {
      ones.alloc(fine.Nlocal);
      launch_fill<double>(fine.Nlocal, 1.0, ones.p, stream);
      d_sum.alloc(1);
    }
  }
  if (opt.nfields > 1) {
    wBlock.alloc(n);
    for (int f = 0; f < opt.nfields; ++f)
      NRSG_CUDA(cudaMemcpyAsync(wBlock.p + (size_t)f * fine.Nlocal, fine.d_invDegree64.p, sizeof(double) * fine.Nlocal,
                                cudaMemcpyDeviceToDevice, stream));
  }
  if (opt.stress) {
    vgeo.alloc((size_t)12 * fine.Nlocal);
    launch_vgeo(fine.N, fine.E, fine.d_VX64.p, fine.d_z64.p, fine.d_w64.p, fine.d_D64.p, vgeo.p, stream);
  }
  p.alloc(n);
  z.alloc(n);
  Ap.alloc(n);
  x0.alloc(n);
  d_scal.alloc(1);
  NRSG_CUDA(cudaMallocHost((void **)&h_scal, sizeof(PcgScalars)));
  red_partials.alloc((size_t)kRedSlots * kRedSegments);
  red_counters.alloc(kRedSlots);
  NRSG_CUDA(cudaMemsetAsync(red_counters.p, 0, sizeof(unsigned) * kRedSlots, stream));
  NRSG_CUDA(cudaMemsetAsync(d_scal.p, 0, sizeof(PcgScalars), stream));
  red.partials = red_partials.p;
  red.counters = red_counters.p;
  red.slots = kRedSlots;
  NRSG_CUDA(cudaEventCreate(&ev0));
  NRSG_CUDA(cudaEventCreate(&ev1));
  NRSG_CUDA(cudaEventCreateWithFlags(&evRead, cudaEventDisableTiming));

  if (opt.axPrecision == "fp32x2") {
    if (opt.trilinear) throw Error(NRSG_ERR_BAD_CONFIG, "axPrecision = fp32x2 needs stored geometric factors");
    ggeoPairs.alloc(fine.d_ggeo64.n);
    launch_split_pairs((long long)fine.d_ggeo64.n, fine.d_ggeo64.p, ggeoPairs.p, stream);
    std::vector<float2> dp(fine.Dh.size());
    for (size_t q = 0; q < dp.size(); ++q) {
      dp[q].x = (float)fine.Dh[q];
      dp[q].y = (float)(fine.Dh[q] - (double)dp[q].x);
    }
    DPairs.upload(dp);
  }
  if (opt.precon == "jacobi") {
    invDiag.alloc(n);
    build_jacobi();
  } else if (opt.precon == "multigrid") {
    mg_setup();
  } else if (opt.precon == "semfem") {
    semfem_setup();
  }
  if (opt.solver == "pgmres" || opt.solver == "pfgmres") gmres_setup();
  if (opt.projection) {
    if (opt.projVecs < 1 || opt.projVecs > 64) throw Error(NRSG_ERR_BAD_CONFIG, "residualProjectionVectors must be 1..64");
    projXX.alloc((size_t)opt.projVecs * n);
    projBB.alloc((size_t)(opt.projection == 1 ? opt.projVecs : 1) * n);
    projXbar.alloc(n);
    projAlpha.alloc(opt.projVecs);
  }
  NRSG_CUDA(cudaStreamSynchronize(stream));
}

Elliptic::~Elliptic()
{
  if (stream) cudaStreamSynchronize(stream);
  if (h_scal) cudaFreeHost(h_scal);
  if (h_y) cudaFreeHost(h_y);
  if (ev0) cudaEventDestroy(ev0);
  if (ev1) cudaEventDestroy(ev1);
  if (evRead) cudaEventDestroy(evRead);
  graph_release();
  mg_release();
  if (ownStream && stream) cudaStreamDestroy(stream);
}

void Elliptic::ax(const double *q, double *Aq)
{
  if (block_mode()) {
    const double *l0p = coef ? lam0.p : nullptr, *l1p = coef ? lam1.p : nullptr;
    if (opt.stress)
      launch_stress_ax(fine.N, fine.E, fine.Nlocal, loffset, vgeo.p, fine.d_D64.p, l0p, l1p, opt.lambda0,
                       opt.poisson ? 0.0 : opt.lambda1, q, Aq, stream);
    else
      launch_block_ax(fine.N, fine.E, opt.nfields, fine.Nlocal, loffset, fine.d_ggeo64.p, fine.d_D64.p, l0p, l1p,
                      opt.lambda0, opt.lambda1, opt.poisson, q, Aq, stream);
    return;
  }
  if (ggeoPairs.p)
    launch_ax_fp32x2(fine.N, fine.E, ggeoPairs.p, DPairs.p, opt.lambda0, opt.lambda1, opt.poisson, q, Aq, stream);
  else if (opt.trilinear)
    launch_ax_trilinear<double>(fine.N, fine.E, fine.d_VX64.p, fine.d_z64.p, fine.d_w64.p, fine.d_D64.p, opt.lambda0,
                                opt.lambda1, opt.poisson, q, Aq, stream, opt.trilinearLambda0All);
  else
    launch_ax_stored<double>(fine.N, fine.E, fine.d_ggeo64.p, fine.d_D64.p, opt.lambda0, opt.lambda1, opt.poisson, q,
                             Aq, stream);
}

void Elliptic::op(const double *q, double *Aq)
{
  ax(q, Aq);
  gs_mask_fields(Aq); // mask and gather-scatter
}

void Elliptic::gs_mask_fields(double *v)
{
  // zero-normal boundaries first, as ellipticApplyMask (ellipticApplyMask.cpp:19-23)
  if (znNode.n)
    launch_zero_normal((long long)znNode.n, znNode.p, znReps.p, znFrame.p, znMask.p, fine.Nlocal, v, stream);
  for (int f = 0; f < opt.nfields; ++f)
    launch_gs_mask<double>(fieldPlans.empty() ? fine.gsPlan : fieldPlans[f].plan, v + (size_t)f * fine.Nlocal, true,
                           stream);
}

void build_mask_plan(const FieldLevel &L, const int *EToB, FieldMaskPlan &P)
{
  dirichlet_nodes(L.N, L.E, EToB, L.um, P.maskIds);
  std::vector<long long> masked = L.ids;
  for (int m : P.maskIds) masked[m] = 0;
  build_gather(masked, P.gm);
  P.gsOff.upload(P.gm.devOff);
  P.gsIds.upload(P.gm.devIds);
  P.mask.upload(P.maskIds);
  P.ngroups = (long long)P.gm.devOff.size() - 1;
  std::vector<int2> pairs;
  std::vector<int> roff(1, 0), rids;
  for (long long g = 0; g < P.ngroups; ++g) {
    const int s0 = P.gm.devOff[g], s1 = P.gm.devOff[g + 1];
    if (s1 - s0 == 2) {
      pairs.push_back(make_int2(P.gm.devIds[s0], P.gm.devIds[s0 + 1]));
    } else {
      rids.insert(rids.end(), P.gm.devIds.begin() + s0, P.gm.devIds.begin() + s1);
      roff.push_back((int)rids.size());
    }
  }
  P.pairs.upload(pairs);
  P.restOff.upload(roff);
  P.restIds.upload(rids);
  P.plan.npairs = (long long)pairs.size();
  P.plan.nrest = (long long)roff.size() - 1;
  P.plan.nmask = (long long)P.maskIds.size();
  P.plan.pairs = P.pairs.p;
  P.plan.restOff = P.restOff.p;
  P.plan.restIds = P.restIds.p;
  P.plan.mask = P.mask.p;
}

// boundary types per field ([nfields][E][6], nekRS face order): each field gets
// its own mask and gather groups; the Jacobi diagonal is rebuilt
void Elliptic::set_field_bcs(const int *h_EToB)
{
  if (!h_EToB) throw Error(NRSG_ERR_INVALID, "EToB of the fields required");
  if (opt.nfields < 2) throw Error(NRSG_ERR_BAD_CONFIG, "per-field boundary types need the block solver");
  bool zeroNormal = false;
  for (long long q = 0; q < (long long)opt.nfields * fine.E * 6; ++q) {
    if (h_EToB[q] == 3) throw Error(NRSG_ERR_BAD_CONFIG, "zero-tangential boundaries (type 3) are not supported");
    zeroNormal = zeroNormal || h_EToB[q] == 2;
  }
  // the reference takes unaligned boundaries with the three-component block solver only
  // (ellipticSetup.cpp:94-110) and reads their faces from the first field's types (setup.cpp:810-817)
  if (zeroNormal && opt.nfields != 3)
    throw Error(NRSG_ERR_BAD_CONFIG, "zero-normal boundaries (type 2) need the three-field block solver");
  std::vector<FieldMaskPlan> plans(opt.nfields);
  for (int f = 0; f < opt.nfields; ++f) build_mask_plan(fine, h_EToB + (size_t)f * fine.E * 6, plans[f]);
  ZeroNormalPlan zn;
  if (zeroNormal) build_zero_normal(fine, h_EToB, zn);
  NRSG_CUDA(cudaStreamSynchronize(stream));
  graph_release();
  fieldPlans.swap(plans);
  znNode = DevBuf<int>();
  znReps = DevBuf<unsigned char>();
  znFrame = DevBuf<double>();
  znMask = DevBuf<double>();
  if (!zn.node.empty()) {
    znNode.upload(zn.node);
    znReps.upload(zn.reps);
    znFrame.upload(zn.frame);
    znMask.upload(zn.mask);
  }
  if (opt.precon == "jacobi") build_jacobi();
  NRSG_CUDA(cudaStreamSynchronize(stream));
}

// Jacobi: diag(A) per field, gather-scatter, reciprocal
// (ellipticUpdateJacobi.cpp:32-90; block form ellipticBlockBuildDiagonalHex3D)
void Elliptic::build_jacobi()
{
  if (block_mode())
    launch_block_diag(fine.N, fine.E, opt.nfields, fine.Nlocal, loffset, fine.d_ggeo64.p, fine.d_D64.p,
                      coef ? lam0.p : nullptr, coef ? lam1.p : nullptr, opt.lambda0, opt.lambda1, opt.poisson,
                      invDiag.p, stream);
  else
    launch_build_diag<double>(fine.N, fine.E, fine.d_ggeo64.p, fine.d_D64.p, opt.lambda0, opt.lambda1, opt.poisson,
                              invDiag.p, stream);
  for (int f = 0; f < opt.nfields; ++f) {
    if (fieldPlans.empty())
      launch_gs<double>(fine.ngroups, fine.d_gsOff.p, fine.d_gsIds.p, invDiag.p + (size_t)f * fine.Nlocal, stream);
    else
      launch_gs<double>(fieldPlans[f].ngroups, fieldPlans[f].gsOff.p, fieldPlans[f].gsIds.p,
                        invDiag.p + (size_t)f * fine.Nlocal, stream);
  }
  launch_recip<double>(nT(), invDiag.p, stream);
}

// per-node coefficient fields (elliptic->o_lambda0 / o_lambda1, p_lambda = 1):
// loff = 0 shares one array between the fields, loff = Nlocal gives each its own
void Elliptic::set_coefficients(const double *d_lambda0, const double *d_lambda1, long long loff)
{
  if (!d_lambda0) throw Error(NRSG_ERR_INVALID, "lambda0 field required");
  if (loff != 0 && loff != fine.Nlocal) throw Error(NRSG_ERR_INVALID, "loffset must be 0 or E*Np");
  if (opt.precon == "multigrid") throw Error(NRSG_ERR_BAD_CONFIG, "coefficient fields need preconditioner = jacobi or none");
  const size_t n = (size_t)(loff ? opt.nfields : 1) * fine.Nlocal;
  if (lam0.n != n) {
    lam0.alloc(n);
    lam1.alloc(n);
  }
  NRSG_CUDA(cudaMemcpyAsync(lam0.p, d_lambda0, n * sizeof(double), cudaMemcpyDeviceToDevice, stream));
  if (d_lambda1)
    NRSG_CUDA(cudaMemcpyAsync(lam1.p, d_lambda1, n * sizeof(double), cudaMemcpyDeviceToDevice, stream));
  else
    launch_fill<double>((long long)n, 0.0, lam1.p, stream);
  loffset = loff;
  coef = true;
  graph_release();
  if (opt.precon == "jacobi") build_jacobi();
  NRSG_CUDA(cudaStreamSynchronize(stream));
}

void Elliptic::precondition(const double *r, double *zz)
{
  const long long n = nT();
  if (opt.precon == "jacobi") {
    launch_axmyz<double>(n, r, invDiag.p, zz, stream);
  } else if (opt.precon == "multigrid") {
    mg_apply(r, zz);
  } else if (opt.precon == "semfem") {
    // E -> assembled rows (a representative copy), one V-cycle, rows -> every copy (SEMFEMSolver_t::run)
    launch_rows_gather_f64_f32(sfNrow, sfRep.p, r, sfRows.p, stream);
    const float *zr = amg_vcycle<float>(*semfem, sfRows.p, stream);
    launch_rows_scatter_f32_f64(fine.Nlocal, sfRowOf.p, zr, zz, stream);
  } else {
    NRSG_CUDA(cudaMemcpyAsync(zz, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, stream));
  }
  if (allNeumann) zero_mean(zz); // ellipticPreconditioner.cpp:82-83
}

// SEMFEM preconditioner (SEMFEMSolver.cpp:9-158, SEMFEMSolverBuild.cpp): the linear-tetrahedra operator of the
// fine level's GLL nodes, unmasked nodes as unknowns, solved by one algebraic-multigrid V-cycle in FP32
void Elliptic::semfem_setup()
{
  if (block_mode()) throw Error(NRSG_ERR_BAD_CONFIG, "preconditioner = semfem takes the scalar solve");
  if (allNeumann)
    throw Error(NRSG_ERR_BAD_CONFIG, "preconditioner = semfem does not take all-Neumann problems");
  std::vector<double> X, Y, Z;
  trilinear_nodes(fine.N, fine.E, fine.VXh.data(), fine.z, X, Y, Z);
  CsrMatrix A;
  semfem_assemble(fine.N, fine.E, X.data(), Y.data(), Z.data(), fine.gm, fine.maskIds, opt.lambda0, A);
  AmgHierarchy H;
  amg_build(A.nrow, A.rowPtr.data(), A.col.data(), A.val.data(), H);
  if (!H.invertible) throw Error(NRSG_ERR_INVALID, "algebraic multigrid: singular coarsest operator");
  semfem.reset(new AmgDevice<float>());
  amg_upload<float>(H, *semfem);
  std::vector<int> rep((size_t)A.nrow, -1), rowOf(A.rowOfNode.size());
  for (size_t i = 0; i < rowOf.size(); ++i) {
    rowOf[i] = (int)A.rowOfNode[i];
    if (rowOf[i] >= 0 && rep[(size_t)rowOf[i]] < 0) rep[(size_t)rowOf[i]] = (int)i;
  }
  sfRep.upload(rep);
  sfRowOf.upload(rowOf);
  sfNrow = A.nrow;
  sfRows.alloc((size_t)std::max(A.nrow, 1LL));
  sfInfo.clear();
  for (const auto &L : H.levels) {
    sfInfo.push_back(L.A.n);
    sfInfo.push_back((double)L.A.ci.size());
  }
  sfInfo.push_back(H.coarse.n);
  sfInfo.push_back((double)H.coarse.ci.size());
}

// ellipticZeroMean (ellipticZeroMean.cpp:31-44): q -= sum(q) / (E Np) over the E-vector
void Elliptic::zero_mean(double *q)
{
  launch_wdot<double>(fine.Nlocal, nullptr, q, ones.p, d_sum.p, red, 4, stream);
  launch_sub_mean<double>(fine.Nlocal, d_sum.p, (double)fine.Nlocal, q, stream);
}

double Elliptic::read_scalar(const double *d_src)
{
  NRSG_CUDA(cudaMemcpyAsync(&h_scal->pad, d_src, sizeof(double), cudaMemcpyDeviceToHost, stream));
  NRSG_CUDA(cudaStreamSynchronize(stream));
  return h_scal->pad;
}

// PCG / flexible PCG (PCG.cpp:86-203); scalars live in d_scal.  One
// iteration: z = M r, (r, z), (z, Ap_old) for the flexible form, p update,
// A p, (p, A p), x and r update with (r, r); then the 8-byte residual copy to
// pinned host memory and its event.
void Elliptic::pcg_issue_iteration()
{
  const int it = ++st.it;
  if (it >= 2 && graphs_usable()) {
    if (iterGraph.empty() || graphR != st.r || graphX != st.x) {
      try {
        build_iteration_graph();
      } catch (const Error &) {
        graph_release();
        graphsFailed = true; // capture not possible here: stay on ordinary launches
      }
    }
    if (!graphsFailed) {
      for (auto &g : iterGraph) {
        if (g.coarse) {
          mg_coarse_launch();
        } else {
          NRSG_CUDA(cudaGraphLaunch(g.exec, stream));
          add_launches(g.kernels);
        }
      }
      NRSG_CUDA(cudaEventRecord(evRead, stream));
      return;
    }
  }
  issue_iteration_kernels(it == 1);
  NRSG_CUDA(cudaEventRecord(evRead, stream));
}

bool Elliptic::graphs_usable()
{
  if (!opt.graphs || graphsFailed || stream == nullptr) return false;
  if (opt.solver != "pcg" && opt.solver != "pfcg") return false;
  return opt.precon != "multigrid" || mg_graph_capturable();
}

void Elliptic::end_segment()
{
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(stream, &g);
  if (e != cudaSuccess || !g) {
    if (g) cudaGraphDestroy(g);
    capturing = false;
    set_launch_tally(nullptr);
    throw Error(NRSG_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  }
  GraphSeg seg;
  const cudaError_t ei = cudaGraphInstantiate(&seg.exec, g, 0);
  cudaGraphDestroy(g);
  if (ei != cudaSuccess) {
    capturing = false;
    set_launch_tally(nullptr);
    throw Error(NRSG_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ei));
  }
  seg.kernels = capTally;
  iterGraph.push_back(seg);
}

// called by the multigrid at the coarse solve while an iteration is captured
void Elliptic::capture_split()
{
  end_segment();
  GraphSeg c;
  c.coarse = true;
  iterGraph.push_back(c);
  capTally = 0;
  NRSG_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
}

void Elliptic::build_iteration_graph()
{
  graph_release();
  capTally = 0;
  set_launch_tally(&capTally);
  capturing = true;
  const cudaError_t e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    capturing = false;
    set_launch_tally(nullptr);
    throw Error(NRSG_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  }
  try {
    issue_iteration_kernels(false);
  } catch (...) {
    cudaGraph_t g = nullptr;
    cudaStreamEndCapture(stream, &g);
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    capturing = false;
    set_launch_tally(nullptr);
    throw;
  }
  end_segment();
  capturing = false;
  set_launch_tally(nullptr);
  graphR = st.r;
  graphX = st.x;
}

void Elliptic::graph_release()
{
  for (auto &g : iterGraph)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  iterGraph.clear();
  graphR = graphX = nullptr;
}

void Elliptic::issue_iteration_kernels(bool first)
{
  const long long n = nT();
  const double *wt = wT();
  const bool flexible = (opt.solver == "pfcg");
  PcgScalars *sc = d_scal.p;
  double *r = st.r, *x = st.x;
  if (opt.precon == "jacobi" && !allNeumann) {
    launch_jacobi_rdotz(n, wt, invDiag.p, r, z.p, sc, red, 0, stream);
  } else {
    const double *zz = r;
    if (opt.precon != "none") {
      precondition(r, z.p);
      zz = z.p;
    } else {
      NRSG_CUDA(cudaMemcpyAsync(z.p, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, stream));
    }
    launch_scalar_move(&sc->rdotz_old, &sc->rdotz, nullptr, stream);
    launch_wdot<double>(n, wt, r, zz, &sc->rdotz, red, 0, stream);
  }
  if (flexible && !first) launch_wdot<double>(n, wt, z.p, Ap.p, &sc->zAp, red, 1, stream);
  launch_update_p(n, z.p, p.p, sc, first, flexible, stream);
  op(p.p, Ap.p);
  launch_wdot<double>(n, wt, p.p, Ap.p, &sc->pAp, red, 2, stream);
  launch_update_xr(n, wt, p.p, Ap.p, x, r, sc, red, 3, stream);
  NRSG_CUDA(cudaMemcpyAsync(&h_scal->rdotr, &sc->rdotr, sizeof(double), cudaMemcpyDeviceToHost, stream));
}

void Elliptic::finish_issue()
{
  if (opt.projection) proj_post(st.x);
  launch_axpby<double>(nT(), 1.0, x0.p, 1.0, st.x, stream);
  if (allNeumann) zero_mean(st.x); // ellipticSolve.cpp:188-189
  NRSG_CUDA(cudaEventRecord(ev1, stream));
  st.phase = 3;
}

// ---- solution projection (ellipticSolutionProjection.cpp) ----------------
// pre (:143-182, :262-272): alpha_k = (x_k, r)_invDegree, xbar = sum alpha_k x_k,
// r -= A xbar (A-conjugate) or r -= sum alpha_k b_k (classic, b_k = A x_k).
void Elliptic::proj_pre(double *r)
{
  const long long n = nT();
  ++projStep;
  if (projStep < opt.projStart || projM <= 0) return;
  const double *w = wT();
  launch_multi_wdot(n, w, projXX.p, projM, r, projAlpha.p, red, 0, stream);
  launch_accumulate(n, projM, projAlpha.p, projXX.p, projXbar.p, stream);
  if (opt.projection == 1)
    launch_accumulate(n, projM, projAlpha.p, projBB.p, z.p, stream);
  else
    op(projXbar.p, z.p);
  launch_axpby<double>(n, -1.0, z.p, 1.0, r, stream);
}

// updateProjectionSpace (:40-140): A-orthonormalise the newest basis vector
// by one classical Gram-Schmidt pass; drop it when it is dependent (1e-7).
void Elliptic::proj_update_space()
{
  const long long n = nT();
  const int m = projM;
  if (m <= 0) return;
  const bool classic = opt.projection == 1;
  const double *w = wT();
  const double *b = projBB.p + (size_t)(classic ? m - 1 : 0) * n;
  launch_multi_wdot(n, w, projXX.p, m, b, projAlpha.p, red, 0, stream);
  std::vector<double> alpha(m);
  NRSG_CUDA(cudaMemcpyAsync(alpha.data(), projAlpha.p, sizeof(double) * m, cudaMemcpyDeviceToHost, stream));
  launch_multi_scaled_sub(n, m, projAlpha.p, projXX.p, stream);
  if (classic) launch_multi_scaled_sub(n, m, projAlpha.p, projBB.p, stream);
  NRSG_CUDA(cudaStreamSynchronize(stream));
  const double normOrig = alpha[m - 1];
  double sumAlpha = 0;
  for (int k = 0; k < m - 1; ++k) sumAlpha += alpha[k] * alpha[k];
  const double normNew = std::sqrt(normOrig - sumAlpha);
  if (normNew / normOrig > 1e-7) {
    const double sc = 1.0 / normNew;
    launch_scale_inplace(n, sc, projXX.p + (size_t)(m - 1) * n, stream);
    if (classic) launch_scale_inplace(n, sc, projBB.p + (size_t)(m - 1) * n, stream);
  } else {
    --projM;
  }
}

// post (:183-221, :273-279): the correction x joins the basis; x += xbar
void Elliptic::proj_post(double *x)
{
  const long long n = nT();
  if (projStep < opt.projStart) return;
  const size_t bytes = sizeof(double) * n;
  if (projM == 0) {
    projM = 1;
    NRSG_CUDA(cudaMemcpyAsync(projXX.p, x, bytes, cudaMemcpyDeviceToDevice, stream));
  } else if (projM == opt.projVecs) {
    projM = 1;
    launch_axpby<double>(n, 1.0, projXbar.p, 1.0, x, stream);
    NRSG_CUDA(cudaMemcpyAsync(projXX.p, x, bytes, cudaMemcpyDeviceToDevice, stream));
  } else {
    ++projM;
    NRSG_CUDA(cudaMemcpyAsync(projXX.p + (size_t)(projM - 1) * n, x, bytes, cudaMemcpyDeviceToDevice, stream));
    launch_axpby<double>(n, 1.0, projXbar.p, 1.0, x, stream);
  }
  const int prev = projM;
  const int bOff = opt.projection == 1 ? projM - 1 : 0;
  op(projXX.p + (size_t)(projM - 1) * n, projBB.p + (size_t)bOff * n);
  proj_update_space();
  if (projM < prev) { // the new vector was dependent: restart the space from x
    projM = 1;
    NRSG_CUDA(cudaMemcpyAsync(projXX.p, x, bytes, cudaMemcpyDeviceToDevice, stream));
    op(projXX.p, projBB.p);
    proj_update_space();
  }
}

void Elliptic::begin(double *r, double *x)
{
  if (st.phase != 0 && st.phase != 4) throw Error(NRSG_ERR_INVALID, "a solve is already in progress on this handle");
  const long long n = nT();
  history.clear();
  status = NRSG_OK;
  st = StepState();
  st.r = r;
  st.x = x;
  mg_clear_error();
  NRSG_CUDA(cudaEventRecord(ev0, stream));
  // r = b - A x0 (local Ax, ellipticSolve.cpp:91-103), mask, gather-scatter
  ax(x, Ap.p);
  launch_axpby<double>(n, -1.0, Ap.p, 1.0, r, stream);
  if (allNeumann) zero_mean(r); // ellipticSolve.cpp:101
  gs_mask_fields(r); // mask and gather-scatter
  NRSG_CUDA(cudaMemcpyAsync(x0.p, x, sizeof(double) * n, cudaMemcpyDeviceToDevice, stream));
  launch_fill<double>(n, 0.0, x, stream);
  if (opt.projection) proj_pre(r);
  launch_wdot<double>(n, wT(), r, nullptr, &d_scal.p->rdotr, red, 0, stream);
  NRSG_CUDA(cudaMemcpyAsync(&h_scal->rdotr, &d_scal.p->rdotr, sizeof(double), cudaMemcpyDeviceToHost, stream));
  NRSG_CUDA(cudaEventRecord(evRead, stream));
  st.phase = 1;
}

static bool event_done(cudaEvent_t ev, bool block)
{
  if (block) {
    NRSG_CUDA(cudaEventSynchronize(ev));
    return true;
  }
  const cudaError_t e = cudaEventQuery(ev);
  if (e == cudaErrorNotReady) return false;
  NRSG_CUDA(e);
  return true;
}

bool Elliptic::advance(bool block, nrsg_solve_info *info)
{
  for (;;) {
    if (st.phase == 1) {
      if (!event_done(evRead, block)) return false;
      // res0Norm = weightedNorm2Many * sqrt(resNormFactor) (ellipticSolve.cpp:130-139)
      st.res0 = std::sqrt(h_scal->rdotr) * std::sqrt(1.0 / fine.volume);
      if (!std::isfinite(st.res0)) {
        st.phase = 4;
        throw Error(NRSG_ERR_NAN, "unreasonable res0Norm (NaN/Inf right-hand side)");
      }
      st.tol = opt.relative ? opt.tol * st.res0 : opt.tol;
      st.res = st.res0;
      if (st.res0 > 0 && opt.maxIter > 0) {
        if (opt.solver == "pcg" || opt.solver == "pfcg") {
          launch_fill<double>(nT(), 0.0, p.p, stream);
          pcg_issue_iteration();
          st.phase = 2;
        } else {
          double res = st.res0;
          st.it = pgmres(st.r, st.x, st.tol, opt.maxIter, res);
          st.res = res;
          finish_issue();
        }
      } else {
        finish_issue();
      }
    } else if (st.phase == 2) {
      if (!event_done(evRead, block)) return false;
      // rdotr = sqrt(update() * resNormFactor) (PCG.cpp:189)
      const double rnorm = std::sqrt(h_scal->rdotr * (1.0 / fine.volume));
      history.push_back(rnorm);
      st.res = rnorm;
      if (!std::isfinite(rnorm)) {
        status = NRSG_ERR_NAN;
        finish_issue();
      } else if (rnorm > st.tol && st.it < opt.maxIter) {
        pcg_issue_iteration();
        if (!block) return false;
      } else {
        finish_issue();
      }
    } else if (st.phase == 3) {
      if (!event_done(ev1, block)) return false;
      float ms = 0;
      NRSG_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
      if (status == NRSG_OK && st.it >= opt.maxIter && st.res > st.tol) status = NRSG_ERR_MAXIT;
      if (const int me = mg_error()) {
        status = NRSG_ERR_CUDA;
        set_last_error(me == 2   ? "pipelined axhelm: a bulk copy did not complete within its wait limit"
                       : me == 3 ? "tensor-core FDM: an MMA completion wait exceeded its limit"
                                 : "coarse-level solver: grid barrier wait exceeded its limit");
      }
      lastIters = st.it;
      st.info.iterations = st.it;
      st.info.status = status;
      st.info.res0 = st.res0;
      st.info.res = st.res;
      st.info.solve_ms = ms;
      st.phase = 4;
      if (info) *info = st.info;
      return true;
    } else if (st.phase == 4) {
      if (info) *info = st.info;
      return true;
    } else {
      throw Error(NRSG_ERR_INVALID, "no solve in progress on this handle");
    }
  }
}

int Elliptic::solve(double *r, double *x, nrsg_solve_info *info)
{
  begin(r, x);
  advance(true, info);
  return status;
}

} // namespace nrsg

// ===========================================================================
// C ABI
// ===========================================================================
using nrsg::Elliptic;
using nrsg::Error;

struct nrsg_elliptic {
  std::unique_ptr<Elliptic> impl;
};

#define NRSG_TRY(...)                                                                                     \
  try {                                                                                                    \
    __VA_ARGS__;                                                                                           \
    return NRSG_OK;                                                                                        \
  } catch (const Error &e) {                                                                               \
    nrsg::set_last_error(e.what());                                                                        \
    return e.code;                                                                                         \
  } catch (const std::bad_alloc &) {                                                                       \
    nrsg::set_last_error("host allocation failed");                                                        \
    return NRSG_ERR_OOM;                                                                                   \
  } catch (const std::exception &e) {                                                                      \
    nrsg::set_last_error(e.what());                                                                        \
    return NRSG_ERR_INVALID;                                                                               \
  }

extern "C" {

const char *nrsg_last_error(void) { return nrsg::g_last_error.c_str(); }
int nrsg_version(void) { return 1; }
long long nrsg_kernel_launches(void) { return nrsg::g_launches.load(); }

int nrsg_elliptic_create(const nrsg_mesh_desc *mesh, const char *options, nrsg_elliptic **out)
{
  if (!out) return NRSG_ERR_INVALID;
  *out = nullptr;
  NRSG_TRY({
    auto h = new nrsg_elliptic();
    size_t free0 = 0, free1 = 0, total = 0;
    NRSG_CUDA(cudaDeviceSynchronize());
    NRSG_CUDA(cudaMemGetInfo(&free0, &total));
    try {
      h->impl.reset(new Elliptic(mesh, options));
    } catch (...) {
      delete h;
      throw;
    }
    NRSG_CUDA(cudaDeviceSynchronize());
    NRSG_CUDA(cudaMemGetInfo(&free1, &total));
    h->impl->deviceBytes = free0 > free1 ? (long long)(free0 - free1) : 0;
    *out = h;
  })
}

int nrsg_elliptic_destroy(nrsg_elliptic *el)
{
  NRSG_TRY(delete el)
}

int nrsg_elliptic_set_stream(nrsg_elliptic *el, void *s)
{
  if (!el) return NRSG_ERR_INVALID;
  NRSG_TRY({
    auto &E = *el->impl;
    NRSG_CUDA(cudaStreamSynchronize(E.stream));
    if (E.ownStream) cudaStreamDestroy(E.stream);
    E.stream = (cudaStream_t)s;
    E.ownStream = false;
  })
}

int nrsg_elliptic_solve(nrsg_elliptic *el, double *d_r, double *d_x, nrsg_solve_info *info)
{
  if (!el || !d_r || !d_x) return NRSG_ERR_INVALID;
  try {
    return el->impl->solve(d_r, d_x, info);
  } catch (const Error &e) {
    nrsg::set_last_error(e.what());
    if (info) info->status = e.code;
    return e.code;
  } catch (const std::exception &e) {
    nrsg::set_last_error(e.what());
    return NRSG_ERR_INVALID;
  }
}

int nrsg_elliptic_set_tolerance(nrsg_elliptic *el, double tol, int relative, int maxIterations)
{
  if (!el || !(tol > 0) || maxIterations < 1) return NRSG_ERR_INVALID;
  NRSG_TRY({
    auto &E = *el->impl;
    if (E.st.phase != 0 && E.st.phase != 4) throw Error(NRSG_ERR_INVALID, "a solve is in progress on this handle");
    E.opt.tol = tol;
    E.opt.relative = relative != 0;
    E.opt.maxIter = maxIterations;
  })
}

int nrsg_elliptic_solve_begin(nrsg_elliptic *el, double *d_r, double *d_x)
{
  if (!el || !d_r || !d_x) return NRSG_ERR_INVALID;
  NRSG_TRY(el->impl->begin(d_r, d_x))
}

int nrsg_elliptic_solve_advance(nrsg_elliptic *el, int *done, nrsg_solve_info *info)
{
  if (!el || !done) return NRSG_ERR_INVALID;
  *done = 0;
  try {
    if (el->impl->advance(false, info)) {
      *done = 1;
      return el->impl->st.info.status;
    }
    return NRSG_OK;
  } catch (const Error &e) {
    nrsg::set_last_error(e.what());
    *done = 1;
    return e.code;
  } catch (const std::exception &e) {
    nrsg::set_last_error(e.what());
    *done = 1;
    return NRSG_ERR_INVALID;
  }
}

int nrsg_elliptic_solve_batch(int n, nrsg_elliptic *const *els, double *const *d_r, double *const *d_x,
                              nrsg_solve_info *info)
{
  if (n < 0 || (n > 0 && (!els || !d_r || !d_x))) return NRSG_ERR_INVALID;
  std::vector<int> state(n, 0); // 0 running, 1 done
  std::vector<int> code(n, NRSG_OK);
  for (int k = 0; k < n; ++k) {
    code[k] = nrsg_elliptic_solve_begin(els[k], d_r[k], d_x[k]);
    if (code[k] != NRSG_OK) state[k] = 1;
  }
  int left = 0;
  for (int k = 0; k < n; ++k) left += state[k] == 0;
  while (left > 0) {
    for (int k = 0; k < n; ++k) {
      if (state[k]) continue;
      int done = 0;
      const int c = nrsg_elliptic_solve_advance(els[k], &done, info ? &info[k] : nullptr);
      if (done) {
        state[k] = 1;
        code[k] = c;
        --left;
      }
    }
  }
  for (int k = 0; k < n; ++k)
    if (code[k] != NRSG_OK && code[k] != NRSG_ERR_MAXIT) return code[k];
  for (int k = 0; k < n; ++k)
    if (code[k] != NRSG_OK) return code[k];
  return NRSG_OK;
}

int nrsg_elliptic_solve_host(nrsg_elliptic *el, double *h_r, double *h_x, nrsg_solve_info *info)
{
  if (!el || !h_r || !h_x) return NRSG_ERR_INVALID;
  try {
    auto &E = *el->impl;
    const size_t bytes = sizeof(double) * E.nT();
    if (!E.io_r.p) { E.io_r.alloc(E.nT()); E.io_x.alloc(E.nT()); }
    NRSG_CUDA(cudaMemcpyAsync(E.io_r.p, h_r, bytes, cudaMemcpyHostToDevice, E.stream));
    NRSG_CUDA(cudaMemcpyAsync(E.io_x.p, h_x, bytes, cudaMemcpyHostToDevice, E.stream));
    const int st = E.solve(E.io_r.p, E.io_x.p, info);
    NRSG_CUDA(cudaMemcpyAsync(h_r, E.io_r.p, bytes, cudaMemcpyDeviceToHost, E.stream));
    NRSG_CUDA(cudaMemcpyAsync(h_x, E.io_x.p, bytes, cudaMemcpyDeviceToHost, E.stream));
    NRSG_CUDA(cudaStreamSynchronize(E.stream));
    return st;
  } catch (const Error &e) {
    nrsg::set_last_error(e.what());
    return e.code;
  } catch (const std::exception &e) {
    nrsg::set_last_error(e.what());
    return NRSG_ERR_INVALID;
  }
}

int nrsg_elliptic_operator(nrsg_elliptic *el, const double *d_q, double *d_Aq)
{
  if (!el || !d_q || !d_Aq) return NRSG_ERR_INVALID;
  NRSG_TRY({
    el->impl->op(d_q, d_Aq);
    NRSG_CUDA(cudaStreamSynchronize(el->impl->stream));
  })
}
int nrsg_elliptic_ax(nrsg_elliptic *el, const double *d_q, double *d_Aq)
{
  if (!el || !d_q || !d_Aq) return NRSG_ERR_INVALID;
  NRSG_TRY({
    el->impl->ax(d_q, d_Aq);
    NRSG_CUDA(cudaStreamSynchronize(el->impl->stream));
  })
}
int nrsg_elliptic_gs(nrsg_elliptic *el, double *d_q)
{
  if (!el || !d_q) return NRSG_ERR_INVALID;
  NRSG_TRY({
    auto &E = *el->impl;
    nrsg::launch_gs_mask<double>(E.fine.gsPlan, d_q, false, E.stream);
    NRSG_CUDA(cudaStreamSynchronize(E.stream));
  })
}
int nrsg_elliptic_mask(nrsg_elliptic *el, double *d_q)
{
  if (!el || !d_q) return NRSG_ERR_INVALID;
  NRSG_TRY({
    auto &E = *el->impl;
    nrsg::launch_mask<double>((long long)E.fine.maskIds.size(), E.fine.d_mask.p, d_q, E.stream);
    NRSG_CUDA(cudaStreamSynchronize(E.stream));
  })
}
int nrsg_elliptic_precondition(nrsg_elliptic *el, const double *d_r, double *d_z)
{
  if (!el || !d_r || !d_z) return NRSG_ERR_INVALID;
  NRSG_TRY({
    el->impl->precondition(d_r, d_z);
    NRSG_CUDA(cudaStreamSynchronize(el->impl->stream));
  })
}

int nrsg_elliptic_get(nrsg_elliptic *el, const char *name, void *h_out, long long *count)
{
  if (!el || !name || !count) return NRSG_ERR_INVALID;
  NRSG_TRY({
    auto &E = *el->impl;
    auto &L = E.fine;
    const std::string s(name);
    auto put = [&](const auto &v) {
      *count = (long long)v.size();
      if (h_out && !v.empty()) std::memcpy(h_out, v.data(), v.size() * sizeof(v[0]));
    };
    if (s == "ids") put(L.ids);
    else if (s == "maskedIds") put(L.maskedIds);
    else if (s == "gsOff") put(L.gm.off);
    else if (s == "gsIds") put(L.gm.ids);
    else if (s == "maskIds") put(L.maskIds);
    else if (s == "invDegree") put(L.gm.invDegree);
    else if (s == "D") put(L.Dh);
    else if (s == "history") put(E.history);
    else if (s == "semfemLevels") put(E.sfInfo);
    else if (s == "deviceBytes") put(std::vector<double>{(double)E.deviceBytes});
    else if (s == "allNeumann") put(std::vector<double>{E.allNeumann ? 1.0 : 0.0});
    else if (s == "proj.vectors") put(std::vector<double>{(double)E.projM, (double)E.projStep});
    else if (s == "graph.segments") {
      // segments of the captured steady-state iteration (0: ordinary launches), and how many are coarse solves
      long long nc = 0;
      for (auto &g : E.iterGraph) nc += g.coarse ? 1 : 0;
      put(std::vector<double>{(double)E.iterGraph.size(), (double)nc, E.graphsFailed ? 1.0 : 0.0});
    } else if (s == "ggeo") put(L.d_ggeo64.download());
    else if (s == "invDiag") put(E.invDiag.download());
    else if (s == "x" || s == "y" || s == "z") {
      std::vector<double> X, Y, Z;
      nrsg::trilinear_nodes(L.N, L.E, L.VXh.data(), L.z, X, Y, Z);
      put(s == "x" ? X : (s == "y" ? Y : Z));
    } else if (s.rfind("mg.", 0) == 0) {
      put(E.mg_get(s));
    } else
      throw Error(NRSG_ERR_INVALID, "unknown array '" + s + "'");
  })
}

int nrsg_elliptic_mg_smoother(nrsg_elliptic *el, int level, const double *d_u, double *d_Su)
{
  if (!el || !d_u || !d_Su) return NRSG_ERR_INVALID;
  NRSG_TRY(el->impl->mg_schwarz(level, d_u, d_Su))
}
int nrsg_elliptic_mg_fdm(nrsg_elliptic *el, int level, const void *d_u, void *d_Su)
{
  if (!el || !d_u || !d_Su) return NRSG_ERR_INVALID;
  NRSG_TRY(el->impl->mg_fdm(level, d_u, d_Su))
}
long long nrsg_elliptic_mg_level_size(nrsg_elliptic *el, int level)
{
  if (!el) return -1;
  try {
    return el->impl->mg_level_size(level);
  } catch (const std::exception &e) {
    nrsg::set_last_error(e.what());
    return -1;
  }
}

// ---- host-only setup (no device needed) -----------------------------------
double nrsg_host_hessenberg_rho(int n, const double *h_H)
{
  if (n < 1 || !h_H) return -1.0;
  try {
    return nrsg::hessenberg_spectral_radius(n, std::vector<double>(h_H, h_H + (size_t)n * n));
  } catch (const std::exception &e) {
    nrsg::set_last_error(e.what());
    return -1.0;
  }
}

int nrsg_host_setup_maps(int N, long long E, const long long *h_EToV, const int *h_EToB, long long *h_ids,
                         long long *h_maskedIds, double *h_invDegree, int *h_maskIds, long long *nmask, int *h_gsOff,
                         long long *ngroups, int *h_gsIds)
{
  if (N < 1 || E < 1 || !h_EToV || !h_EToB) return NRSG_ERR_INVALID;
  NRSG_TRY({
    std::vector<long long> ids;
    nrsg::nek_global_ids(N, E, h_EToV, ids);
    nrsg::GatherMap um, gm;
    nrsg::build_gather(ids, um);
    std::vector<int> mask;
    nrsg::dirichlet_nodes(N, E, h_EToB, um, mask);
    std::vector<long long> masked = ids;
    for (int m : mask) masked[m] = 0;
    nrsg::build_gather(masked, gm);
    if (h_ids) std::memcpy(h_ids, ids.data(), ids.size() * sizeof(long long));
    if (h_maskedIds) std::memcpy(h_maskedIds, masked.data(), masked.size() * sizeof(long long));
    if (h_invDegree) std::memcpy(h_invDegree, gm.invDegree.data(), gm.invDegree.size() * sizeof(double));
    if (h_maskIds) std::memcpy(h_maskIds, mask.data(), mask.size() * sizeof(int));
    if (nmask) *nmask = (long long)mask.size();
    if (h_gsOff) std::memcpy(h_gsOff, gm.off.data(), gm.off.size() * sizeof(int));
    if (ngroups) *ngroups = (long long)gm.off.size() - 1;
    if (h_gsIds) std::memcpy(h_gsIds, gm.ids.data(), gm.ids.size() * sizeof(int));
  })
}

int nrsg_host_assemble_operator(int N, long long E, const long long *h_EToV, const int *h_EToB, const double *h_ggeo,
                                double lambda0, double lambda1, int poisson, long long *nrow, long long *nnz,
                                long long *h_rowPtr, long long *h_cols, double *h_vals, long long *h_rowOfNode)
{
  if (N < 1 || E < 1 || !h_EToV || !h_EToB || !h_ggeo || !nrow || !nnz) return NRSG_ERR_INVALID;
  NRSG_TRY({
    std::vector<long long> ids;
    nrsg::nek_global_ids(N, E, h_EToV, ids);
    nrsg::GatherMap um, gm;
    nrsg::build_gather(ids, um);
    std::vector<int> mask;
    nrsg::dirichlet_nodes(N, E, h_EToB, um, mask);
    for (int m : mask) ids[m] = 0;
    nrsg::build_gather(ids, gm);
    std::vector<double> z, w, D;
    nrsg::gll_nodes(N, z, w);
    nrsg::diff_matrix(z, D);
    nrsg::CsrMatrix A;
    nrsg::assemble_level(N, E, D, h_ggeo, lambda0, lambda1, poisson != 0, gm, A);
    *nrow = A.nrow;
    *nnz = A.rowPtr[A.nrow];
    if (h_rowPtr) std::memcpy(h_rowPtr, A.rowPtr.data(), A.rowPtr.size() * sizeof(long long));
    if (h_cols) std::memcpy(h_cols, A.col.data(), A.col.size() * sizeof(long long));
    if (h_vals) std::memcpy(h_vals, A.val.data(), A.val.size() * sizeof(double));
    if (h_rowOfNode) std::memcpy(h_rowOfNode, A.rowOfNode.data(), A.rowOfNode.size() * sizeof(long long));
  })
}

int nrsg_host_assemble_galerkin(int Nf, long long E, const long long *h_EToV, const int *h_EToB,
                                const double *h_ggeo_fine, double lambda0, double lambda1, int poisson,
                                long long *nrow, long long *nnz, long long *h_rowPtr, long long *h_cols,
                                double *h_vals, long long *h_rowOfNode)
{
  if (Nf < 1 || E < 1 || !h_EToV || !h_EToB || !h_ggeo_fine || !nrow || !nnz) return NRSG_ERR_INVALID;
  NRSG_TRY({
    std::vector<long long> ids;
    nrsg::nek_global_ids(1, E, h_EToV, ids);
    nrsg::GatherMap um, gm;
    nrsg::build_gather(ids, um);
    std::vector<int> mask;
    nrsg::dirichlet_nodes(1, E, h_EToB, um, mask);
    for (int m : mask) ids[m] = 0;
    nrsg::build_gather(ids, gm);
    std::vector<double> z, w, D;
    nrsg::gll_nodes(Nf, z, w);
    nrsg::diff_matrix(z, D);
    std::vector<double> Ae;
    nrsg::galerkin_element_matrices(Nf, E, D, z, h_ggeo_fine, lambda0, lambda1, poisson != 0, Ae);
    nrsg::CsrMatrix A;
    nrsg::assemble_rows(8, E, Ae, gm, A);
    *nrow = A.nrow;
    *nnz = A.rowPtr[A.nrow];
    if (h_rowPtr) std::memcpy(h_rowPtr, A.rowPtr.data(), A.rowPtr.size() * sizeof(long long));
    if (h_cols) std::memcpy(h_cols, A.col.data(), A.col.size() * sizeof(long long));
    if (h_vals) std::memcpy(h_vals, A.val.data(), A.val.size() * sizeof(double));
    if (h_rowOfNode) std::memcpy(h_rowOfNode, A.rowOfNode.data(), A.rowOfNode.size() * sizeof(long long));
  })
}

int nrsg_host_assemble_semfem(int N, long long E, const double *h_VX, const long long *h_EToV, const int *h_EToB,
                              double lambda0, long long *nrow, long long *nnz, long long *h_rowPtr, long long *h_cols,
                              double *h_vals, long long *h_rowOfNode)
{
  if (N < 1 || E < 1 || !h_VX || !h_EToV || !h_EToB || !nrow || !nnz) return NRSG_ERR_INVALID;
  NRSG_TRY({
    std::vector<long long> ids;
    nrsg::nek_global_ids(N, E, h_EToV, ids);
    nrsg::GatherMap um, gm;
    nrsg::build_gather(ids, um);
    std::vector<int> mask;
    nrsg::dirichlet_nodes(N, E, h_EToB, um, mask);
    for (int m : mask) ids[m] = 0;
    nrsg::build_gather(ids, gm);
    std::vector<double> z, w, X, Y, Z;
    nrsg::gll_nodes(N, z, w);
    nrsg::trilinear_nodes(N, E, h_VX, z, X, Y, Z);
    nrsg::CsrMatrix A;
    nrsg::semfem_assemble(N, E, X.data(), Y.data(), Z.data(), gm, mask, lambda0, A);
    *nrow = A.nrow;
    *nnz = A.rowPtr[A.nrow];
    if (h_rowPtr) std::memcpy(h_rowPtr, A.rowPtr.data(), A.rowPtr.size() * sizeof(long long));
    if (h_cols) std::memcpy(h_cols, A.col.data(), A.col.size() * sizeof(long long));
    if (h_vals) std::memcpy(h_vals, A.val.data(), A.val.size() * sizeof(double));
    if (h_rowOfNode) std::memcpy(h_rowOfNode, A.rowOfNode.data(), A.rowOfNode.size() * sizeof(long long));
  })
}

// ---- kernel-level entry points --------------------------------------------
int nrsg_ax_stored_f64(int N, long long E, const double *ggeo, const double *D, double l0, double l1, int poisson,
                       const double *q, double *Aq, void *s)
{
  NRSG_TRY(nrsg::launch_ax_stored<double>(N, E, ggeo, D, l0, l1, poisson != 0, q, Aq, (cudaStream_t)s))
}
int nrsg_ax_stored_f32(int N, long long E, const float *ggeo, const float *D, float l0, float l1, int poisson,
                       const float *q, float *Aq, void *s)
{
  NRSG_TRY(nrsg::launch_ax_stored<float>(N, E, ggeo, D, l0, l1, poisson != 0, q, Aq, (cudaStream_t)s))
}

int nrsg_ax_const_f32(int N, long long E, const float *ggeo, const float *D, float l0, float l1, int poisson,
                      const float *q, float *Aq, void *s)
{
  if (N != 7 || E < 1 || !ggeo || !D || !q || !Aq) return NRSG_ERR_INVALID;
  NRSG_TRY(nrsg::launch_ax_const(N, E, ggeo, D, l0, l1, poisson != 0, q, Aq, (cudaStream_t)s))
}
int nrsg_ax_const_prefetch_f32(int N, long long E, const float *ggeo, const float *D, float l0, float l1, int poisson,
                               const float *q, float *Aq, void *s)
{
  if (N != 7 || E < 1 || !ggeo || !D || !q || !Aq) return NRSG_ERR_INVALID;
  NRSG_TRY(nrsg::launch_ax_const(N, E, ggeo, D, l0, l1, poisson != 0, q, Aq, (cudaStream_t)s, true))
}

int nrsg_elliptic_set_field_bcs(nrsg_elliptic *el, const int *h_EToB)
{
  if (!el) return NRSG_ERR_INVALID;
  NRSG_TRY(el->impl->set_field_bcs(h_EToB))
}

int nrsg_elliptic_set_coefficients(nrsg_elliptic *el, const double *d_lambda0, const double *d_lambda1,
                                   long long loffset)
{
  if (!el) return NRSG_ERR_INVALID;
  NRSG_TRY(el->impl->set_coefficients(d_lambda0, d_lambda1, loffset))
}

int nrsg_ax_pipe_f32(int N, long long E, const float *ggeo, const float *D, float l0, float l1, int poisson,
                     const float *q, float *Aq, void *s)
{
  if (N != 7 || E < 1 || !ggeo || !D || !q || !Aq || (((uintptr_t)ggeo | (uintptr_t)q) & 15)) return NRSG_ERR_INVALID;
  NRSG_TRY(nrsg::launch_ax_pipe(N, E, ggeo, D, l0, l1, poisson != 0, q, Aq, (cudaStream_t)s))
}
int nrsg_ax_trilinear_f64(int N, long long E, const double *VX, const double *z, const double *w, const double *D,
                          double l0, double l1, int poisson, const double *q, double *Aq, void *s)
{
  NRSG_TRY(nrsg::launch_ax_trilinear<double>(N, E, VX, z, w, D, l0, l1, poisson != 0, q, Aq, (cudaStream_t)s))
}
int nrsg_ax_trilinear_f32(int N, long long E, const float *VX, const float *z, const float *w, const float *D,
                          float l0, float l1, int poisson, const float *q, float *Aq, void *s)
{
  NRSG_TRY(nrsg::launch_ax_trilinear<float>(N, E, VX, z, w, D, l0, l1, poisson != 0, q, Aq, (cudaStream_t)s))
}
int nrsg_ax_fp32x2(int N, long long E, const void *ggeo_pairs, const void *D_pairs, double l0, double l1, int poisson,
                   const double *q, double *Aq, void *s)
{
  NRSG_TRY(nrsg::launch_ax_fp32x2(N, E, (const float2 *)ggeo_pairs, (const float2 *)D_pairs, l0, l1, poisson != 0, q,
                                  Aq, (cudaStream_t)s))
}
int nrsg_split_pairs(long long n, const double *x, void *pairs, void *s)
{
  NRSG_TRY(nrsg::launch_split_pairs(n, x, (float2 *)pairs, (cudaStream_t)s))
}
int nrsg_gs_add_f64(long long ng, const int *off, const int *ids, double *q, void *s)
{
  NRSG_TRY(nrsg::launch_gs<double>(ng, off, ids, q, (cudaStream_t)s))
}
int nrsg_gs_add_f32(long long ng, const int *off, const int *ids, float *q, void *s)
{
  NRSG_TRY(nrsg::launch_gs<float>(ng, off, ids, q, (cudaStream_t)s))
}
int nrsg_mask_f64(long long n, const int *ids, double *q, void *s)
{
  NRSG_TRY(nrsg::launch_mask<double>(n, ids, q, (cudaStream_t)s))
}

namespace {
// scratch for the kernel-level reduction entry points (one per device)
struct KernelScratch {
  nrsg::DevBuf<double> partials;
  nrsg::DevBuf<unsigned> counters;
  nrsg::Reduce red;
  int device = -1;
};
std::mutex g_ks_mutex;
KernelScratch &kernel_scratch()
{
  static KernelScratch ks[16];
  int dev = 0;
  NRSG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 16) throw Error(NRSG_ERR_INVALID, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_ks_mutex);
  KernelScratch &k = ks[dev];
  if (k.device != dev) {
    k.partials.alloc(nrsg::kRedSegments);
    k.counters.alloc(1);
    NRSG_CUDA(cudaMemset(k.counters.p, 0, sizeof(unsigned)));
    k.red.partials = k.partials.p;
    k.red.counters = k.counters.p;
    k.red.slots = 1;
    k.device = dev;
  }
  return k;
}
} // namespace

int nrsg_update_pcg_f64(long long n, const double *w, const double *p, const double *Ap, double alpha, double *x,
                        double *r, double *rdotr, void *s)
{
  NRSG_TRY({
    auto &k = kernel_scratch();
    nrsg::launch_update_pcg_alpha(n, w, p, Ap, alpha, x, r, rdotr, k.red, 0, (cudaStream_t)s);
  })
}
int nrsg_weighted_inner_prod_f64(long long n, const double *w, const double *a, const double *b, double *out, void *s)
{
  NRSG_TRY({
    auto &k = kernel_scratch();
    nrsg::launch_wdot<double>(n, w, a, b, out, k.red, 0, (cudaStream_t)s);
  })
}
int nrsg_geometric_factors_f64(int N, long long E, const double *VX, double *ggeo, void *s)
{
  NRSG_TRY({
    std::vector<double> z, w, D;
    nrsg::gll_nodes(N, z, w);
    nrsg::diff_matrix(z, D);
    nrsg::DevBuf<double> dz, dw, dD;
    dz.upload(z);
    dw.upload(w);
    dD.upload(D);
    nrsg::launch_geofac(N, E, VX, dz.p, dw.p, dD.p, ggeo, (cudaStream_t)s);
    NRSG_CUDA(cudaStreamSynchronize((cudaStream_t)s));
  })
}

} // extern "C"

// ---------------------------------------------------------------------------
// Algebraic multigrid of an assembled operator (the coarse solve of
// coarseSolver = amg), in the form of the reference's BoomerAMG wrapper
// (hypreWrapper.hpp: boomerAMG_t(nrows, nnz, Ai, Aj, Av, ...) and solve(b, x))
// ---------------------------------------------------------------------------
struct nrsg_amg {
  nrsg::AmgHierarchy H;
  nrsg::AmgDevice<double> D;
  bool uploaded = false;
};

extern "C" {

int nrsg_amg_create(long long nrow, const long long *h_rowPtr, const long long *h_col, const double *h_val,
                    nrsg_amg **out)
{
  NRSG_TRY({
    if (!out || nrow <= 0 || !h_rowPtr || !h_col || !h_val) throw Error(NRSG_ERR_INVALID, "matrix required");
    auto *a = new nrsg_amg();
    try {
      nrsg::amg_build(nrow, h_rowPtr, h_col, h_val, a->H);
      if (!a->H.invertible) throw Error(NRSG_ERR_INVALID, "algebraic multigrid: singular coarsest operator");
    } catch (...) {
      delete a;
      throw;
    }
    *out = a;
  })
}

int nrsg_amg_destroy(nrsg_amg *a) { NRSG_TRY(delete a) }

int nrsg_amg_num_levels(const nrsg_amg *a, int *nlevels)
{
  NRSG_TRY({
    if (!a || !nlevels) throw Error(NRSG_ERR_INVALID, "handle required");
    *nlevels = (int)a->H.levels.size() + 1;
  })
}

int nrsg_amg_level_matrix(const nrsg_amg *a, int level, int which, long long *nrow, long long *ncol, long long *nnz,
                          long long *h_rowPtr, int *h_col, double *h_val, double *lmax)
{
  NRSG_TRY({
    if (!a) throw Error(NRSG_ERR_INVALID, "handle required");
    const int L = (int)a->H.levels.size();
    if (level < 0 || level > L || which < 0 || which > 1 || (level == L && which == 1))
      throw Error(NRSG_ERR_INVALID, "no such level matrix");
    const nrsg::AmgCsr &M = level == L ? a->H.coarse : (which == 0 ? a->H.levels[level].A : a->H.levels[level].P);
    if (nrow) *nrow = M.n;
    if (ncol) *ncol = M.m;
    if (nnz) *nnz = (long long)M.ci.size();
    if (h_rowPtr)
      for (int i = 0; i <= M.n; ++i) h_rowPtr[i] = M.rp[i];
    if (h_col) std::copy(M.ci.begin(), M.ci.end(), h_col);
    if (h_val) std::copy(M.v.begin(), M.v.end(), h_val);
    if (lmax) *lmax = level < L ? a->H.levels[level].lmax : 0.0;
  })
}

int nrsg_amg_vcycle(nrsg_amg *a, const double *d_b, double *d_x, void *stream)
{
  NRSG_TRY({
    if (!a || !d_b || !d_x) throw Error(NRSG_ERR_INVALID, "handle and vectors required");
    cudaStream_t s = (cudaStream_t)stream;
    if (!a->uploaded) {
      nrsg::amg_upload<double>(a->H, a->D);
      a->uploaded = true;
    }
    const double *x = nrsg::amg_vcycle<double>(a->D, d_b, s);
    const long long n = a->H.levels.empty() ? a->H.coarse.n : a->H.levels[0].A.n;
    NRSG_CUDA(cudaMemcpyAsync(d_x, x, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    NRSG_CUDA(cudaStreamSynchronize(s));
  })
}

} // extern "C"
