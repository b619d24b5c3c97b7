/*
 * nekrs_gb300 — C ABI of the GB300-native pressure/Helmholtz elliptic solve.
 *
 * The entry points mirror nekRS's elliptic-solver boundary:
 *   ellipticSolveSetup(elliptic_t*)          src/solvers/elliptic/elliptic.h:193
 *   ellipticSolve(elliptic_t*, o_r, o_x)     src/solvers/elliptic/elliptic.h:191,
 *                                            src/solvers/elliptic/ellipticSolve.cpp:32
 *   ellipticOperator(elliptic, o_q, o_Aq, precision)
 *                                            src/solvers/elliptic/elliptic.h:202-206
 *   ellipticAx(...)                          src/solvers/elliptic/elliptic.h:208-213
 * plus the per-kernel entry points the reference dispatches through OCCA
 * (ellipticPartialAxCoeffHex3D, ellipticPartialAxTrilinearHex3D, oogs
 * gather-scatter, mask, ellipticBlockUpdatePCG).
 *
 * Conventions.  All vectors are element-local "E-vectors" [E][Nq^3] with
 * index i + Nq*(j + Nq*k) + Np*e (the reference's fieldOffset layout for one
 * field).  Geometric factors are [E][7][Np] in the order G00, G01, G11, G12,
 * G02, G22, GWJ (src/mesh/mesh3D.h:96-102).  Pointers named d_* are device
 * pointers on the current CUDA device, h_* are host pointers.  Every entry
 * point returns an int status (NRSG_OK = 0) and never aborts the process;
 * nrsg_last_error() gives the message of the last failure on this thread.
 * A CUDA stream of 0 means the legacy default stream.
 */
#ifndef NEKRS_GB300_H
#define NEKRS_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NRSG_OK 0
#define NRSG_ERR_MAXIT 1       /* iteration limit reached (ellipticSolve.cpp:161-162) */
#define NRSG_ERR_BREAKDOWN 2   /* p.Ap <= 0 or H(k,k) == 0 */
#define NRSG_ERR_NAN 3         /* NaN/Inf residual (PCG.cpp:193-195) */
#define NRSG_ERR_OOM 4         /* device allocation failed */
#define NRSG_ERR_BAD_CONFIG 5  /* invalid options or mesh description */
#define NRSG_ERR_CUDA 6        /* CUDA runtime error */
#define NRSG_ERR_NO_DEVICE 7   /* no CUDA device */
#define NRSG_ERR_INVALID 8     /* invalid argument */

/* Face boundary types (elliptic.h:46-49); lower id wins at shared nodes. */
#define NRSG_BC_NONE 0
#define NRSG_BC_DIRICHLET 1
#define NRSG_BC_ZERO_NORMAL 2 /* symmetry on a boundary of any orientation (three-field block solve) */
#define NRSG_BC_NEUMANN 4

typedef struct nrsg_elliptic nrsg_elliptic;

/* Mesh description filled by the caller before setup (the data
 * ellipticSolveSetup reads from mesh_t / elliptic_t, setup.cpp:893-915). */
typedef struct {
  int N;                    /* polynomial order, 1..9 */
  long long Nelements;
  const double *h_VX;       /* [E][8][3] vertex coordinates, hypercube vertex order v = i + 2j + 4k */
  const long long *h_EToV;  /* [E][8] global vertex ids (> 0), same order; drive the Nek5000 numbering */
  const int *h_EToB;        /* [E][6] face BC per nekRS face order (t-, s-, r+, s+, r-, t+) */
  const double *h_ggeo;     /* optional [E][7][Np]; NULL = computed on the device from the vertices */
} nrsg_mesh_desc;

typedef struct {
  int iterations;      /* elliptic->Niter */
  int status;          /* NRSG_* */
  double res0;         /* elliptic->res0Norm: sqrt((r,r)_invDegree / volume) */
  double res;          /* elliptic->resNorm at exit */
  double solve_ms;     /* device time of the solve */
} nrsg_solve_info;

/* Library / device */
const char *nrsg_last_error(void);
int nrsg_version(void);
/* Number of kernels this library has launched in the process so far. */
long long nrsg_kernel_launches(void);

/* Setup: mirrors ellipticSolveSetup.  `options` holds .par [PRESSURE]-section
 * style "key = value" lines (or ';'-separated): solver (pcg | pcg+flexible |
 * pfcg | pgmres+nVector=15 | pfgmres), residualTol (1e-8+relative),
 * maxIterations, preconditioner (none | jacobi | multigrid), smootherType,
 * pMGSchedule, coarseSolver, mgPrecision (fp64 | fp32 | mixed), axPrecision
 * (fp64 | fp32x2), lambda0,
 * lambda1, poisson, elementMap (trilinear), initialGuess (previous |
 * projectionAconj | projection: solution projection of
 * ellipticSolutionProjection.cpp, with residualProjectionVectors (8) and
 * residualProjectionStart (5)), cudaGraphs, nFields, stressFormulation,
 * axPipeline, axConst, coarseGridDiscretization (fem | fem+galerkin | semfem). */
int nrsg_elliptic_create(const nrsg_mesh_desc *mesh, const char *options, nrsg_elliptic **out);
/* Block (vector) Helmholtz, the velocity solve (tombo.cpp:224-228): options
 * "solver = pcg+block" (or nFields = 2 | 3) and stressFormulation = true.
 * Every vector of the handle (solve, operator, preconditioner) then holds
 * nFields fields one after another, fieldOffset = E*Np; norms sum over the
 * fields (weightedNorm2Many).  Preconditioner jacobi (block diagonal,
 * ellipticBlockBuildDiagonalHex3D) or none.  The per-field entry points
 * nrsg_elliptic_gs / _mask act on one field. */
/* Per-node coefficient fields (elliptic->o_lambda0 / o_lambda1, the
 * p_lambda = 1 kernels; ELLIPTIC COEFF FIELD): device arrays of E*Np doubles
 * shared by the fields (loffset = 0) or nFields*E*Np with loffset = E*Np.
 * d_lambda1 NULL means 0.  Copied into the handle; rebuilds the Jacobi
 * diagonal (ellipticUpdateJacobi).  Needs preconditioner jacobi or none. */
int nrsg_elliptic_set_coefficients(nrsg_elliptic *el, const double *d_lambda0, const double *d_lambda1,
                                   long long loffset);
/* Boundary types per field for the block solver (elliptic->EToB with Nfields
 * sections, ellipticSetup.cpp:190-199): h_EToB [nFields][E][6] in nekRS face
 * order, e.g. a symmetry plane normal to x masks only the first component.
 * Each field gets its own mask and gather groups; the Jacobi diagonal is
 * rebuilt.  Without this call every field takes the mesh descriptor's EToB.
 * NRSG_BC_ZERO_NORMAL faces of the first field (three fields only) remove the
 * normal component of the velocity on boundaries of any orientation: the
 * node's normal is the average of its zero-normal faces' normals and every
 * application of the mask projects (u, v, w) onto its tangent plane before
 * the Dirichlet mask and the gather-scatter (ellipticApplyMask.cpp:19-23,
 * applyZeroNormalMask.okl, createZeroNormalMask in applyDirichlet.cpp:7-33).
 * Type 3 (zero-tangential) is rejected with NRSG_ERR_BAD_CONFIG. */
int nrsg_elliptic_set_field_bcs(nrsg_elliptic *el, const int *h_EToB);
int nrsg_elliptic_destroy(nrsg_elliptic *el);
/* Run all later work of `el` on `cuda_stream` (a cudaStream_t; NULL = the
 * legacy default stream) instead of the library's own non-blocking stream,
 * which does not wait for work the caller queued elsewhere.  Waits for the
 * previous stream to drain.  No reference counterpart (OCCA's device stream). */
int nrsg_elliptic_set_stream(nrsg_elliptic *el, void *cuda_stream);

/* Solve: mirrors ellipticSolve(elliptic, o_r, o_x).  d_r holds the RHS on
 * entry and is overwritten with the final residual; d_x holds x0 on entry
 * and the solution on exit.  Both are device E-vectors of E*Np doubles. */
int nrsg_elliptic_solve(nrsg_elliptic *el, double *d_r, double *d_x, nrsg_solve_info *info);
/* Change the residual tolerance (residualTol, "+relative" when relative != 0)
 * and maxIterations of a handle between solves (the .par SOLVER TOLERANCE /
 * MAXIMUM ITERATIONS of the next ellipticSolve). */
int nrsg_elliptic_set_tolerance(nrsg_elliptic *el, double tol, int relative, int maxIterations);
/* Resumable form of the same solve (PCG / flexible PCG; GMRES runs to
 * completion inside the first advance).  begin() queues the initial residual
 * on the solver's stream and returns; each advance() call returns without
 * waiting on the device: it consumes the residual norm of the last queued
 * iteration once that has landed, queues the next iteration, and sets *done
 * = 1 (with *info filled and the solve's status returned) when the solve has
 * finished.  One solve per handle at a time.  Handles on different streams
 * advance concurrently (nrsg_elliptic_solve_batch, serving loops).  No
 * reference counterpart (ellipticSolve is blocking).  With solution
 * projection (initialGuess = projection*) the advance() that finishes a solve
 * waits for the basis update, which reads its Gram-Schmidt coefficients. */
int nrsg_elliptic_solve_begin(nrsg_elliptic *el, double *d_r, double *d_x);
int nrsg_elliptic_solve_advance(nrsg_elliptic *el, int *done, nrsg_solve_info *info);
/* n independent solves, each on its own handle (and stream), stepped together
 * one Krylov iteration at a time until all have finished.  info[k] receives
 * each solve's result; returns the first hard error, else the first
 * NRSG_ERR_MAXIT, else NRSG_OK. */
int nrsg_elliptic_solve_batch(int n, nrsg_elliptic *const *els, double *const *d_r, double *const *d_x,
                              nrsg_solve_info *info);

/* Serving: a request scheduler over resident operator handles.  The
 * reference has no counterpart (its ellipticSolve is blocking,
 * src/solvers/elliptic/ellipticSolve.cpp:32-190); these calls sequence the
 * resumable solve above for many requests.
 *   create   hbm_budget_bytes: the most device memory the handles of requests
 *            in flight may hold together (a request always starts when none
 *            is in flight).
 *   submit   queue a solve on a resident handle: d_r (right-hand side,
 *            overwritten by the residual) and d_x (initial guess, then the
 *            solution) stay the caller's and must not be touched until the
 *            request is polled; tol / relative / maxIterations as
 *            nrsg_elliptic_set_tolerance; footprint_bytes is the handle's
 *            device memory (nrsg_elliptic_get "deviceBytes").  Returns the
 *            request id.
 *   step     admit queued requests in arrival order (a request whose handle
 *            is busy waits without blocking the ones behind it; the budget
 *            stops admission), then advance every request in flight by at
 *            most one Krylov iteration without waiting on the device.  Returns
 *            the numbers in flight and queued.
 *   poll     take one finished request (*got = 1): its id and solve info; the
 *            return value is the solve's hard error, if any (an exhausted
 *            iteration budget shows as info->status = NRSG_ERR_MAXIT).
 *   destroy  fails with NRSG_ERR_INVALID while requests are in flight.
 * One thread at a time per server (calls are serialised by a mutex). */
typedef struct nrsg_server nrsg_server;
int nrsg_server_create(long long hbm_budget_bytes, nrsg_server **out);
int nrsg_server_destroy(nrsg_server *s);
int nrsg_server_submit(nrsg_server *s, nrsg_elliptic *el, double *d_r, double *d_x, double tol, int relative,
                       int maxIterations, long long footprint_bytes, long long *request_id);
int nrsg_server_step(nrsg_server *s, int *in_flight, int *queued);
int nrsg_server_poll(nrsg_server *s, long long *request_id, nrsg_solve_info *info, int *got);
/* Same solve on host buffers: copies in, solves, copies back. */
int nrsg_elliptic_solve_host(nrsg_elliptic *el, double *h_r, double *h_x, nrsg_solve_info *info);

/* ellipticOperator(elliptic, q, Aq, dfloatString): Ax -> mask -> gs-sum. */
int nrsg_elliptic_operator(nrsg_elliptic *el, const double *d_q, double *d_Aq);
/* ellipticAx(elliptic, E, elementList, q, Aq, dfloatString): local Ax only. */
int nrsg_elliptic_ax(nrsg_elliptic *el, const double *d_q, double *d_Aq);
/* oogs::startFinish(q, ..., ogsDfloat, ogsAdd) on the masked handle. */
int nrsg_elliptic_gs(nrsg_elliptic *el, double *d_q);
/* ellipticApplyMask(elliptic, q, dfloatString). */
int nrsg_elliptic_mask(nrsg_elliptic *el, double *d_q);
/* ellipticPreconditioner(elliptic, r, z). */
int nrsg_elliptic_precondition(nrsg_elliptic *el, const double *d_r, double *d_z);

/* Setup data for parity checks, copied to host.  Names: "ids", "maskedIds"
 * (int64), "gsOff", "gsIds", "maskIds" (int32), "invDegree", "ggeo",
 * "invDiag", "x", "y", "z", "D" (float64), "history" (float64, last solve),
 * "mg.levels", "mg.rho", "mg.degrees", "mg.coarseIters" (float64).  With h_out == NULL only *count is set. */
int nrsg_elliptic_get(nrsg_elliptic *el, const char *name, void *h_out, long long *count);

/* Schwarz smoother of pMG level `level` (pMGLevel::smoothSchwarz,
 * ellipticMultiGridSchwarz.cpp:1056-1156) applied once: Su = S u, FP64 in
 * and out (computed in the multigrid precision).  For parity checks. */
int nrsg_elliptic_mg_smoother(nrsg_elliptic *el, int level, const double *d_u, double *d_Su);
/* One launch of the fused FDM local solve of pMG level `level`
 * (fusedFDM in pMGLevel::smoothSchwarz, ellipticMultiGridSchwarz.cpp:1064-1130)
 * on device buffers of the multigrid precision (get "mg.bytes": 4 or 8) with
 * mg_level_size(level) entries: d_Su = the element-local FDM result on the own
 * nodes (RAS: times the overlap weights; ASM: the halo results stay inside
 * the library for the combine step).  Asynchronous on the solver's stream; no
 * gather-scatter or mask.  For kernel timing and parity checks. */
int nrsg_elliptic_mg_fdm(nrsg_elliptic *el, int level, const void *d_u, void *d_Su);
/* Number of E-vector nodes of pMG level `level` (-1 on error). */
long long nrsg_elliptic_mg_level_size(nrsg_elliptic *el, int level);

/* Host-only setup (no device needed): Nek5000 global numbering (setvert3d,
 * 3rd_party/nek5000/core/navier8.f:2004-2350), the Dirichlet mask
 * (ellipticOgs.cpp:4-134) and the masked gather maps (ogsSetup.cpp:111-397).
 * Output capacities: ids, maskedIds, invDegree, maskIds, gsIds: E*Np;
 * gsOff: E*Np+1.  Any output pointer may be NULL. */
int nrsg_host_setup_maps(int N, long long E, const long long *h_EToV, const int *h_EToB, long long *h_ids,
                         long long *h_maskedIds, double *h_invDegree, int *h_maskIds, long long *nmask, int *h_gsOff,
                         long long *ngroups, int *h_gsIds);

/* Spectral radius of an n x n upper-Hessenberg matrix (column-major), the
 * eigenvalue step of the Arnoldi lambda_max estimate
 * (ellipticMultiGridLevelSetup.cpp:415-438, LAPACK dgeev there).  -1 on error. */
double nrsg_host_hessenberg_rho(int n, const double *h_H);

/* Host-only: the assembled matrix of the level operator
 * lambda0 * (stiffness) + lambda1 * JW (lambda1 ignored when poisson != 0)
 * over the unmasked unique nodes, the matrix the reference hands to its
 * coarse solver (ellipticBuildFEMHex3D, src/solvers/elliptic/MG/
 * ellipticBuildFEM.cpp:73-230; coarseLevel_t::setupSolver,
 * src/solvers/elliptic/MG/coarseLevel.cpp:47).  Row r is the r-th masked
 * gather group, CSR with columns ascending.  h_ggeo is [E][7][Np].  Call with
 * h_rowPtr == NULL to get *nrow and *nnz; then capacities are nrow+1
 * (h_rowPtr), nnz (h_cols, h_vals) and E*Np (h_rowOfNode: row of each E-vector
 * node, -1 where masked).  The solver uses it on an order-1 coarsest level. */
/* Algebraic multigrid of an assembled SPD operator: the coarse solve of
 * coarseSolver = amg, in the form of the reference's BoomerAMG wrapper
 * (hypreWrapper.hpp: boomerAMG_t(nrows, nnz, Ai, Aj, Av, ...), solve(b, x);
 * the settings of coarseLevel.cpp:79-92): classical strength 0.25,
 * Ruge-Stueben first-pass coarsening, extended+i interpolation (4 entries per
 * row), Galerkin coarse operators, degree-1 Chebyshev smoothing, dense
 * coarsest solve.  nrsg_amg_create builds the hierarchy on the host (CSR,
 * 0-based); nrsg_amg_vcycle runs one V-cycle from x = 0 on the device (FP64
 * vectors of nrow entries) and synchronises the stream.
 * nrsg_amg_level_matrix returns level `level`'s operator (which = 0) or its
 * interpolation from the next level (which = 1); null arrays query the sizes;
 * lmax is the largest eigenvalue of D^-1 A the smoother uses.  The coarsest
 * level is level nlevels - 1 (operator only). */
typedef struct nrsg_amg nrsg_amg;
int nrsg_amg_create(long long nrow, const long long *h_rowPtr, const long long *h_col, const double *h_val,
                    nrsg_amg **out);
int nrsg_amg_destroy(nrsg_amg *a);
int nrsg_amg_num_levels(const nrsg_amg *a, int *nlevels);
int nrsg_amg_level_matrix(const nrsg_amg *a, int level, int which, long long *nrow, long long *ncol, long long *nnz,
                          long long *h_rowPtr, int *h_col, double *h_val, double *lmax);
int nrsg_amg_vcycle(nrsg_amg *a, const double *d_b, double *d_x, void *stream);

int nrsg_host_assemble_operator(int N, long long E, const long long *h_EToV, const int *h_EToB, const double *h_ggeo,
                                double lambda0, double lambda1, int poisson, long long *nrow, long long *nnz,
                                long long *h_rowPtr, long long *h_cols, double *h_vals, long long *h_rowOfNode);

/* Galerkin coarse operator (coarseGridDiscretization = FEM+Galerkin;
 * ellipticBuildFEMGalerkinHex3D, src/solvers/elliptic/MG/ellipticBuildFEM.cpp:
 * 384-520): the order-1 system B^T A_f B, A_f the order-Nf operator in FP32
 * on h_ggeo_fine ([E][7][(Nf+1)^3]), B the trilinear basis at the order-Nf
 * GLL nodes; rows are the order-1 level's masked gather groups.  Same calling
 * convention as nrsg_host_assemble_operator (h_rowOfNode: E*8 entries). */
int nrsg_host_assemble_galerkin(int Nf, long long E, const long long *h_EToV, const int *h_EToB,
                                const double *h_ggeo_fine, double lambda0, double lambda1, int poisson,
                                long long *nrow, long long *nnz, long long *h_rowPtr, long long *h_cols,
                                double *h_vals, long long *h_rowOfNode);

/* SEMFEM operator (coarseGridDiscretization = SEMFEM; SEMFEMSolver_t::build,
 * src/solvers/elliptic/SEMFEMSolverBuild.cpp:218-335, 551-700): linear
 * tetrahedra (the eight corner tetrahedra of every sub-hexahedron of the
 * order-N GLL grid) on the trilinear nodes of h_VX, lambda0 times the
 * stiffness, accumulated in FP32 as the reference does; rows are the order-N
 * level's masked gather groups.  Same calling convention as
 * nrsg_host_assemble_operator. */
int nrsg_host_assemble_semfem(int N, long long E, const double *h_VX, const long long *h_EToV, const int *h_EToB,
                              double lambda0, long long *nrow, long long *nnz, long long *h_rowPtr, long long *h_cols,
                              double *h_vals, long long *h_rowOfNode);

/* ---- mesh ingestion: Nek5000 binary .re2 files (host only) --------------
 * Replaces the mesh read nekRS delegates to Nek5000 (src/io/re2Reader.cpp:4-41
 * for the header; Nek5000 core/reader_re2.f: read_re2_hdr :543-620,
 * readp_re2_mesh :68-157, readp_re2_curve :159-286, readp_re2_bc :288-428)
 * and the vertex numbering parCon computes from the coordinates
 * (core/map2.f:471-540 calling parrsb_conn_mesh).  Versions v002, v003 and
 * v004 (8-byte words), either byte order, 3-D meshes. */
typedef struct {
  int version;       /* 2, 3 or 4 */
  int ndim;          /* 3 */
  long long nelgt;   /* elements */
  long long nelgv;   /* fluid elements (the first nelgv) */
  long long ncurve;  /* curved-side records */
  int nbcFields;     /* boundary sections in the file */
  int byteSwapped;   /* written with the other byte order */
} nrsg_re2_header;

int nrsg_re2_read_header(const char *path, nrsg_re2_header *hdr);
/* Element corners [nelgt][8][3] in hypercube order v = i + 2j + 4k (the
 * file's pre-processor corners 3<->4 and 7<->8 swapped, as meshNekReader.cpp:30
 * maps them) and group ids [nelgt]; either output may be NULL. */
int nrsg_re2_read_elements(const char *path, double *h_VX, int *h_group);
/* Curved sides, ncurve records: element (0-based), pre-processor face
 * (0-based), 5 parameters, type character; any output may be NULL. */
int nrsg_re2_read_curves(const char *path, long long *h_elem, int *h_face, double *h_params, char *h_type);
/* Boundary section `field` (0-based): per element and pre-processor face the
 * 3-character code, NUL-terminated in 4 bytes (h_cbc [nelgt][6][4]; faces
 * without a record read "E  "), and its 5 parameters (h_bc [nelgt][6][5]). */
int nrsg_re2_read_bc(const char *path, int field, char *h_cbc, double *h_bc);
/* Boundary ids in nekRS face order (t-, s-, r+, s+, r-, t+), the mapping of
 * meshNekReader.cpp:66-80: a face whose code equals codes[k] (trailing blanks
 * optional) gets ids[k], every other face 0.  Pass the result as h_EToB with
 * ids that are boundary types (NRSG_BC_*), as a .usr / boundaryTypeMap pair
 * would assign them. */
int nrsg_re2_boundary_ids(long long E, const char *h_cbc, int ncodes, const char *const *codes, const int *ids,
                          int *h_EToB);
/* Global vertex ids from corner coordinates (parrsb_conn_mesh, parRSB
 * con.c:221-321: findMinNeighborDistance :85-117, find_unique_vertices
 * con-unique-vertices.c:385-446, matchPeriodicFaces con-periodic.c:266-281),
 * for one process: corners closer than tol x their nearest-edge length in
 * every coordinate share an id; ids are numbered in the order of the sorted
 * segments (x, then y, then z); faces coded "P  " are matched with the
 * element and face their parameters name (h_cbc / h_bc as read by
 * nrsg_re2_read_bc, or NULL for none).  h_VX hypercube order; h_EToV [E][8]
 * receives 1-based ids, *nvertices their count.  tol = 0.2 is Nek5000's
 * default (core/reader_rea.f:50). */
int nrsg_mesh_connect(long long E, const double *h_VX, double tol, const char *h_cbc, const double *h_bc,
                      long long *h_EToV, long long *nvertices);

/* ---- kernel-level entry points (one launch each, on `stream`) ---------- */

/* ellipticPartialAxCoeffHex3D (kernels/elliptic/ellipticPartialAxCoeffHex3D.okl),
 * all elements, scalar lambda (p_lambda = 0), poisson = 1 drops the GWJ term. */
int nrsg_ax_stored_f64(int N, long long E, const double *d_ggeo, const double *d_D, double lambda0,
                       double lambda1, int poisson, const double *d_q, double *d_Aq, void *stream);
int nrsg_ax_stored_f32(int N, long long E, const float *d_ggeo, const float *d_D, float lambda0,
                       float lambda1, int poisson, const float *d_q, float *d_Aq, void *stream);
/* The same FP32 operator for N = 7 through a bulk-copy pipeline: persistent
 * CTAs stream each chunk of 3 elements' geometric factors and q into shared
 * memory (cp.async.bulk, completion on an mbarrier) one stage ahead of the
 * compute; results are bit-identical to nrsg_ax_stored_f32.  d_ggeo and d_q
 * must be 16-byte aligned; other N or unaligned pointers return
 * NRSG_ERR_INVALID. */
int nrsg_ax_pipe_f32(int N, long long E, const float *d_ggeo, const float *d_D, float lambda0, float lambda1,
                     int poisson, const float *d_q, float *d_Aq, void *stream);
/* The same FP32 operator for N = 7 with D held in constant memory (the row
 * every thread of a plane reads) and registers (the rows and columns a thread
 * contracts against), so that only the q and G planes pass through shared
 * memory; bit-identical to nrsg_ax_stored_f32.  D (64 floats on the device) is
 * copied into one constant bank on `stream` before the launch: launches that
 * may overlap must pass the same D.  Other N return NRSG_ERR_INVALID. */
int nrsg_ax_const_f32(int N, long long E, const float *d_ggeo, const float *d_D, float lambda0, float lambda1,
                      int poisson, const float *d_q, float *d_Aq, void *stream);
/* nrsg_ax_const_f32 as persistent CTAs (every resident slot of the device)
 * walking the element pairs; before computing a pair a CTA asks L2 for its
 * next pair's q and geometric factors (cp.async.bulk.prefetch.L2), so DRAM
 * reads overlap the contractions.  Bit-identical to nrsg_ax_const_f32; with
 * d_ggeo or d_q not 16-byte aligned nothing is prefetched.  Other N return
 * NRSG_ERR_INVALID. */
int nrsg_ax_const_prefetch_f32(int N, long long E, const float *d_ggeo, const float *d_D, float lambda0,
                               float lambda1, int poisson, const float *d_q, float *d_Aq, void *stream);
/* ellipticPartialAxTrilinearHex3D: geometry recomputed from d_VX [E][8][3]. */
int nrsg_ax_trilinear_f64(int N, long long E, const double *d_VX, const double *d_gllz, const double *d_gllw,
                          const double *d_D, double lambda0, double lambda1, int poisson, const double *d_q,
                          double *d_Aq, void *stream);
int nrsg_ax_trilinear_f32(int N, long long E, const float *d_VX, const float *d_gllz, const float *d_gllw,
                          const float *d_D, float lambda0, float lambda1, int poisson, const float *d_q,
                          float *d_Aq, void *stream);

/* FP64-accurate axhelm computed in FP32-pair arithmetic (about 48
 * significant bits; GB300 runs FP32 at 64x its FP64 rate).  ggeo_pairs /
 * D_pairs hold each FP64 value v as the float pair (hi, lo) with
 * hi = (float)v, lo = (float)(v - hi) (see nrsg_split_pairs); q and Aq are
 * FP64.  Same operator as nrsg_ax_stored_f64. */
int nrsg_ax_fp32x2(int N, long long E, const void *d_ggeo_pairs, const void *d_D_pairs, double lambda0,
                   double lambda1, int poisson, const double *d_q, double *d_Aq, void *stream);
/* (hi, lo) float-pair split of n doubles (8 bytes per pair). */
int nrsg_split_pairs(long long n, const double *d_x, void *d_pairs, void *stream);

/* gatherScatterMany_doubleAdd (3rd_party/gslib/ogs/okl/gatherScatterMany.okl):
 * q[ids[off[g]..off[g+1]]] = sum over the group, for every group g. */
int nrsg_gs_add_f64(long long ngroups, const int *d_off, const int *d_ids, double *d_q, void *stream);
int nrsg_gs_add_f32(long long ngroups, const int *d_off, const int *d_ids, float *d_q, void *stream);
/* mask.okl: q[maskIds[n]] = 0. */
int nrsg_mask_f64(long long n, const int *d_ids, double *d_q, void *stream);

/* ellipticBlockUpdatePCG + axpbyMany (PCG.cpp:33-83), fused: r -= alpha Ap,
 * x += alpha p, and *d_rdotr = sum invDegree r^2 (one launch, deterministic). */
int nrsg_update_pcg_f64(long long n, const double *d_invDegree, const double *d_p, const double *d_Ap,
                        double alpha, double *d_x, double *d_r, double *d_rdotr, void *stream);
/* weightedInnerProdMany (kernels/linAlg/weightedInnerProdMany.okl), one field:
 * *d_out = sum w a b (deterministic two-level reduction, one launch). */
int nrsg_weighted_inner_prod_f64(long long n, const double *d_w, const double *d_a, const double *d_b,
                                 double *d_out, void *stream);

/* Allocation-free variant of nrsg_weighted_inner_prod_f64 for callers that
 * cannot call cudaMalloc (their device memory is owned by another allocator,
 * or they must not take an allocation's implicit device synchronisation).
 * This entry point has no counterpart in the reference.  Its scratch (8192
 * partial sums + a counter, 64 KiB per GPU, held until exit) is a fixed
 * array inside this library; n is limited to 67,108,864 and larger n returns
 * NRSG_ERR_INVALID.  The first call on a device looks up the array's device
 * address and should come before any stream capture.  Calls share the array:
 * calls that overlap on the GPU race. */
int nrsg_weighted_inner_prod_f64_noalloc(long long n, const double *d_w, const double *d_a, const double *d_b,
                                         double *d_out, void *stream);

/* Geometric factors (kernels/mesh/geometricFactorsHex3D.okl) from trilinear
 * vertices: writes ggeo [E][7][Np]. */
int nrsg_geometric_factors_f64(int N, long long E, const double *d_VX, double *d_ggeo, void *stream);

#ifdef __cplusplus
}
#endif
#endif
