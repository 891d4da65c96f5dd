/*
 * sgfem.h - C ABI of the GB300 (sm_103a) stochastic-Galerkin hot path.
 *
 * Drop-in boundary for the Julia package ExtendableASGFEM.jl: every entry
 * point replaces one reference routine (cited as path:line inside that
 * project) and takes the reference's own data as plain pointers:
 *   - sparse matrices as Julia SparseMatrixCSC{Float64,Int64} arrays
 *     (1-based colptr / rowval, nzval), i.e. ExtendableSparseMatrix.cscmatrix;
 *   - SG vectors as SGFEVector.entries: Float64[n*P], column-major n x P
 *     (mode mu occupies entries[mu*n : (mu+1)*n], src/sgfevector.jl:94-103);
 *   - index lists 1-based Int64.
 * Host pointers are borrowed for the duration of a call only; the library
 * copies what it needs into device memory owned by the context and never
 * writes to caller data except the documented outputs.
 *
 * Every function returns an int status (SGFEM_OK = 0); on failure
 * sgfem_last_error() returns a message.  One context per host thread; all
 * calls on a context are synchronous with respect to the host.
 */
#ifndef SGFEM_H
#define SGFEM_H

#include <stdint.h>

#if defined(__GNUC__)
#define SGFEM_API __attribute__((visibility("default")))
#else
#define SGFEM_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define SGFEM_OK 0
#define SGFEM_ERR_ARGUMENT 1    /* bad size, null pointer, index out of range */
#define SGFEM_ERR_STATE 2       /* call order violated (e.g. apply before finalize) */
#define SGFEM_ERR_CUDA 3        /* CUDA runtime error (message has the detail) */
#define SGFEM_ERR_NONFINITE 4   /* NaN/Inf met in an input or an iterate */
#define SGFEM_ERR_BREAKDOWN 5   /* Krylov breakdown (p'Ap <= 0 or r'z <= 0) */
#define SGFEM_ERR_MAXIT 6       /* tolerance not reached within maxit */
#define SGFEM_ERR_UNSUPPORTED 7 /* configuration the library does not handle */

#define SGFEM_FP64 0            /* all arithmetic in FP64 */
#define SGFEM_FP32 1            /* FP32 operator values, vectors and accumulation */
#define SGFEM_MIXED 2           /* FP32 inner PCG inside FP64 iterative refinement */

#define SGFEM_PREC_NONE 0
#define SGFEM_PREC_LATTICE 1    /* mean-based I (x) (a0 L)^-1, L = 5-point lattice Laplacian */
#define SGFEM_PREC_JACOBI 2     /* I (x) diag(K_0)^-1 */
#define SGFEM_PREC_CHOLESKY 3   /* mean-based I (x) K_0^-1 on any mesh: sparse Cholesky of K_0 on the
                                   interior dofs (nested-dissection order), factored at the first use;
                                   the reference's LU(K_0) solve, solvers_poisson_primal.jl:23-78 */

typedef struct sgfem_context sgfem_context;

typedef struct {
    int precision;      /* SGFEM_FP64 or SGFEM_MIXED (SGFEM_FP32: FP32 PCG, no refinement) */
    int preconditioner; /* SGFEM_PREC_* ; LATTICE needs sgfem_set_dof_coordinates */
    double rtol;        /* stop when ||b - A x||_2 <= rtol ||b||_2 (FP64 true residual) */
    int maxit;          /* total PCG iterations (inner ones for MIXED) */
    double inner_rtol;  /* MIXED: relative reduction asked of each FP32 inner solve */
    int reference_rhs;  /* 1: b = x0 + e_1 (x) b0 as solvers_poisson_primal.jl:149-150 does;
                           0: b = e_1 (x) b0.  Boundary rows of b are zeroed either way. */
    int check_every;    /* PCG iterations per body of the device-side loop (1..64, default 4): the
                           whole PCG is one CUDA graph launch whose conditional WHILE node runs
                           bodies until the device-side convergence flag is set; iterations of a
                           body after convergence return at once */
} sgfem_solve_options;

typedef struct {
    int iterations;        /* PCG iterations (inner ones for MIXED) */
    int outer_iterations;  /* MIXED: refinement steps; FP64: 1 */
    int fp64_applies;      /* FP64 operator applications made */
    double relres;         /* final ||b - A x|| / ||b|| in FP64 */
    double time_ms;        /* device time of the solve (CUDA events) */
    double apply_ms;       /* device time spent in operator applications */
    double precond_ms;     /* device time spent in the preconditioner */
    long long kernel_launches; /* kernels this solve launched (graph replays included) */
} sgfem_solve_stats;

/* context */
SGFEM_API int sgfem_create(sgfem_context** ctx, int device);
SGFEM_API int sgfem_destroy(sgfem_context* ctx);
SGFEM_API const char* sgfem_last_error(const sgfem_context* ctx);
SGFEM_API int sgfem_version(void);

/*
 * Operator setup.  Replaces the construction of MySystemPrimal and
 * MyPreconditionerPrimal (src/modelproblems/solvers_poisson_primal.jl:14-44,
 * :136-146): K_0..K_M from poisson_primal.jl:56-63, G from
 * TensorizedBasis.G (src/tensorizedbasis.jl:193-218), boundary dofs from
 * FES[BFaceDofs].
 */
SGFEM_API int sgfem_set_spatial_matrix(sgfem_context* ctx, int m, int64_t n, const int64_t* colptr,
                             const int64_t* rowval, const double* nzval);
SGFEM_API int sgfem_set_coupling(sgfem_context* ctx, int64_t P, int64_t M, const int64_t* colptr,
                       const int64_t* rowval, const double* nzval);
SGFEM_API int sgfem_set_boundary_dofs(sgfem_context* ctx, int64_t count, const int64_t* bdofs);
/* dof coordinates, 2 x n column-major (Julia's xgrid[Coordinates] layout); when they
   form a uniform lattice of the unit square the lattice preconditioner is enabled
   and the device numbering follows the lattice. */
SGFEM_API int sgfem_set_dof_coordinates(sgfem_context* ctx, int64_t n, const double* xy);
SGFEM_API int sgfem_finalize(sgfem_context* ctx);
/* the adaptive loop appended modes (scripts/poisson.jl:341-420): new coupling G
   ((M*P) x P, 1-based CSC as for sgfem_set_coupling) on a finalized context.  Only
   the coupling-dependent state is rebuilt (device column order, pair and
   combination tables, the specialised FP32 apply); the K_m, the dof numbering and
   the lattice preconditioner stay resident.  M must not exceed the number of K_m
   set before finalize minus one.  Device vectors of the old layout are invalid
   afterwards. */
SGFEM_API int sgfem_update_coupling(sgfem_context* ctx, int64_t P, int64_t M, const int64_t* colptr,
                                    const int64_t* rowval, const double* nzval);
/* 1 if the lattice preconditioner is available after finalize */
SGFEM_API int sgfem_has_lattice(const sgfem_context* ctx);
/* which mean-based lattice preconditioner a finalized context applies: the exact
   K_0^-1 (4x4 blocks of the 2-D sine transform; K_0 translation invariant on the
   lattice, as for P1/P2 with a constant mean) or the 5-point Laplacian scaled by
   the mean diagonal, with the reason */
SGFEM_API const char* sgfem_lattice_log(const sgfem_context* ctx);
/* the sparse-Cholesky mean preconditioner (SGFEM_PREC_CHOLESKY) of a finalized
   context: "not factored yet" before its first use, then the factor's size (nodes
   and heights of the nested-dissection tree, nnz(L)) or why the factorisation
   failed.  Replaces the reference's lu(A0.cscmatrix), solvers_poisson_primal.jl:41. */
SGFEM_API const char* sgfem_cholesky_log(const sgfem_context* ctx);
/* Whether the mixed-precision solve of a finalized context runs its inner FP32 PCG
   (the iterations of solve_primal!, solvers_poisson_primal.jl:130-169, on the
   refinement residual) as ONE thread-block-cluster launch per refinement step:
   "one-cluster FP32 PCG: <CTAs> CTAs, <KB> KB shared memory each; launches: <n>"
   for small P1 problems on a power-of-two dof lattice (K_0 = a0 x 5-point
   Laplacian, at most 32 modes and 16 KLE terms, couplings to neighbouring lines
   only, the vectors in the cluster's shared memory; n counts the launches so far),
   else the reason it does not (then one launch per phase).  SGFEM_SMALL=0 at
   finalize disables it. */
SGFEM_API const char* sgfem_small_solve_log(const sgfem_context* ctx);
/* Host-only (no GPU needed): the SGFEM_PREC_CHOLESKY factorisation of K_0
   (1-based CSC, n x n, boundary dofs 1-based) and both triangular solves in the
   device kernels' order of summation, applied to B (column-major n x P) into Z:
   Z = K_0^-1 B on the interior rows, zero on the boundary rows, as ldiv! of
   solvers_poisson_primal.jl:47-78 with the LU of K_0 (1e60 on the boundary
   diagonals, :30-44).  msg (msglen bytes) receives the factor summary or the
   error.  For checking the ordering and factorisation on a CPU. */
SGFEM_API int sgfem_cholesky_host_solve(int64_t n, const int64_t* colptr, const int64_t* rowval,
                                        const double* nzval, int64_t nb, const int64_t* bdofs, int64_t P,
                                        const double* B, double* Z, char* msg, int msglen);

/*
 * mul!(Ax, S::MySystemPrimal, x), solvers_poisson_primal.jl:86-124:
 *   Y_mu = K_0 X_mu + sum_{m,nu} G[(m-1)P+mu, nu] K_m X_nu, boundary rows zeroed.
 * x, y: host SGFEVector.entries (n*P doubles).  precision: SGFEM_FP64 / SGFEM_FP32.
 */
SGFEM_API int sgfem_apply(sgfem_context* ctx, const double* x, double* y, int precision);

/*
 * ldiv!(y, P::MyPreconditionerPrimal, b), solvers_poisson_primal.jl:47-78, with the
 * mean-based operator selected by `kind` (SGFEM_PREC_*).  For P1 lattices
 * SGFEM_PREC_LATTICE equals the reference's LU solve on interior rows.
 */
SGFEM_API int sgfem_precondition(sgfem_context* ctx, const double* b, double* y, int kind, int precision);

/*
 * solve_primal!(sol, A0, Am, b0, G, nmodes, 1), solvers_poisson_primal.jl:130-169:
 * solves S x = b with b built from b0 (n doubles, the assembled (f, v)) and the
 * warm start x_inout (SGFEVector.entries, in/out).  Uses PCG (the SG operator of
 * PoissonProblemPrimal is SPD on interior dofs) instead of the reference's GMRES.
 * x_inout receives the solution on SGFEM_OK and SGFEM_ERR_MAXIT.  When x_inout is
 * pinned host memory (cudaHostAlloc / cudaHostRegister), the solution of a step
 * expected to end the solve is copied to it while the final convergence check runs;
 * after an error other than SGFEM_ERR_MAXIT it may then hold that last iterate.
 * The call returns only once every copy into x_inout has ended.
 */
SGFEM_API int sgfem_solve(sgfem_context* ctx, const double* b0, double* x_inout,
                const sgfem_solve_options* opts, sgfem_solve_stats* stats);
SGFEM_API void sgfem_default_options(sgfem_solve_options* opts);

/*
 * solve_logpoisson_primal!(sol, A, N0, Nm, b0, G, nmodes, bfac),
 * src/modelproblems/solvers_logpoisson_primal.jl:130-172: the same SG operator
 * structure with non-symmetric blocks (K_0 = A + N_0, K_m = N_m =
 * -(grad a_m . grad u, v) of LogTransformedPoissonProblemPrimal, set with
 * sgfem_set_spatial_matrix).  b0 is n x P column-major (the assembled
 * (lambda_mu f, v) of every mode); b = x0 + b0 (reference_rhs = 1, as :149-155)
 * or b0, Dirichlet rows zeroed.  Right-preconditioned restarted GMRES(restart)
 * (restart <= 0: 20, the Krylov.jl default memory) with the mean-based
 * preconditioner opts->preconditioner, stopping on ||b - A x|| <= rtol ||b||
 * (FP64 true residual).  SGFEM_MIXED: FP64 iterative refinement, each step one
 * FP32 GMRES(restart) cycle to max(inner_rtol, 1e-4) (about the accuracy FP32
 * GMRES reaches).  Also valid for symmetric operators.
 */
SGFEM_API int sgfem_solve_gmres(sgfem_context* ctx, const double* b0, double* x_inout,
                                const sgfem_solve_options* opts, int restart, sgfem_solve_stats* stats);

/*
 * Device-resident variants for callers that keep SG vectors on the GPU.  Vectors
 * are in the device layout: n_dev rows (device dof order) x ld columns, row-major,
 * where sgfem_device_layout() reports n_dev, ld and the element size.
 * Pointers are device pointers; calls are ordered on the context's stream and
 * return after the work has completed.
 */
SGFEM_API int sgfem_device_layout(const sgfem_context* ctx, int64_t* n_dev, int64_t* ld);
SGFEM_API int sgfem_apply_device(sgfem_context* ctx, const void* x_dev, void* y_dev, int precision);
SGFEM_API int sgfem_to_device_layout(sgfem_context* ctx, const double* x_host, void* x_dev, int precision);
SGFEM_API int sgfem_from_device_layout(sgfem_context* ctx, const void* x_dev, double* x_host, int precision);
/* solve with b0 (n doubles, host) and a device-resident FP64 solution x_dev (in/out) */
SGFEM_API int sgfem_solve_device(sgfem_context* ctx, const double* b0, void* x_dev,
                       const sgfem_solve_options* opts, sgfem_solve_stats* stats);

/* time (ms, CUDA events on the context stream) of `reps` back-to-back device applies */
SGFEM_API int sgfem_time_apply(sgfem_context* ctx, int precision, int reps, double* ms_per_apply);
/* device time of the residual r = b - A x that ends every mixed refinement step:
   double-FP32 arithmetic (difference form, error-free products and sums on the
   FP32 pipe) when every K_m has vanishing row sums, else the FP64 apply plus
   the subtraction; *kind = 1 for the double-FP32 form, 0 for FP64 */
SGFEM_API int sgfem_time_residual(sgfem_context* ctx, int reps, double* ms_per_residual, int* kind);
/* the same for the lattice preconditioner (three passes per application) */
SGFEM_API int sgfem_time_precondition(sgfem_context* ctx, int precision, int reps, double* ms_per_application);
/*
 * Batched deterministic sample problems, deterministic_problem(problem, C, y_s)
 * + ExtendableFEM.solve (src/modelproblems/poisson_primal.jl:14-35,
 * src/sampling_error.jl:118-128): -div(a(y_s) grad u_s) = f, homogeneous
 * Dirichlet data, s = 1..S, a(y) = a_0 + sum_{m<=M} y_m a_m.  Instead of
 * sgfem_set_coupling, a context gets the samples (y: M x S, column-major) and
 * K_0..K_M of the deterministic space; its operator is then block diagonal,
 * column s holding K_0 + sum_m y_{s,m} K_m, and the SG entry points (apply,
 * preconditioner, solve) act on n x S vectors.  sgfem_solve_samples solves all
 * S problems with b0 in every column and reports the largest per-sample
 * relative residual in stats->relres.  After finalize, sgfem_set_samples with
 * the same S and M replaces the samples (the next batch) without rebuilding
 * the context.  x_inout = NULL: start from zero and keep the solutions on the
 * device only (for sgfem_sampling_error).  M <= 64.
 */
SGFEM_API int sgfem_set_samples(sgfem_context* ctx, int64_t S, int64_t M, const double* y);
SGFEM_API int sgfem_solve_samples(sgfem_context* ctx, const double* b0, double* x_inout,
                                  const sgfem_solve_options* opts, sgfem_solve_stats* stats);


/*
 * Residual error estimator, estimate(::Type{PoissonProblemPrimal}, sol, C; rhs,
 * bonus_quadorder, tail_extension), src/estimate.jl:260-418.  The caller (the
 * host layer, which also runs the integer work add_boundary_modes /
 * get_neighbours of mopcontrol.jl:60-132, estimate.jl:1-22) passes the mesh in
 * ExtendableGrids' layout, the quadrature rules, f at the cell quadrature
 * points, the cosine coefficient and, for every extended mode j, the list of
 * its couplings to ACTIVE modes (the terms the reference adds):
 *   (m = 0, nu = j, g = 1) if j is active, and (m, nu, g = G_ext[(m-1)P_ext+j, nu])
 *   for every active neighbour nu = j +/- e_m, m = 1..M_ext.
 * Outputs follow the reference: eta4modes[P_ext], eta4cell (ncells x P_ext,
 * column-major).  The jump term integrates |sum_m a_m [[grad w_{j,m}]]|^2 on
 * every interior face with the given face rule (the reference projects onto a
 * face space first, ExtendableFEM's FaceInterpolator; that projection is not
 * restated).  All arithmetic in FP64.
 */
typedef struct {
    int order;                     /* 1 or 2: H1 Pk on triangles */
    int64_t nnodes, ncells, nfaces;
    const double* coords;          /* 2 x nnodes (xgrid[Coordinates]) */
    const int64_t* cell_nodes;     /* 3 x ncells, 1-based (xgrid[CellNodes]) */
    const int64_t* cell_dofs;      /* nd x ncells, 1-based (FES[CellDofs]); P2: vertex dofs then the
                                      dofs of faces (1,2), (2,3), (3,1) */
    const int64_t* face_nodes;     /* 2 x nfaces, 1-based (xgrid[FaceNodes]) */
    const int64_t* face_cells;     /* 2 x nfaces, 1-based, 0 = none (xgrid[FaceCells]) */
    const int64_t* cell_faces;     /* 3 x ncells, 1-based (xgrid[CellFaces]) */
    const double* cell_volumes;    /* ncells */
    const double* face_volumes;    /* nfaces */
} sgfem_mesh;

typedef struct {
    int nq;                        /* cell rule: reference points (xi, eta) 2 x nq, weights (sum 1) */
    const double* xref;
    const double* w;
    int nqf;                       /* face rule on [0, 1]: points, weights (sum 1) */
    const double* tref;
    const double* wf;
} sgfem_quadrature;

typedef struct {                   /* StochasticCoefficientCosinus, src/coefficients/cosinus.jl:11-76 */
    int maxm;
    double mean;                   /* a_0 */
    double freq;                   /* multiplies pi (1 in the reference) */
    const double* decay_factors;   /* maxm */
    const int64_t* b1;             /* maxm */
    const int64_t* b2;             /* maxm */
} sgfem_cosine;

typedef struct {
    int64_t P_ext;                 /* extended modes, the active ones first */
    int64_t M_ext;                 /* length of the extended multi-indices */
    const int64_t* ptr;            /* P_ext + 1, 0-based offsets into the lists */
    const int32_t* m;              /* coupling term: 0..M_ext */
    const int32_t* nu;             /* active mode, 0-based */
    const double* g;
} sgfem_extension;

SGFEM_API int sgfem_estimate_primal(sgfem_context* ctx, const double* sol, const sgfem_mesh* mesh,
                                    const sgfem_quadrature* quad, const double* f_qp /* nq x ncells */,
                                    const sgfem_cosine* coef, const sgfem_extension* ext, double* eta4modes,
                                    double* eta4cell);

/*
 * estimate(::Type{LogTransformedPoissonProblemPrimal}, sol, C; rhs,
 * bonus_quadorder, tail_extension), src/estimate.jl:70-257, for a context whose
 * operator is the log-transformed one (K_0 = A, K_m = N_m).  mesh, quad, f_qp,
 * coef and ext as for sgfem_estimate_primal (ext's (0, j, 1) entries are not
 * used; coef must hold all maxm terms: the data term sums a_m^2 over them).
 * lam: the interpolant of the Hermite chaos coefficients lambda_j of exp(-a)
 * (expa_PCE_mop with factor -1, coefficients.jl:219-260) on an H1Pk space of
 * degree 1 or 2 over the same cells, values P_ext x ndofs (mode j at
 * [j * ndofs]).  Outputs: eta4modes[P_ext], eta4cell (ncells x P_ext,
 * column-major) and zeta[2] = (zeta1, zeta2); the reference returns
 * zeta1 - zeta2.  eta4modes[j] = sqrt(V_j) + sqrt(V_j + J_j) for active j (the
 * reference's update at :244) and sqrt(V_j) otherwise.
 */
typedef struct {
    int order;                     /* 1 or 2 */
    int64_t ndofs;
    const int64_t* cell_dofs;      /* nd x ncells, 1-based */
    const double* values;          /* ndofs x P_ext column-major */
} sgfem_interpolant;

SGFEM_API int sgfem_estimate_logpoisson(sgfem_context* ctx, const double* sol, const sgfem_mesh* mesh,
                                        const sgfem_quadrature* quad, const double* f_qp, const sgfem_cosine* coef,
                                        const sgfem_extension* ext, const sgfem_interpolant* lam,
                                        double* eta4modes, double* eta4cell, double* zeta);

/*
 * estimate_equilibration(::Type{PoissonProblemPrimal}, sol, C; rhs,
 * tail_extension), src/estimate.jl:607-954: for every node z and extended mode
 * j the flux sigma_{z,j} in RT_k (k = mesh->order, HDIVRTk{2, k}) on the node
 * patch that minimises ||sigma - phi_z F_j||^2 + sum_T div_penalty sqrt|T|
 * ||div sigma - (F_j . grad phi_z - f phi_z [j = 1])||_T^2 with zero normal flux
 * on the edges the patch shares with outside cells, F_j = sum over ext's list j
 * of g a_m grad u_nu; then eta4cell[c + j ncells] = sum_q w_q |T| (|F_j -
 * sigma_j|^2 + (f [j = 1] + div sigma_j)^2 / pi^2), sigma_j = sum_z sigma_{z,j},
 * eta4modes[j] = sqrt(sum_c eta4cell[c + j ncells]).  The reference's penalty is
 * div_penalty = 1e5 and its cell rule has order 2 (k + 1).  mesh: coords,
 * cell_nodes, cell_dofs, cell_faces, face_nodes, face_cells, cell_volumes;
 * quad: the cell rule (the face rule is not used); f_qp: nq x ncells.  Each
 * node patch is solved on its own (the reference groups disjoint patches
 * into one system, NodePatchGroups).  A patch may hold at most 120 flux dofs.
 */
SGFEM_API int sgfem_estimate_equilibration(sgfem_context* ctx, const double* sol, const sgfem_mesh* mesh,
                                           const sgfem_quadrature* quad, const double* f_qp,
                                           const sgfem_cosine* coef, const sgfem_extension* ext, double div_penalty,
                                           double* eta4modes, double* eta4cell);
/* the RT_k basis of the reference cell that sgfem_estimate_equilibration maps to
   every cell (k = 1 or 2): dual to the edge moments int_0^1 sigma(x(t)) . R x'(t)
   L_l(2t - 1) dt on the edges (v0,v1), (v1,v2), (v2,v0) of the reference cell
   (R the rotation by -90 degrees, L_l Legendre, l = 0..k; dofs e (k + 1) + l)
   and the interior moments int sigma_c q, q in {1} (k = 1) or {1, xi, eta}
   (k = 2; dofs 3 (k + 1) + c * nq + iq).  At np points (xi, eta): values
   np x nb x 2, divs np x nb, nb = 8 (k = 1) or 15 (k = 2).  Host only. */
SGFEM_API int sgfem_rt_reference_basis(int k, int np, const double* pts, double* values, double* divs);

/*
 * Evaluation of an SG solution at parameter samples and the sampling error.
 *
 * sgfem_evaluate_samples: batched set_sample!(SGFEV, y[1:m])
 * (src/sgfevector.jl:43-69, src/tensorizedbasis.jl:226-252):
 *   out[:, s] = sum_k Psi_k(y_s) U[:, k],  Psi_k(y) = prod_{d<M} v_d[mu_k[d]],
 *   v_d[j] = p_j(y_d) / ||p_j|| for d < m and v_d = (1, 0, 0, ...) for d >= m,
 * p_j from the three-term recurrence (orthogonal_polynomials.jl:63-73).
 * U: n x P column-major (SGFEVector entries); y: Ms x S column-major, Ms >= m;
 * out: n x S column-major.  Any finalized context serves (device and stream).
 *
 * sgfem_sampling_error: the error integrals of calculate_sampling_error
 * (src/sampling_error.jl:2-44, :149-191) for a batch of samples,
 *   errH1[s][m] = sum_T int_T |grad(u_s - u_sg,m(y_s))|^2
 *   errL2[s][m] = sum_T int_T (u_s - u_sg,m(y_s))^2,    m = 0..basis->M,
 * with u_sg,m the SG solution evaluated at y_s[1:m] and u_s the deterministic
 * solution of sample s.  ctx is a samples context (sgfem_set_samples) whose
 * samples are the y_s; det_solutions = NULL takes the solutions of its last
 * sgfem_solve_samples from the device, otherwise n_det x S (column-major,
 * host).  mesh: geometry (coords, cell_nodes, cell_volumes) and the
 * deterministic space (order, cell_dofs); sg_space: order and cell_dofs of
 * the SG space on the same cells.  quad: the cell rule (2 * order of the
 * deterministic space in the reference).  Outputs are (M+1) x S column-major.
 * The SG part is evaluated with Psi_k at the full sample (m = M); for modes
 * active at truncation m this differs from the reference's truncated product
 * only by the factors 1/||p_0|| of the dimensions m..M-1 (1 up to rounding).
 * Where the SG space embeds in the deterministic one (P1 in P2, equal orders)
 * the rule's sums are evaluated as quadratic forms in the local coefficients of
 * the error, with matrices built from the same rule (equal up to rounding);
 * otherwise point by point.  sgfem_sampling_error_log names the form of the
 * last call; SGFEM_SAMPLING_QF=0 keeps the point-by-point form.
 */
typedef struct {                   /* TensorizedBasis + ONBasis, src/tensorizedbasis.jl:28-34, onbasis.jl:13-18 */
    int64_t P;                     /* multi-indices */
    int64_t M;                     /* their length (maxlength_multiindices) */
    const int32_t* multi_indices;  /* M x P column-major: entry d of multi-index k at [k * M + d] */
    int32_t maxorder;              /* highest degree in the multi-indices */
    const double* recurrence;      /* 3 x maxorder: (a_j, b_j, c_j), p_{j+1} = (a_j + b_j y) p_j - c_j p_{j-1} */
    const double* norms;           /* maxorder + 1: ||p_j|| */
} sgfem_sg_basis;

typedef struct {                   /* H1Pk space on the cells of an sgfem_mesh */
    int order;                     /* 1 or 2 */
    int64_t ndofs;
    const int64_t* cell_dofs;      /* nd x ncells, 1-based */
} sgfem_fe_space;

SGFEM_API int sgfem_evaluate_samples(sgfem_context* ctx, const double* U, int64_t n, const sgfem_sg_basis* basis,
                                     const double* y, int64_t Ms, int64_t S, int64_t m, double* out);
SGFEM_API int sgfem_sampling_error(sgfem_context* ctx, const double* det_solutions, const sgfem_mesh* mesh,
                                   const sgfem_fe_space* sg_space, const double* U, const sgfem_sg_basis* basis,
                                   const sgfem_quadrature* quad, double* errH1, double* errL2);
/* "quadratic forms", "quadrature points" or "none" (no call yet): the form of the
   last sgfem_sampling_error on this context. */
SGFEM_API const char* sgfem_sampling_error_log(const sgfem_context* ctx);

/*
 * No counterpart in the reference package.  Applies the mean-based lattice
 * preconditioner (what sgfem_precondition does with SGFEM_PREC_LATTICE) to
 * device vectors without allocating any device memory.  It is meant for
 * callers that cannot allocate at that point: a Julia process whose CUDA.jl
 * memory pool already owns the GPU, an application held to a fixed
 * device-memory budget, or a loop in which the implicit synchronisation of
 * cudaMalloc is not acceptable.  r_dev (input) and z_dev (output) are vectors
 * in the device layout (sgfem_device_layout).  The intermediate buffer is a
 * static device array of SGFEM_STATIC_SCRATCH_BYTES that every GPU loading the
 * library holds until the process exits; a vector needing more than that
 * (n_dev * ld * element size) is rejected with SGFEM_ERR_ARGUMENT.  The work
 * runs on the context's own stream, which does not wait for other streams:
 * finish every write to r_dev and z_dev (e.g. synchronise the stream that
 * made them) before the call.  The call is synchronous: it returns after the
 * result is in z_dev.  The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress), so make that first call before any stream
 * capture.  All calls share the one array and it keeps the last call's
 * contents: calls that overlap on the same GPU (from other contexts or host
 * threads) race on it.
 */
#define SGFEM_STATIC_SCRATCH_BYTES (32u * 1024u * 1024u)
SGFEM_API int sgfem_precondition_device_static(sgfem_context* ctx, const void* r_dev, void* z_dev, int precision);

/*
 * Adjoint gradient of a mean quantity of interest J = l . U_0 (no counterpart in
 * the reference package; the reference's Julia API has no derivative).  For the
 * symmetric SG operator S = I (x) K_0 + sum_m G_m (x) K_m of the context, U the
 * solution of S U = b and Lambda the adjoint solution of S Lambda = e_1 (x) l
 * (both n x P column-major, host):
 *   dblocks[m-1] = -Lambda^T (G_m (x) K_m) U, the derivative of J with respect
 *                  to a factor multiplying K_m (m = 1..M);
 *   dalpha[i]    = -sum_mu Lambda_mu^T K_0^(i) U_mu, K_0^(i) = (phi_i grad u, grad v):
 *                  the derivative with respect to the nodal values of a P1 mean
 *                  field a_0 = sum_i alpha_i phi_i (mesh: the P1 space of the
 *                  context, one dof per node).
 * Either output may be NULL.  FP64; reductions in a fixed order.
 */
SGFEM_API int sgfem_adjoint_gradient(sgfem_context* ctx, const double* U, const double* Lambda, double* dblocks,
                                     const sgfem_mesh* mesh, double* dalpha);

/*
 * Batches of independent SG problems (no counterpart in the reference, which
 * solves one problem per solve! call, poisson_primal.jl:38-81).  Each problem
 * is the PoissonProblemPrimal system of solve_primal! with b = e_1 (x) b0 and a
 * zero start: its own n, K_0..K_M on one shared pattern (1-based CSC, values
 * (M+1) x nnz column-major), coupling G ((M*P) x P, 1-based CSC), boundary dofs
 * and b0.  sgfem_batch_solve runs preconditioned CG (mean-based by sine transforms on
 * problems marked with sgfem_batch_set_lattice, Jacobi otherwise) on all problems in
 * lock step: each phase of an iteration is one launch over every problem, a
 * batch of check_every iterations is a captured CUDA graph, converged problems
 * skip their blocks.  The apply's form (pair passes, or column slots when every
 * problem has M + 1 <= 31) and launch shape are chosen at finalize by timing
 * the candidates (sgfem_batch_tuning reports them).  x_out receives the
 * solutions, problem after problem, each n x P column-major (may be NULL).
 * Mixed precision by default: iterative refinement whose residuals are FP64
 * applies of every unconverged problem, with an FP32 PCG (FP32 operator and
 * preconditioner tables, FP64 solution accumulation) as the correction solve;
 * stats report the FP64 residuals.  SGFEM_BATCH_PRECISION=fp64 in the
 * environment selects the plain FP64 PCG.  Per-problem reductions run in a
 * fixed order.  M <= 255.
 */
typedef struct sgfem_batch sgfem_batch;
typedef struct {
    int iterations_max;            /* largest iteration count over the problems */
    int converged;                 /* problems that reached rtol */
    int graph_replays;
    double relres_max;             /* largest final ||b - A x|| / ||b|| */
    double time_ms;                /* device time of the solve (CUDA events) */
    long long kernel_launches;
} sgfem_batch_stats;
SGFEM_API int sgfem_batch_create(sgfem_batch** batch, int device);
SGFEM_API int sgfem_batch_destroy(sgfem_batch* batch);
SGFEM_API const char* sgfem_batch_last_error(const sgfem_batch* batch);
SGFEM_API int sgfem_batch_add(sgfem_batch* batch, int64_t n, int64_t M, int64_t P, const int64_t* colptr,
                              const int64_t* rowval, const double* vals, const int64_t* Gcolptr,
                              const int64_t* Growval, const double* Gval, int64_t nbdofs, const int64_t* bdofs,
                              const double* b0);
SGFEM_API int sgfem_batch_count(const sgfem_batch* batch);
/* problem i's dofs are the (nl+1)^2 points of a uniform lattice, x fastest, Dirichlet rows on its
   boundary (P1 on the unit square): it gets the mean-based preconditioner (a0 L)^-1 by sine transforms
   (L the 5-point Laplacian, exact for P1 with a constant mean) instead of Jacobi */
SGFEM_API int sgfem_batch_set_lattice(sgfem_batch* batch, int i, int64_t nl);
SGFEM_API int sgfem_batch_finalize(sgfem_batch* batch);
SGFEM_API const char* sgfem_batch_tuning(const sgfem_batch* batch);
SGFEM_API int sgfem_batch_solve(sgfem_batch* batch, double rtol, int maxit, int check_every, double* x_out,
                                sgfem_batch_stats* stats);
SGFEM_API int sgfem_batch_problem_stats(const sgfem_batch* batch, int i, int* iterations, double* relres);
/* Host check of the batch apply's column-slot form (no device work, no counterpart in
   the reference; its result is mul! of solvers_poisson_primal.jl:86-124): one problem,
   given as to sgfem_batch_add, is scheduled as sgfem_batch_finalize schedules it and
   Y = S X is evaluated on the host in FP64 from the pass structure of the FP32
   (precision 1) or FP64 (precision 0) kernel, pass area and combination entries
   included.  X, Y: n x P column-major.  msg receives a summary of the schedule;
   SGFEM_ERR_UNSUPPORTED when M + 1 > 31 (the form does not apply). */
/* Host check of the batch sine-transform preconditioner's split tables (no device
   work, no counterpart in the reference): y = S x, S_ik = sin(pi i k / nl), i, k =
   1..nl-1, for ncols lines (x, y: (nl-1) x ncols column-major), computed as the batch
   kernel computes it (pairs (x_k, x_{nl-k}) into sums and differences, odd outputs
   from the sums, even outputs from the differences) with its FP32 table values, in
   FP64.  2 <= nl <= 128. */
SGFEM_API int sgfem_batch_host_dst(int64_t nl, int64_t ncols, const double* x, double* y);
SGFEM_API int sgfem_batch_host_apply(int64_t n, int64_t M, int64_t P, const int64_t* colptr, const int64_t* rowval,
                                     const double* vals, const int64_t* Gcolptr, const int64_t* Growval,
                                     const double* Gval, int64_t nbdofs, const int64_t* bdofs, int precision,
                                     const double* X, double* Y, char* msg, int msglen);

/*
 * Stiffness matrices of the cosine coefficient assembled on the GPU (the
 * reference assembles them on the host with ExtendableFEM, poisson_primal.jl:
 * 56-68): K_m = (a_m grad u, grad v) for m = m0..m1 (a_0 = coef->mean) on the
 * H1Pk space `space` (order 1 or 2) of `mesh` (coords, cell_nodes and
 * cell_volumes are used), with the cell rule of `quad` (weights summing to
 * one).  The sparsity pattern is the caller's CSC (1-based colptr[n + 1],
 * rowval[nnz], every cell coupling present); values receives the nonzeros of
 * K_m0..K_m1 in that pattern, (m1 - m0 + 1) x nnz column-major.  Each nonzero
 * sums its cells' contributions in increasing cell order (no atomics).  ctx only
 * names the GPU, the stream and the error message; it need not be finalized.
 */
SGFEM_API int sgfem_assemble_stiffness(sgfem_context* ctx, const sgfem_mesh* mesh, const sgfem_fe_space* space,
                                       const sgfem_cosine* coef, int m0, int m1, const sgfem_quadrature* quad,
                                       int64_t nnz, const int64_t* colptr, const int64_t* rowval, double* values);
/* the convection blocks of solve!(LogTransformedPoissonProblemPrimal),
   N_m[i, j] = -(grad a_m . grad phi_j, phi_i) for m = m0..m1 (logpoisson_primal.jl:
   101-107; N_0 = 0), same arguments and layout as sgfem_assemble_stiffness (row i
   of the CSC pattern tests with phi_i, column j is the ansatz) */
SGFEM_API int sgfem_assemble_convection(sgfem_context* ctx, const sgfem_mesh* mesh, const sgfem_fe_space* space,
                                        const sgfem_cosine* coef, int m0, int m1, const sgfem_quadrature* quad,
                                        int64_t nnz, const int64_t* colptr, const int64_t* rowval, double* values);

/*
 * Right-hand sides assembled on the GPU (the reference assembles them on the
 * host with ExtendableFEM's LinearOperator).  f_qp: the caller's f at the points
 * of the cell rule `quad`, nq x ncells (f_qp[c * nq + q]), as for the
 * estimators.  Each dof sums its cells in increasing cell order (no atomics).
 * sgfem_assemble_rhs: b = (f, v), b[ndofs], of solve!(PoissonProblemPrimal)
 *   (poisson_primal.jl:65-68).
 * sgfem_assemble_pce_rhs: b[:, k] = (lambda_k f, v) for the P multi-indices of
 *   solve!(LogTransformedPoissonProblemPrimal) (logpoisson_primal.jl:109-131),
 *   lambda_mu(x) = exp(sum_{m <= N_truncate} a_m(x)^2 / 2) exp(factor a_0)
 *   prod_d a_d(x)^mu_d / (sqrt(prod_d mu_d!) factor^|mu|) (lambda_mu of
 *   expa_PCE_mop, coefficients.jl:219-260; the reference passes factor = -1 and
 *   N_truncate = maxm).  multi_indices: M x P column-major (entry d of mode k at
 *   [k * M + d]), M, N_truncate <= coef->maxm; b: ndofs x P column-major
 *   (SGFEVector entries).
 * ctx only names the GPU, the stream and the error message.
 */
SGFEM_API int sgfem_assemble_rhs(sgfem_context* ctx, const sgfem_mesh* mesh, const sgfem_fe_space* space,
                                 const sgfem_quadrature* quad, const double* f_qp, double* b);
SGFEM_API int sgfem_assemble_pce_rhs(sgfem_context* ctx, const sgfem_mesh* mesh, const sgfem_fe_space* space,
                                     const sgfem_quadrature* quad, const double* f_qp, const sgfem_cosine* coef,
                                     int64_t M, int64_t P, const int32_t* multi_indices, double factor,
                                     int64_t N_truncate, double* b);

/* which FP32 apply kernel a finalized context uses: 1 = specialised to the coupling
   structure (compiled with NVRTC at finalize), 0 = generic; the log says why */
SGFEM_API int sgfem_apply_variant(const sgfem_context* ctx);
SGFEM_API const char* sgfem_apply_variant_log(const sgfem_context* ctx);

/* kernels launched by this context so far (graph replays included) */
SGFEM_API long long sgfem_kernel_launches(const sgfem_context* ctx);

#ifdef __cplusplus
}
#endif
#endif /* SGFEM_H */
