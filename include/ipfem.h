/*
 * ipfem.h -- C-ABI of the GB300 (sm_103a) integration-point FEM library.
 *
 * Drop-in boundary for the integration-point residual / tangent / Newton-CG
 * path of labmec/IntPointsFEM.  The entry points replace the reference's
 * TPZCudaCalls (TPZCudaCalls.h:12-51) and back the public API of
 * TPZElastoPlasticIntPointsStructMatrix (TPZElastoPlasticIntPointsStructMatrix.h:33-42).
 * Plain C types only: pointers, sizes, status codes.  No exceptions cross the
 * boundary; every call returns an ipfem_status and the context keeps a
 * message for ipfem_last_error().
 *
 * Memory: a context owns every device buffer it needs (the reference's
 * TPZVecGPU members of TPZNumericalIntegrator, TPZIrregularBlocksMatrix and
 * TPZConstitutiveLawProcessor) and one CUDA stream.  Vector arguments are
 * host or device pointers as selected by the IPFEM_HOST / IPFEM_DEVICE flag
 * of the call.  One context per host thread; no global mutable state.
 *
 * Element type: quadrilateral, order 2 (9 connects x 2 dofs), 3x3 Gauss
 * points, plane strain.
 */
#ifndef IPFEM_H
#define IPFEM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    IPFEM_OK = 0,
    IPFEM_NONCONVERGED = 1,   /* Newton or CG iteration limit reached */
    IPFEM_NAN = 2,            /* non-finite value detected */
    IPFEM_BREAKDOWN = 3,      /* CG: p.Kp <= 0 */
    IPFEM_OOM = 4,            /* device allocation failed */
    IPFEM_INVALID = 5,        /* bad argument / inconsistent mesh */
    IPFEM_CUDA = 6,           /* CUDA runtime error */
    IPFEM_NO_DEVICE = 7       /* no usable sm_100-family device */
} ipfem_status;

enum { IPFEM_HOST = 0, IPFEM_DEVICE = 1 };
enum { IPFEM_PLAIN_FP64 = 0, IPFEM_MIXED = 1 };
enum { IPFEM_PREC_JACOBI = 0, IPFEM_PREC_MLP = 1, IPFEM_PREC_BLOCK_JACOBI = 2 };

/* Element order p = 1, 2 or 3 (the reference's O_LINEAR, O_QUADRATIC and
 * O_CUBIC builds, KernelsMatrixAssemble.h:3-12): (p+1)^2 connects and
 * (p+1)^2 Gauss points per quadrilateral, 2 (p+1)^2 dofs.  The sizes below
 * are those of order 2, the default. */
#define IPFEM_NPTS 9     /* integration points per element (order 2) */
#define IPFEM_NNODE 9    /* connects per element (order 2) */
#define IPFEM_NDOF 18    /* dofs per element (order 2) */
#define IPFEM_MAX_ORDER 3

typedef struct ipfem_ctx ipfem_ctx;

/* ------------------------------------------------------------------ mesh */
/* Host description of the integration-point data that the reference builds
 * in TPZElastoPlasticIntPointsStructMatrix::SetUpDataStructure
 * (TPZElastoPlasticIntPointsStructMatrix.cpp:80-97).  All arrays are read
 * during ipfem_create only.  nn = nq = (order+1)^2 connects and points per
 * element. */
typedef struct {
    int32_t n_elements;
    int32_t n_nodes;          /* connects; equations = 2*n_nodes, dof = 2*node+comp */
    const int32_t *connects;  /* [n_elements*nn] connect order of the element: 4 vertices, the
                                 order-1 nodes of each edge in traversal order (edges v0v1, v1v2,
                                 v2v3, v3v0), interior nodes row by row */
    /* Element blocks, one of the two forms:
     *  dphi:          [n_elements*nq*2*nn] d(phi_n)/d(x_d) at point q, index ((e*nq+q)*2+d)*nn+n
     *  block_storage: [n_elements*(3*nq)*(2*nn)] the reference's fStorage, row-major
     *                 (3*npts) x (2*nshape) (TPZNumericalIntegrator.cpp:371-386) */
    const double *dphi;
    const double *block_storage;
    const double *weight;     /* [n_elements*nq] w*|detJ| (TPZNumericalIntegrator.cpp:425) */
    const uint8_t *fixed;     /* [2*n_nodes] 1 = Dirichlet dof (may be NULL) */
    const double *f0;         /* [2*n_nodes] external load at load factor 0 (may be NULL) */
    const double *df;         /* [2*n_nodes] external load per unit load factor (may be NULL) */
    int32_t order;            /* element order 1, 2 or 3 (0 = 2) */
} ipfem_mesh;

/* Mohr-Coulomb / elastic material (TPZPlasticStepPV<TPZYCMohrCoulombPV,
 * TPZElasticResponse>, main.cpp:550-561).  Per-element arrays override the
 * uniform values when not NULL. */
typedef struct {
    double E, nu;
    double cohesion, phi, psi;        /* radians */
    const double *el_cohesion;        /* [n_elements] or NULL */
    const double *el_phi;             /* [n_elements] or NULL; psi = phi per element */
    double sigma0[4];                 /* in-situ stress xx, xy, yy, zz (seeded as eps_p = -C^{-1} sigma0) */
} ipfem_material;

/* ------------------------------------------------------------- lifecycle */
ipfem_status ipfem_create(const ipfem_mesh *mesh, const ipfem_material *mat, ipfem_ctx **out);
void ipfem_destroy(ipfem_ctx *ctx);
/* message of the last failure on ctx; with ctx == NULL, of the last failed
 * ipfem_create on the calling thread */
const char *ipfem_last_error(const ipfem_ctx *ctx);
const char *ipfem_status_string(ipfem_status s);
/* sizes: n_elements, n_ip, n_nodes, neq, n_colors, n_blocks (nodal 2x2 blocks) */
ipfem_status ipfem_sizes(const ipfem_ctx *ctx, int64_t out[6]);
/* the context's CUDA stream (cudaStream_t), for callers that order their own work */
void *ipfem_stream(ipfem_ctx *ctx);

/* ----------------------------------- TPZElastoPlasticIntPointsStructMatrix */
/* External load factor: rhs_linear = f0 + lambda*df (the reference's
 * fRhsLinear, built by AssembleBoundaryData,
 * TPZElastoPlasticIntPointsStructMatrix.cpp:156-167, and added to the
 * residual at :118 and :147). */
ipfem_status ipfem_set_load_factor(ipfem_ctx *ctx, double lambda);
/* Precision of the tangent and the linear solve (no counterpart in the
 * reference, whose tangent and solve are FP64):
 *  IPFEM_PLAIN_FP64  FP64 tangent and Jacobi-CG (default; bit-exact with the oracle)
 *  IPFEM_MIXED       FP32 tangent (FP32 element blocks and w*Dep, FP32 fma) and
 *                    FP32 Jacobi-CG with FP32 accumulation on the right-hand side
 *                    scaled to unit norm; the residual, the return mapping and
 *                    the Newton update stay FP64, so Newton acts as FP64
 *                    iterative refinement.  cg_rtol is then the inner FP32
 *                    tolerance (1e-4 is a good choice). */
ipfem_status ipfem_set_precision(ipfem_ctx *ctx, int mode);
/* Precision of the residual evaluations in IPFEM_MIXED (no counterpart in
 * the reference): bits = 64 (default) or 32.  With 32 the strain gather
 * (FP32 element blocks, u rounded to FP32 as it is gathered), the weighted
 * stresses and the residual scatter with its colour sums run in FP32 with
 * FP32 accumulation; the return mapping and tangent operator stay FP64 (on
 * the widened FP32 strain), the external load is added in FP64 and the
 * residual norm is FP64.  In the Newton iteration a load step evaluates
 * FP32 residuals until |R| <= switch_rtol |R0| or |R| stops halving, then
 * refines with FP64 residuals (the first at the same u, the tangent kept);
 * the convergence test and the state commit only ever use FP64 residuals.
 * Direct ipfem_assemble / ipfem_assemble_residual calls return the FP32
 * residual (widened) while 32 is set, except when committing. */
ipfem_status ipfem_set_residual_precision(ipfem_ctx *ctx, int bits, double switch_rtol);
/* TPZMatWithMem::SetUpdateMem: when set, the next residual commits the
 * integration-point state (main.cpp:487-522). */
ipfem_status ipfem_set_update_mem(ipfem_ctx *ctx, int update);
/* Assemble(rhs) (TPZElastoPlasticIntPointsStructMatrix.cpp:137-154):
 * rhs = -B^T sigma(u) + rhs_linear, Dirichlet rows zeroed. */
ipfem_status ipfem_assemble_residual(ipfem_ctx *ctx, const double *u, double *rhs, int where);
/* Assemble(K, rhs) (TPZElastoPlasticIntPointsStructMatrix.cpp:99-135):
 * rhs as above; the tangent K stays on the device for ipfem_solve. */
ipfem_status ipfem_assemble(ipfem_ctx *ctx, const double *u, double *rhs, int where);
/* K as nodal 2x2 blocks, rows ascending, columns ascending per row:
 * row_ptr[n_nodes+1], col[n_blocks], vals[4*n_blocks] (row-major blocks);
 * in IPFEM_MIXED mode the FP32 tangent, widened to double. */
ipfem_status ipfem_get_stiffness(ipfem_ctx *ctx, int64_t *row_ptr, int32_t *col, double *vals);
/* K in the reference's matrix form: the upper triangle (column >= row) of
 * the scalar dof matrix in CSR, rows ascending, columns ascending per row,
 * 0-based, int64 indices -- TPZSYsmpMatrix's IA, JA and A, the positions the
 * reference's colour-ordered assembly writes (TPZNumericalIntegrator.cpp:
 * 538-606, FillLIndexes / me), which Assemble(K, rhs) copies back
 * (TPZElastoPlasticIntPointsStructMatrix.cpp:122).  With ia, ja and a all
 * NULL, *nnz receives the number of entries; otherwise *nnz gives the
 * capacity of ja and a (ia holds 2*n_nodes+1) and receives the count; with a
 * NULL only the pattern (ia, ja) is written, which needs no assembled
 * tangent.  Dirichlet rows and columns are stored as assembled (the solves
 * mask them). */
ipfem_status ipfem_get_stiffness_sym_csr(ipfem_ctx *ctx, int64_t *nnz, int64_t *ia, int64_t *ja, double *a);
/* Jacobi-preconditioned CG on the current K (replaces the reference's
 * TPZCudaCalls::SolveCG, TPZCudaCalls.cu:213-290, and the Pardiso solve):
 * stops when |r|^2 <= rtol^2 |b|^2.  *iters receives the iteration count. */
ipfem_status ipfem_solve(ipfem_ctx *ctx, const double *b, double *x, double rtol, int max_it,
                         int where, int *iters);

/* Newton with load stepping (main.cpp:160-262 per step, accept main.cpp:487-522). */
typedef struct {
    int32_t n_steps;
    double newton_rtol;       /* |R| <= newton_rtol |R_0| per step */
    int32_t newton_max_it;
    double cg_rtol;
    int32_t cg_max_it;
} ipfem_solve_opts;

typedef struct {
    int32_t newton_iters;
    int64_t cg_iters;
    int32_t last_step_iters;
    int32_t converged;
    double final_res;
    double ms_assemble, ms_solve, ms_commit;
    int64_t fcg_fallbacks;   /* learned-preconditioner solves that fell back to Jacobi-PCG */
} ipfem_solve_stats;

/* Runs steps [step_begin, step_end); u (neq, host or device per `where`)
 * holds the displacement on entry and exit.  log (3 doubles per Newton
 * iteration: step, cg iterations, |R|) may be NULL. */
ipfem_status ipfem_newton_solve(ipfem_ctx *ctx, const ipfem_solve_opts *opts, int32_t step_begin,
                                int32_t step_end, double *u, int where, ipfem_solve_stats *stats,
                                double *log, int32_t log_cap);

/* Newton variant of the load-stepped solve: 0 = the plain iteration (below),
 * 1 = the modified-Thomas accelerated iteration of Solution(...,
 * modified_thomas_accel_Q = true) (main.cpp:194-217): u += alpha du, residual
 * at u, a second solve with the same tangent for du~, alpha += (alpha du .
 * du~) / (alpha du . alpha du), u += du~; alpha starts at 1 in every load
 * step.  Convergence is still judged on |R| / |R0| after the tangent
 * assembly at the new u.  Refused while the adaptive inner tolerance is on
 * (ipfem_set_inner_tolerance mode 1): with inner solves stopped at up to
 * eta_max the step factor is wrong and the iteration diverged in a measured
 * plastic step. */
ipfem_status ipfem_set_newton_accel(ipfem_ctx *ctx, int mode);

/* Tangent of the Newton iteration: 0 = Assemble(K, rhs) at every iteration
 * (the shipped Solution(), main.cpp:229-233); 1 = initial stiffness, the
 * iteration of the reference's logged runs (the Results folders
 * CPU_NOT_MODIFIED, CPU_MODIFIED and their GPU and PZ twins: K assembled once,
 * then only AssembleResidual per iteration: main.cpp:218-222 with
 * AssembleResidual in place of the Assemble of main.cpp:229-233): the
 * tangent of the first assembly after ipfem_newton_begin is kept for every
 * later linear solve, and later assemblies compute the residual only. */
ipfem_status ipfem_set_newton_tangent(ipfem_ctx *ctx, int mode);
/* Tangent operator of the assemblies: 0 (default) the reference's
 * TangentOperator (FunctionsTangentOperator.h:37-123), bit-identical to it;
 * 1 the consistent spectral tangent, which differs in two places: the spin
 * factor of each eigen-pair (s_i - s_j) / (e_i - e_j) takes the projected
 * principal stresses instead of the trial ones, and each pair's ProdT terms
 * start from zero instead of accumulating over the pairs.  It matches finite
 * differences of the residual in plastic states (the reference's tangent is
 * off by 1e-3 to 1e-2 there) and Newton then converges at its quadratic rate:
 * 45 -> 27 Newton iterations for the plain 40 x 40 ramp and 108 -> 56 for
 * 80 x 80, the same solution to 1e-10; 95 -> 51 for the whole 400 x 400
 * solve of the mixed method with the learned preconditioner.  The residual
 * and the accepted solutions are unchanged; only the iteration differs from
 * the reference's. */
ipfem_status ipfem_set_consistent_tangent(ipfem_ctx *ctx, int on);
/* Spectral decomposition of the trial stress and the elastic strain: 0
 * (default) the reference's SpectralDecomposition
 * (FunctionsSpectralDecomp.h:261-268), bit-identical to it; 1 the closed form
 * of a plane-strain tensor, zz with (0, 0, 1) and the eigen-pairs of the
 * in-plane 2x2 block.  Within about 1e-6 (relative) of a repeated eigenvalue
 * the reference's cubic roots are about 3e-6 off and Multiplicity1 can return
 * the same eigenvector twice; the reconstructed stress is then wrong by the
 * size of the stress, and the residual jumps as a Newton iterate crosses such
 * a state (an in-plane principal stress crossing sigma_zz).  Mode 1 has
 * orthonormal vectors at any gap and no iteration; elsewhere it agrees with
 * the reference to about 1e-7 (the reference's own accuracy there) and turns
 * the reference's NaN at an exactly repeated in-plane eigenvalue into the
 * right stress.  Invalidates the stored tangent. */
ipfem_status ipfem_set_spectral_mode(ipfem_ctx *ctx, int mode);
/* Secant predictor of the load steps (no counterpart in the reference, whose
 * load steps start from the last accepted solution): with on = 1 each load
 * step after the first of a newton_begin run starts from
 *   u_s = u_{s-1} + (u_{s-1} - u_{s-2})
 * (equal load increments), the solutions of the two previous accepted steps.
 * The step's convergence target stays newton_rtol times |R| at u_{s-1} (one
 * more residual evaluation per step), so the accepted solutions meet the
 * same residual bound as without the predictor.  Off by default: the plain
 * method then follows the reference's iterates bit for bit. */
ipfem_status ipfem_set_newton_predictor(ipfem_ctx *ctx, int on);
/* Inner tolerance of the Newton iterations (no counterpart in the reference,
 * whose solve is to a fixed tolerance).  mode 0 (default): every linear
 * solve to opts.cg_rtol.  mode 1: an adaptive forcing term (Eisenstat and
 * Walker's choice 2 with the safeguards of Kelley, "Iterative Methods for
 * Linear and Nonlinear Equations", 1995, ch. 6): the first solve of a load
 * step to opts.cg_rtol, then
 *   eta_k = gamma (|R_k| / |R_k-1|)^alpha, at least gamma eta_k-1^alpha when
 *   that is above 0.1, at least 0.5 newton_rtol |R0| / |R_k| (no solve
 *   beyond what convergence needs), clamped to [eta_min, eta_max];
 *   eta_k = eta_min after an iteration that reduced |R| by less than a
 *   factor 0.9 (stagnation: the rule alone would loosen the solve there).
 * The inner solves stop at relative residual eta_k, so no solve is tighter
 * than the Newton contraction it serves (slow where the tangent is
 * inconsistent).  Eisenstat and Walker suggest gamma 0.9, alpha 2 or
 * (1 + sqrt 5) / 2; eta_min keeps FP32 inner solves above their precision
 * floor. */
ipfem_status ipfem_set_inner_tolerance(ipfem_ctx *ctx, int mode, double gamma, double alpha, double eta_min,
                                       double eta_max);

/* Row stencils of the SpMVs.  On a structured node grid every row of the
 * block tangent has one of a few dozen column-offset patterns (interior
 * vertex, edge and centre nodes and their boundary variants); the SpMVs then
 * form each block's column as node + offset from an 8-bit pattern id instead
 * of loading the column index stored with the block.  Same blocks in the
 * same order: the results are equal bit for bit.  on = 1 (default) uses the
 * stencils wherever the layout has them, 0 the stored indices.  No
 * counterpart in the reference (its solve is Pardiso). */
ipfem_status ipfem_set_row_stencils(ipfem_ctx *ctx, int on);
/* stencils of the FP64 and FP32 (IPFEM_MIXED, else 0) layouts; 0 = explicit
 * columns only (rows longer than 32 blocks or more than 255 patterns) */
ipfem_status ipfem_row_stencil_count(ipfem_ctx *ctx, int32_t *n_fp64, int32_t *n_fp32);
/* The tangent layout the SpMVs read now: fp32 = 0 the FP64 tangent, 1 the
 * FP32 one (IPFEM_MIXED only, else IPFEM_INVALID).  stored_blocks = 2x2
 * blocks held, slots = padded SELL slots, upper_only = 1 when the FP32
 * tangent holds only the blocks (i, j >= i) and reads the lower ones as
 * transposes (structured grids with row stencils on).  Any output may be
 * null.  No counterpart in the reference. */
ipfem_status ipfem_layout_info(ipfem_ctx *ctx, int fp32, int64_t *stored_blocks, int64_t *slots,
                               int32_t *upper_only);

/* Resumable form of the same loop: begin sets the options and the step range;
 * each advance performs n_iters Newton iterations (0 = until the last step is
 * accepted).  An iteration is: CG on the current tangent, u += du,
 * Assemble(K, rhs), convergence test; a converged step is accepted (state
 * committed) inside the iteration that converged, and the next step's first
 * assembly opens the following iteration.  *n_done receives the iterations
 * performed. */
ipfem_status ipfem_newton_begin(ipfem_ctx *ctx, const ipfem_solve_opts *opts, int32_t step_begin, int32_t step_end);
ipfem_status ipfem_newton_advance(ipfem_ctx *ctx, int32_t n_iters, double *u, int where, ipfem_solve_stats *stats,
                                  double *log, int32_t log_cap, int32_t *n_done);

/* ------------------------------------------------ TPZCudaCalls replacements */
/* Canonical deterministic dot product of two device vectors of length neq
 * (the reduction order of the CG; replaces cublasDdot in
 * TPZCudaCalls::SolveCG, TPZCudaCalls.cu:245-286).  *out is a host double.
 * d_a and d_b must be 16-byte aligned (cudaMalloc'd memory is; a slice at an
 * odd double offset is not): misaligned vectors are rejected with
 * IPFEM_INVALID before anything is launched. */
ipfem_status ipfem_dot(ipfem_ctx *ctx, const double *d_a, const double *d_b, double *out);
/* TPZNumericalIntegrator::Multiply (TPZNumericalIntegrator.cpp:25-37):
 * gather + B*u.  d_strain: device, SoA [3][n_ip] (eps_xx, gamma_xy, eps_yy). */
ipfem_status ipfem_gather_strain(ipfem_ctx *ctx, const double *d_u, double *d_strain);
/* TPZCudaCalls::ComputeSigma / ComputeSigmaDep (TPZCudaCalls.cu:165-191):
 * d_sigma_w SoA [3][n_ip]; d_dep SoA [9][n_ip] or NULL (no tangent).  Uses
 * and, if update_mem, commits the context's integration-point state. */
ipfem_status ipfem_compute_sigma(ipfem_ctx *ctx, int update_mem, const double *d_strain,
                                 double *d_sigma_w, double *d_dep);
/* TPZNumericalIntegrator::MultiplyTranspose (TPZNumericalIntegrator.cpp:54-78):
 * -B^T sigma_w, scattered and reduced over colours (no load, no masking). */
ipfem_status ipfem_scatter_residual(ipfem_ctx *ctx, const double *d_sigma_w, double *d_res);
/* The FP32 kernels of the same two steps (IPFEM_MIXED after
 * ipfem_set_residual_precision(ctx, 32, ...)): d_strain float SoA [3][n_ip],
 * each displacement taken relative to its element's first connect (same
 * component) in FP64 and rounded to FP32, FP32 fma; d_sigma_w float SoA
 * [3][n_ip], FP32 element forces summed over colours in FP32, widened into
 * the FP64 d_res (no load, no masking). */
ipfem_status ipfem_gather_strain32(ipfem_ctx *ctx, const double *d_u, float *d_strain);
ipfem_status ipfem_scatter_residual32(ipfem_ctx *ctx, const float *d_sigma_w, double *d_res);

/* The same canonical dot product for callers that cannot allocate device
 * memory (an application that serves all device memory from its own
 * preallocated pool, or a latency-critical pipeline that must not call
 * cudaMalloc, which synchronises the device).  No counterpart in the
 * reference.  Needs no context: d_a and d_b are device vectors of n doubles
 * (n even, n <= 33,554,432), both 16-byte aligned; the result is written to
 * the device double *d_out (8-byte aligned), asynchronously on `stream`
 * (cudaStream_t, NULL = legacy default stream).  Bad arguments (null,
 * misaligned, odd or too large n) are rejected with IPFEM_INVALID before
 * anything touches the device; the message is in ipfem_last_error(NULL).
 * The scratch lives in a 512 KiB array inside the library that every device
 * keeps until process exit; the call allocates nothing and calls no
 * allocating routine.  Every call looks up that array's device address in
 * the current device's context (a lookup, not an allocation); the first call
 * on a device may also load the library's device code, so make it before any
 * stream capture.  Calls share the array: calls that overlap on the GPU (on
 * different streams without ordering) race and give wrong results. */
ipfem_status ipfem_dot_noalloc(const double *d_a, const double *d_b, int64_t n, double *d_out, void *stream);

/* Integration-point state (TPZConstitutiveLawProcessor members), host copies.
 * field: 0 plastic strain [4][n_ip] (xx, xy, yy, zz), 1 stress [4][n_ip],
 *        2 alpha [n_ip], 3 m_type as double [n_ip]. */
ipfem_status ipfem_get_state(ipfem_ctx *ctx, int field, double *out);
ipfem_status ipfem_set_state(ipfem_ctx *ctx, int field, const double *in);

/* Setup arrays computed by the library (for verification):
 * field 0 element colour [n_elements] int32, 1 number of colours (int32),
 * 2 dof indexes [n_elements*2*nn] int32 (fDoFIndexes),
 * 3 dphi [n_elements*nq*2*nn] double, 4 weights [n_ip] double. */
ipfem_status ipfem_get_setup(ipfem_ctx *ctx, int field, void *out);

/* Greedy element colouring of TPZNumericalIntegrator::SetUpColoredIndexes
 * (TPZNumericalIntegrator.cpp:452-536), host only: element e takes, in
 * repeated passes over the elements in index order, the current colour iff
 * none of its 9 connects is marked in this pass.  Returns the number of
 * colours, or -1 on bad arguments. */
int32_t ipfem_color_elements(int32_t n_elements, int32_t n_nodes, const int32_t *connects, int32_t *el_color);
/* the same for nn connects per element */
int32_t ipfem_color_elements_nn(int32_t n_elements, int32_t n_nodes, int32_t nn, const int32_t *connects,
                                int32_t *el_color);

/* ------------------------------------------------- learned preconditioner */
/* None of these has a counterpart in the reference.  A per-node MLP
 * (32 -> 128 -> 128 -> 20, BF16 weights, FP32 accumulation on the tensor
 * cores) maps the FP32 tangent around node i of a structured node grid
 * (node = b*gr + a) to its block row of a sparse triangular factor G
 * (patch position k = 3*(db+1) + (da+1), da, db in {-1, 0, 1}).  Features:
 * X_i[4m + 2p + q] = K_ij[p][q] s_i[p] s_j[q] for the 8 neighbours j in k
 * order without the centre, s = sqrt(Jacobi inverse diagonal), 0 on Dirichlet
 * dofs.  Factor: G_ik = O_i[4k..4k+3] (row-major 2x2) for k = 0..3,
 * G_i4 = [[exp(O_i[16]), 0], [O_i[17], exp(O_i[18])]], entries touching a
 * Dirichlet dof 0.  Operator: M = diag(s) G^T G diag(s), symmetric positive
 * definite on the free dofs by construction; O = 0 is Jacobi.  The network
 * runs once per tangent; G and G^T are applied (two stencil passes) in every
 * iteration of flexible CG (Polak-Ribiere), which falls back to Jacobi-PCG
 * when it stagnates.  Requires IPFEM_MIXED.  Parameters are one FP32 vector
 * of 23316 values: W1[32][128] b1[128] W2[128][128] b2[128] W3[128][20]
 * b3[20]. */
ipfem_status ipfem_set_node_grid(ipfem_ctx *ctx, int32_t gr, int32_t gt);
/* allocates the network (He-uniform W1, W2; W3 = 0, zero biases) */
ipfem_status ipfem_mlp_init(ipfem_ctx *ctx, uint64_t seed);
/* Preconditioner of the CG solves: IPFEM_PREC_JACOBI (default; z_i = r_i / K_ii
 * on free dofs), IPFEM_PREC_BLOCK_JACOBI (z = B_i^-1 r at every node, B_i the
 * 2x2 diagonal block of the tangent restricted to the node's free dofs; plain
 * and mixed precision), IPFEM_PREC_MLP (the learned factor above, IPFEM_MIXED
 * only).  No counterpart in the reference, which factorises K (Pardiso). */
ipfem_status ipfem_set_preconditioner(ipfem_ctx *ctx, int kind);
ipfem_status ipfem_mlp_get_params(ipfem_ctx *ctx, float *out);
ipfem_status ipfem_mlp_set_params(ipfem_ctx *ctx, const float *in);
/* features [n_nodes][32] (device) of the current FP32 tangent */
ipfem_status ipfem_mlp_features(ipfem_ctx *ctx, float *d_X);
/* network output [rows][20] (device) for device feature rows [rows][32] */
ipfem_status ipfem_mlp_forward(ipfem_ctx *ctx, const float *d_X, int64_t rows, float *d_O);
/* the factor G[5][n_nodes][2][2] of the current tangent (device) */
ipfem_status ipfem_mlp_operator(ipfem_ctx *ctx, float *d_M);
/* training pass on the current FP32 tangent: the loss
 *   w_kaporin * (log(tr(G A G^T) / nf) - (2/nf) log det G)
 *   + w_pairs * (1/n_pairs) sum_p |K e_p - K M r_p|^2 / |K e_p|^2
 * (A = diag(s) K diag(s), nf free dofs; the first line is the log of
 * Kaporin's condition number of M K up to a constant) over n_pairs >= 0
 * (residual r_p, solution increment e_p) pairs, FP32 device arrays
 * [n_pairs][neq], and its gradient (host, 23316 floats; grads and loss may
 * be NULL) */
ipfem_status ipfem_learn_grad(ipfem_ctx *ctx, const float *d_r, const float *d_e, int n_pairs, float w_kaporin,
                              float w_pairs, float *grads, float *loss);
/* one Adam step (beta 0.9, 0.999) with the host gradient, or with the
 * context's last gradient when grads is NULL */
ipfem_status ipfem_mlp_adam(ipfem_ctx *ctx, const float *grads, float lr);
/* FP32 Jacobi-CG with (x_k, r_k) snapshots at iterations that are multiples of
 * 32, plus the final iterate (training data: residual / solution increment) */
ipfem_status ipfem_cg_snapshots(ipfem_ctx *ctx, const double *d_b, double rtol, int max_it, int n_snap,
                                const int32_t *snap_iters, float *d_xs, float *d_rs, float *d_xfinal, int *iters);

/* ------------------------------------------------------------ diagnostics */
/* JSON-lines record of the Newton iterations of ipfem_newton_solve /
 * ipfem_newton_advance, appended to the file at `path` (NULL or "" closes
 * it): per iteration {"step", "iter", "cg_iters", "res" (|R|), "res_rel"
 * (|R| / |R0| of the load step), "ms_solve", "ms_assemble", "ips_assemble"
 * (integration points per second of the iteration's assembly),
 * "fcg_fallback"}, and per accepted load step {"step", "accepted",
 * "newton_iters", "converged", "res_rel", "ms_commit", "ms_step_total"}.
 * The reference prints its residual norms to stdout (main.cpp:239-252). */
ipfem_status ipfem_set_iteration_log(ipfem_ctx *ctx, const char *path);
/* number of kernels this context has launched (graph nodes included) */
uint64_t ipfem_launch_count(const ipfem_ctx *ctx);
/* average duration of the CG block SpMV on the current tangent, timed with
 * CUDA events on the context's stream over `reps` back-to-back launches */
ipfem_status ipfem_profile_spmv(ipfem_ctx *ctx, int reps, double *ms_per_launch);
/* average durations (ms) of the four kernels of one residual evaluation at
 * the device displacement d_u, in the order they run: ms[0] strain
 * gather, ms[1] return mapping (no tangent, no commit), ms[2] stress to
 * element forces, ms[3] colour reduction + load.  bits = 64: the FP64
 * kernels; 32: the FP32 gather and scatter (IPFEM_MIXED after
 * ipfem_set_residual_precision(ctx, 32, ...)).  The chain runs `reps` times;
 * CUDA events between the kernels on the context's stream time each one with
 * the cache state the others leave.  The integration-point state is not
 * changed. */
ipfem_status ipfem_profile_residual(ipfem_ctx *ctx, const double *d_u, int bits, int reps, double *ms);
/* FP64 fma issue rate of this device (TFLOP/s, 2 flops per fma), measured with
 * a dependent-chain probe kernel timed by CUDA events */
ipfem_status ipfem_measure_fp64_peak(ipfem_ctx *ctx, double *tflops);

/* --------------------------------------------------- wellbore mesh provider */
/* Structured quarter annulus standing in for the reference's NeoPZ/Gmsh mesh
 * (main.cpp:447-464, 542-607): nr x nt order-2 quads, radial grading,
 * in-situ stress sigma0 on the outer arc, well traction ramped from sigma0
 * to pw_final*I, symmetry u_y = 0 on y = 0 and u_x = 0 on x = 0. */
typedef struct {
    int32_t nr, nt;
    double r_in, r_out, grading;
    double E, nu, cohesion, phi_deg, psi_deg;
    double sxx0, syy0, sxy0, szz0;
    double pw_final;
    int32_t material_mode;    /* 0 uniform, 1 lognormal cohesion, 2 + uniform friction angle */
    double c_cv, phi_lo_deg, phi_hi_deg;
    uint64_t seed;
} ipfem_wellbore_params;

typedef struct {
    ipfem_mesh mesh;
    ipfem_material material;
    double *node_xy;          /* [n_nodes*2] */
    /* owned storage behind mesh / material */
    int32_t *connects;
    double *dphi, *weight, *f0, *df, *el_cohesion, *el_phi;
    uint8_t *fixed;
    uint8_t *el_shape;        /* [n_elements] 0 quadrilateral, 1 triangle (NULL: all quadrilaterals) */
    int32_t n_ghost;          /* ghost connects of the triangles (fixed, zero shape functions) */
} ipfem_wellbore;

void ipfem_wellbore_default(ipfem_wellbore_params *p, int32_t n);
ipfem_status ipfem_wellbore_build(const ipfem_wellbore_params *p, ipfem_wellbore **out);
void ipfem_wellbore_free(ipfem_wellbore *w);

/* ------------------------------------------------------------ Gmsh meshes */
/* The reference reads its geometry with NeoPZ's TPZGmshReader
 * (ReadGeometry, main.cpp:447-464; gmsh/wellbore_*.msh).  This reads the
 * same files: Gmsh 4.1 ASCII with 4-node quadrilaterals (element type 3),
 * 3-node triangles (type 2; the reference's wellbore_mix.msh mixes both),
 * 2-node lines (type 1) and points (type 15); every element carries the first
 * physical tag of its entity (0 when it has none).  Node indices are 0-based
 * in file order.  Other element types, binary files and other format versions
 * are rejected (IPFEM_INVALID, message in ipfem_last_error(NULL)). */
typedef struct {
    int32_t n_nodes;
    double *xy;                       /* [2*n_nodes] */
    int32_t n_quads;
    int32_t *quads, *quad_phys;       /* [4*n_quads] (file node order), [n_quads] */
    int32_t n_lines;
    int32_t *lines, *line_phys;       /* [2*n_lines], [n_lines] */
    int32_t n_points;
    int32_t *points, *point_phys;     /* [n_points], [n_points] */
    int32_t n_phys;
    int32_t *phys_dim, *phys_tag;     /* [n_phys] $PhysicalNames */
    char **phys_name;                 /* [n_phys] */
    int32_t n_tris;
    int32_t *tris, *tri_phys;         /* [3*n_tris] 3-node triangles (element type 2), [n_tris] */
} ipfem_gmsh;

ipfem_status ipfem_gmsh_read(const char *path, ipfem_gmsh **out);
void ipfem_gmsh_free(ipfem_gmsh *g);

/* A boundary condition on the lines and points of one physical tag: the
 * reference's TBCData (id, type, value; main.cpp:374-446) as NeoPZ's
 * elastoplastic material applies it:
 *   0  u = 0 (both components; non-zero values are rejected)
 *   1  traction (val[0], val[1]) per unit length
 *   3  directional Dirichlet: u_k = 0 for every k with val[k] != 0
 *   6  normal stress: traction val[0] * n, n the outward unit normal
 * The Dirichlet types act on every node of the tagged entities (for a line,
 * its two vertices and its edge connects). */
typedef struct {
    int32_t phys;
    int32_t type;
    double val[2];
} ipfem_bc;

/* Problem of order 1, 2 or 3 on a Gmsh mesh (CmeshElastoplasticity with
 * p_order = order, main.cpp:546-601): every quadrilateral whose physical tag
 * is domain_phys (every quadrilateral if domain_phys < 0) becomes an element
 * of (order+1)^2 connects, its edge connects equally spaced on the straight
 * edges and its interior connects on the bilinear map (the geometric elements
 * are linear); a shared edge's connects are numbered from its lower-numbered
 * vertex, so that both elements use the same ones.  Triangles of the domain tag
 * (the reference's mixed mesh wellbore_mix.msh) become order-p Lagrange
 * triangles carried in the block shape of the order-p quadrilateral: their
 * (p+1)(p+2)/2 connects, then ghost connects with zero shape functions and
 * fixed dofs up to (p+1)^2, and (p+1)^2 collapsed-Gauss points; el_shape
 * marks them and n_ghost counts the ghosts.  Connects are numbered
 * in order of first use by the elements, so that elements close in file
 * order share nearby rows.  Loads go into df (f0 = 0): load factor 1 applies
 * them in full.  mat supplies E, nu, cohesion, phi, psi and sigma0
 * (el_cohesion and el_phi must be NULL).  The result has the layout of the
 * wellbore provider's and is released with ipfem_wellbore_free. */
ipfem_status ipfem_gmsh_problem(const ipfem_gmsh *g, int32_t order, int32_t domain_phys, const ipfem_bc *bcs,
                                int32_t n_bc, const ipfem_material *mat, ipfem_wellbore **out);

#ifdef __cplusplus
}
#endif

#endif /* IPFEM_H */
