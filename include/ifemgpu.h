/*
 * ifemgpu.h -- C ABI of the GB300 element-integration, assembly and solve
 * path for tensor-product spline (B-spline / NURBS) patches.
 *
 * One context (ifemgpu_ctx) is one simulator model: a set of structured
 * spline patches, their SAM-style DOF numbering, one sparse system matrix in
 * compressed-column storage and its right-hand side, all resident in the
 * memory of one GPU.  Every entry point returns an ifemgpu_status; the text
 * of the last failure is available from ifemgpu_last_error().  There is no
 * CPU fallback: a configuration the GPU path cannot handle is rejected with
 * IFEMGPU_UNSUPPORTED.
 *
 * Each declaration names the IFEM interface it replaces (file:line within
 * the IFEM source tree).  Conventions that follow IFEM exactly:
 *   - nodes of a patch are numbered with the first parametric index fastest
 *     (ASMs3D::generateFEMTopology, src/ASM/ASMs3D.C:487-509);
 *   - element-to-node lists are ascending, first index fastest
 *     (ASMs3D::createMNPC, src/ASM/ASMs3D.C:3899-3924);
 *   - DOFs are node-major, free DOFs are numbered in DOF order
 *     (SAM::initSystemEquations, src/LinAlg/SAM.C:317-323);
 *   - the matrix pattern is SuperLU compressed-column storage with 0-based,
 *     ascending row indices (SparseMatrix::optimiseCols, SparseMatrix.C:984).
 * Equation numbers returned by this API are 1-based like IFEM's MEQN;
 * 0 marks a fixed DOF and a negative value -i marks the i-th prescribed DOF.
 *
 * Threading: a context is used by one host thread at a time.  All device
 * work of a context is ordered on one CUDA stream owned by the context.
 */
#ifndef IFEMGPU_H
#define IFEMGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define IFEMGPU_ABI_VERSION 2

typedef enum ifemgpu_status {
  IFEMGPU_OK = 0,
  IFEMGPU_INVALID_ARG = 1,       /* bad argument or call order            */
  IFEMGPU_OUT_OF_MEMORY = 2,     /* device or host allocation failed      */
  IFEMGPU_SINGULAR_JACOBIAN = 3, /* |det J| <= 1e-12 at an integration pt */
  IFEMGPU_NOT_CONVERGED = 4,     /* iterative solve hit its iteration cap */
  IFEMGPU_DEVICE_TIMEOUT = 5,    /* a bounded device wait gave up          */
  IFEMGPU_CUDA_ERROR = 6,        /* CUDA runtime error                    */
  IFEMGPU_NOT_READY = 7,         /* step required before this call missing */
  IFEMGPU_UNSUPPORTED = 8        /* configuration not handled on the GPU  */
} ifemgpu_status;

typedef struct ifemgpu_ctx ifemgpu_ctx;

/* Arithmetic of the element matrices. */
enum ifemgpu_ke_precision {
  IFEMGPU_KE_FP64 = 0,       /* FP64 on CUDA cores (exact-parity mode)     */
  IFEMGPU_KE_SPLIT_TF32 = 1  /* FP32 via 3xTF32 tcgen05 products, FP32 acc */
};

typedef struct ifemgpu_options {
  int device;        /* CUDA device ordinal; -1 = host-only context (model
                        input, numbering and pattern; no device work)       */
  int ke_precision;  /* enum ifemgpu_ke_precision                            */
  int n_gauss;       /* IFEM nGauss: 1..10 points per direction, or 10+k for
                        degree+1+k points (ASMbase::getNoGaussPt,
                        src/ASM/ASMbase.C:1788-1798)                          */
  int verbose;       /* 0 silent, 1 model summary on stdout                  */
  int colour_passes; /* generic element kernel (patches off the tensor-core
                        kernel): 0 the first assembly times one persistent
                        colour-major launch ordered by per-element done flags
                        (every element must have a volume) against one launch
                        per colour and keeps the faster; 1 one launch per
                        colour; 2 the persistent launch                     */
} ifemgpu_options;

typedef struct ifemgpu_sizes {
  int npatch;
  int nnod;          /* total nodes                                  */
  int nel;           /* total elements (non-zero parametric volume)  */
  int ndof;          /* total DOFs                                   */
  int neq;           /* free equations                               */
  int nceq;          /* prescribed (constraint) equations            */
  int64_t nnz;       /* non-zeros of the system matrix               */
} ifemgpu_sizes;

/* Weak form of a patch: the GPU counterpart of the application Integrand.
 * Poisson:     -div(kappa grad u) = f,   Ke = sum_q kappa dNdX dNdX^T detJxW
 *              (EqualOrderOperators::Weak::LaplacianCoeff,
 *               Apps/Utils/EqualOrderOperators.C:194-211; Source :243-265)
 * Elasticity:  isotropic linear elasticity, Ke = sum_q B^T D B detJxW with
 *              node-interleaved DOFs (IntegrandBase.C:68-77,
 *              EqualOrderOperators.C:27-33 for the component ordering).     */
enum ifemgpu_kind { IFEMGPU_POISSON = 1, IFEMGPU_ELASTICITY = 2 };
enum ifemgpu_source_shape {
  IFEMGPU_SOURCE_CONSTANT = 0,  /* f = source                           */
  IFEMGPU_SOURCE_SINE = 1       /* f = source * prod_d sin(pi x_d)      */
};
enum ifemgpu_field {
  IFEMGPU_FIELD_LOG_KAPPA = 1,   /* g_a: kappa = kappa0 * exp(sum_a R_a g_a) */
  IFEMGPU_FIELD_SOURCE_NOISE = 2 /* eta_a: f *= (1 + sum_a R_a eta_a)        */
};

typedef struct ifemgpu_material {
  int kind;            /* enum ifemgpu_kind                               */
  double kappa;        /* Poisson conductivity (scale of the field)       */
  double source;       /* Poisson source scale f0                         */
  int source_shape;    /* enum ifemgpu_source_shape                       */
  double E, nu;        /* elasticity: Young's modulus, Poisson's ratio    */
  double body[3];      /* elasticity: body force per unit volume          */
} ifemgpu_material;

/* ---- context ---------------------------------------------------------- */

/* Replaces IFEM::Init + SIMbase construction (src/IFEM.C:41-46). */
ifemgpu_status ifemgpu_ctx_create(ifemgpu_ctx** ctx, const ifemgpu_options* opts);
void ifemgpu_ctx_destroy(ifemgpu_ctx* ctx);
const char* ifemgpu_last_error(const ifemgpu_ctx* ctx);
int ifemgpu_abi_version(void);

/* ---- model input ------------------------------------------------------ */

/* Adds one structured spline patch; replaces ASMs3D::read/ASMs2D::read plus
 * generateFEMTopology (src/ASM/ASMs3D.C:433-516, ASMs2D.C:501).
 *   dim       2 or 3 (parametric = spatial dimension)
 *   degree    polynomial degree per direction (GoTools order minus one)
 *   ncoef     control points per direction
 *   knots     per direction, ncoef+degree+1 non-decreasing values
 *   coefs     node-major, first index fastest; per node dim Euclidean
 *             coordinates followed by the weight when rational != 0
 * The arrays are copied.  patch_id receives a 1-based patch index.        */
ifemgpu_status ifemgpu_patch_add(ifemgpu_ctx* ctx, int dim, const int* degree,
                                 const int* ncoef, const double* const* knots,
                                 const double* coefs, int rational,
                                 int* patch_id);

/* Sets the weak form integrated over a patch (Integrand / IntegrandBase::npv,
 * src/ASM/IntegrandBase.h:363).  Must precede ifemgpu_preprocess.        */
ifemgpu_status ifemgpu_patch_set_material(ifemgpu_ctx* ctx, int patch_id,
                                          const ifemgpu_material* mat);

/* Identifies face (3D, 1..6) or edge (2D, 1..4) slave_face of patch slave
 * with face master_face of patch master: the slave's nodes there take the
 * master's global node numbers, so the patches couple conformingly.
 * orient: 0..7 in 3D as in ASMs3D::connectPatch (bit 2 swaps the face's
 * parameter directions, then bits 1 and 0 reverse them), 0/1 in 2D
 * (reversed edge).  Global nodes are numbered as SIMbase::renumberNodes
 * does after connections (first appearance, patch by patch).  Replaces
 * SIM3D/SIM2D::connectPatches -> ASMs3D::connectPatch (src/SIM/SIM3D.C:
 * 44-95, src/ASM/ASMs3D.C:700-796).  Must precede ifemgpu_preprocess.
 * Connected models assemble with per-patch colour passes; the Kronecker
 * preconditioner needs unconnected patches.                              */
ifemgpu_status ifemgpu_patch_connect(ifemgpu_ctx* ctx, int master, int master_face,
                                     int slave, int slave_face, int orient);

/* Adds scale x the consistent mass matrix to the patch's element matrices,
 * K_eff = K + scale M with M_ab = integral N_a N_b (per solution component),
 * the effective stiffness of implicit time stepping (Newmark: scale =
 * density / (beta dt^2)).  M is EqualOrderOperators::Weak::Mass
 * (Apps/Utils/EqualOrderOperators.C:214-227) as NewmarkMats combines it with
 * K (src/ASM/NewmarkMats.C).  scale = 0 removes it.  Must precede
 * ifemgpu_preprocess.                                                      */
ifemgpu_status ifemgpu_patch_set_mass(ifemgpu_ctx* ctx, int patch_id, double scale);

/* Per-control-point coefficient field (enum ifemgpu_field), nnod values.  */
ifemgpu_status ifemgpu_patch_set_field(ifemgpu_ctx* ctx, int patch_id,
                                       int which, const double* values);

/* Dirichlet condition on a patch face; replaces ASMs3D::constrainFace
 * (src/ASM/ASMs3D.C:1025-1102) and ASMs2D::constrainEdge.  face follows the
 * IFEM face index (1:-u 2:+u 3:-v 4:+v 5:-w 6:+w), dofs is a digit list
 * such as 123.  value 0 fixes the DOFs (MSC=0, ASMbase::fix,
 * src/ASM/ASMbase.C:963); a non-zero value prescribes them through a
 * constraint equation with coefficient c0=value (ASMbase::prescribe, :884). */
ifemgpu_status ifemgpu_patch_constrain_face(ifemgpu_ctx* ctx, int patch_id,
                                            int face, int dofs, double value);

/* Constant Neumann data on a face: traction vector (elasticity, npv values)
 * or normal flux (Poisson, 1 value); integrated by the face overload of
 * ASMs3D::integrate (src/ASM/ASMs3D.C:2547-2812).                        */
ifemgpu_status ifemgpu_patch_add_neumann(ifemgpu_ctx* ctx, int patch_id,
                                         int face, const double* values);

/* ---- preprocessing ---------------------------------------------------- */

/* Node/DOF numbering and matrix pattern; replaces SIMbase::preprocessC
 * (src/SIM/SIMbase.C:209-443) -> SAMpatch::init (src/ASM/SAMpatch.C:21-81)
 * and SIMbase::initSystem -> SparseMatrix::preAssemble/optimiseCols
 * (src/LinAlg/SparseMatrix.C:731-762, :984-1023).  Uploads the model to the
 * device and builds the element colouring.                                */
ifemgpu_status ifemgpu_preprocess(ifemgpu_ctx* ctx);

ifemgpu_status ifemgpu_get_sizes(const ifemgpu_ctx* ctx, ifemgpu_sizes* out);

/* SAM arrays (src/LinAlg/SAM.h:333-342): MADOF (nnod+1, 1-based
 * accumulated DOFs) and MEQN (ndof).                                      */
ifemgpu_status ifemgpu_get_madof(const ifemgpu_ctx* ctx, int* madof);
ifemgpu_status ifemgpu_get_meqn(const ifemgpu_ctx* ctx, int* meqn);

/* Element connectivity of a patch: nel x nen patch-local 0-based nodes
 * (ASMbase::MNPC, src/ASM/ASMbase.h:1085).                                */
ifemgpu_status ifemgpu_get_mnpc(const ifemgpu_ctx* ctx, int patch_id,
                                int* mnpc);

/* Compressed-column pattern (SparseMatrix IA/JA, SparseMatrix.h:294-297):
 * colptr has neq+1 entries, rowidx nnz entries.                           */
ifemgpu_status ifemgpu_get_pattern(const ifemgpu_ctx* ctx, int* colptr,
                                   int* rowidx);

/* Replaces the control net of a preprocessed patch (same layout as
 * ifemgpu_patch_add), e.g. for a moved or optimised geometry; the topology
 * and numbering are kept.  The host array is read by an asynchronous copy
 * on the context's stream: it must stay valid until the next synchronising
 * call (pinned memory makes the copy truly asynchronous).  Counterpart of
 * updating the spline coefficients of ASMs3D's Go::SplineVolume before the
 * next SIMbase::assembleSystem.                                           */
ifemgpu_status ifemgpu_patch_update_coefs(ifemgpu_ctx* ctx, int patch_id,
                                          const double* coefs);

/* The CUDA stream (cudaStream_t) all device work of the context runs on. */
ifemgpu_status ifemgpu_get_stream(const ifemgpu_ctx* ctx, void** stream);

/* ---- assembly --------------------------------------------------------- */

/* Zeroes the system and integrates every patch (interior and Neumann
 * faces), scattering into the matrix and right-hand side; replaces
 * SIMbase::assembleSystem (src/SIM/SIMbase.C:1229-1429) with
 * ASMs3D::integrate (src/ASM/ASMs3D.C:2071-2335) and
 * AlgEqSystem::assemble -> SAM::assembleSystem -> assemSparse
 * (src/ASM/AlgEqSystem.C:215-303, src/LinAlg/SAM.C:430-467,
 * src/LinAlg/SparseMatrix.C:614-688).  Stream-ordered; returns once the
 * work is enqueued unless sync != 0.                                      */
ifemgpu_status ifemgpu_assemble(ifemgpu_ctx* ctx, int sync);

/* Copies the assembled matrix values (nnz, FP64, compressed-column order)
 * and the right-hand side (neq) to host memory.                           */
ifemgpu_status ifemgpu_copy_matrix(ifemgpu_ctx* ctx, double* values);
ifemgpu_status ifemgpu_copy_rhs(ifemgpu_ctx* ctx, double* rhs);

/* The same copies without waiting: the matrix values and the right-hand side
 * (rhs may be null) are snapshotted on the device, stream-ordered after the
 * last assembly, and copied to the host buffers on a copy stream, so the
 * next ifemgpu_assemble runs while the copy proceeds (pinned host memory
 * lets the two overlap).  The buffers must stay untouched until
 * ifemgpu_copy_wait returns; copies complete in the order they were made.
 * A time loop that hands every step's system to the host this way runs at
 * the pace of the slower of assembly and copy instead of their sum.       */
ifemgpu_status ifemgpu_copy_system_async(ifemgpu_ctx* ctx, double* values, double* rhs);
ifemgpu_status ifemgpu_copy_wait(ifemgpu_ctx* ctx);

/* Text dumps of the system in the formats of SparseMatrix::dump and
 * StdVector::dump (src/LinAlg/SparseMatrix.C:341-396, SystemMatrix.C:78-102)
 * as SIMbase::dumpEqSys writes them (src/SIM/SIMbase.C:2863-2925): precision
 * 17, matrix label "A" in IFEM's column-oriented (SuperLU) entry order,
 * vector label "b", vector entries with |v| <= zero_tol printed as 0 where
 * IFEM applies utl::trunc.  The format numbers are LinAlg::StorageFormat's
 * (src/LinAlg/LinAlgenums.h:42-48).  Either path may be NULL.             */
enum ifemgpu_dump_format {
  IFEMGPU_DUMP_FLAT = 1,
  IFEMGPU_DUMP_MATLAB = 2,
  IFEMGPU_DUMP_MATRIX_MARKET = 3
};
ifemgpu_status ifemgpu_dump_system(ifemgpu_ctx* ctx, const char* matrix_path,
                                   const char* rhs_path, int format, double zero_tol);
/* The same writer on caller arrays (0-based compressed columns of an n x n
 * matrix with nnz = colptr[n] entries); needs no context or GPU.          */
ifemgpu_status ifemgpu_write_system(int n, const int* colptr, const int* rowidx,
                                    const double* values, const double* rhs,
                                    const char* matrix_path, const char* rhs_path,
                                    int format, double zero_tol);

/* Norms of a solution field u (DOF order, ndof values, e.g. from
 * ifemgpu_expand_solution), integrated with the Gauss rules of the last
 * assembly: totals[0] = a(u, u) (Poisson: int kappa grad u . grad u;
 * elasticity: int sigma(u) : eps(u)), totals[1] = int u . u; element
 * (optional, 2 values per element, patches in order, patch-local elements
 * first index fastest) the same per element.  Replaces SIMbase::
 * solutionNorms (src/SIM/SIMbase.C:1838-1967) with the applications'
 * energy and L2 norm integrands.  Needs an assembly first.               */
ifemgpu_status ifemgpu_solution_norms(ifemgpu_ctx* ctx, const double* u_dof,
                                      double* totals, double* element);

/* Secondary solution of u at every Gauss point of one patch: Poisson flux
 * -kappa grad u (dim values), elasticity stress (6 values, Voigt order
 * xx yy zz xy yz zx).  out: nel x nq x values, elements and points first
 * index fastest; zero at singular points.  Replaces the integrand path of
 * ASMs3D::evalSolution (src/ASM/ASMs3D.C:3179-3500) at the Gauss points. */
ifemgpu_status ifemgpu_secondary_solution(ifemgpu_ctx* ctx, int patch_id,
                                          const double* u_dof, double* out);

/* Device pointers of the system, owned by the context (read-only use).   */
ifemgpu_status ifemgpu_device_system(ifemgpu_ctx* ctx, const double** values,
                                     const int** colptr, const int** rowidx,
                                     const double** rhs);

/* Statistics of the last ifemgpu_assemble: device time in milliseconds of
 * the whole assembly and of its volume integration + scatter passes alone,
 * and the number of integration points skipped because |det J| <= 1e-12
 * (IFEM skips them the same way, src/ASM/ASMs3D.C:2286), and the number of
 * kernels one assembly launches.  Synchronises.  Null pointers are skipped. */
ifemgpu_status ifemgpu_last_assembly_stats(ifemgpu_ctx* ctx, double* total_ms,
                                           double* volume_ms,
                                           long long* singular_points,
                                           int* kernel_launches);

/* Device time of the last assembly's two phases on the tensor-core path:
 * the element kernels (with the generic volume passes of other patches)
 * and the node-wise gathers, from events between the captured segments.
 * No IFEM counterpart (timing diagnostics).                               */
ifemgpu_status ifemgpu_last_assembly_phases(ifemgpu_ctx* ctx, double* element_ms,
                                            double* gather_ms);

/* Block-CSR copy of the assembled matrix for models whose free DOFs come in
 * whole nodes of `block` DOFs (e.g. block 3 for elasticity with fully
 * clamped faces): block rows in equation order, column indices ascending,
 * blocks row-major (block (I, J)[k][l] = K(I*block + k, J*block + l)).
 * Pass null arrays to get *nbrows and *nnzb only.  No IFEM counterpart in
 * this form (IFEM's SparseMatrix is scalar CSC/CSR; PETSc's BAIJ matrices
 * take this layout).                                                      */
ifemgpu_status ifemgpu_copy_matrix_bsr(ifemgpu_ctx* ctx, int block, int* nbrows,
                                       int64_t* nnzb, int* browptr, int* bcolind,
                                       double* bvals);

/* ---- solve ------------------------------------------------------------ */

enum ifemgpu_solver_method {
  IFEMGPU_PCG_MIXED = 1,  /* FP32 Jacobi-PCG inner, FP64 residual refinement */
  IFEMGPU_PCG_FP64 = 2,   /* FP64 Jacobi-PCG                                 */
  IFEMGPU_FCG_LEARNED = 3 /* FP32 flexible CG preconditioned by the fine
                             level (precond) plus the learned coarse
                             correction (ifemgpu_learn_*), FP64 residual
                             refinement; an inner solve that breaks down or
                             does not lower the FP64 residual is undone and
                             the solve continues without the network
                             (counted in info->fallbacks)                  */
};

enum ifemgpu_precond {
  IFEMGPU_PRECOND_JACOBI = 0,    /* point Jacobi                              */
  IFEMGPU_PRECOND_KRONECKER = 1  /* per patch and component: the parameter-cube
                                    Laplacian K0xM1xM2 + M0xK1xM2 + M0xM1xK2 of
                                    the 1D spline stiffness K_d and mass M_d,
                                    inverted by fast diagonalisation and scaled
                                    to the matrix diagonal; 3D patches whose
                                    free DOFs form boxes, no shared nodes,
                                    FP32 methods only                         */
};

typedef struct ifemgpu_solver_options {
  int method;          /* enum ifemgpu_solver_method                     */
  double rtol;         /* target ||b - A x|| / ||b|| in FP64 (e.g. 1e-10) */
  int max_outer;       /* refinement steps (mixed)                       */
  int max_inner;       /* PCG iterations per refinement step / total     */
  double inner_rtol;   /* FP32 residual reduction per refinement step    */
  int precond;         /* enum ifemgpu_precond (fine level of the FP32
                          methods; IFEMGPU_PCG_FP64 takes Jacobi only)    */
} ifemgpu_solver_options;

typedef struct ifemgpu_solve_info {
  int outer_iters;
  int inner_iters;     /* total PCG iterations                           */
  double relres;       /* final FP64 relative residual                   */
  double device_ms;    /* device time of the solve                       */
  int fallbacks;       /* learned inner solves replaced by plain PCG     */
} ifemgpu_solve_info;

/* Solves K x = b with the assembled system; replaces SIMbase::solveSystem
 * -> SparseMatrix::solve (src/SIM/SIMbase.C:1487-1550,
 * src/LinAlg/SparseMatrix.C:1026-1042).  x (neq) is host memory.          */
ifemgpu_status ifemgpu_solve(ifemgpu_ctx* ctx,
                             const ifemgpu_solver_options* opts, double* x,
                             ifemgpu_solve_info* info);

/* FP64 Jacobi-PCG solve of the assembled system that allocates nothing, for
 * callers that cannot allocate device or pinned host memory at solve time:
 * an application that hands its whole device memory to its own pool, a
 * time-stepping or Newton loop that must not synchronise on cudaMalloc, or a
 * host framework that owns the allocator.  No IFEM counterpart: it is the
 * IFEMGPU_PCG_FP64 branch of ifemgpu_solve with a fixed workspace.
 *   - The workspace is a file-scope device array of the library, about
 *     5.8 MB, held by every GPU that loads the library until the process
 *     exits; it limits the system to 65,536 equations (larger systems are
 *     rejected with IFEMGPU_INVALID_ARG).
 *   - The first call on a device looks the array's device address up and
 *     keeps it; make that first call before any stream capture, and do not
 *     reset the device (cudaDeviceReset) while the library is in use.
 *   - All calls share the one array: calls that overlap on the GPU (two
 *     contexts of one device on different streams, or from several host
 *     threads) race and give wrong results.  Calls of one context are
 *     ordered on its stream and are safe.  Calls on different GPUs use
 *     different arrays and share no host memory.
 * rtol is the FP64 relative residual target, max_iter the PCG iteration cap,
 * x (neq, host) receives the solution; info is optional.                   */
ifemgpu_status ifemgpu_solve_noalloc(ifemgpu_ctx* ctx, double rtol, int max_iter,
                                     double* x, ifemgpu_solve_info* info);

/* ---- captured assemble -> solve step ----------------------------------- */

/* Captures one assembly of the model followed by a solve of the assembled
 * system into a single CUDA graph owned by the context, for loops that
 * re-assemble and re-solve a model whose values change between steps
 * (ifemgpu_patch_update_coefs, ifemgpu_patch_update_field): the assembly's
 * kernels, the solver's prologue, and the FP64 refinement loop as a
 * device-driven conditional loop (CUDA conditional WHILE nodes) around the
 * FP32 inner solve, itself a conditional loop over blocks of iterations.  The
 * device takes the loop decisions from the same FP64 quantities as
 * ifemgpu_solve, so a replay gives the bits of ifemgpu_assemble followed by
 * ifemgpu_solve with the same options.  Method IFEMGPU_PCG_MIXED with the
 * Jacobi or Kronecker preconditioner.  The first capture of a context runs
 * one assembly (it settles the assembly's launch tuning).  Replaces the pair
 * SIMbase::assembleSystem -> SIMbase::solveEqSystem
 * (src/SIM/SIMbase.C:1229-1429, :1487-1550) of IFEM's time and parameter
 * loops.                                                                   */
ifemgpu_status ifemgpu_graph_capture(ifemgpu_ctx* ctx, const ifemgpu_solver_options* opts);

/* Replays the captured step on the context's stream and copies the solution
 * (neq values, FP64, equation order) to x (may be null); info as for
 * ifemgpu_solve (device_ms covers assembly and solve).  The assembled system
 * stays on the device as after ifemgpu_assemble.                          */
ifemgpu_status ifemgpu_graph_launch(ifemgpu_ctx* ctx, double* x, ifemgpu_solve_info* info);

/* Equation order -> DOF order, fixed DOFs 0 and prescribed DOFs their value
 * times scale; replaces SAM::expandSolution (src/LinAlg/SAM.C:768-810).   */
ifemgpu_status ifemgpu_expand_solution(const ifemgpu_ctx* ctx, const double* x,
                                       double* u, double scale);

/* ---- learned coarse correction ---------------------------------------- */
/* No IFEM counterpart: IFEM's solvers are SuperLU and PETSc/ISTL Krylov
 * methods with algebraic preconditioners.  For a context of one 3D patch a
 * small network maps the residual, restricted to a coarse grid of
 * (m+1)^3 vertices over the patch's parameter domain (trilinear weights at
 * the Greville points, R; npv values per vertex), to a coarse direction y.
 * Flexible CG (IFEMGPU_FCG_LEARNED) applies it as a two-level step after
 * the fine preconditioner's z1 (Jacobi or Kronecker):
 *   t = A z1,  y = net(R r) or net(R (r - t)),
 *   z = z1 + alpha R^T y,  alpha = (y, R (r - t)) / (y, Ac y),
 * Ac = R A R^T the Galerkin coarse matrix of the assembly (formed on the
 * device at the first learned solve after each assembly): alpha minimises
 * the energy norm of the error after the step, so a poor direction costs
 * its work but no convergence.  The network (3 layers of width `hidden`,
 * ReLU) is trained on the device by the library's own kernels on
 * (residual, error) pairs that solves of the same patch generate.  The
 * coarse cells must be at least as wide as the matrix coupling (p
 * Greville spacings), else the learned solve reports IFEMGPU_UNSUPPORTED. */

typedef struct ifemgpu_learn_options {
  int coarse_cells;   /* m, coarse cells per direction (1..32)            */
  int hidden;         /* hidden width (8..1024)                           */
  int capacity;       /* training pairs kept on the device                */
  unsigned seed;      /* initial weights                                  */
  int field_inputs;   /* 1: the network also reads the patch's
                         log-conductivity field averaged onto the coarse
                         vertices (one network for many fields)          */
} ifemgpu_learn_options;

/* Builds the coarse transfer operators and a freshly initialised network
 * for the preprocessed one-patch 3D model (discards earlier training).    */
ifemgpu_status ifemgpu_learn_setup(ifemgpu_ctx* ctx, const ifemgpu_learn_options* o);

/* Solves A x = rhs (rhs: neq host values, or null for the assembled b)
 * from x = 0 to the relative residual rtol (at most max_iter iterations)
 * with FP32 Jacobi-PCG (precond IFEMGPU_PRECOND_JACOBI) or flexible CG with
 * the Kronecker preconditioner (IFEMGPU_PRECOND_KRONECKER: the iteration the
 * network is added to) and stores one pair per stride-th iterate (see
 * ifemgpu_learn_set_target; Rn is the weight-normalised restriction).  x*
 * is xstar (neq host values) or, when null, the library's FP64-refined
 * solve to 1e-12 with the same preconditioner.  *pairs receives the
 * stored total.                                                           */
ifemgpu_status ifemgpu_learn_collect(ifemgpu_ctx* ctx, const double* rhs,
                                     const double* xstar, int stride,
                                     int max_iter, double rtol, int precond,
                                     int* pairs);

/* Forgets the stored pairs (the network is kept).                         */
ifemgpu_status ifemgpu_learn_clear(ifemgpu_ctx* ctx);

/* What the stored pairs are (default IFEMGPU_LEARN_TARGET_ERROR):
 *   ERROR       input R r_k, target Rn (x* - x_k) / |R r_k|: the whole
 *               coarse error;
 *   COMPLEMENT  input R (r_k - A z_k), target Rn (x* - x_k - z_k) /
 *               |R (r_k - A z_k)|, z_k = M r_k the collecting iteration's
 *               fine preconditioner output (Kronecker along flexible CG,
 *               Jacobi along PCG): the part of the error that the fine step
 *               leaves, seen through the residual it leaves.
 * The learned solve feeds the network the input of the same mode.
 * Changing the mode forgets the stored pairs; learn_setup restores the
 * default.                                                                */
enum ifemgpu_learn_target {
  IFEMGPU_LEARN_TARGET_ERROR = 0,
  IFEMGPU_LEARN_TARGET_COMPLEMENT = 1
};
ifemgpu_status ifemgpu_learn_set_target(ifemgpu_ctx* ctx, int mode);

/* Copies stored pairs first .. first+count-1 to host rows X (`inputs`
 * floats each) and Y (`coarse_unknowns` floats each): the training set's
 * checkpoint, and the check of the restriction.                           */
ifemgpu_status ifemgpu_learn_get_pairs(ifemgpu_ctx* ctx, int first, int count,
                                       float* X, float* Y);

/* Adam on the stored pairs: mean squared error against targets divided by
 * their RMS S, minibatches of `batch`, `epochs` passes, shuffled from seed.
 * The last batch's loss goes to *final_loss (optional).                   */
ifemgpu_status ifemgpu_learn_train(ifemgpu_ctx* ctx, int epochs, int batch,
                                   float lr, unsigned seed, float* final_loss);

/* Mean squared error (targets / S) of the FP32 network on the stored pairs. */
ifemgpu_status ifemgpu_learn_evaluate(ifemgpu_ctx* ctx, float* mse);

/* Loss mean((net(X) - Y)^2) over n host pairs (rows of X hold `inputs`
 * floats, rows of Y `coarse_unknowns`, targets taken as they are) and its
 * gradient with respect to all parameters (layout of
 * ifemgpu_learn_get_weights).                                             */
ifemgpu_status ifemgpu_learn_gradients(ifemgpu_ctx* ctx, const float* X,
                                       const float* Y, int n, float* grad,
                                       float* loss);

/* The trained network's output y (coarse_unknowns floats) for a coarse
 * input rc (coarse_unknowns floats, normalised inside as in the solve; the
 * field features of the current field appended) through the solve's
 * inference path: BF16 tcgen05 products with FP32 accumulation, weights and
 * inputs of each layer rounded to BF16.  Diagnostic; no IFEM counterpart. */
ifemgpu_status ifemgpu_learn_forward(ifemgpu_ctx* ctx, const float* rc, float* y);

/* The Galerkin coarse matrix Ac = R A R^T of the assembled system as a
 * dense row-major nc x nc FP32 array (nc = coarse_unknowns): the matrix
 * the learned step prices its direction with, formed on the device from
 * the FP64 matrix.  Diagnostic; no IFEM counterpart.                       */
ifemgpu_status ifemgpu_learn_coarse_matrix(ifemgpu_ctx* ctx, float* Ac);

/* Sizes of the coarse problem and the network; null pointers skipped.     */
ifemgpu_status ifemgpu_learn_info(const ifemgpu_ctx* ctx, int* coarse_unknowns,
                                  int* inputs, int* hidden, int* nparam,
                                  int* pairs);

/* Parameters as one FP32 array: W1 (hidden x inputs, row-major), b1, W2
 * (hidden x hidden), b2, W3 (nc x hidden), b3, and the target scale S.
 * get with theta null returns only the count; set marks the network
 * trained (checkpoint restore).                                           */
ifemgpu_status ifemgpu_learn_get_weights(ifemgpu_ctx* ctx, float* theta,
                                         int* count, float* scale);
ifemgpu_status ifemgpu_learn_set_weights(ifemgpu_ctx* ctx, const float* theta,
                                         int count, float scale);

/* Replaces the values of a field set before preprocessing (same length),
 * for a new assembly of the same model; the random-coefficient solves that
 * feed the network use it.  No IFEM counterpart (IFEM re-reads a field
 * function per assembly).                                                 */
ifemgpu_status ifemgpu_patch_update_field(ifemgpu_ctx* ctx, int patch_id,
                                          int which, const double* values);

/* ---- diagnostics ------------------------------------------------------ */

/* z = M r with the FP32 preconditioner `precond` (enum ifemgpu_precond) of
 * the assembled matrix, r and z neq host values.  No IFEM counterpart: it
 * checks the preconditioner kernels in isolation.                         */
ifemgpu_status ifemgpu_apply_preconditioner(ifemgpu_ctx* ctx, int precond,
                                            const double* r, double* z);

/* Test hooks of the bounded device waits.  Every wait of a device kernel on
 * another's progress is bounded; one that gives up counts a timeout, the
 * kernel returns, and the next call that needs the assembled system
 * (ifemgpu_assemble with sync, ifemgpu_copy_matrix, ifemgpu_solve, ...)
 * reports IFEMGPU_DEVICE_TIMEOUT and marks the system invalid.  This sets
 * the limits -- flag_spin polls per wait for a neighbour's done flag in the
 * persistent generic pass (0: the default, about 0.1 s), copy_spin polls per
 * wait for a tensor-core kernel's control-point copy (0: the default) -- and
 * picks one element (patch_id 1-based, patch-local element; patch_id 0:
 * none) whose done flag is never published and whose copy is never issued,
 * so that the waits for it run out.  No IFEM counterpart: it exercises the
 * failure path without faulting the GPU.                                  */
ifemgpu_status ifemgpu_debug_waits(ifemgpu_ctx* ctx, unsigned flag_spin, unsigned copy_spin,
                                   int patch_id, int element);

/* Runs the tensor-core building block of the element kernel once on the
 * current device: D (128 x 96) = A (128 x 32) * B (96 x 32)^T in 3xTF32
 * split precision with FP32 accumulation, all row-major host arrays.  No
 * IFEM counterpart: it checks the sm_103a MMA path in isolation.          */
ifemgpu_status ifemgpu_selftest_tc_gemm(const float* A, const float* B, float* D);

#ifdef __cplusplus
}
#endif

#endif /* IFEMGPU_H */
