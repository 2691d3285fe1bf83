/*
 * te_gpu.h -- C ABI of the GB300 geometric-multigrid hot path.
 *
 * Every entry point is plain C: opaque handles, device pointers, sizes and an
 * int status (TE_OK == 0).  No CUDA, torch or C++ types cross this boundary,
 * so a C++ adapter (see include/thunderegg_gb300/adapters.hpp), ctypes or any
 * other FFI can bind it.  Each function names the ThunderEgg interface it
 * replaces (paths are inside the ThunderEgg source tree, src/ThunderEgg/...).
 *
 * Data layout (identical to ThunderEgg's Vector<D>, Vector.h:133-153):
 *   one level vector = num_patches patches, contiguous;
 *   one patch        = [component][z][y][x], x fastest, every spatial axis
 *                      padded by num_ghost cells on both sides.
 * So a device level buffer can be wrapped by ThunderEgg's unmanaged Vector
 * constructor (Vector.h:199) with patch_starts[i] = base + i * patch_stride.
 *
 * Mesh tables (te_level_desc) are the flattened Domain<D>/PatchInfo<D>/NbrInfo
 * data (PatchInfo.h:66-126): local index == position in the arrays.  Face
 * slots follow PatchInfo's nbr_infos indexing, Face<D,M>::sum_of_faces +
 * face index (Face.h:75-78): 2D corners 0..3, sides 4..7; 3D corners 0..7,
 * edges 8..19, sides 20..25.  Side index = 2*axis + is_upper (Face.h:558-584).
 *
 * Threading: a handle is bound to the stream that was current (te_set_stream)
 * in the creating thread when it was created; calls on one handle are not
 * thread safe, handles of different streams may be used from different threads.
 */
#ifndef TE_GPU_H
#define TE_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
enum {
  TE_OK = 0,
  TE_ERR_INVALID = 1,     /* bad argument (null handle, size mismatch, ...) */
  TE_ERR_CUDA = 2,        /* a CUDA runtime call failed                     */
  TE_ERR_BREAKDOWN = 3,   /* Krylov breakdown: rho == 0, or (BiCGStab) a non-
                             finite residual or rho (BreakdownError.h)      */
  TE_ERR_UNSUPPORTED = 4, /* combination not supported (e.g. odd n trilinear) */
  TE_ERR_BUDGET = 5,      /* serving admission: request over memory budget  */
  TE_ERR_TIMEOUT = 6,     /* bounded device-side wait ran out               */
  TE_ERR_NOT_CONVERGED = 7
};

/* arithmetic type of a level vector */
enum { TE_F64 = 0, TE_F32 = 1 };

/* neighbour types (NbrType.h); -1 = no neighbour on that face */
enum { TE_NBR_NONE = -1, TE_NBR_NORMAL = 0, TE_NBR_COARSE = 1, TE_NBR_FINE = 2 };

/* ghost schemes and GhostFillingType (GhostFillingType.h:33-47) */
enum { TE_GHOST_BILINEAR = 0, TE_GHOST_BIQUADRATIC = 1, TE_GHOST_TRILINEAR = 2 };
enum { TE_FILL_FACES = 0, TE_FILL_EDGES = 1, TE_FILL_CORNERS = 2 };

/* One level of the mesh: the flattened PatchInfo<D> vector of a Domain<D>.
 * All pointers are HOST pointers; the arrays are copied at te_domain_create. */
typedef struct te_level_desc {
  int dim;            /* D = 2 or 3                                        */
  int ns[3];          /* cells per patch along each axis                   */
  int num_ghost;      /* ghost layers per side (>= 1)                      */
  int num_patches;    /* P                                                 */
  const int* id;             /* [P]                                        */
  const int* refine_level;   /* [P]                                        */
  const int* parent_id;      /* [P]      -1 = none                         */
  const int* orth_on_parent; /* [P]      -1 = Orthant::null()              */
  const int* child_ids;      /* [P*2^D]  -1 = none                         */
  const double* starts;      /* [P*D]                                      */
  const double* spacings;    /* [P*D]                                      */
  const int* nbr_type;       /* [P*F]    TE_NBR_*, F = 8 (2D) / 26 (3D)    */
  const int* nbr_ids;        /* [P*F*4]  neighbour ids (fine: by orthant)  */
  const int* nbr_orth;       /* [P*F]    orth_on_coarse for coarse nbrs    */
} te_level_desc;

typedef struct te_domain te_domain;
typedef struct te_ghost_filler te_ghost_filler;
typedef struct te_operator te_operator;
typedef struct te_patch_solver te_patch_solver;
typedef struct te_restrictor te_restrictor;
typedef struct te_interpolator te_interpolator;
typedef struct te_cycle te_cycle;

/* ---- library ------------------------------------------------------------ */
const char* te_last_error_message(void);
/* Stream used by handles this thread creates after this call (a cudaStream_t,
 * or NULL for the legacy default stream); each thread has its own.  The text
 * of te_last_error_message is per thread as well. */
int te_set_stream(void* cuda_stream);
int te_synchronize(void);
/* Number of kernels this library has launched since load (for accounting). */
long long te_kernel_launch_count(void);

/* ---- Domain<D> (Domain.h:94-248) ---------------------------------------- */
/* Uploads the level's flattened metadata; resolves neighbour ids to local
 * indexes exactly as Domain::indexPatchesLocal (Domain.h:94-110). */
int te_domain_create(const te_level_desc* desc, te_domain** out);
int te_domain_destroy(te_domain* d);
/* doubles (or floats) of one patch with ncomp components, ghosts included */
long long te_domain_patch_stride(const te_domain* d, int ncomp);
int te_domain_num_patches(const te_domain* d);
/* A zero-filled device level buffer of the domain (num_patches * patch_stride
 * elements of TE_F64 or TE_F32), for a Vector<D> made with the unmanaged
 * constructor (Vector.h:199-215); free it with te_level_free. */
int te_level_alloc(const te_domain* d, int ncomp, int dtype, void** out);
int te_level_free(void* buffer);
/* Plain device memory and a synchronous copy in either direction (host or
 * device pointers, unified addressing), for callers without the CUDA runtime
 * headers (the C++ adapters' boundary-data arrays). */
int te_device_alloc(size_t bytes, void** out);
int te_device_free(void* p);
int te_copy(void* dst, const void* src, size_t bytes);

/* ---- Vector<D> algebra (Vector.h:391-611); interior cells only unless
 *      with_ghost.  x, a, b, c are device level buffers of the domain. ---- */
int te_vec_set(const te_domain* d, int ncomp, int dtype, void* x, double alpha, int with_ghost);
int te_vec_scale(const te_domain* d, int ncomp, int dtype, void* x, double alpha);
int te_vec_shift(const te_domain* d, int ncomp, int dtype, void* x, double delta);
int te_vec_copy(const te_domain* d, int ncomp, int dtype, void* x, const void* b, int with_ghost);
int te_vec_add(const te_domain* d, int ncomp, int dtype, void* x, const void* b);
/* x += alpha*a */
int te_vec_add_scaled(const te_domain* d, int ncomp, int dtype, void* x, double alpha, const void* a);
/* x += alpha*a + beta*b */
int te_vec_add_scaled2(const te_domain* d, int ncomp, int dtype, void* x, double alpha,
                       const void* a, double beta, const void* b);
/* x = alpha*x + b */
int te_vec_scale_then_add(const te_domain* d, int ncomp, int dtype, void* x, double alpha,
                          const void* b);
/* x = alpha*x + beta*b */
int te_vec_scale_then_add_scaled(const te_domain* d, int ncomp, int dtype, void* x,
                                 double alpha, double beta, const void* b);
/* x = alpha*x + beta*b + gamma*c */
int te_vec_scale_then_add_scaled2(const te_domain* d, int ncomp, int dtype, void* x,
                                  double alpha, double beta, const void* b, double gamma,
                                  const void* c);
/* reductions return a host double; accumulation is FP64, fixed order */
int te_vec_two_norm(const te_domain* d, int ncomp, int dtype, const void* x, double* out);
int te_vec_inf_norm(const te_domain* d, int ncomp, int dtype, const void* x, double* out);
int te_vec_dot(const te_domain* d, int ncomp, int dtype, const void* x, const void* b,
               double* out);
/* precision conversion between level buffers of the same domain (all cells) */
int te_vec_convert(const te_domain* d, int ncomp, int dst_dtype, void* dst, int src_dtype,
                   const void* src);

/* ---- GhostFiller<D> (GhostFiller.h:46, MPIGhostFiller.h:956-1092) -------- */
int te_ghost_filler_create(const te_domain* d, int scheme, int fill_type, te_ghost_filler** out);
int te_ghost_filler_destroy(te_ghost_filler* g);
int te_ghost_fill(const te_ghost_filler* g, int ncomp, int dtype, void* u);
/* Length of the call list (number of fillGhostCellsFor*NbrPatch calls per
 * fill) and the list itself, in the reference's enumeration order
 * (MPIGhostFiller.h:821-895): rows of
 * {caller local index, nbr local index, face dimensionality M, face index,
 *  nbr type, orthant}. */
int te_ghost_filler_num_calls(const te_ghost_filler* g);
int te_ghost_filler_calls(const te_ghost_filler* g, int* rows6);

/* ---- PatchOperator<D> (PatchOperator.h:126-143) ------------------------- */
/* Poisson::StarPatchOperator (Poisson/StarPatchOperator.h:52-63) */
int te_poisson_operator_create(const te_domain* d, const te_ghost_filler* g, int neumann,
                               te_operator** out);
/* VarPoisson::StarPatchOperator (VarPoisson/StarPatchOperator.h:61-71):
 * coeffs is a device FP64 level buffer with 1 component, ghosts included;
 * it is copied and its ghosts filled with g. */
int te_varpoisson_operator_create(const te_domain* d, const te_ghost_filler* g,
                                  const void* coeffs, te_operator** out);
int te_operator_destroy(te_operator* op);
/* f = A u  (f.setWithGhost(0); fillGhost(u); applySinglePatch per patch) */
int te_operator_apply(const te_operator* op, int ncomp, int dtype, void* u, void* f);
/* modifyRHSForInternalBoundaryConditions on every patch: f_in -= ... using
 * u's ghosts (which the caller has filled) */
int te_operator_modify_rhs(const te_operator* op, int ncomp, int dtype, const void* u, void* f);

/* ---- right-hand-side boundary helpers -------------------------------------
 * The reference's helpers take the boundary data as functions of a point
 * (std::function); across the ABI the caller evaluates them at the boundary
 * points and passes the values.  Boundary data arrays are device FP64
 * [P][2D][FS] with FS = te_domain_face_stride: side s = 2 * axis + is_upper,
 * face cell e = the tangential cell indices in increasing axis order, the
 * first fastest; entries of sides with a neighbour are ignored.
 * te_domain_boundary_points writes the points themselves into a device array
 * [P][2D][FS][D], as DomainTools::GetRealCoordBound (DomainTools.h:179-210)
 * computes them: the side's own coordinate on the patch boundary, cell
 * centres in the other directions.  Sides are processed in the reference's
 * order and each term in its operation order, so FP64 results match the
 * reference bit for bit. */
long long te_domain_face_stride(const te_domain* d);
int te_domain_boundary_points(const te_domain* d, double* coords);
/* Poisson::StarPatchOperator::addDrichletBCToRHS (Poisson/StarPatchOperator.h:187-204):
 * f += -2 g / h^2 on the interior cells next to every side without a neighbour;
 * VarPoisson::StarPatchOperator::addDrichletBCToRHS (VarPoisson/StarPatchOperator.h:194-219):
 * f -= 2 g c / h^2 with cvals the coefficient at the boundary points (NULL for
 * the Poisson operator, required for VarPoisson). */
int te_operator_add_dirichlet_bc_to_rhs(const te_operator* op, int dtype, void* f, const double* gvals,
                                        const double* cvals);
/* Poisson::StarPatchOperator::addNeumannBCToRHS (Poisson/StarPatchOperator.h:212-242):
 * f += dg / h on lower sides and f -= dg / h on upper sides, dgvals = the
 * derivative of g along the side's axis at the boundary points.  The
 * VarPoisson operator has no Neumann helper (TE_ERR_UNSUPPORTED), as in the
 * reference. */
int te_operator_add_neumann_bc_to_rhs(const te_operator* op, int dtype, void* f, const double* dgvals);

/* ---- PatchSolver<D> / GMG::Smoother<D> (PatchSolver.h:107-170) ---------- */
/* Poisson::DFTPatchSolver (Poisson/DFTPatchSolver.h:385-450); neumann_mask
 * bit i = Side index i is Neumann (when it has no neighbour). */
int te_dft_patch_solver_create(const te_operator* op, int neumann_mask, te_patch_solver** out);
/* Poisson::FFTWPatchSolver (Poisson/FFTWPatchSolver.h:189-308) computes the
 * same solve (FFTW's RODFT/REDFT kinds are the same DST/DCT families, the
 * eigenvalues and the prod 1/(2n) scale match): a caller of that class binds
 * te_dft_patch_solver_create. */
/* Iterative::PatchSolver with an inner BiCGStab (Iterative/PatchSolver.h:121-175) */
int te_bicgstab_patch_solver_create(const te_operator* op, double tol, int max_iterations,
                                    int continue_on_breakdown, te_patch_solver** out);
int te_patch_solver_destroy(te_patch_solver* s);
/* smooth: fillGhost(u), then solveSinglePatch on every patch (block Jacobi) */
int te_patch_solver_smooth(const te_patch_solver* s, int ncomp, int dtype, const void* f, void* u);
/* apply: u.setWithGhost(0), then solveSinglePatch on every patch */
int te_patch_solver_apply(const te_patch_solver* s, int ncomp, int dtype, const void* f, void* u);
/* *out = 1 when the FP32 DFT solves of this solver run on the tensor cores
 * (3xTF32 tcgen05 contractions: cubic patches, n = 16, 32 or 64 in 2D or 16 in
 * 3D, one set of transform matrices for the level; TE_NO_TC=1 at creation
 * turns it off).  No counterpart in the reference. */
int te_patch_solver_uses_tensor_cores(const te_patch_solver* s, int* out);
/* Poisson::DFTPatchSolver (Poisson/DFTPatchSolver.h:385-450) with the arithmetic
 * of its FP32 tensor-core transforms chosen (no counterpart in the reference):
 * TE_TC_TF32X3 = 3xTF32 split products (what te_dft_patch_solver_create uses,
 * about FP32 accuracy), TE_TC_BF16 = BF16 operands with FP32 accumulation, each
 * patch's right-hand side scaled by a power of two that brings its largest
 * magnitude into [1, 2) and the result scaled back (8 significant bits per
 * operand: a preconditioner for an FP64 outer loop, te_ir_solve or BiCGStab).
 * FP64 solves of the same solver stay FP64.  TE_TC_BF16 where the tensor-core
 * path does not apply gives TE_ERR_UNSUPPORTED. */
enum { TE_TC_TF32X3 = 0, TE_TC_BF16 = 1 };
int te_dft_patch_solver_create_tc(const te_operator* op, int neumann_mask, int tc_precision,
                                  te_patch_solver** out);

/* ---- GMG transfers -------------------------------------------------------- */
/* GMG::LinearRestrictor (GMG/LinearRestrictor.h:166-191, MPIRestrictor.h:55-83)
 * coarse_out is overwritten (ghosts included). */
int te_linear_restrictor_create(const te_domain* fine, const te_domain* coarse,
                                int extrapolate_boundary_ghosts, te_restrictor** out);
int te_restrictor_destroy(te_restrictor* r);
int te_restrict(const te_restrictor* r, int ncomp, int dtype, const void* fine, void* coarse_out);
/* GMG::DirectInterpolator (GMG/DirectInterpolator.h:60-91): fine += P coarse */
int te_direct_interpolator_create(const te_domain* coarse, const te_domain* fine,
                                  te_interpolator** out);
int te_interpolator_destroy(te_interpolator* i);
int te_interpolate(const te_interpolator* i, int ncomp, int dtype, const void* coarse, void* fine);

/* ---- GMG::Cycle (GMG/Cycle.h:94-98, VCycle.h:46-70, CycleBuilder.h:97-192) */
typedef struct te_cycle_level {
  const te_operator* op;           /* level operator                        */
  const te_patch_solver* smoother; /* level smoother                        */
  const te_restrictor* restrictor; /* to the next coarser level (NULL at coarsest) */
  const te_interpolator* interpolator; /* from this level to the next finer (NULL at finest) */
} te_cycle_level;
typedef struct te_cycle_opts {
  int pre_sweeps, post_sweeps, mid_sweeps, coarse_sweeps; /* CycleOpts.h:33-55 */
} te_cycle_opts;
/* levels[0] is the finest.  All level objects must be FP64-capable; the
 * cycle runs in `dtype` internally (TE_F32 = mixed-precision V-cycle: the
 * cycle converts f to FP32, cycles in FP32 and writes FP64 u). */
int te_vcycle_create(const te_cycle_level* levels, int num_levels, te_cycle_opts opts, int dtype,
                     te_cycle** out);
/* CycleBuilder::getCycle (CycleBuilder.h:176-191): cycle_type TE_CYCLE_V
 * ("V", VCycle.h), TE_CYCLE_W ("W", WCycle.h:50-84: a mid_sweeps smooth and
 * a second coarse visit per level) or TE_CYCLE_FMG ("F", FMGCycle.h:43-104).
 * te_vcycle_create(...) is te_cycle_create(..., TE_CYCLE_V, ...); other types
 * give TE_ERR_UNSUPPORTED. */
enum { TE_CYCLE_V = 0, TE_CYCLE_W = 1, TE_CYCLE_FMG = 2 };
int te_cycle_create(const te_cycle_level* levels, int num_levels, te_cycle_opts opts, int cycle_type, int dtype,
                    te_cycle** out);
int te_cycle_destroy(te_cycle* c);
/* u = M f  (u.setWithGhost(0); visit(finest, f, u)); f and u are FP64 */
int te_cycle_apply(const te_cycle* c, int ncomp, const void* f, void* u);

/* Per-kernel device times of one eager application of the cycle (the GPU
 * counterpart of the reference's per-level Timer, Timer.h:60-202): fills up to
 * max_entries names (32 chars each, "L<k> <phase>") and milliseconds measured
 * with CUDA events between consecutive kernels.  Only the fused DFT-smoother
 * cycle records phases; *count = 0 otherwise.  An FP32 cycle is timed as the
 * mixed-precision BiCGStab runs it, with FP32 input and output (f is
 * converted before the first event and the result into u after the last). */
int te_cycle_timings(const te_cycle* c, int ncomp, const void* f, void* u, int max_entries, char* names,
                     double* ms, int* count);

/* ---- Iterative::BiCGStab (Iterative/BiCGStab.h:111-203) ------------------- */
/* Right-preconditioned BiCGStab on FP64 device vectors of A's domain.
 * M may be NULL.  Stops when ||r||/||b|| <= tol.  Returns TE_ERR_BREAKDOWN
 * when rho == 0 (the reference throws BreakdownError), and when the right-hand
 * side, a residual or rho is not finite (no reference counterpart: its NaN
 * comparisons are false, so it returns at once or runs to max_iterations).
 * With an FP32 cycle as M (mixed precision) the iteration runs in float-float
 * arithmetic (pairs of FP32 numbers, ~48 significant bits) on the FP32 pipes;
 * the initial residual and x in and out stay FP64.  When the float-float
 * recurrence has converged, every solve's true residual b - A x is computed
 * in FP64; a solve still above tol restarts from it (residual replacement),
 * and the final residual reported is that FP64 residual.  With an FP64 cycle
 * or no preconditioner the iteration runs in FP64.
 * flags: 0 = the reference's update rule exactly; TE_BICGSTAB_PRECONDITIONED_EXIT
 * = on the early exit (||s|| small) add alpha * M p instead of alpha * p
 * (the reference adds alpha * p, BiCGStab.h:160-168, which leaves the true
 * residual of a preconditioned solve well above tol); TE_BICGSTAB_FP64_OUTER
 * = run the iteration in FP64 even with an FP32 cycle (no counterpart in the
 * reference). */
enum { TE_BICGSTAB_PRECONDITIONED_EXIT = 1, TE_BICGSTAB_FP64_OUTER = 2, TE_BICGSTAB_SLOTS = 4 };
int te_bicgstab_solve(const te_operator* A, int ncomp, void* x, const void* b, const te_cycle* M,
                      double tol, int max_iterations, int flags, int* iterations,
                      double* final_residual);

/* ---- Iterative::CG (Iterative/CG.h:126-194) ------------------------------- */
/* CG on FP64 device vectors of A's domain in the reference's form: the
 * iteration runs on a correction started at zero, applies M to each search
 * direction before A, and ends with x = M y + x0.  M may be NULL (any cycle
 * type and precision).  Stops when ||r||/||b|| <= tol; *final_residual is
 * that recursive residual.  TE_ERR_BREAKDOWN when rho == 0 (the reference
 * throws BreakdownError).  A zero b returns at once with x's interior zero. */
int te_cg_solve(const te_operator* A, int ncomp, void* x, const void* b, const te_cycle* M, double tol,
                int max_iterations, int* iterations, double* final_residual);

/* ---- iterative refinement (no counterpart in the reference) ----------------
 * FP64 iterative refinement around a cycle, behind the Iterative::Solver
 * signature (Iterative/Solver.h:64-69): r = b - A x in FP64; while
 * ||r||/||b|| > tol: x += M r, r = b - A x.  The stopping test is on the true
 * FP64 residual every iteration; *final_residual is that residual.  M is
 * required (typically an FP32 cycle, whose tensor-core transforms may run in
 * BF16, te_patch_solver_set_tc_precision).  A zero b returns at once with x
 * unchanged; a non-finite b or residual returns TE_ERR_BREAKDOWN. */
int te_ir_solve(const te_operator* A, int ncomp, void* x, const void* b, const te_cycle* M, double tol,
                int max_iterations, int* iterations, double* final_residual);

/* Batched form: num_solves independent systems whose finest-level patches
 * are the contiguous ranges [patch_offsets[i], patch_offsets[i+1]) of A's
 * domain (a union of meshes of equal depth; M a V-cycle on the union).  Each
 * solve keeps its own scalars, stops on its own tolerance and reports its own
 * iterations, residual and status (TE_OK / TE_ERR_BREAKDOWN).  A solve's
 * result does not depend on the other solves in the batch.  No counterpart in
 * the reference (one solve per BiCGStab::solve call). */
int te_bicgstab_solve_batched(const te_operator* A, int ncomp, void* x, const void* b, const te_cycle* M,
                              double tol, int max_iterations, int flags, int num_solves,
                              const int* patch_offsets, int* iterations, double* final_residuals,
                              int* statuses);

/* A batched BiCGStab run that the caller advances a few iterations at a time
 * (the serving loop's unit of work; no counterpart in the reference, whose
 * Iterative::BiCGStab::solve runs to the end).  create computes the initial
 * residuals of all solves (same arguments as te_bicgstab_solve_batched; x, b,
 * A and M must outlive the handle); step runs up to max_iterations iterations
 * of the solves still iterating and sets *num_running (0: every solve has
 * finished, x holds the results); state reports per solve the iterations,
 * the last residual (the FP64 true residual once finished in the float-float
 * loop), the status and whether it is still iterating; sync_x waits for the
 * batch's work to finish (x holds every solve's current iterate between
 * steps). */
typedef struct te_bicgstab_batch te_bicgstab_batch;
int te_bicgstab_batch_create(const te_operator* A, int ncomp, void* x, const void* b, const te_cycle* M, double tol,
                             int max_iterations, int flags, int num_solves, const int* patch_offsets,
                             te_bicgstab_batch** out);
int te_bicgstab_batch_step(te_bicgstab_batch* batch, int max_iterations, int* num_running);
int te_bicgstab_batch_state(const te_bicgstab_batch* batch, int* iterations, double* residuals, int* statuses,
                            int* running);
int te_bicgstab_batch_sync_x(te_bicgstab_batch* batch);
/* Slot mode (a batch created with flags | TE_BICGSTAB_SLOTS; no reference
 * counterpart): continuous batching of the solves.  _step only iterates.
 * Solves that stopped on their recurrences are finished together by
 * _finish_slots: one FP64 residual pass gives each listed solve's true
 * residual, and per solve either reports it finished (finished[k] = 1; x holds
 * its result in its patch range) or restarts it from that residual (at most 8
 * times per solve).  _reset puts a new system into a solve that is not
 * iterating: the caller has written its right-hand side and initial iterate
 * into the solve's patch range of b and x; it starts at iteration 0 while the
 * other solves keep their state. */
int te_bicgstab_batch_finish_slots(te_bicgstab_batch* batch, int num_slots, const int* slots, int* finished);
int te_bicgstab_batch_reset(te_bicgstab_batch* batch, int slot);
int te_bicgstab_batch_destroy(te_bicgstab_batch* batch);

/* ---- autotuner (no counterpart in the reference) ---------------------------
 * Launch shapes and kernel variants of the tunable kernels (the tensor-core
 * patch solve: operand placement and resident CTAs per SM; the BiCGStab patch
 * smoother: threads per patch) are chosen per (device, kernel, shape key) by
 * timing every candidate with CUDA events the first time the shape is met
 * outside a stream capture; cycles tune their levels before capturing their
 * graphs.  TE_TUNE=0 keeps the defaults; TE_TUNE_CACHE=<file> keeps choices
 * across processes.  te_tune_report writes the choices and each candidate's
 * median milliseconds as JSON into buf (len bytes) and the length needed
 * (with the terminating zero) into *needed; te_tune_reset forgets them. */
int te_tune_report(char* buf, int len, int* needed);
int te_tune_reset(void);

/* ---- serving: continuous batching of independent solves --------------------
 * No counterpart in the reference (one solve per Iterative::BiCGStab::solve
 * call, BiCGStab.h:111-203); the native form of thunderegg_gb300.serve.Server.
 * A request is one GMG-preconditioned BiCGStab solve of -Lap u = f (Poisson
 * star operator, Dirichlet sides, V-cycle) on its own hierarchy, finest level
 * first, with its right-hand side on the host (finest level, padded layout,
 * FP64).  te_serve_submit copies the tables and f and queues the request
 * (TE_ERR_BUDGET when it alone needs more device memory than the budget).
 * Each te_serve_step is one scheduling round: it admits queued requests while
 * the estimated device memory of the admitted ones and of cached idle unions
 * fits the budget; packs the admitted requests of one class (equal patch shape
 * and te_solve_opts, any depth) into one union hierarchy so that every
 * per-level kernel covers all of them; starts waiting requests in free slots
 * built on their mesh while the others iterate; re-forms a class's batch when
 * requests wait without such a slot (running solves continue from their
 * current iterates); runs steps_per_round BiCGStab iterations of every batch;
 * and finishes the solves that stopped (FP64 true residual; restart when it
 * is above tol).  *unfinished = requests queued or still solving.
 * te_serve_poll returns TE_PENDING until the request has finished, then
 * TE_OK once, with u (finest level, padded layout, FP64, host) and the
 * result.  A request's result matches the same solve run alone within the
 * solver tolerance.  One thread drives a server; its handles bind to the
 * stream that was current (te_set_stream) at te_serve_create. */
enum { TE_PENDING = 8 };
typedef struct te_server te_server;
typedef struct te_serve_opts {
  double budget_bytes; /* device memory the admitted requests may hold (estimated) */
  int steps_per_round; /* BiCGStab iterations per batch per round (>= 1)             */
  int max_batch;       /* most solves in one batch (>= 1)                            */
} te_serve_opts;
typedef struct te_solve_opts {
  int scheme;                      /* TE_GHOST_*                                   */
  int fill_type;                   /* TE_FILL_*                                    */
  int smoother;                    /* 0 DFT patch solver, 1 BiCGStab patch solver  */
  double inner_tol;                /* BiCGStab patch solver: tolerance,            */
  int inner_max_iterations;        /*   iteration limit,                           */
  int inner_continue_on_breakdown; /*   continue on breakdown                      */
  int pre_sweeps, post_sweeps, coarse_sweeps;
  double tol;                      /* outer BiCGStab: relative residual            */
  int max_iterations;
  int cycle_dtype;                 /* TE_F32 mixed precision, TE_F64 plain         */
  int flags;                       /* TE_BICGSTAB_PRECONDITIONED_EXIT, ..._FP64_OUTER */
  int tc_precision;                /* TE_TC_TF32X3 or TE_TC_BF16                    */
} te_solve_opts;
typedef struct te_serve_result {
  int status;        /* TE_OK or TE_ERR_BREAKDOWN                             */
  int iterations;    /* outer iterations, over every batch it was in          */
  double residual;   /* final relative residual (FP64 true residual with an FP32 cycle) */
  double latency_s;  /* submit to result                                      */
  int restarts;      /* batch re-formations the request went through          */
} te_serve_result;
typedef struct te_serve_counters {
  long long submitted, admitted, completed, rejected;
  long long union_builds, union_cache_hits, slot_fills, reforms, rounds;
  int queued, active, classes;
  double bytes_in_use; /* estimate: admitted requests and cached idle unions */
  double build_s;      /* host seconds spent building unions (device objects)   */
  double step_s;       /* host seconds in te_bicgstab_batch_step                 */
  double finish_s;     /* host seconds finishing solves and copying results out  */
  double form_s;       /* host seconds forming batches (iterates, uploads), without builds */
} te_serve_counters;
int te_serve_create(const te_serve_opts* opts, te_server** out);
int te_serve_destroy(te_server* s);
int te_serve_submit(te_server* s, const te_level_desc* levels, int num_levels, const te_solve_opts* opts,
                    const double* f, long long* request_id);
int te_serve_step(te_server* s, int* unfinished);
int te_serve_poll(te_server* s, long long request_id, double* u, te_serve_result* result);
int te_serve_stats(const te_server* s, te_serve_counters* out);

/* ---- dot product without allocation ---------------------------------------
 * No counterpart in the reference (ThunderEgg reduces on the host).
 * For callers that cannot call cudaMalloc when they need a reduction: hosts
 * whose device memory belongs to another allocator (a pool that reserved the
 * GPU at start-up), or callers that must not trigger the device-wide
 * synchronisation an allocation can cause.  Computes the
 * interior dot product of two level buffers of the given layout (the same
 * result as te_vec_dot) and allocates nothing: its scratch is a fixed device
 * array of TE_NOALLOC_MAX_PARTIALS + 1 doubles that every GPU using this
 * library holds until exit.  num_patches * ncomp above TE_NOALLOC_MAX_PARTIALS
 * is rejected with TE_ERR_UNSUPPORTED.  Calls share the array: calls that
 * overlap on the GPU race, so serialise them.  The first call on a device
 * looks up the array's device address; make it before any stream capture.
 * Synchronises `cuda_stream` (NULL = legacy default stream) to return *out. */
#define TE_NOALLOC_MAX_PARTIALS 65536
int te_level_dot_noalloc(int dim, const int* ns, int num_ghost, int num_patches, int ncomp, int dtype,
                         const void* x, const void* y, double* out, void* cuda_stream);

#ifdef __cplusplus
}
#endif
#endif /* TE_GPU_H */
