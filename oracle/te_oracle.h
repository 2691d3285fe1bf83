/* te_oracle.h -- TEST INFRASTRUCTURE ONLY: C API shared by the oracle
 * restatement (te_oracle.cpp, prefix teo_) and by the reference driver
 * (ref/teref.cpp, prefix teref_).  Host pointers throughout; vectors use the
 * level layout of include/te_gpu.h. */
#ifndef TE_ORACLE_H
#define TE_ORACLE_H
#include "te_gpu.h"
#ifdef __cplusplus
extern "C" {
#endif
typedef struct teo_gmg_config {
  int scheme, fill_type;  /* ghost filler of every level                   */
  int op_kind;            /* 0 Poisson::StarPatchOperator, 1 VarPoisson     */
  int neumann;            /* Poisson operator neumann flag                  */
  int smoother;           /* 0 DFTPatchSolver, 1 Iterative::PatchSolver     */
  int dft_neumann_mask;
  double inner_tol;       /* inner BiCGStab of the patch solver             */
  int inner_max_it, inner_continue_on_breakdown;
  int pre_sweeps, post_sweeps, coarse_sweeps;
  int extrapolate_boundary_ghosts;
  double tol;             /* outer BiCGStab                                 */
  int max_it;
  int use_precond;        /* 0: BiCGStab without the V-cycle                */
  int mid_sweeps;         /* W and FMG cycles (CycleOpts.h:45)              */
  int cycle_type;         /* 0 "V", 1 "W", 2 "F" (CycleBuilder.h:176-191)   */
  int krylov;             /* outer solver: 0 Iterative::BiCGStab, 1 Iterative::CG */
  int precond_exit;       /* BiCGStab early exit adds alpha*M p instead of the
                             reference's alpha*p (te_gpu.h flag
                             TE_BICGSTAB_PRECONDITIONED_EXIT); 0 = reference */
} teo_gmg_config;

/* A function of a point of the domain (x[0..D-1]): the boundary data of the
 * right-hand-side helpers (addDrichletBCToRHS / addNeumannBCToRHS). */
typedef double (*teo_point_fn)(const double* x);
#ifdef __cplusplus
}
#endif
#endif
