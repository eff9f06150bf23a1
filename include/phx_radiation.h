/*
 * phx_radiation.h -- C ABI of the GB300 (sm_103a) radiation moment (M1 /
 * Eddington) transport of phoebus.
 *
 * Each entry point replaces one task of the reference's radiation package
 * (src/radiation/moments.cpp, moments_source.cpp, radiation.cpp; paths
 * relative to the phoebus source tree) for the "moment_m1" and
 * "moment_eddington" methods with one neutrino species, on a Minkowski block:
 * with a static fluid background (physics/hydro = false; the reference then
 * calls MomentFluidSource with update_fluid = false), or coupled to the
 * evolved fluid (update_fluid = true: phx_rad_fluid_stage).
 *
 * Conventions are those of phx_fluid.h: caller-owned device memory, FP64,
 * structure of arrays with i fastest, ghost-inclusive inclusive ranges, every
 * call asynchronous on the given stream, no allocation inside a call.  The
 * fluid block (phx_block) supplies the mesh, the coordinates and the fluid
 * primitives the moments read (density, W v^i, internal energy,
 * temperature); the radiation fields live in a phx_rad_block.
 */
#ifndef PHX_RADIATION_H_
#define PHX_RADIATION_H_

#include "phx_fluid.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Conserved radiation moments (cons[PHX_RNCONS][N]), densitised by
 * sqrt(gamma), in the reference's flux order.  Like the fluid's conserved
 * variables they have one copy per RK stage container. */
enum {
  PHX_RE = 0,  /* sqrt(gamma) E                 */
  PHX_RF = 1,  /* sqrt(gamma) F_i (3 entries)   */
  PHX_RNCONS = 4
};
/* Radiation fields with a single copy shared by all stage containers
 * (Metadata::OneCopy in radiation.cpp:471-520): prim[PHX_RNPRIM][N]. */
enum {
  PHX_RJ = 0,       /* J, fluid-frame energy density (radmoment_prim::J)        */
  PHX_RH = 1,       /* H_i / J (3 entries; radmoment_prim::H stores the ratio)  */
  PHX_RXI = 4,      /* closure guess xi = |H| / J (radmoment_internal::xi)      */
  PHX_RPHI = 5,     /* closure guess phi (radmoment_internal::phi)              */
  PHX_RFAIL = 6,    /* c2pfail: 1.0 success, 0.0 failure                        */
  PHX_RKAPPAJ = 7,  /* absorption coefficient (radmoment_internal::kappaJ)      */
  PHX_RKAPPAH = 8,  /* total coefficient (radmoment_internal::kappaH)           */
  PHX_RJBB = 9,     /* black-body energy density (radmoment_internal::JBB)      */
  PHX_RNPRIM = 10
};

typedef enum { PHX_RAD_M1 = 0, PHX_RAD_EDDINGTON = 1 } phx_rad_method; /* radiation.cpp:51-59 */

typedef enum { /* radiation.hpp SourceSolver, radiation.cpp:403-415 (zerod is disabled there) */
  PHX_RAD_SRC_ONED = 0,
  PHX_RAD_SRC_FOURD = 1
} phx_rad_src_solver;

typedef enum { /* fixup/rad_floor_type, fixup.cpp:188-200, fixup.hpp:150-182 */
  PHX_RAD_FLOOR_CONSTANT_J = 0, /* J_floor = J0_floor                          */
  PHX_RAD_FLOOR_EXPX1_J = 1     /* J_floor = J0_floor exp(J_exp_floor X1)     */
} phx_rad_floor_type;

typedef enum { /* radiation.hpp OneDFixupStrategy, radiation.cpp:432-445 */
  PHX_RAD_ONED_FIXUP_NONE = 0,
  PHX_RAD_ONED_FIXUP_IGNORE_DJ = 1,
  PHX_RAD_ONED_FIXUP_IGNORE_ALL = 2
} phx_rad_oned_fixup;

/* Radiation package Params (radiation.cpp:340-450) and the radiation
 * bounds of the fixup package (fixup.cpp:75-76, 188-215).  Fill with
 * phx_rad_params_default() and override. */
typedef struct {
  int method;                 /* phx_rad_method                           */
  int recon;                  /* phx_recon; reference default: linear    */
  double cfl;                 /* radiation/cfl (default 0.8)             */
  int closure_frail;          /* closure_c2p_strategy: 0 robust, 1 frail */
  int recon_fixup_bounds;     /* recon_fixup_strategy: 1 bounds, 0 none  */
  double src_rootfind_tol;    /* radiation/src_rootfind_tol (1e-12)      */
  int src_rootfind_maxiter;   /* radiation/src_rootfind_maxiter (100)    */
  int oned_fixup_strategy;    /* phx_rad_oned_fixup                      */
  /* Gray opacities in the run's code units.  kappaJ = rho kappa_a,
   * kappaH = kappaJ + rho kappa_s, JBB = jbb_coeff T^4.  The reference takes
   * Rosseland means from singularity-opac tables; for gray opacities they
   * are these constants. */
  double kappa_a, kappa_s, jbb_coeff;
  /* fixup/enable_rad_floors (rad_floor_type below), and
   * fixup/enable_rad_ceilings with ConstantXi0 */
  int enable_rad_floors;
  double J0_floor;
  int enable_rad_ceilings;
  double xi0_ceiling, tau0_ceiling;
  /* MomentFluidSource's update_fluid: 0, the fluid is not evolved
   * (physics/hydro = false); 1, the source hands the exchanged energy and
   * momentum to the fluid and inverts it (phx_rad_fluid_stage sets it). */
  int update_fluid;
  /* fixup/rad_c2p_failure_strategy: 0 interpolate (default), 1 floors */
  int rad_c2p_failure_floors;
  /* radiation/src_solver (phx_rad_src_solver, default oned), and for fourd
   * radiation/src_rootfind_eps (finite-difference step, 1e-8) and
   * radiation/src_use_oned_backup (0).  fourd iterates to src_rootfind_tol
   * within src_rootfind_maxiter Newton steps. */
  int src_solver;
  double src_rootfind_eps;
  int src_use_oned_backup;
  /* fixup/rad_floor_type (phx_rad_floor_type, with enable_rad_floors) and
   * fixup/J_exp_floor (-2) of the ExpX1J floor, evaluated at the X1 of the
   * zone (ApplyFloors) or of the face (the flux's reconstructed J) */
  int rad_floor_type;
  double J_exp_floor;
} phx_rad_params;

/* Radiation fields of one block.  Same shape and var_stride convention as
 * the fluid block it is paired with (var_stride 0 = the block's cell count). */
typedef struct {
  long long var_stride;
  double *cons; /* [PHX_RNCONS][N]  stage input E, F_i (the reference's sc0) */
  double *prim; /* [PHX_RNPRIM][N]                                          */
  double *flux; /* [3][PHX_RNCONS][N]  flux(d, m, k, j, i)                  */
  double *dudt; /* [PHX_RNCONS][N]     right-hand side (scratch)            */
} phx_rad_block;

void phx_rad_params_default(phx_rad_params *p);

/* radiation::MomentPrim2Con (moments.cpp:198-275): E, F_i from J, H_i/J and
 * the fluid velocity over the range. */
phx_status phx_rad_prim_to_con(phx_ctx *ctx, const phx_rad_params *rp, const phx_params *p, const phx_block *fb,
                               const phx_rad_block *rb, phx_range ib, phx_range jb, phx_range kb, void *stream);

/* radiation::MomentCon2Prim (moments.cpp:61-192): the closure solve from the
 * stored xi guess, then J, H_i/J, xi, phi, c2pfail (and E, F_i when the
 * robust inversion modified the state) over the range. */
phx_status phx_rad_con_to_prim(phx_ctx *ctx, const phx_rad_params *rp, const phx_params *p, const phx_block *fb,
                               const phx_rad_block *rb, phx_range ib, phx_range jb, phx_range kb, void *stream);

/* radiation::MomentCalculateOpacities (moments.cpp:919-995): kappaJ, kappaH,
 * JBB over the entire block. */
phx_status phx_rad_calculate_opacities(phx_ctx *ctx, const phx_rad_params *rp, const phx_params *p,
                                       const phx_block *fb, const phx_rad_block *rb, void *stream);

/* radiation::ReconstructEdgeStates + radiation::CalculateFluxes
 * (moments.cpp:280-736), fused: flux of E and F_i on every face the
 * interior update reads. */
phx_status phx_rad_calculate_fluxes(phx_ctx *ctx, const phx_rad_params *rp, const phx_params *p,
                                    const phx_block *fb, const phx_rad_block *rb, void *stream);

/* Parthenon FluxDivergence + SumData with CalculateGeometricSource
 * (moments.cpp:764-885: zero on Minkowski; on an FMKS block computed per
 * zone from the stage input E, F_i, the stored J, H_i and the derivative
 * table) + AverageIndependentData + UpdateIndependentData on E, F_i
 * (interior):
 *   cons = beta cons + (1 - beta) base;  out = cons + beta dt dudt.
 * base and out are [PHX_RNCONS][N] arrays with the block's var_stride. */
phx_status phx_rad_update(phx_ctx *ctx, const phx_rad_params *rp, const phx_block *fb, const phx_rad_block *rb,
                          const double *base, double *out, double beta, double dt, void *stream);

/* radiation::MomentFluidSource with the "oned" source solver
 * (moments_source.cpp:203-490, 786-965): the implicit absorption/scattering
 * update of E, F_i over dt, then the frail closure inversion that sets
 * J, H_i/J (or the failure state).  With rp->update_fluid the fluid's tau
 * and S_i lose what the radiation gained, the fluid is inverted (robust
 * con2prim with p's tolerance, iteration cap and floor scale, failing on
 * floors and ceilings: prims, cell speeds, cons where bounds were used), and
 * the closure inversion uses the new fluid velocity; when either inversion
 * fails the fluid becomes rho = u = 10 SMALL at rest (with the bulk modulus
 * stored in the gamma1 slot, as the reference stores it) with its D, S_i,
 * tau from prim2con, and the radiation the J = SMALL, H = 0 state. */
phx_status phx_rad_fluid_source(phx_ctx *ctx, const phx_rad_params *rp, const phx_params *p, const phx_block *fb,
                                const phx_rad_block *rb, double dt, void *stream);

/* Periodic ghost exchange of the radiation fields (E, F_i, J, H_i, xi, phi,
 * c2pfail: every radiation field with Metadata::FillGhost) of a block that
 * is periodic on every active axis. */
phx_status phx_rad_fill_ghosts_periodic(phx_ctx *ctx, const phx_block *fb, const phx_rad_block *rb, void *stream);

/* The radiation fields' part of the boundary exchange of a tiled mesh
 * (phoebus_driver.cpp:646-668; phoebus_boundaries.cpp:42-254, 303-445), on
 * every FillGhost radiation field (E, F_i, J, H_i/J, xi, phi, c2pfail;
 * radiation.cpp:448-474, 506-508).  rblocks[n] pairs with blocks[n]; mesh
 * and blocks as for phx_mesh_exchange, which must have run first (the
 * primitive rebuild reads the fluid ghosts' velocities).  Ghosts inside the
 * domain copy the owning block's fields.  Beyond a physical face each field
 * takes the mapped cell's value: with bc_vars = conserved scaled by the
 * DetGamma ratios, as every FillGhost field (the radiation primitives
 * included); F_d and H_d negated across a reflect face on axis d; polar faces
 * negate no radiation field.  Then, in the outer-X1 slab of an FMKS mesh with
 * p->enable_ox1_fmks_inflow_check, H^1 < 0 is set to 0 with |H| capped at
 * 0.99 (:383-411), and with bc_vars = primitive E and F_i are rebuilt from J,
 * H_i and the ghost's fluid velocity (MomentPrim2Con over the physical
 * slabs, :436-445). */
phx_status phx_rad_mesh_exchange(phx_ctx *ctx, const phx_rad_params *rp, const phx_params *p, const phx_mesh *mesh,
                                 const phx_block *blocks, const phx_rad_block *rblocks, int nblocks, void *stream);

/* FixFluxes' radiation part (fixup.cpp:728-1078) on every block of a tiled
 * mesh that touches a physical boundary, in place on the radiation flux
 * arrays; a no-op unless p->enable_flux_fixup.  Boundary faces only, over
 * the interior of the other axes: reflect faces set the normal flux of E to
 * 0 (X2 faces also those of F_1 and F_3); polar X2 faces set the X2 fluxes
 * of E, F_1 and F_3 to 0; gr_outflow leaves the radiation fluxes alone. */
phx_status phx_rad_fix_fluxes(phx_ctx *ctx, const phx_rad_params *rp, const phx_params *p, const phx_mesh *mesh,
                              const phx_block *blocks, const phx_rad_block *rblocks, int nblocks, void *stream);

/* radiation::EstimateTimestepBlock (radiation.cpp:585-648): cfl * the
 * minimum over interior zones and active directions of dx / csig, written to
 * dt_out_device. */
phx_status phx_rad_estimate_timestep(phx_ctx *ctx, const phx_rad_params *rp, const phx_params *p,
                                     const phx_block *fb, const phx_rad_block *rb, double *dt_out_device,
                                     void *stream);

/* fixup::RadConservedToPrimitiveFixup (fixup_radc2p.cpp:45-225), with
 * p->enable_c2p_fixup: interior zones whose closure inversion failed take the
 * c2pfail-weighted average of their face neighbours' J and H_i / J (or, with
 * rp->rad_c2p_failure_floors or no valid neighbour, J = 10 SMALL, H = 0),
 * H / J held to the xi ceiling, and E, F_i from prim2con. */
phx_status phx_rad_c2p_fixup(phx_ctx *ctx, const phx_rad_params *rp, const phx_params *p, const phx_block *fb,
                             const phx_rad_block *rb, void *stream);

/* fixup::ApplyFloors with the radiation active (fixup.cpp:285-678) over the
 * range: the fluid part (as phx_apply_floors), then, with
 * rp->enable_rad_floors (which needs p->enable_floors), the radiation part:
 * the closure inversion again where the fluid floors or ceilings acted, the
 * J floor as an added isotropic normal-observer field, the xi ceiling.
 * rb->dudt is used as scratch. */
phx_status phx_rad_apply_floors(phx_ctx *ctx, const phx_rad_params *rp, const phx_params *p, const phx_block *fb,
                                const phx_rad_block *rb, phx_range ib, phx_range jb, phx_range kb, void *stream);

/* One RK stage of the moment transport on a periodic block, in the task
 * order of PhoebusDriver::RungeKuttaStage with hydro off
 * (phoebus_driver.cpp:349-362, 547-620, 640-668): opacities, fluxes,
 * update into out, FillDerived (con2prim over the entire block; over the
 * interior when the c2p fixup is off, since nothing reads the ghosts'
 * inversion before the exchange rewrites them), RadConservedToPrimitiveFixup,
 * ApplyFloors, fluid source (beta dt), ApplyFloors, ghost exchange,
 * FillDerived, the fixup and the floors again (the fixups and floors as
 * p / rp enable them).  rb->cons is the stage input (the reference's sc0), base the
 * step's initial state, out the stage output (sc1); everything after the
 * update acts on out and the shared prim fields. */
phx_status phx_rad_stage(phx_ctx *ctx, const phx_rad_params *rp, const phx_params *p, const phx_block *fb,
                         const phx_rad_block *rb, const double *base, double *out, double beta, double dt,
                         void *stream);

/* One RK stage of the fluid and the moments together on a periodic block
 * (physics/hydro = true, phoebus_driver.cpp:318-362, 547-620, 640-680):
 * fluid source terms, fluid fluxes, FluxCT, opacities, radiation fluxes;
 * both updates (fluid_base/fluid_out and rad_base/rad_out, each [nvar][N]
 * like its block's cons); FillDerived (the fluid's con2prim over the entire
 * block, then MomentCon2Prim), ConservedToPrimitiveFixup,
 * RadConservedToPrimitiveFixup, ApplyFloors; MomentFluidSource over beta dt
 * with update_fluid; ApplyFloors; the periodic exchange of the fluid's
 * conserved variables and the radiation fields; FillDerived, the fixups and
 * the floors again.  fb->cons and rb->cons are the stage inputs;
 * rp->update_fluid is implied. */
phx_status phx_rad_fluid_stage(phx_ctx *ctx, const phx_rad_params *rp, const phx_params *p, const phx_block *fb,
                               const phx_rad_block *rb, const double *fluid_base, double *fluid_out,
                               const double *rad_base, double *rad_out, double beta, double dt, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* PHX_RADIATION_H_ */
