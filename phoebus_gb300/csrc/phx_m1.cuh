// phx_m1.cuh -- declarations of the radiation moment kernels (phx_m1.cu).
#pragma once
#include "phx_kernels.cuh"
#include "../../include/phx_radiation.h"

namespace phx {
namespace rad {

// Radiation package parameters resolved for the device (phx_rad_params plus
// the fluid ceiling and the EOS heat capacity).
struct RPar {
  int m1;          // 1 M1 closure, 0 Eddington
  int robust;      // closure_c2p_strategy robust (MomentCon2Prim)
  int bounds;      // recon_fixup_strategy bounds
  int recon;       // phx_recon
  int maxiter;     // src_rootfind_maxiter
  int oned_fixup;  // phx_rad_oned_fixup
  int update_fluid;  // MomentFluidSource also updates and inverts the fluid
  int rad_fixup_floors;  // rad_c2p_failure_strategy floors (else interpolate)
  int fourd;       // src_solver fourd (else oned)
  int oned_backup;  // src_use_oned_backup
  double fd_eps;   // src_rootfind_eps
  double cfl, tol, kappa_a, kappa_s, jbb;
  double J_floor, xi_ceiling, tau_max, W_ceiling, Cv;
  int floor_expx1;  // rad_floor_type ExpX1J: J_floor exp(J_alpha X1)
  double J_alpha;
};

// Radiation fields of one block.
struct RView {
  double *cons, *prim, *flux, *dudt;
  long long vs;
};

void launch_p2c(const RPar &p, const BView &b, const RView &r, Range3 rg, cudaStream_t s);
void launch_c2p(const RPar &p, const BView &b, const RView &r, Range3 rg, cudaStream_t s);
void launch_opacities(const RPar &p, const BView &b, const RView &r, cudaStream_t s);
void launch_fluxes(const RPar &p, const BView &b, const RView &r, cudaStream_t s);
// FluxDivergence + SumData (the geometric source on FMKS blocks) + the RK
// update of the interior
void launch_update(const RPar &p, const BView &b, const RView &r, const double *base, double *out, double beta,
                   double dt, cudaStream_t s);
// fp: the fluid's con2prim settings for update_fluid (failure on floors and
// ceilings, as MomentFluidSourceImpl sets them up)
void launch_source(const RPar &p, const Par &fp, const BView &b, const RView &r, double dt, cudaStream_t s);
void launch_ghosts(const BView &b, const RView &r, cudaStream_t s);
// The radiation fields' boundary exchange of block blk of a tiled mesh
// (views / rviews: device arrays over the mesh's blocks); inflow: the FMKS
// outer-X1 inflow check is on.  Reads the fluid ghosts' primitives, so it runs
// after the fluid's exchange.
void launch_mesh_ghosts(const RPar &p, bool mink, const BView &b, const BView *views, const RView *rviews,
                        const MeshDev &m, int blk, int inflow, cudaStream_t s);
// the direction-d radiation fluxes of the moments in mask (bit m: moment m)
// zeroed on local face index f over the interior of the other axes
void launch_fix_face(const BView &b, const RView &r, int d, int f, unsigned mask, cudaStream_t s);
// RadConservedToPrimitiveFixup over the interior
void launch_rad_c2p_fixup(const RPar &p, const BView &b, const RView &r, cudaStream_t s);
// the radiation part of ApplyFloors over rg; flag[N]: nonzero where the fluid
// part floored or ceilinged the zone (launch_floors' flag output)
void launch_rad_floors(const RPar &p, const BView &b, const RView &r, const double *flag, Range3 rg,
                       cudaStream_t s);
void launch_dt(const RPar &p, const BView &b, const RView &r, unsigned long long *scratch, double *dt_out,
               cudaStream_t s);

}  // namespace rad
}  // namespace phx
