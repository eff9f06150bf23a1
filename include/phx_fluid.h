/*
 * phx_fluid.h -- C ABI of the GB300 (sm_103a) GRMHD fluid hot path.
 *
 * This is the drop-in boundary for the fluid update of phoebus (lanl/phoebus).
 * Every entry point below replaces one Parthenon task of the reference fluid
 * package (file:line cited beside each declaration, paths relative to the
 * phoebus source tree).  The C++ shim in phx_parthenon_shim.hpp keeps the
 * reference's task signatures and forwards to these functions.
 *
 * Conventions
 *   - All arrays are caller-owned DEVICE memory, FP64, structure-of-arrays:
 *     field(v, k, j, i) = base[v * var_stride + (k * n2t + j) * n1t + i],
 *     with i fastest.  n1t = nx1 + 2 ng, n2t = nx2 + 2 ng (1 when ndim < 2),
 *     n3t = nx3 + 2 ng (1 when ndim < 3).  This is Parthenon's per-variable
 *     View layout, so packs can be passed through without copies.
 *   - Index ranges (phx_range) are inclusive, in ghost-inclusive indices,
 *     exactly like Parthenon's IndexRange.
 *   - Every call is asynchronous on the given CUDA stream (cudaStream_t passed
 *     as void*; NULL = legacy default stream).  Nothing is allocated inside a
 *     call; scratch lives in the phx_ctx or in caller-owned block fields.
 *   - Device code never traps.  Per-zone failures are written as the
 *     reference's fail flags (1.0 success / 0.0 failure).  Conditions the
 *     reference aborts on (an unbracketed con2prim root) are recorded in the
 *     context's sticky error word, read with phx_ctx_check().
 */
#ifndef PHX_FLUID_H_
#define PHX_FLUID_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PHX_ABI_VERSION 1

/* ---- variable indices ------------------------------------------------- */
/* Primitive block (prim[PHX_NPRIM][N]).  The first PHX_NRECON entries are the
 * reconstructed variables, in the order the reference registers them
 * (fluid.cpp:272-286: density, velocity(3), energy, bfield(3), pressure,
 * gamma1).  The reference takes its flux (conserved) indices from this same
 * map (riemann.hpp:240-245). */
enum {
  PHX_PRHO = 0,  /* rest-mass density rho                           */
  PHX_PVEL = 1,  /* W v^i (3 entries, normal-observer 3-velocity * W) */
  PHX_PENG = 4,  /* internal energy density u = rho * eps            */
  PHX_PB = 5,    /* B^i (3 entries)                                  */
  PHX_PPRS = 8,  /* pressure                                         */
  PHX_PGM1 = 9,  /* gamma1 = bulk modulus / pressure                 */
  PHX_PTMP = 10, /* temperature                                      */
  PHX_PMU = 11,  /* c2p_mu: last con2prim root (warm-start guess)    */
  PHX_NPRIM = 12,
  PHX_NRECON = 10
};
/* Conserved block (cons[PHX_NCONS][N]), densitized by sqrt(gamma). */
enum {
  PHX_CRHO = 0, /* D = sqrt(gamma) rho W            */
  PHX_CMOM = 1, /* S_i (3 entries)                  */
  PHX_CENG = 4, /* tau (Valencia energy)            */
  PHX_CB = 5,   /* sqrt(gamma) B^i (3 entries)      */
  PHX_NCONS = 8
};

typedef enum {
  PHX_OK = 0,
  PHX_ERR_INVALID_ARG = 1,
  PHX_ERR_UNBRACKETED = 2, /* con2prim root not bracketed (reference aborts) */
  PHX_ERR_NAN_INPUT = 3,
  PHX_ERR_TIMEOUT = 4,     /* a bounded device wait gave up                */
  PHX_ERR_CUDA = 5,
  PHX_ERR_NO_DEVICE = 6,
  PHX_ERR_CAPACITY = 7,    /* request larger than a fixed-size buffer      */
  PHX_ERR_UNSUPPORTED = 8
} phx_status;

typedef enum { /* reconstruction.hpp:23 ReconType */
  PHX_RECON_CONSTANT = 0,
  PHX_RECON_LINEAR = 1, /* PLM, MC limiter with alpha = 1.5            */
  PHX_RECON_WENO5Z = 2, /* WENO5-Z blended with MC (alpha = 2)         */
  PHX_RECON_MP5 = 3
} phx_recon;

typedef enum { PHX_RIEMANN_LLF = 0, PHX_RIEMANN_HLL = 1 } phx_riemann; /* riemann.hpp:30 */

typedef enum { PHX_GEOM_MINKOWSKI = 0, PHX_GEOM_FMKS = 1 } phx_geom_kind;

typedef enum { /* fixup.hpp FloorFlag */
  PHX_FLOOR_CONSTANT_RHO_SIE = 0,
  PHX_FLOOR_EXPX1_RHO_SIE = 1,
  PHX_FLOOR_EXPX1_RHO_U = 2,
  PHX_FLOOR_X1_RHO_SIE = 3,
  PHX_FLOOR_R_RHO_SIE = 4
} phx_floor_type;

typedef struct {
  int s, e; /* inclusive, ghost-inclusive */
} phx_range;

/* Physics parameters: the fluid, fixup and eos package Params the hot path
 * reads (fluid.cpp:53-136, fixup.cpp:48-280, eos_phoebus.cpp:73-95).  Fill
 * with phx_params_default() and override. */
typedef struct {
  /* ideal-gas EOS (singularity-eos IdealGas in scale-free units) */
  double gm1;  /* Gamma - 1 */
  double Cv;
  double rho_min_eos, sie_min_eos; /* eos/rho_min, eos/sie_min (default 0) */
  /* con2prim (fluid.cpp:76-94) */
  double c2p_tol;
  int c2p_max_iter;
  double c2p_floor_scale_fac;
  int c2p_fail_on_floors;
  int c2p_fail_on_ceilings;
  /* reconstruction / Riemann solver / timestep */
  int recon;   /* phx_recon   */
  int riemann; /* phx_riemann */
  double cfl;
  int mhd;     /* fluid/mhd: 1 = B evolved (FluxCT applied) */
  /* fixup package */
  int enable_floors, enable_ceilings, enable_mhd_floors, enable_c2p_fixup;
  int c2p_failure_strategy_floors; /* 0 = interpolate (default), 1 = floors */
  int floor_type;                  /* phx_floor_type */
  double rho0_floor, sie0_floor, rho_exp_floor, sie_exp_floor;
  double gam0_ceiling, sie0_ceiling;         /* ConstantGamSie ceilings */
  double bsqorho0_ceiling, bsqou0_ceiling;   /* ConstantBsqRat ceilings */
  /* physical-boundary fixups of a tiled mesh (fixup.cpp:56-60; both off by
   * default, both on in the torus deck) */
  int enable_flux_fixup;            /* FixFluxes after FluxCT                 */
  int enable_ox1_fmks_inflow_check; /* u^1 >= 0 in outer-X1 ghosts (FMKS)     */
} phx_params;

/* Geometry.  Minkowski is constant-folded into the kernels.  FMKS
 * (Modified<SphericalKerrSchild, McKinneyGammieRyan>, fmks.hpp:44) is read
 * from axisymmetric per-block tables, the layout of the reference's cached
 * geometry (cached_system.hpp:474-560 with geometry/axisymmetric = true).
 * Each location table holds PHX_GEOM_NLOC values per (j, i):
 *   alpha, beta^1..3, gcov (10, symmetric, Flatten2 order), gamcon (6,
 *   symmetric), sqrt(gamma).
 * Cell-centre derivative table: dlnalpha/dX^1..3 (3), dg_{mu nu}/dX^1..3
 * (10 x 3).  Tables are filled by phx_geometry_fill_fmks or by the caller. */
enum {
  PHX_G_ALPHA = 0,
  PHX_G_BETA = 1,
  PHX_G_GCOV = 4,
  PHX_G_GAMCON = 14,
  PHX_G_DETGAM = 20,
  PHX_GEOM_NLOC = 21,
  PHX_GD_DALPHA = 0,
  PHX_GD_DG = 3,
  PHX_GEOM_NDER = 33
};

typedef struct {
  int kind; /* phx_geom_kind */
  /* FMKS parameters (fmks.cpp:37-88 defaults in phx_geometry_default) */
  double a, hslope, poly_xt, poly_alpha, x0, smooth, hexp_br, hexp_nsq, hexp_csq;
  int derefine_poles;
  /* tables (device pointers; NULL for Minkowski).  Leading dimension is
   * the variable, then j, then i. */
  double *cent;  /* [PHX_GEOM_NLOC][n2t][n1t]     cell centres (and X3 faces)   */
  double *face1; /* [PHX_GEOM_NLOC][n2t][n1t + 1] X1 faces                      */
  double *face2; /* [PHX_GEOM_NLOC][n2t + 1][n1t] X2 faces                      */
  double *deriv; /* [PHX_GEOM_NDER][n2t][n1t]     cell-centre derivatives       */
} phx_geometry;

/* One meshblock.  Coordinates are Parthenon UniformCartesian:
 * Xf(i) = (xmin - ng dx) + i dx, Xc(i) = (xmin - ng dx) + (i + 1/2) dx for
 * active dimensions (xmin is the interior lower edge); an inactive
 * dimension has a single zone with Xc = xmin + dx/2. */
typedef struct {
  int nx1, nx2, nx3; /* interior zones (1 for inactive dimensions) */
  int ng;            /* ghost zones per side (4 for WENO5-Z / MP5)  */
  int ndim;          /* 1, 2 or 3 */
  long long var_stride; /* elements between variables; 0 = n1t*n2t*n3t */
  double x1min, x2min, x3min;
  double dx1, dx2, dx3;
  double *prim;     /* [PHX_NPRIM][N]                                   */
  double *cons;     /* [PHX_NCONS][N]                                   */
  double *flux;     /* [3][PHX_NCONS][N]  flux(d, m, k, j, i)           */
  double *face_sig; /* [3][N] face signal speed                        */
  double *cell_sig; /* [3][N] cell signal speed                        */
  double *fail;     /* [N]    1.0 = con2prim success, 0.0 = failure     */
  double *src;      /* [4][N] geometric sources for S_1..3 and tau      */
  double *emf;      /* [3][N] FluxCT edge EMFs (scratch)                */
  double *dudt;     /* [PHX_NCONS][N] right-hand side (scratch)         */
  const phx_geometry *geom; /* NULL = Minkowski */
} phx_block;

/* con2prim statistics, accumulated on the device by every con2prim call
 * (the reference's CON2PRIM_STATISTICS histogram, con2prim_statistics.hpp). */
#define PHX_C2P_HIST 128
typedef struct {
  unsigned long long zones;
  unsigned long long iterations;     /* sum of root-find iterations      */
  unsigned long long residual_evals; /* sum of residual evaluations      */
  unsigned long long failures;       /* zones flagged fail = 0.0         */
  unsigned long long unbracketed;    /* zones whose root was not bracketed */
  unsigned long long learned_accepted; /* learned brackets that bracketed */
  unsigned long long hist[PHX_C2P_HIST]; /* iteration-count histogram     */
} phx_c2p_stats;

typedef struct phx_ctx phx_ctx;

/* ---- context ----------------------------------------------------------- */
phx_status phx_ctx_create(int device, phx_ctx **out);
phx_status phx_ctx_destroy(phx_ctx *ctx);
/* Synchronise the device and return (and clear) the sticky error word. */
phx_status phx_ctx_check(phx_ctx *ctx);
/* Copy (and optionally reset) the device-side con2prim statistics. */
phx_status phx_ctx_c2p_stats(phx_ctx *ctx, phx_c2p_stats *out, int reset);
const char *phx_status_string(phx_status s);
/* Human-readable detail of the last host-side error in this thread. */
const char *phx_last_error(void);
int phx_abi_version(void);
/* Build flavour: 1 when compiled without FMA contraction (bit-exact parity
 * build), 0 for the production build. */
int phx_build_exact(void);

void phx_params_default(phx_params *p);
void phx_geometry_default(phx_geometry *g, int kind);

/* ---- hot-path entry points -------------------------------------------- */

/* fluid::PrimitiveToConservedRegion (fluid.cpp:368-449).  Writes cons and
 * cell_sig over the range. */
phx_status phx_prim_to_con(phx_ctx *ctx, const phx_params *p, const phx_block *b,
                           phx_range ib, phx_range jb, phx_range kb, void *stream);

/* fluid::ConservedToPrimitiveRegion with the robust solver
 * (fluid.cpp:451-517, con2prim_robust.hpp:299-453).  Reads cons and the
 * c2p_mu guess, writes prims, fail, cell_sig and (when bounds were applied)
 * cons. */
phx_status phx_con_to_prim(phx_ctx *ctx, const phx_params *p, const phx_block *b,
                           phx_range ib, phx_range jb, phx_range kb, void *stream);

/* Same as phx_con_to_prim, but the starting bracket comes from the learned
 * guess network loaded into ctx (phx_mlp_set_weights).  The FP64 root find
 * and its fallback to the reference bracket are unchanged. */
phx_status phx_con_to_prim_learned(phx_ctx *ctx, const phx_params *p, const phx_block *b,
                                   phx_range ib, phx_range jb, phx_range kb,
                                   void *stream);

/* prim2con::p2c (prim2con.hpp:25-102) over a list of independent zones, the
 * generator of con2prim inputs and training pairs.  prim[PHX_NPRIM][n] ->
 * cons[PHX_NCONS][n]; geom[PHX_GEOM_NLOC][n] as below (NULL = Minkowski);
 * cell_sig[3][n] may be NULL. */
phx_status phx_prim_to_con_zones(phx_ctx *ctx, const phx_params *p, long long n, const double *prim,
                                 const double *geom, double *cons, double *cell_sig, void *stream);

/* con2prim over a list of independent zones with per-zone geometry (the
 * isolated-zone form of ConservedToPrimitiveRobust used to benchmark the
 * inversion itself).  Arrays are SoA with stride n: cons[PHX_NCONS][n] (read;
 * rewritten where bounds were applied), prim[PHX_NPRIM][n] (c2p_mu read as the
 * guess, the rest written), geom[PHX_GEOM_NLOC][n] (point geometry as in the
 * cell-centre table; NULL = Minkowski), fail[n], cell_sig[3][n] (may be NULL), coords[3][n]
 * (X1..X3 for the floors; may be NULL = 0).  learned = 1 takes the starting
 * bracket from the loaded network (phx_mlp_set_weights). */
phx_status phx_con_to_prim_zones(phx_ctx *ctx, const phx_params *p, long long n, double *cons,
                                 double *prim, const double *geom, double *fail,
                                 double *cell_sig, const double *coords, int learned,
                                 void *stream);

/* Point FMKS geometry for a list of zones at coordinates (X1, X2): writes
 * geom[PHX_GEOM_NLOC][n] as phx_geometry_fill_fmks does for cell centres. */
phx_status phx_geometry_fmks_points(phx_ctx *ctx, const phx_geometry *g, long long n,
                                    const double *x1, const double *x2, double *geom,
                                    void *stream);

/* fluid::CalculateFluxes (fluid.cpp:659-773): reconstruction + LLF/HLL.
 * Writes flux(d, m) and face_sig(d) on every face the reference's divergence
 * and FluxCT read. */
phx_status phx_calculate_fluxes(phx_ctx *ctx, const phx_params *p, const phx_block *b,
                                void *stream);

/* fluid::FluxCT (fluid.cpp:775-841). */
phx_status phx_flux_ct(phx_ctx *ctx, const phx_params *p, const phx_block *b,
                       void *stream);

/* fluid::CalculateFluidSourceTerms (fluid.cpp:566-657) over nblocks blocks
 * (a MeshData pack).  Writes src. */
phx_status phx_calculate_fluid_source_terms(phx_ctx *ctx, const phx_params *p,
                                            const phx_block *blocks, int nblocks,
                                            void *stream);

/* Stage glue of PhoebusDriver::RungeKuttaStage (phoebus_driver.cpp:547-577):
 * dudt = FluxDivergence + src (SumData), cons0 = beta cons0 + (1-beta) base
 * (AverageIndependentData), out = cons0 + beta dt dudt (UpdateIndependentData).
 * base may equal cons0 (first stage); out may equal base. */
phx_status phx_update_stage(phx_ctx *ctx, const phx_block *b, const double *cons_base,
                            double *cons_out, double beta, double dt, void *stream);

/* Periodic ghost fill of nvar variables starting at field (Parthenon's
 * periodic boundary exchange for a single block). */
phx_status phx_fill_ghosts_periodic(phx_ctx *ctx, const phx_block *b, double *field,
                                    int nvar, void *stream);

/* fluid::EstimateTimestepBlock (fluid.cpp:899-944).  use_face_speeds selects
 * the reference's second form.  The result (cfl * min dt) is written to
 * *dt_out_device (device memory) without synchronising. */
phx_status phx_estimate_timestep(phx_ctx *ctx, const phx_params *p, const phx_block *b,
                                 int use_face_speeds, double *dt_out_device,
                                 void *stream);

/* Allocation-free variant of phx_estimate_timestep.  It has no counterpart in
 * the reference.  It is for callers that cannot allocate device memory (and so
 * cannot create a phx_ctx, which calls cudaMalloc): hosts whose device memory
 * all comes from their own pool and that forbid libraries from allocating, or
 * loops that must not risk the device synchronisation an allocation can cause
 * mid-step.  Same inputs, output and result as phx_estimate_timestep; it uses
 * the current device and calls no cudaMalloc, cudaFree or allocating routine.
 * Its scratch is a file-scope __device__ array of PHX_DT_STATIC_MAX_PARTIALS
 * doubles (512 KiB) that every device loading the library keeps until exit,
 * so blocks with more than PHX_DT_STATIC_MAX_ZONES interior zones are
 * rejected with PHX_ERR_CAPACITY.  The block checks are those of
 * phx_estimate_timestep that do not involve prim/cons (ng >= 3, var_stride 0
 * or at least the block's size); errors are described by phx_last_error().
 * The first call on each device looks up the array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * The address is kept with the id of the CUDA context it was found in and
 * looked up again when another context is current (after cudaDeviceReset).
 * All calls share the array: calls that overlap on the GPU (different
 * streams, concurrent host threads) race on it. */
#define PHX_DT_STATIC_MAX_PARTIALS 65536
#define PHX_DT_STATIC_MAX_ZONES (65536LL * 256LL)
phx_status phx_estimate_timestep_static(const phx_params *p, const phx_block *b,
                                        int use_face_speeds, double *dt_out_device,
                                        void *stream);

/* fixup::ConservedToPrimitiveFixup (fixup_c2p.cpp:44-356), interior zones. */
phx_status phx_c2p_fixup(phx_ctx *ctx, const phx_params *p, const phx_block *b,
                         void *stream);

/* fixup::ApplyFloors (fixup.cpp:285-687), range as in the reference. */
phx_status phx_apply_floors(phx_ctx *ctx, const phx_params *p, const phx_block *b,
                            phx_range ib, phx_range jb, phx_range kb, void *stream);

/* Fill the FMKS geometry tables of g for block b (cached_system.hpp:560-640
 * "analytic" branch: point evaluations and finite-difference derivatives). */
phx_status phx_geometry_fill_fmks(phx_ctx *ctx, const phx_geometry *g, const phx_block *b,
                                  void *stream);

/* One full RK stage for one block with periodic boundaries, in the order
 * of PhoebusDriver::RungeKuttaStage (phoebus_driver.cpp:204-738): sources,
 * fluxes, FluxCT, divergence + SumData + Average + Update, con2prim over the
 * entire block, [c2p fixup, floors], ghost exchange of the conserved
 * variables, con2prim over the entire block again, [c2p fixup, floors].
 * b->cons is the stage input (prims consistent with it), cons_base the state
 * at the start of the step, cons_out receives the stage result (it may alias
 * cons_base); on return the prims are consistent with cons_out.  Heun RK2:
 * stage 1 (beta = 1) cons = base -> out = second buffer; stage 2
 * (beta = 1/2) cons = second buffer -> out = base. */
phx_status phx_stage(phx_ctx *ctx, const phx_params *p, const phx_block *b,
                     const double *cons_base, double *cons_out, double beta, double dt,
                     int use_learned_guess, void *stream);

/* Batched uneven meshblocks: the stage of phx_stage over nblocks independent
 * (periodic) blocks of mixed sizes, with one persistent launch per phase
 * walking a device work list of (block, index range) items, the whole stage
 * replayed as a CUDA graph.  cons_base[n] / cons_out[n] per block.  The
 * first call for a set of blocks and buffers builds a plan: device tables,
 * work lists, tile shapes chosen by timing candidates (cached per process,
 * and in the JSON file PHX_AUTOTUNE_CACHE names, if set) and the captured
 * graph; later calls with the same blocks, buffers and params only update
 * beta and dt in device memory and launch the graph.  Blocks must share ndim
 * and geometry kind; c2p fixup and floors run as in phx_stage; with
 * use_learned_guess each con2prim pass is a tensor-core bracket launch and a
 * root-find launch over all blocks.  No counterpart in the reference, which
 * launches every block's tasks separately. */
phx_status phx_stage_batched(phx_ctx *ctx, const phx_params *p, const phx_block *blocks,
                             int nblocks, const double *const *cons_base,
                             double *const *cons_out, double beta, double dt,
                             int use_learned_guess, void *stream);

/* A domain tiled by blocks as a tensor product of per-axis segments, for
 * phx_stage_mesh.  Block (s1, s2, s3) (segment indices) is blocks[(s3 *
 * nseg[1] + s2) * nseg[0] + s1]; its interior covers global cells
 * seg_start[d][s_d] .. seg_start[d][s_d + 1] - 1 on axis d.  All blocks share
 * ndim; an inactive axis has n = 1 and one segment.
 * Physical boundaries (phoebus_boundaries.cpp) fill a ghost from the cell
 * that the rule maps it to:
 *   PHX_BC_OUTFLOW  gr_outflow: the boundary cell (OutflowInnerX1 & co.)
 *   PHX_BC_REFLECT  the mirror cell, vector components along the axis
 *                   negated (GenericBC<..., Reflect>)
 *   PHX_BC_POLAR    X2 faces only, bc_vars = primitive only: the mirror
 *                   cell, v^2 and B^2 negated (PolarInnerX2 / PolarOuterX2)
 * with bc_vars (fluid.cpp:153-165):
 *   PHX_BC_VARS_CONSERVED  the conserved variables are exchanged and copied,
 *                   each copy scaled by robust::ratio(DetGamma(ghost),
 *                   DetGamma(source)) (the reference's default);
 *   PHX_BC_VARS_PRIMITIVE  primitives and conserved variables are exchanged,
 *                   physical ghosts take the primitives and prim2con.
 * Periodic axes must be periodic on both faces (Parthenon's rule). */
#define PHX_BC_PERIODIC 0
#define PHX_BC_OUTFLOW 1
#define PHX_BC_REFLECT 2
#define PHX_BC_POLAR 3
#define PHX_BC_VARS_CONSERVED 0
#define PHX_BC_VARS_PRIMITIVE 1
typedef struct {
  int n[3];                  /* global interior cells per axis            */
  int nseg[3];               /* segments (blocks) per axis                */
  const int *seg_start[3];   /* host arrays of nseg[d] + 1 entries         */
  int bc_lo[3], bc_hi[3];    /* PHX_BC_* of each face                      */
  int bc_vars;               /* PHX_BC_VARS_*                              */
} phx_mesh;

/* The stage of phx_stage over a tiled mesh, in the reference's task order:
 * sources, fluxes, FluxCT, FixFluxes (p->enable_flux_fixup), update, then
 * twice con2prim + c2p fixup + floors with the boundary exchange between the
 * two passes.  The exchange is phx_mesh_exchange's.  batched = 1: one
 * persistent launch per phase replayed as a CUDA graph (as
 * phx_stage_batched); batched = 0: the same kernels launched block by block
 * (the launch structure of per-block tasks).  Plans are built and cached as
 * in phx_stage_batched. */
phx_status phx_stage_mesh(phx_ctx *ctx, const phx_params *p, const phx_mesh *mesh, const phx_block *blocks,
                          int nblocks, const double *const *cons_base, double *const *cons_out, double beta,
                          double dt, int use_learned_guess, int batched, void *stream);

/* The boundary exchange of a tiled mesh (phoebus_driver.cpp:646-668:
 * AddBoundaryExchangeTasks, ApplyBoundaryConditions,
 * ConvertBoundaryConditions).  A ghost whose cell lies inside the domain,
 * across a block face or a periodic wrap, receives the owning block's
 * exchanged variables (bc_vars).  A ghost in a physical boundary slab
 * receives the values of the cell its boundary rule maps it to, the rules of
 * all axes composed as the face-by-face application in X1, X2, X3 order
 * leaves them (with bc_vars = conserved, the product of the DetGamma ratios
 * along that path).  With bc_vars = primitive it then gets, with
 * p->enable_ox1_fmks_inflow_check on an FMKS mesh, the outer-X1 inflow check
 * (phoebus_boundaries.cpp:366-397), and prim2con with its own metric
 * (PrimitiveToConservedRegion: conserved variables and cell signal speeds).
 * With bc_vars = conserved and the inflow check on an FMKS mesh, the
 * outer-X1 slab of a block on the physical outer X1 face is first inverted
 * (ConservedToPrimitiveRegion, phoebus_boundaries.cpp:333-340: primitives,
 * floors, fail flags), then checked and prim2con'd the same way. */
phx_status phx_mesh_exchange(phx_ctx *ctx, const phx_params *p, const phx_mesh *mesh, const phx_block *blocks,
                             int nblocks, void *stream);

/* fixup::FixFluxes (fixup.cpp:728-1078) on every block of a tiled mesh
 * that touches a physical boundary, in place on the blocks' flux arrays; a
 * no-op unless p->enable_flux_fixup.  Boundary faces only:
 *   gr_outflow  the density flux may only leave: min(F, 0) on lower faces,
 *               max(F, 0) on upper faces;
 *   reflect     density and energy fluxes 0 (X2 faces also S_1 and S_3);
 *   polar       X2 fluxes of density, energy, momentum and B set to 0, and the
 *               X1 and X3 fluxes of B^2 in the ghost row outside the pole
 *               set to minus those of the row inside. */
phx_status phx_fix_fluxes(phx_ctx *ctx, const phx_params *p, const phx_mesh *mesh, const phx_block *blocks,
                          int nblocks, void *stream);

/* FixFluxes as the reference's per-block task: bc_lo[d] / bc_hi[d] give the
 * boundary kind of the block's lower / upper face on axis d
 * (PHX_BC_OUTFLOW, PHX_BC_REFLECT, PHX_BC_POLAR on a physical boundary;
 * PHX_BC_PERIODIC for a face with a neighbouring block or a periodic wrap).
 * A no-op unless p->enable_flux_fixup. */
phx_status phx_fix_fluxes_block(phx_ctx *ctx, const phx_params *p, const phx_block *b, const int bc_lo[3],
                                const int bc_hi[3], void *stream);

/* Tile shapes and graph size of the most recent batched plan (0 if none). */
phx_status phx_batch_info(phx_ctx *ctx, int *x1_cells, int *sweep_seg, int *graph_nodes);

/* ---- learned con2prim guess (no reference counterpart) ---------------- */
/* Network 6 -> 64 -> 64 -> 64 -> 2, GELU, BF16 weights, FP32 accumulate. */
#define PHX_MLP_IN 6
#define PHX_MLP_HID 64
#define PHX_MLP_OUT 2
#define PHX_MLP_NPARAM (PHX_MLP_IN * PHX_MLP_HID + PHX_MLP_HID + \
                        2 * (PHX_MLP_HID * PHX_MLP_HID + PHX_MLP_HID) + \
                        PHX_MLP_HID * PHX_MLP_OUT + PHX_MLP_OUT)
/* Parameter order (weights [out][in]): W1[64][6], b1[64], W2[64][64], b2[64],
 * W3[64][64], b3[64], W4[2][64], b4[2].  GELU (tanh form) after each hidden
 * layer.  Outputs: o0 = predicted ln(mu), o1 = ln(sigma) of its error, mu the
 * con2prim unknown 1 / (h W).  The learned start is the bracket
 * [e^{o0 - 3 s}, e^{o0 + 3 s}] (s = e^{o1}, clipped to [0, 1]) around
 * m = e^{o0}; the root find evaluates f(m), then the outer end of the half
 * that should hold the root, and starts the reference's Illinois iterations
 * from that half if it changes sign -- otherwise from the reference's own
 * [0, 1] + guess start.  Inference multiplies BF16 weights and activations on
 * the tensor cores with FP32 accumulation. */

/* Load FP32 master parameters (host memory, PHX_MLP_NPARAM floats); resets
 * the optimiser state and the input box (unbounded). */
phx_status phx_mlp_set_weights(phx_ctx *ctx, const float *params_host);
phx_status phx_mlp_get_weights(phx_ctx *ctx, float *params_host);

/* Input box of the learned start (6 floats each, host): a cold zone whose
 * features (phx_mlp_features_zones) fall outside [lo, hi] gets no learned
 * bracket and keeps the reference's start, so the network is not consulted
 * outside the states it was trained on.  phx_mlp_train sets the box to the
 * training features' range widened by 2% of it on each side; NULL lo or hi
 * leaves that side unbounded. */
phx_status phx_mlp_set_input_box(phx_ctx *ctx, const float *lo_host, const float *hi_host);
phx_status phx_mlp_get_input_box(phx_ctx *ctx, float *lo_host, float *hi_host);

/* The 6 FP32 network inputs of independent zones, x[6][n] (device), from the
 * con2prim setup invariants of cons/geom/coords as in
 * phx_con_to_prim_zones: log10 q / 4, log10 r^2 / 4, log10 b^2 / 4,
 * (b.r)^2 / (b^2 r^2), v0^2, log10 D / 8 (q = tau / D, r_i = S_i / D,
 * b^i = B^i / sqrt(D)). */
phx_status phx_mlp_features_zones(phx_ctx *ctx, const phx_params *p, long long n, const double *cons,
                                  const double *geom, const double *coords, float *x, void *stream);

/* Network outputs out[2][n] for inputs x[6][n] (device), on the tensor cores. */
phx_status phx_mlp_forward(phx_ctx *ctx, long long n, const float *x, float *out, void *stream);

/* The learned start (m, lo, hi) per zone, bracket[3][n] (device, NaN where
 * the con2prim setup rejects the zone): what phx_con_to_prim_zones with
 * learned = 1 starts its root find from. */
phx_status phx_mlp_bracket_zones(phx_ctx *ctx, const phx_params *p, long long n, const double *cons,
                                 const double *geom, const double *coords, double *bracket, void *stream);

/* Mean loss over n samples and its gradient for the loaded parameters:
 * grad[PHX_MLP_NPARAM] and loss[1] (device; overwritten).  x[6][n], y[n]
 * (device) with y = ln(mu) of the exact primitive state.  Loss: Gaussian
 * negative log-likelihood 0.5 (y - o0)^2 e^{-2 o1} + o1.  The forward pass
 * multiplies BF16-rounded weights and inputs; the gradient passes straight
 * through the rounding. */
phx_status phx_mlp_loss_grad(phx_ctx *ctx, long long n, const float *x, const float *y, float *grad,
                             float *loss, void *stream);

typedef struct phx_mlp_train_opts {
  int batch;          /* samples per step (a multiple of 64 is best)   */
  int epochs;         /* passes over the n samples (in order)          */
  float lr, lr_min;   /* cosine schedule from lr to lr_min             */
  float beta1, beta2, eps, weight_decay; /* AdamW (decay on weights)   */
} phx_mlp_train_opts;

void phx_mlp_train_opts_default(phx_mlp_train_opts *o);

#define PHX_MLP_MAX_EPOCHS 1024

/* Train the loaded parameters on n samples (x[6][n], y[n], device) with
 * AdamW, floor(n / batch) steps per epoch, on the GPU; then pack the
 * parameters for inference and set the input box from x (phx_mlp_set_input_box).
 * epoch_loss (host, may be NULL) receives the mean
 * training loss of each epoch.  Synchronises the stream. */
phx_status phx_mlp_train(phx_ctx *ctx, long long n, const float *x, const float *y, const phx_mlp_train_opts *o,
                         float *epoch_loss, void *stream);

/* ---- problem generator: the magnetised Fishbone-Moncrief torus --------- */
typedef struct phx_torus_params {
  double rin;               /* inner edge of the torus (torus/rin, 6)                */
  double rmax;              /* radius of the pressure maximum (torus/rmax, 12)       */
  double kappa;             /* polytropic constant (torus/kappa, 1e-2)               */
  double u_jitter;          /* u *= 1 + u_jitter (U - 0.5) (torus/u_jitter, 1e-2)    */
  double target_beta;       /* max P / max (b^2 / 2) after normalisation (100)       */
  int magnetized;           /* torus/magnetized (1): 0 leaves B = 0                  */
  unsigned long long seed;  /* counter seed of the noise draws U                     */
} phx_torus_params;

void phx_torus_params_default(phx_torus_params *tp);

/* torus::ProblemGenerator (pgen/torus.cpp:130-474) on every block, then
 * torus::PostInitializationModifier's HARM-style field normalisation
 * (torus.cpp:525-740, ComputeBetas :844-924), for the ideal gas with
 * nsub = 1 and no radiation or tracers.  Per block, over its entire index
 * range: the Fishbone-Moncrief solution (torus.cpp:743-843) at the cell
 * centres in FMKS coordinates, u^phi transformed BL -> FMKS, the pressure
 * noise, the floors, T, P, gamma1; A_phi at the corners from the floored
 * density and the poloidal field from it; PrimitiveToConserved and
 * ApplyFloors.  Then the maxima of P and b^2 over all blocks' interiors give
 * the field factor sqrt(beta_pmax / target_beta) (written to *field_factor,
 * host, may be NULL), the interior field is scaled and PrimitiveToConserved
 * runs again.  The blocks need FMKS geometry tables (phx_geometry_fill_fmks)
 * and share one geometry.  U is a counter-based uniform (SplitMix64 of
 * (seed, zone)), zones numbered block after block over the entire ranges (the
 * reference's Kokkos pool is seeded by the clock).  Synchronises the stream
 * once, for the maxima.  Blocks wider than 3 x 2^21 / 7 cells per (j, i)
 * plane return PHX_ERR_CAPACITY. */
phx_status phx_torus_init(phx_ctx *ctx, const phx_params *p, const phx_torus_params *tp,
                          const phx_block *blocks, int nblocks, double *field_factor, void *stream);

/* ---- the library's transcendental functions ----------------------------- */
/* The FMKS geometry tables and the exponential floors evaluate exp, sin, cos
 * and pow written out from their series with IEEE operations only (no
 * counterpart in the reference, which calls the C library's): the oracle
 * evaluates the same operations, so tables and floors compare bit for bit.
 * out[q] = f(x[q]) (pow: x[q]^y[q]) for device arrays of n doubles, for
 * validating them against other implementations. */
enum { PHX_MATH_EXP = 0, PHX_MATH_LOG = 1, PHX_MATH_SIN = 2, PHX_MATH_COS = 3, PHX_MATH_POW = 4,
       /* the kernels' 1/x and 1/sqrt(x): IEEE division and square root in the
        * exact build; in the production build the hardware seed with one
        * third-order correction (normal x; others divide) */
       PHX_MATH_RCP = 5, PHX_MATH_RSQRT = 6 };
phx_status phx_math_eval(int fn, long long n, const double *x, const double *y, double *out, void *stream);

/* ---- measurement probe -------------------------------------------------- */
/* Time a dependent-chain-free FP64 FMA loop and report FLOP/s (2 per FMA).
 * Used to measure the FP64 roofline of the device the library runs on. */
phx_status phx_probe_fp64_peak(phx_ctx *ctx, double *flops_out);

/* Drive the failure path of the library's bounded device waits (no
 * counterpart in the reference): one thread block arms an mbarrier for 16
 * bytes and issues no copy, so the wait can never complete and nothing is in
 * flight; after `polls` polls (1 .. 2^20) the block gives up exactly as the
 * bulk-copy staging of the flux and learned-start kernels does, sets the
 * context's timeout bit and returns.  The next phx_ctx_check on ctx returns
 * PHX_ERR_TIMEOUT (and clears the bit); the context stays usable. */
phx_status phx_probe_bounded_wait(phx_ctx *ctx, long long polls, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* PHX_FLUID_H_ */
