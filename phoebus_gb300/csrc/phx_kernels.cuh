// phx_kernels.cuh -- kernel declarations shared by the translation units.
#pragma once
#include <cuda.h>  // CUtensorMap (the type only; the encode goes through the runtime)

#include "phx_c2p.cuh"

namespace phx {

// Sticky error bits (device word in the context).
enum : unsigned int {
  ERR_UNBRACKETED = 1u,
  ERR_NAN_INPUT = 2u,
  ERR_TIMEOUT = 4u,  // MBAR_ERR_TIMEOUT of phx_bulk.cuh
  ERR_BOUNDS = 8u,
};

struct DevStats {  // mirrors phx_c2p_stats
  unsigned long long zones, iterations, residual_evals, failures, unbracketed, learned_accepted;
  unsigned long long hist[PHX_C2P_HIST];
};

struct Range3 {
  int is, ie, js, je, ks, ke;
};

// One CTA's share of a batched launch: indices [first, last) of one block's
// index space for that phase (zones, faces, pencils or sweep threads).
struct WorkItem {
  int block;
  int pad;
  long long first, last;
};

// Sets the text phx_last_error() returns on this host thread.
void set_last_error(const char *msg);

void launch_p2c(const Par &p, const BView &b, Range3 r, cudaStream_t s);
struct MlpPacked;
// con2prim works in chunks of C2P_CHUNK zones; per chunk the context holds
// the learned brackets [3][C2P_CHUNK] and the retry list of zones deferred
// past the first kernel's iteration cap.
constexpr long long C2P_CHUNK = 1ll << 21;
struct C2PScratch {
  double *brk;                  // [3][C2P_CHUNK]
  int *count;                   // [1]
  int *idx;                     // [C2P_CHUNK]
  double *a, *b, *ya, *yb;      // [C2P_CHUNK] each
  unsigned long long *packed;   // [C2P_CHUNK]
};
void launch_c2p(const Par &p, const BView &b, Range3 r, DevStats *stats, unsigned int *err,
                const MlpPacked *mlp, const C2PScratch &scr, cudaStream_t s);
void launch_fluxes(const Par &p, const BView &b, cudaStream_t s);
void launch_fluxct(const BView &b, cudaStream_t s);
void launch_sources(const Par &p, const BView &b, cudaStream_t s);
void launch_update(const Par &p, const BView &b, const double *base, double *out, double beta,
                   double dt, cudaStream_t s);
void launch_ghost_periodic(const BView &b, double *field, int nvar, cudaStream_t s);
void launch_dt(const Par &p, const BView &b, int use_face, unsigned long long *scratch,
               double *dt_out, cudaStream_t s);
void launch_c2p_fixup(const Par &p, const BView &b, cudaStream_t s);
// flag (optional, [N]): 1 where floors or ceilings acted, else 0
void launch_floors(const Par &p, const BView &b, Range3 r, DevStats *stats, unsigned int *err,
                   cudaStream_t s, double *flag = nullptr);
void launch_geom_fmks(const phx_geometry &g, const BView &b, cudaStream_t s);
void launch_geom_points(const phx_geometry &g, long long n, const double *x1, const double *x2, double *geom,
                        cudaStream_t s);
void launch_math_eval(int fn, long long n, const double *x, const double *y, double *out, cudaStream_t s);
void launch_wait_probe(long long limit, unsigned int *err, cudaStream_t s);
// The torus problem generator and its field normalisation (phx_torus.cu) over
// the blocks of a mesh: scratch holds 7 x n1t x n2t doubles of the largest
// block, red 2 words; synchronises s once (the mesh-wide maxima).
constexpr int TORUS_PLANE_VARS = 7;
cudaError_t torus_init(const Par &p, const phx_geometry &g, const phx_torus_params &tp, const BView *views, int n,
                       double *scratch, unsigned long long *red, DevStats *stats, unsigned int *err, double *fac_out,
                       cudaStream_t s);
void launch_p2c_zones(const Par &p, long long n, const double *prim, const double *geom, double *cons,
                      double *cell_sig, cudaStream_t s);
void launch_c2p_zones(const Par &p, long long n, double *cons, double *prim, const double *geom, double *fail,
                      double *cell_sig, const double *coords, DevStats *stats, unsigned int *err,
                      const MlpPacked *mlp, const C2PScratch &scr, cudaStream_t s);
void launch_mlp_bracket(const Par &p, long long n, const double *cons, const double *geom, const double *coords,
                        const MlpPacked *mlp, double *bracket, unsigned int *err, cudaStream_t s);
// learned-start network (phx_mlp.cu)
void launch_mlp_pack(const float *theta, MlpPacked *out, cudaStream_t s);
// The input box: reset to (-inf, inf), or the range of the features x[6][n]
// widened by `margin` of the range on each side (keys: 12 ints of device
// scratch).
void launch_mlp_box_reset(MlpPacked *out, cudaStream_t s);
void launch_mlp_box_from(const float *x, long long n, float margin, int *keys, MlpPacked *out, cudaStream_t s);
void launch_mlp_features(const Par &p, long long n, const double *cons, const double *geom, const double *coords,
                         float *x, cudaStream_t s);
void launch_mlp_forward(const MlpPacked *mlp, long long n, const float *x, float *out, unsigned int *err,
                        cudaStream_t s);
void launch_mlp_grad(const float *theta, const float *x, const float *y, long long stride, long long off,
                     long long count, float inv_batch, float *grad, float *loss, cudaStream_t s);
void launch_mlp_adamw(float *theta, float *grad, float *m, float *v, float lr, float b1, float b2, float eps,
                      float wd, float c1, float c2, cudaStream_t s);
void launch_fp64_probe(double *out, int iters, cudaStream_t s, int *nthreads_out);

// ---- batched (many blocks, one persistent launch per phase; phx_batch.cu)
// Grid of a persistent launch: as many CTAs as fit on the GPU at once (or
// fewer when there are fewer items); grid > 0 is taken as given.
template <class K>
inline int persistent_grid(K kernel, int threads, size_t smem, int nitems, int grid) {
  if (grid > 0) return grid < nitems ? grid : nitems;
  int dev = 0, nsm = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, threads, smem);
  const long long g = (long long)(nsm > 0 ? nsm : 1) * (occ > 0 ? occ : 1);
  return (int)(g < nitems ? g : nitems);
}
// A tiled mesh on the device (phx_mesh): per-axis global cell -> segment
// maps, the owner block of each segment triple, each block's origin.
struct MeshDev {
  int n[3], nseg[3], bc_lo[3], bc_hi[3];
  int bc_vars;           // PHX_BC_VARS_*
  const int *seg_of[3];  // [n[d]]
  const int *owner;      // [nseg[2]][nseg[1]][nseg[0]]
  const int *origin;     // [nblocks][3] global index of the first interior cell
};
// Where ghost cell t of block blk takes its values from.  Periodic axes
// wrap; beyond a physical face gr_outflow clamps to the boundary cell and
// reflect / polar mirror about the face.  src / sid: the owner block and cell
// of the mapped global cell; mloc[d]: the mapped local index on each axis
// (the cell Parthenon's face loop reads); phys[d]: axis d crossed a physical
// face; reflect[d]: that face is reflect (vector components along d flip);
// mirror[d]: reflect or polar.
struct GhostMap {
  bool ghost, physical, outer_x1;
  bool phys[3], reflect[3], mirror[3];
  int loc[3], mloc[3];
  int src;
  long long id, sid;
};
#ifdef __CUDACC__
__device__ __forceinline__ GhostMap map_ghost(const BView *views, const MeshDev &m, int blk, long long t) {
  const BView &b = views[blk];
  GhostMap q;
  q.loc[0] = (int)(t % b.n1t);
  q.loc[1] = (int)((t / b.n1t) % b.n2t);
  q.loc[2] = (int)(t / ((long long)b.n1t * b.n2t));
  const int nx[3] = {b.nx1, b.nx2, b.nx3};
  const int nd = b.ndim;
  q.ghost = q.physical = q.outer_x1 = false;
  int g[3];
  for (int d = 0; d < 3; d++) {
    q.mloc[d] = q.loc[d];
    q.phys[d] = q.reflect[d] = q.mirror[d] = false;
    g[d] = 0;
    if (d >= nd) continue;  // inactive axis: one cell, no ghosts
    if (q.loc[d] < b.ng || q.loc[d] >= b.ng + nx[d]) q.ghost = true;
    int gg = m.origin[blk * 3 + d] + q.loc[d] - b.ng;
    if (gg < 0 || gg >= m.n[d]) {
      const bool lo = gg < 0;
      const int bc = lo ? m.bc_lo[d] : m.bc_hi[d];
      if (bc == PHX_BC_PERIODIC) {
        gg += lo ? m.n[d] : -m.n[d];
      } else {
        q.physical = q.phys[d] = true;
        if (d == 0 && !lo) q.outer_x1 = true;
        const int ref = lo ? b.ng : b.ng + nx[d] - 1;  // interior cell next to the face (local)
        if (bc == PHX_BC_OUTFLOW) {
          gg = lo ? 0 : m.n[d] - 1;
          q.mloc[d] = ref;
        } else {  // reflect / polar: mirror about the face
          gg = lo ? -1 - gg : 2 * m.n[d] - 1 - gg;
          q.mloc[d] = 2 * ref + (lo ? -1 : 1) - q.loc[d];
          q.mirror[d] = true;
          q.reflect[d] = bc == PHX_BC_REFLECT;
        }
      }
    }
    g[d] = gg;
  }
  q.src = -1;
  q.id = q.sid = 0;
  if (!q.ghost) return q;
  q.src = m.owner[(m.seg_of[2][g[2]] * m.nseg[1] + m.seg_of[1][g[1]]) * m.nseg[0] + m.seg_of[0][g[0]]];
  const BView &sb = views[q.src];
  int sl[3];
  for (int d = 0; d < 3; d++) sl[d] = d < nd ? g[d] - m.origin[q.src * 3 + d] + sb.ng : 0;
  q.sid = sb.idx(sl[2], sl[1], sl[0]);
  q.id = b.idx(q.loc[2], q.loc[1], q.loc[0]);
  return q;
}
// robust::ratio(DetGamma(c), DetGamma(r)) of face d's boundary loop (FMKS):
// c is the cell that loop sets (axes before d at the ghost's own index, axes
// after it already mapped), r the cell it reads (c mapped on axis d).
__device__ __forceinline__ double ghost_gratio(const BView &b, const GhostMap &q, int d) {
  int c[3], r[3];
  for (int e = 0; e < 3; e++) c[e] = e < d ? q.loc[e] : (e == d ? q.loc[d] : q.mloc[e]);
  for (int e = 0; e < 3; e++) r[e] = e == d ? q.mloc[d] : c[e];
  const double *detg = b.gcent + (long long)PHX_G_DETGAM * b.n2t * b.n1t;
  return ratio_p(detg[(long long)c[1] * b.n1t + c[0]], detg[(long long)r[1] * b.n1t + r[0]]);
}
#endif
void launch_mesh_exchange(const Par &p, bool mink, const BView *views, const MeshDev &m, const WorkItem *items,
                          int nitems, int grid, cudaStream_t s);
// FixFluxes: the physical-boundary faces of a block, per face (X1 lo, X1 hi,
// X2 lo, X2 hi, X3 lo, X3 hi; 0 where the face is not physical).
__host__ __device__ inline void fix_face_counts(int ndim, const int nx[3], const int origin[3], const int n[3],
                                                const int bc_lo[3], const int bc_hi[3], long long cnt[6]) {
  const long long e1 = nx[0], e2 = ndim >= 2 ? nx[1] : 1, e3 = ndim >= 3 ? nx[2] : 1;
  const long long area[3] = {e2 * e3, e1 * e3, e1 * e2};
  for (int d = 0; d < 3; d++) {
    const bool on = d < ndim;
    cnt[2 * d] = (on && origin[d] == 0 && bc_lo[d] != PHX_BC_PERIODIC) ? area[d] : 0;
    cnt[2 * d + 1] = (on && origin[d] + nx[d] == n[d] && bc_hi[d] != PHX_BC_PERIODIC) ? area[d] : 0;
  }
}
void launch_fix_fluxes(const Par &p, const BView *views, const MeshDev &m, const WorkItem *items, int nitems,
                       int grid, cudaStream_t s);
void launch_fix_fluxes_block(const Par &p, const BView &b, const int bc_lo[3], const int bc_hi[3], cudaStream_t s);
struct BatchCache;
BatchCache *batch_cache_create();
void batch_cache_destroy(BatchCache *c);
// mesh: null for independent periodic blocks.  batched = false launches each
// phase block by block (no graph).  only: BATCH_STAGE the whole stage,
// BATCH_EXCHANGE the mesh ghost fill alone, BATCH_FIXFLUX FixFluxes alone.
enum { BATCH_STAGE = 0, BATCH_EXCHANGE = 1, BATCH_FIXFLUX = 2 };
cudaError_t batch_stage(BatchCache *cache, const Par &par, const phx_block *blocks, const BView *views, int n,
                        const double *const *base, double *const *out, double beta, double dt,
                        const MlpPacked *mlp, const phx_mesh *mesh, bool batched, int only,
                        DevStats *stats, unsigned int *err, cudaStream_t s, const char **why);
void batch_last_tuning(BatchCache *cache, int *x1_cells, int *seg, int *launches);
long long interior_count(const BView &b);
long long fluxct_count(const BView &b);
void launch_sources_batched(const Par &p, bool mink, const BView *views, const WorkItem *items, int nitems, int grid,
                            cudaStream_t s);
void launch_fluxct_batched(int ndim, const BView *views, const WorkItem *items, int nitems, int grid, cudaStream_t s);
void launch_update_batched(const Par &p, const BView *views, const double *const *base, double *const *out,
                           const double *beta_dt, const WorkItem *items, int nitems, int grid, cudaStream_t s);
void launch_ghost_batched(const BView *views, int nvar, const WorkItem *items, int nitems, int grid, cudaStream_t s);
// mlp non-null: the learned start; brk holds 4 x nitems x 128 + 1 doubles
// (the brackets, each zone's warm / cold pass, the cold-zone count).
void launch_c2p_batched(const Par &p, bool mink, const BView *views, const WorkItem *items, int nitems, int grid,
                        const MlpPacked *mlp, double *brk, DevStats *stats, unsigned int *err, cudaStream_t s);
// bc_vars = conserved, outer-X1 inflow check (FMKS): con2prim, u^1 >= 0 and
// prim2con over the outer-X1 ghost slabs; items over ng * n2t * n3t zones.
void launch_ox1_inflow(const Par &p, const BView *views, const WorkItem *items, int nitems, int grid,
                       unsigned int *err, cudaStream_t s);
// maps / modes: per block, the X1 tensor map and staging mode from x1_mode
void launch_flux_x1_batched(const Par &p, bool mink, const BView *views, const WorkItem *items, int nitems, int grid,
                            size_t smem, const CUtensorMap *maps, const int *modes, unsigned int *err,
                            cudaStream_t s);
void prepare_flux_x1_batched(const Par &p, bool mink, size_t smem);
void launch_flux_sweep_batched(const Par &p, bool mink, int dir, const BView *views, const WorkItem *items,
                               int nitems, int grid, int seg_target, cudaStream_t s);
void launch_c2p_fixup_batched(const Par &p, bool mink, const BView *views, const WorkItem *items, int nitems,
                              cudaStream_t s);
void launch_floors_batched(const Par &p, bool mink, const BView *views, const WorkItem *items, int nitems,
                           DevStats *stats, unsigned int *err, cudaStream_t s);
int x1_npencil(const BView &b);
long long sweep_threads(const BView &b, int dir, int seg_target);
bool x1_tma_ok_host(const BView &b);
// Shared-memory doubles per staged X1 pencil (rows rounded up to 128 bytes).
long long x1_pencil_stride_host(const BView &b);
// X1 staging mode of a block: 2 tiled TMA through *map (encoded here), 1
// 1-D bulk copies, 0 plain loads.
int x1_mode(const BView &b, CUtensorMap *map);

}  // namespace phx
