// phx_batch.cu -- batched uneven meshblocks.
//
// One RK stage over many independent (periodic) blocks of mixed sizes, in
// the order of PhoebusDriver::RungeKuttaStage (phoebus_driver.cpp:204-738):
// each phase is ONE persistent launch over a device work list of
// (block, index range) items covering every block, and the whole stage is
// captured once as a CUDA graph and replayed.  A plan (device tables, work
// lists, tuned tile shapes, graph) is built on the first call for a given set
// of blocks and buffers and reused by later calls; beta and dt live in device
// memory so the graph serves every step.
//
// Autotuner: before capture, the X1 flux kernel's tile (cells staged per
// CTA, converted to pencils per block size) and the X2/X3 sweeps' segment
// length are chosen by timing each candidate on the plan's own blocks.
// Results are cached per (reconstruction, geometry, block-size mix) in the
// process and, when PHX_AUTOTUNE_CACHE names a file, in that JSON file.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "phx_kernels.cuh"

namespace phx {

namespace {

struct PhaseList {
  WorkItem *d_items = nullptr;
  int n = 0;
  std::vector<int> boff;  // items of block b: [boff[b], boff[b + 1])
};

struct Tuning {
  int x1_cells = 288;  // cells staged per X1 CTA (pencils x n1t)
  int seg = 32;        // faces per thread along an X2/X3 sweep
};

std::mutex g_tune_mu;
std::map<std::string, Tuning> g_tune;  // process-wide autotune results
bool g_tune_loaded = false;

void load_tune_file() {
  if (g_tune_loaded) return;
  g_tune_loaded = true;
  const char *path = getenv("PHX_AUTOTUNE_CACHE");
  if (!path) return;
  std::ifstream f(path);
  std::string line;
  // one entry per line: "key": {"x1_cells": N, "seg": M},
  while (std::getline(f, line)) {
    const size_t k0 = line.find('"'), k1 = line.find('"', k0 + 1);
    if (k0 == std::string::npos || k1 == std::string::npos) continue;
    const std::string key = line.substr(k0 + 1, k1 - k0 - 1);
    Tuning t;
    const size_t a = line.find("\"x1_cells\":"), b = line.find("\"seg\":");
    if (a == std::string::npos || b == std::string::npos) continue;
    t.x1_cells = atoi(line.c_str() + a + 11);
    t.seg = atoi(line.c_str() + b + 6);
    if (t.x1_cells > 0 && t.seg > 0) g_tune[key] = t;
  }
}

void save_tune_file() {
  const char *path = getenv("PHX_AUTOTUNE_CACHE");
  if (!path) return;
  std::ofstream f(path);
  f << "{\n";
  size_t i = 0;
  for (const auto &kv : g_tune) {
    f << "  \"" << kv.first << "\": {\"x1_cells\": " << kv.second.x1_cells << ", \"seg\": " << kv.second.seg << "}"
      << (++i < g_tune.size() ? "," : "") << "\n";
  }
  f << "}\n";
}

}  // namespace

struct BatchPlan {
  // identity
  std::vector<phx_block> blocks;   // geom pointers re-pointed into geoms
  std::vector<phx_geometry> geoms;
  std::vector<const double *> base;
  std::vector<double *> out;
  Par par;
  // device state (one allocation for the tables)
  void *mem = nullptr;
  BView *views_in = nullptr, *views_out = nullptr;
  CUtensorMap *x1_maps = nullptr;  // per block: X1 tensor map (64-byte aligned) and staging mode
  int *x1_modes = nullptr;
  const double **base_tab = nullptr;
  double **out_tab = nullptr;
  double *beta_dt = nullptr;
  std::vector<void *> item_mem;  // work-list allocations
  PhaseList sources, x1, x2, x3, fluxct, fixflux, update, ghost, c2p, inflow;
  size_t x1_smem = 0;
  Tuning tune;
  bool mink = true;
  int ndim = 3;
  const MlpPacked *mlp = nullptr;  // learned start (packed weights in the context) or null
  double *brk = nullptr;           // learned brackets + pass marker, 4 x c2p items x 128
  bool batched = true;             // one persistent launch per phase in a graph; else block by block
  bool has_mesh = false;           // tiled mesh exchange instead of per-block periodic ghosts
  int mesh_n[3] = {0, 0, 0}, mesh_nseg[3] = {0, 0, 0}, mesh_bc[6] = {0, 0, 0, 0, 0, 0}, mesh_bc_vars = 0;
  std::vector<int> mesh_seg[3];    // host copy of the segment starts
  MeshDev md{};
  void *mesh_mem = nullptr;
  std::vector<BView> vin;          // host copy of views_in
  bool staged = false;             // tuned, flux lists built, graph captured
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  ~BatchPlan() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (void *m : item_mem) cudaFree(m);
    cudaFree(brk);
    cudaFree(mesh_mem);
    cudaFree(mem);
  }
};

struct BatchCache {
  std::vector<std::unique_ptr<BatchPlan>> plans;  // most recent last
};

BatchCache *batch_cache_create() { return new BatchCache(); }
void batch_cache_destroy(BatchCache *c) { delete c; }

// Items of size T over counts[b] indices per block.
static std::vector<WorkItem> make_items(const std::vector<long long> &counts, long long T) {
  std::vector<WorkItem> v;
  for (size_t b = 0; b < counts.size(); b++)
    for (long long f = 0; f < counts[b]; f += T) v.push_back(WorkItem{(int)b, 0, f, std::min(f + T, counts[b])});
  return v;
}

static cudaError_t upload_items(BatchPlan &pl, PhaseList &ph, const std::vector<WorkItem> &items) {
  ph.n = (int)items.size();
  ph.boff.assign(pl.blocks.size() + 1, 0);
  for (const WorkItem &w : items) ph.boff[w.block + 1]++;
  for (size_t b = 0; b < pl.blocks.size(); b++) ph.boff[b + 1] += ph.boff[b];
  if (items.empty()) return cudaSuccess;
  void *m = nullptr;
  cudaError_t e = cudaMalloc(&m, sizeof(WorkItem) * items.size());
  if (e != cudaSuccess) return e;
  pl.item_mem.push_back(m);
  ph.d_items = static_cast<WorkItem *>(m);
  return cudaMemcpy(m, items.data(), sizeof(WorkItem) * items.size(), cudaMemcpyHostToDevice);
}

// X1 items: per block ceil(npencil / pencils) items of `pencils` pencils,
// pencils = clamp(round(x1_cells / n1t), 1, 32) and the shared memory bound.
static std::vector<WorkItem> x1_items(const std::vector<BView> &v, int x1_cells, size_t &smem) {
  std::vector<WorkItem> items;
  smem = 0;
  for (size_t b = 0; b < v.size(); b++) {
    int pen = (x1_cells + v[b].n1t / 2) / v[b].n1t;
    pen = std::max(1, std::min(32, pen));
    const size_t pst = (size_t)x1_pencil_stride_host(v[b]) * sizeof(double);
    while (pen > 1 && (size_t)pen * pst > 200 * 1024) pen--;
    smem = std::max(smem, (size_t)pen * pst);
    const int np = x1_npencil(v[b]);
    for (int f = 0; f < np; f += pen) items.push_back(WorkItem{(int)b, 0, f, std::min(f + pen, np)});
  }
  return items;
}

static std::string tune_key(const Par &p, const std::vector<BView> &v, bool mink) {
  std::map<int, int> sizes;
  for (const BView &b : v) sizes[b.n1t * 1000000 + b.n2t * 1000 + b.n3t]++;
  std::ostringstream k;
  k << "recon" << p.recon << (mink ? "-mink" : "-fmks") << "-mhd" << p.mhd;
  for (const auto &kv : sizes) k << "-" << kv.first << "x" << kv.second;
  return k.str();
}

static float time_launch(cudaStream_t s, const std::function<void()> &fn, int reps) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  fn();  // warm-up
  cudaEventRecord(a, s);
  for (int r = 0; r < reps; r++) fn();
  cudaEventRecord(b, s);
  cudaEventSynchronize(b);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms / reps;
}

// Time the candidate tile shapes on the plan's blocks (flux outputs only are
// written; the stage recomputes them).
static Tuning autotune(BatchPlan &pl, const std::vector<BView> &v, unsigned int *err, cudaStream_t s) {
  Tuning best;
  float best_ms = 1e30f;
  for (int cells : {96, 192, 288, 384, 576, 768, 1152}) {
    size_t smem;
    std::vector<WorkItem> items = x1_items(v, cells, smem);
    PhaseList ph;
    if (upload_items(pl, ph, items) != cudaSuccess) break;
    const float ms = time_launch(
        s,
        [&] {
          launch_flux_x1_batched(pl.par, pl.mink, pl.views_in, ph.d_items, ph.n, 0, smem, pl.x1_maps, pl.x1_modes,
                                 err, s);
        },
        3);
    if (ms < best_ms) {
      best_ms = ms;
      best.x1_cells = cells;
    }
  }
  best_ms = 1e30f;
  for (int seg : {8, 16, 32, 64}) {
    float ms = 0.f;
    for (int dir = 1; dir <= pl.ndim - 1; dir++) {
      std::vector<long long> counts;
      for (const BView &b : v) counts.push_back(sweep_threads(b, dir, seg));
      PhaseList ph;
      if (upload_items(pl, ph, make_items(counts, 128)) != cudaSuccess) break;
      ms += time_launch(
          s, [&] { launch_flux_sweep_batched(pl.par, pl.mink, dir, pl.views_in, ph.d_items, ph.n, 0, seg, s); }, 3);
    }
    if (ms < best_ms) {
      best_ms = ms;
      best.seg = seg;
    }
  }
  return best;
}

// The stage's launches, in order.  Batched: one persistent launch per phase
// over all items (captured into the plan's graph).  Per block: phase by phase,
// each block's items in a launch of its own (one item per CTA).
static void stage_launches(BatchPlan &pl, DevStats *stats, unsigned int *err, cudaStream_t s,
                           int only = BATCH_STAGE) {
  const Par &p = pl.par;
  const int nb = (int)pl.blocks.size();
  // run fn(items, count, grid) for all items, or block by block
  auto each = [&](const PhaseList &ph, const std::function<void(const WorkItem *, int, int)> &fn) {
    if (pl.batched) {
      fn(ph.d_items, ph.n, 0);
      return;
    }
    for (int b = 0; b < nb; b++) {
      const int c = ph.boff[b + 1] - ph.boff[b];
      if (c > 0) fn(ph.d_items + ph.boff[b], c, c);
    }
  };
  auto exchange = [&] {
    if (pl.has_mesh) {
      each(pl.c2p, [&](const WorkItem *it, int n, int g) {
        launch_mesh_exchange(p, pl.mink, pl.views_out, pl.md, it, n, g, s);
      });
      each(pl.inflow, [&](const WorkItem *it, int n, int g) {
        launch_ox1_inflow(p, pl.views_out, it, n, g, err, s);
      });
    } else
      each(pl.ghost, [&](const WorkItem *it, int n, int g) {
        launch_ghost_batched(pl.views_out, p.mhd ? PHX_NCONS : 5, it, n, g, s);
      });
  };
  auto fix_fluxes = [&] {
    if (pl.has_mesh && p.fix_flux)
      each(pl.fixflux, [&](const WorkItem *it, int n, int g) {
        launch_fix_fluxes(p, pl.views_in, pl.md, it, n, g, s);
      });
  };
  if (only == BATCH_EXCHANGE) {
    exchange();
    return;
  }
  if (only == BATCH_FIXFLUX) {
    fix_fluxes();
    return;
  }
  each(pl.sources, [&](const WorkItem *it, int n, int g) { launch_sources_batched(p, pl.mink, pl.views_in, it, n, g, s); });
  each(pl.x1, [&](const WorkItem *it, int n, int g) {
    launch_flux_x1_batched(p, pl.mink, pl.views_in, it, n, g, pl.x1_smem, pl.x1_maps, pl.x1_modes, err, s);
  });
  if (pl.ndim >= 2)
    each(pl.x2, [&](const WorkItem *it, int n, int g) {
      launch_flux_sweep_batched(p, pl.mink, 1, pl.views_in, it, n, g, pl.tune.seg, s);
    });
  if (pl.ndim >= 3)
    each(pl.x3, [&](const WorkItem *it, int n, int g) {
      launch_flux_sweep_batched(p, pl.mink, 2, pl.views_in, it, n, g, pl.tune.seg, s);
    });
  if (p.mhd && pl.ndim > 1)
    each(pl.fluxct, [&](const WorkItem *it, int n, int g) { launch_fluxct_batched(pl.ndim, pl.views_in, it, n, g, s); });
  fix_fluxes();
  each(pl.update, [&](const WorkItem *it, int n, int g) {
    launch_update_batched(p, pl.views_in, pl.base_tab, pl.out_tab, pl.beta_dt, it, n, g, s);
  });
  for (int pass = 0; pass < 2; pass++) {  // FillDerived over MeshData, then per block after the exchange
    if (pass == 1) exchange();
    each(pl.c2p, [&](const WorkItem *it, int n, int g) {
      launch_c2p_batched(p, pl.mink, pl.views_out, it, n, g, pl.mlp, pl.brk, stats, err, s);
    });
    each(pl.update, [&](const WorkItem *it, int n, int g) {  // interior zones
      launch_c2p_fixup_batched(p, pl.mink, pl.views_out, it, n, s);
    });
    each(pl.c2p, [&](const WorkItem *it, int n, int g) {  // entire blocks
      launch_floors_batched(p, pl.mink, pl.views_out, it, n, stats, err, s);
    });
  }
}

static bool same_mesh(const BatchPlan &pl, const phx_mesh *m) {
  if (!m) return !pl.has_mesh;
  if (!pl.has_mesh || pl.mesh_bc_vars != m->bc_vars) return false;
  for (int d = 0; d < 3; d++) {
    if (pl.mesh_n[d] != m->n[d] || pl.mesh_nseg[d] != m->nseg[d] || pl.mesh_bc[2 * d] != m->bc_lo[d] ||
        pl.mesh_bc[2 * d + 1] != m->bc_hi[d])
      return false;
    for (int k = 0; k <= m->nseg[d]; k++)
      if (pl.mesh_seg[d][k] != m->seg_start[d][k]) return false;
  }
  return true;
}

// Upload the mesh maps: per-axis cell -> segment, segment triple -> block,
// block -> origin.
static cudaError_t upload_mesh(BatchPlan &P, const phx_mesh *m, int nblocks) {
  P.has_mesh = true;
  P.mesh_bc_vars = m->bc_vars;
  P.md.bc_vars = m->bc_vars;
  size_t ints = 0;
  for (int d = 0; d < 3; d++) {
    P.mesh_n[d] = m->n[d];
    P.mesh_nseg[d] = m->nseg[d];
    P.mesh_bc[2 * d] = m->bc_lo[d];
    P.mesh_bc[2 * d + 1] = m->bc_hi[d];
    P.mesh_seg[d].assign(m->seg_start[d], m->seg_start[d] + m->nseg[d] + 1);
    ints += m->n[d];
  }
  ints += (size_t)nblocks + 3 * (size_t)nblocks;
  std::vector<int> host;
  host.reserve(ints);
  size_t off_seg[3], off_owner, off_origin;
  for (int d = 0; d < 3; d++) {
    off_seg[d] = host.size();
    for (int s = 0; s < m->nseg[d]; s++)
      for (int c = m->seg_start[d][s]; c < m->seg_start[d][s + 1]; c++) host.push_back(s);
  }
  off_owner = host.size();
  for (int b = 0; b < nblocks; b++) host.push_back(b);  // blocks are ordered by segment triple
  off_origin = host.size();
  for (int s3 = 0; s3 < m->nseg[2]; s3++)
    for (int s2 = 0; s2 < m->nseg[1]; s2++)
      for (int s1 = 0; s1 < m->nseg[0]; s1++) {
        host.push_back(m->seg_start[0][s1]);
        host.push_back(m->seg_start[1][s2]);
        host.push_back(m->seg_start[2][s3]);
      }
  cudaError_t e = cudaMalloc(&P.mesh_mem, sizeof(int) * host.size());
  if (e != cudaSuccess) return e;
  if ((e = cudaMemcpy(P.mesh_mem, host.data(), sizeof(int) * host.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
    return e;
  const int *base = static_cast<const int *>(P.mesh_mem);
  for (int d = 0; d < 3; d++) {
    P.md.n[d] = m->n[d];
    P.md.nseg[d] = m->nseg[d];
    P.md.bc_lo[d] = m->bc_lo[d];
    P.md.bc_hi[d] = m->bc_hi[d];
    P.md.seg_of[d] = base + off_seg[d];
  }
  P.md.owner = base + off_owner;
  P.md.origin = base + off_origin;
  return cudaSuccess;
}

// Field-wise (phx_block has padding bytes the caller need not initialise).
static bool same_block(const phx_block &a, const phx_block &b) {
  if (a.nx1 != b.nx1 || a.nx2 != b.nx2 || a.nx3 != b.nx3 || a.ng != b.ng || a.ndim != b.ndim ||
      a.var_stride != b.var_stride)
    return false;
  if (a.x1min != b.x1min || a.x2min != b.x2min || a.x3min != b.x3min || a.dx1 != b.dx1 || a.dx2 != b.dx2 ||
      a.dx3 != b.dx3)
    return false;
  if (a.prim != b.prim || a.cons != b.cons || a.flux != b.flux || a.face_sig != b.face_sig ||
      a.cell_sig != b.cell_sig || a.fail != b.fail || a.src != b.src || a.emf != b.emf || a.dudt != b.dudt)
    return false;
  // geometry by content: the caller may pass a fresh phx_geometry each call
  const bool fa = a.geom && a.geom->kind == PHX_GEOM_FMKS, fb = b.geom && b.geom->kind == PHX_GEOM_FMKS;
  if (fa != fb) return false;
  if (fa && (a.geom->cent != b.geom->cent || a.geom->face1 != b.geom->face1 || a.geom->face2 != b.geom->face2 ||
             a.geom->deriv != b.geom->deriv))
    return false;
  return true;
}

static bool same_plan(const BatchPlan &pl, const phx_block *blocks, int n, const double *const *base,
                      double *const *out, const Par &par, const MlpPacked *mlp, const phx_mesh *mesh,
                      bool batched) {
  if ((int)pl.blocks.size() != n || pl.mlp != mlp || pl.batched != batched || !same_mesh(pl, mesh)) return false;
  if (memcmp(&pl.par, &par, sizeof(Par)) != 0) return false;  // Par is zero-filled before assignment
  for (int i = 0; i < n; i++) {
    if (!same_block(pl.blocks[i], blocks[i])) return false;
    if (pl.base[i] != base[i] || pl.out[i] != out[i]) return false;
  }
  return true;
}

// Tile shapes (tuned on the plan's own blocks: the flux arrays are
// overwritten), flux work lists and the captured graph of the stage.  A plan
// first built for the exchange or FixFluxes alone gets these at its first
// stage.
static cudaError_t prepare_stage(BatchPlan &P, DevStats *stats, unsigned int *err, cudaStream_t s) {
  cudaError_t e;
  const Par &par = P.par;
  const std::vector<BView> &vin = P.vin;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    load_tune_file();
    const std::string key = tune_key(par, vin, P.mink);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
      P.tune = it->second;
    } else {
      P.tune = autotune(P, vin, err, s);
      g_tune[key] = P.tune;
      save_tune_file();
    }
  }
  if ((e = upload_items(P, P.x1, x1_items(vin, P.tune.x1_cells, P.x1_smem))) != cudaSuccess) return e;
  for (int dir = 1; dir <= 2; dir++) {
    std::vector<long long> counts;
    for (const BView &b : vin) counts.push_back(dir < P.ndim ? sweep_threads(b, dir, P.tune.seg) : 0);
    if ((e = upload_items(P, dir == 1 ? P.x2 : P.x3, make_items(counts, 128))) != cudaSuccess) return e;
  }
  prepare_flux_x1_batched(par, P.mink, P.x1_smem);  // kernel attributes are set outside the capture
  if ((e = cudaDeviceSynchronize()) != cudaSuccess) return e;
  if (P.batched) {  // capture the stage
    cudaStream_t cs;
    if ((e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)) != cudaSuccess) return e;
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      stage_launches(P, stats, err, cs);
      e = cudaStreamEndCapture(cs, &P.graph);
    }
    cudaStreamDestroy(cs);
    if (e != cudaSuccess) return e;
    if ((e = cudaGraphInstantiate(&P.exec, P.graph, 0)) != cudaSuccess) return e;
  }
  P.staged = true;
  return cudaSuccess;
}

// Build (or find) the plan of this block set and launch its graph.
// views: validated views of the blocks (cons = stage input).
cudaError_t batch_stage(BatchCache *cache, const Par &par, const phx_block *blocks, const BView *views, int n,
                        const double *const *base, double *const *out, double beta, double dt,
                        const MlpPacked *mlp, const phx_mesh *mesh, bool batched, int only,
                        DevStats *stats, unsigned int *err, cudaStream_t s, const char **why) {
  *why = nullptr;
  BatchPlan *pl = nullptr;
  for (auto &q : cache->plans)
    if (same_plan(*q, blocks, n, base, out, par, mlp, mesh, batched)) pl = q.get();
  cudaError_t e = cudaSuccess;
  if (!pl) {
    auto np = std::make_unique<BatchPlan>();
    BatchPlan &P = *np;
    P.blocks.assign(blocks, blocks + n);
    P.geoms.resize(n);
    for (int i = 0; i < n; i++)
      if (blocks[i].geom) {
        P.geoms[i] = *blocks[i].geom;
        P.blocks[i].geom = &P.geoms[i];
      }
    P.base.assign(base, base + n);
    P.out.assign(out, out + n);
    P.par = par;
    P.mlp = mlp;
    P.batched = batched;
    P.mink = !views[0].fmks;
    P.ndim = views[0].ndim;
    std::vector<BView> vin(views, views + n), vout(views, views + n);
    for (int i = 0; i < n; i++) vout[i].cons = out[i];
    const size_t bytes = 2 * sizeof(BView) * n + 2 * sizeof(double *) * n + 2 * sizeof(double) +
                         sizeof(CUtensorMap) * n + sizeof(int) * n + 256 * 10;
    if ((e = cudaMalloc(&P.mem, bytes)) != cudaSuccess) return e;
    char *m = static_cast<char *>(P.mem);
    auto take = [&](size_t b) {
      char *r = m;
      m += (b + 255) & ~size_t(255);
      return r;
    };
    P.views_in = reinterpret_cast<BView *>(take(sizeof(BView) * n));
    P.views_out = reinterpret_cast<BView *>(take(sizeof(BView) * n));
    P.base_tab = reinterpret_cast<const double **>(take(sizeof(double *) * n));
    P.out_tab = reinterpret_cast<double **>(take(sizeof(double *) * n));
    P.beta_dt = reinterpret_cast<double *>(take(2 * sizeof(double)));
    P.x1_maps = reinterpret_cast<CUtensorMap *>(take(sizeof(CUtensorMap) * n));
    P.x1_modes = reinterpret_cast<int *>(take(sizeof(int) * n));
    {
      std::vector<CUtensorMap> maps(n);
      std::vector<int> modes(n);
      for (int i = 0; i < n; i++) {
        memset(&maps[i], 0, sizeof(CUtensorMap));
        modes[i] = x1_mode(vin[i], &maps[i]);
      }
      cudaMemcpy(P.x1_maps, maps.data(), sizeof(CUtensorMap) * n, cudaMemcpyHostToDevice);
      cudaMemcpy(P.x1_modes, modes.data(), sizeof(int) * n, cudaMemcpyHostToDevice);
    }
    cudaMemcpy(P.views_in, vin.data(), sizeof(BView) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(P.views_out, vout.data(), sizeof(BView) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(P.base_tab, base, sizeof(double *) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(P.out_tab, out, sizeof(double *) * n, cudaMemcpyHostToDevice);
    // work lists
    std::vector<long long> interior, faces, all;
    for (const BView &b : vin) {
      interior.push_back(interior_count(b));
      faces.push_back(fluxct_count(b));
      all.push_back((long long)b.n1t * b.n2t * b.n3t);
    }
    if ((e = upload_items(P, P.sources, make_items(interior, 128))) != cudaSuccess) return e;
    if ((e = upload_items(P, P.fluxct, make_items(faces, 256))) != cudaSuccess) return e;
    if ((e = upload_items(P, P.update, make_items(interior, 256))) != cudaSuccess) return e;
    if ((e = upload_items(P, P.ghost, make_items(all, 256))) != cudaSuccess) return e;
    if ((e = upload_items(P, P.c2p, make_items(all, 128))) != cudaSuccess) return e;
    // learned brackets (3 planes), each zone's warm / cold pass (plane 3) and
    // the count of cold zones (one word after)
    if (mlp && (e = cudaMalloc(&P.brk, sizeof(double) * (4 * (size_t)P.c2p.n * 128 + 1))) != cudaSuccess) return e;
    if (mesh) {
      if ((e = upload_mesh(P, mesh, n)) != cudaSuccess) return e;
      std::vector<long long> fix;
      for (int s3 = 0, b = 0; s3 < mesh->nseg[2]; s3++)
        for (int s2 = 0; s2 < mesh->nseg[1]; s2++)
          for (int s1 = 0; s1 < mesh->nseg[0]; s1++, b++) {
            const int nx[3] = {vin[b].nx1, vin[b].nx2, vin[b].nx3};
            const int org[3] = {mesh->seg_start[0][s1], mesh->seg_start[1][s2], mesh->seg_start[2][s3]};
            long long cnt[6], tot = 0;
            fix_face_counts(vin[b].ndim, nx, org, mesh->n, mesh->bc_lo, mesh->bc_hi, cnt);
            for (long long c : cnt) tot += c;
            fix.push_back(tot);
          }
      if ((e = upload_items(P, P.fixflux, make_items(fix, 128))) != cudaSuccess) return e;
      // bc_vars = conserved: the inflow check's slabs (blocks on the physical outer X1 face)
      std::vector<long long> slab(n, 0);
      if (mesh->bc_vars == PHX_BC_VARS_CONSERVED && par.inflow_check && !P.mink &&
          mesh->bc_hi[0] != PHX_BC_PERIODIC)
        for (int s3 = 0, b = 0; s3 < mesh->nseg[2]; s3++)
          for (int s2 = 0; s2 < mesh->nseg[1]; s2++)
            for (int s1 = 0; s1 < mesh->nseg[0]; s1++, b++)
              if (s1 == mesh->nseg[0] - 1) slab[b] = (long long)vin[b].ng * vin[b].n2t * vin[b].n3t;
      if ((e = upload_items(P, P.inflow, make_items(slab, 128))) != cudaSuccess) return e;
    }
    P.vin = vin;
    if (only == BATCH_STAGE && (e = prepare_stage(P, stats, err, s)) != cudaSuccess) return e;
    if (cache->plans.size() >= 8) cache->plans.erase(cache->plans.begin());
    cache->plans.push_back(std::move(np));
    pl = cache->plans.back().get();
  }
  if (only != BATCH_STAGE) {
    stage_launches(*pl, stats, err, s, only);
    return cudaGetLastError();
  }
  if (!pl->staged && (e = prepare_stage(*pl, stats, err, s)) != cudaSuccess) return e;
  const double bd[2] = {beta, dt};
  if ((e = cudaMemcpyAsync(pl->beta_dt, bd, sizeof(bd), cudaMemcpyHostToDevice, s)) != cudaSuccess) return e;
  if (pl->batched) return cudaGraphLaunch(pl->exec, s);
  stage_launches(*pl, stats, err, s);
  return cudaGetLastError();
}

// The tuned shapes of the most recent plan (for reporting).
void batch_last_tuning(BatchCache *cache, int *x1_cells, int *seg, int *launches) {
  if (cache->plans.empty()) {
    *x1_cells = *seg = *launches = 0;
    return;
  }
  const BatchPlan &p = *cache->plans.back();
  *x1_cells = p.tune.x1_cells;
  *seg = p.tune.seg;
  size_t nn = 0;
  if (p.graph) cudaGraphGetNodes(p.graph, nullptr, &nn);
  *launches = (int)nn;
}

}  // namespace phx
