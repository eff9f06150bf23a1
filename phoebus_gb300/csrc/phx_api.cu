// phx_api.cu -- the extern "C" entry points of phx_fluid.h.
//
// Host-side validation, parameter resolution (the fixup package defaults of
// fixup.cpp:120-180), and dispatch to the kernels.  All calls are
// asynchronous on the caller's stream; nothing is allocated per call.
#include <cmath>
#include <cstdarg>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "phx_m1.cuh"
#include "phx_mlp.cuh"

struct phx_ctx {
  int device;
  phx::DevStats *stats;        // device
  unsigned int *err;           // device sticky error word
  unsigned long long *dt_scr;  // device scratch for the dt reduction
  float *mlp_w;                // device FP32 master parameters of the learned start
  float *mlp_grad, *mlp_m, *mlp_v;  // device gradient and AdamW moments
  float *mlp_loss;             // device per-epoch loss sums [PHX_MLP_MAX_EPOCHS]
  phx::MlpPacked *mlp_packed;  // device BF16 fragments for inference (and the input box)
  int *mlp_boxkeys;            // device scratch of the input-box reduction [12]
  unsigned long long *red;     // device scratch of mesh-wide maxima [2]
  phx::C2PScratch c2p;         // device con2prim chunk scratch (brackets, retry list)
  void *c2p_mem;               // its single allocation
  long long mlp_step;          // AdamW step count
  int mlp_loaded;
  phx::BatchCache *batch;      // plans of phx_stage_batched (host)
};

namespace {
thread_local std::string g_last_error;

phx_status fail(phx_status s, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return s;
}

}  // namespace

namespace phx {
// Records msg as phx_last_error()'s text for entry points defined in other
// translation units (phx_noalloc.cu).
void set_last_error(const char *msg) { g_last_error = msg ? msg : ""; }
}  // namespace phx

namespace {
phx_status cuda_status(const char *where) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(PHX_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
  return PHX_OK;
}

phx::Par make_par(const phx_params &p) {
  phx::Par d;
  std::memset(&d, 0, sizeof(d));  // all bytes defined: batched plans compare Par bytewise
  d.gm1 = p.gm1;
  d.Cv = p.Cv;
  d.rho_min_eos = p.rho_min_eos;
  d.sie_min_eos = p.sie_min_eos;
  d.c2p_tol = p.c2p_tol;
  d.c2p_max_iter = p.c2p_max_iter;
  d.fsf = p.c2p_floor_scale_fac;
  d.fail_on_floors = p.c2p_fail_on_floors;
  d.fail_on_ceilings = p.c2p_fail_on_ceilings;
  d.mhd = p.mhd;
  if (p.enable_floors || p.enable_c2p_fixup || (p.enable_mhd_floors && p.mhd)) {
    d.floor_type = p.floor_type;
    d.r0 = p.rho0_floor;
    d.s0 = p.sie0_floor;
    d.ralpha = p.rho_exp_floor;
    d.salpha = p.sie_exp_floor;
    d.enable_floors = 1;
  } else {  // Floors(): ConstantRhoSie with -max (fixup.hpp:75-78)
    d.floor_type = PHX_FLOOR_CONSTANT_RHO_SIE;
    d.r0 = -phx::kDBLMAX;
    d.s0 = -phx::kDBLMAX;
    d.ralpha = d.salpha = 0.0;
    d.enable_floors = 0;
  }
  if (p.enable_ceilings) {
    d.g0 = p.gam0_ceiling;
    d.smax0 = p.sie0_ceiling;
  } else {
    d.g0 = phx::kDBLMAX;
    d.smax0 = phx::kDBLMAX;
  }
  d.enable_mhd_floors = (p.enable_mhd_floors && p.mhd) ? 1 : 0;
  if (d.enable_mhd_floors) {
    d.bsqorho0 = p.bsqorho0_ceiling;
    d.bsqou0 = p.bsqou0_ceiling;
  } else {
    d.bsqorho0 = phx::kDBLMAX;
    d.bsqou0 = phx::kDBLMAX;
  }
  d.recon = p.recon;
  d.riemann = p.riemann;
  d.cfl = p.cfl;
  d.c2p_fixup = p.enable_c2p_fixup;
  d.strategy_floors = p.c2p_failure_strategy_floors;
  d.vsq_max = 1.0 - 1.0 / (d.g0 * d.g0);
  d.iCv = 1.0 / p.Cv;
  d.fix_flux = p.enable_flux_fixup ? 1 : 0;
  d.inflow_check = p.enable_ox1_fmks_inflow_check ? 1 : 0;
  return d;
}

phx_status check_params(const phx_params *p) {
  if (!p) return fail(PHX_ERR_INVALID_ARG, "params is NULL");
  if (p->recon < PHX_RECON_CONSTANT || p->recon > PHX_RECON_MP5)
    return fail(PHX_ERR_INVALID_ARG, "invalid recon %d", p->recon);
  if (p->riemann != PHX_RIEMANN_LLF && p->riemann != PHX_RIEMANN_HLL)
    return fail(PHX_ERR_INVALID_ARG, "invalid riemann solver %d (choose llf or hll)", p->riemann);
  if (!(p->c2p_floor_scale_fac <= 1. && p->c2p_floor_scale_fac > 0.))
    return fail(PHX_ERR_INVALID_ARG, "fluid/c2p_floor_scale_fac must be between 0 and 1!");
  if (p->c2p_max_iter < 0) return fail(PHX_ERR_INVALID_ARG, "c2p_max_iter < 0");
  return PHX_OK;
}

phx_status make_view(const phx_block *b, phx::BView &v) {
  if (!b) return fail(PHX_ERR_INVALID_ARG, "block is NULL");
  if (b->ndim < 1 || b->ndim > 3) return fail(PHX_ERR_INVALID_ARG, "ndim must be 1..3");
  if (b->ng < 3) return fail(PHX_ERR_INVALID_ARG, "ng must be >= 3 (got %d)", b->ng);
  if (b->nx1 < 1 || b->nx2 < 1 || b->nx3 < 1) return fail(PHX_ERR_INVALID_ARG, "nx must be >= 1");
  if ((b->ndim < 2 && b->nx2 != 1) || (b->ndim < 3 && b->nx3 != 1))
    return fail(PHX_ERR_INVALID_ARG, "inactive dimensions must have nx = 1");
  if (!b->prim || !b->cons) return fail(PHX_ERR_INVALID_ARG, "prim/cons pointers are NULL");
  v.ndim = b->ndim;
  v.ng = b->ng;
  v.nx1 = b->nx1;
  v.nx2 = b->nx2;
  v.nx3 = b->nx3;
  v.n1t = b->nx1 + 2 * b->ng;
  v.n2t = b->ndim >= 2 ? b->nx2 + 2 * b->ng : 1;
  v.n3t = b->ndim >= 3 ? b->nx3 + 2 * b->ng : 1;
  const long long N = (long long)v.n1t * v.n2t * v.n3t;
  v.vs = b->var_stride ? b->var_stride : N;
  if (v.vs < N) return fail(PHX_ERR_INVALID_ARG, "var_stride smaller than the block");
  const double xmin[3] = {b->x1min, b->x2min, b->x3min};
  const double dx[3] = {b->dx1, b->dx2, b->dx3};
  for (int d = 0; d < 3; d++) {
    v.dx[d] = dx[d];
    v.x0[d] = d < b->ndim ? xmin[d] - b->ng * dx[d] : xmin[d];
  }
  v.prim = b->prim;
  v.cons = b->cons;
  v.flux = b->flux;
  v.face_sig = b->face_sig;
  v.cell_sig = b->cell_sig;
  v.fail = b->fail;
  v.src = b->src;
  v.emf = b->emf;
  v.dudt = b->dudt;
  v.fmks = 0;
  v.gcent = v.gface1 = v.gface2 = v.gderiv = nullptr;
  if (b->geom && b->geom->kind == PHX_GEOM_FMKS) {
    if (!b->geom->cent || !b->geom->face1 || !b->geom->face2 || !b->geom->deriv)
      return fail(PHX_ERR_INVALID_ARG, "FMKS geometry tables are NULL");
    v.fmks = 1;
    v.gcent = b->geom->cent;
    v.gface1 = b->geom->face1;
    v.gface2 = b->geom->face2;
    v.gderiv = b->geom->deriv;
  }
  return PHX_OK;
}

phx_status check_range(const phx::BView &v, phx_range ib, phx_range jb, phx_range kb, phx::Range3 &r) {
  if (ib.s < 0 || ib.e >= v.n1t || jb.s < 0 || jb.e >= v.n2t || kb.s < 0 || kb.e >= v.n3t)
    return fail(PHX_ERR_INVALID_ARG, "index range outside the block");
  r = {ib.s, ib.e, jb.s, jb.e, kb.s, kb.e};
  return PHX_OK;
}

phx::Range3 entire(const phx::BView &v) { return {0, v.n1t - 1, 0, v.n2t - 1, 0, v.n3t - 1}; }
phx::Range3 interior(const phx::BView &v) {
  return {v.ng, v.ng + v.nx1 - 1, v.ndim >= 2 ? v.ng : 0, v.ndim >= 2 ? v.ng + v.nx2 - 1 : 0,
          v.ndim >= 3 ? v.ng : 0, v.ndim >= 3 ? v.ng + v.nx3 - 1 : 0};
}

inline cudaStream_t S(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// The con2prim chunk scratch as one allocation, 256-byte aligned pieces.
size_t c2p_scratch_bytes() {
  const size_t C = (size_t)phx::C2P_CHUNK;
  return 256 * 9 + sizeof(double) * (3 * C + 4 * C) + sizeof(int) * (1 + C) + sizeof(unsigned long long) * C;
}

phx::C2PScratch c2p_scratch_carve(void *mem) {
  const size_t C = (size_t)phx::C2P_CHUNK;
  char *p = static_cast<char *>(mem);
  auto take = [&](size_t bytes) {
    char *r = p;
    p += (bytes + 255) & ~size_t(255);
    return r;
  };
  phx::C2PScratch s;
  s.brk = reinterpret_cast<double *>(take(sizeof(double) * 3 * C));
  s.count = reinterpret_cast<int *>(take(sizeof(int)));
  s.idx = reinterpret_cast<int *>(take(sizeof(int) * C));
  s.a = reinterpret_cast<double *>(take(sizeof(double) * C));
  s.b = reinterpret_cast<double *>(take(sizeof(double) * C));
  s.ya = reinterpret_cast<double *>(take(sizeof(double) * C));
  s.yb = reinterpret_cast<double *>(take(sizeof(double) * C));
  s.packed = reinterpret_cast<unsigned long long *>(take(sizeof(unsigned long long) * C));
  return s;
}

phx_status ctx_device(phx_ctx *ctx) {
  if (!ctx) return fail(PHX_ERR_INVALID_ARG, "ctx is NULL");
  int cur = -1;
  cudaGetDevice(&cur);
  if (cur != ctx->device) {
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return fail(PHX_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
  }
  return PHX_OK;
}
}  // namespace

namespace phx {
void launch_fluxes_err(const Par &p, const BView &b, unsigned int *err, cudaStream_t s);
}

extern "C" {

int phx_abi_version(void) { return PHX_ABI_VERSION; }

int phx_build_exact(void) {
#ifdef PHX_EXACT
  return 1;
#else
  return 0;
#endif
}

const char *phx_status_string(phx_status s) {
  switch (s) {
  case PHX_OK: return "ok";
  case PHX_ERR_INVALID_ARG: return "invalid argument";
  case PHX_ERR_UNBRACKETED: return "con2prim root not bracketed";
  case PHX_ERR_NAN_INPUT: return "NaN input";
  case PHX_ERR_TIMEOUT: return "device wait timed out";
  case PHX_ERR_CUDA: return "CUDA error";
  case PHX_ERR_NO_DEVICE: return "no CUDA device";
  case PHX_ERR_CAPACITY: return "request exceeds a fixed capacity";
  case PHX_ERR_UNSUPPORTED: return "unsupported";
  }
  return "unknown status";
}

const char *phx_last_error(void) { return g_last_error.c_str(); }

void phx_params_default(phx_params *p) {
  std::memset(p, 0, sizeof(*p));
  p->gm1 = 4.0 / 3.0 - 1.0;
  p->Cv = 1.0;
  p->rho_min_eos = 0.0;
  p->sie_min_eos = 0.0;
  p->c2p_tol = 1.e-8;       // fluid.cpp:76
  p->c2p_max_iter = 20;     // fluid.cpp:79
  p->c2p_floor_scale_fac = 1.0;
  p->recon = PHX_RECON_LINEAR;  // fluid.cpp:96
  p->riemann = PHX_RIEMANN_HLL; // fluid.cpp:119
  p->cfl = 0.8;                 // fluid.cpp:63
  p->mhd = 1;
  p->floor_type = PHX_FLOOR_CONSTANT_RHO_SIE;
  p->rho_exp_floor = -2.0;
  p->sie_exp_floor = -1.0;
  p->gam0_ceiling = 1000.0;
  p->sie0_ceiling = 100.0;
  p->bsqorho0_ceiling = 50.0;
  p->bsqou0_ceiling = 2500.0;
}

void phx_geometry_default(phx_geometry *g, int kind) {
  std::memset(g, 0, sizeof(*g));
  g->kind = kind;
  g->a = 0.0;
  g->hslope = 0.3;       // fmks.cpp:41-47
  g->poly_xt = 0.82;
  g->poly_alpha = 14.0;
  g->x0 = 0.0;
  g->smooth = 0.5;
  g->hexp_br = 1.e30;
  g->hexp_nsq = 4.0;
  g->hexp_csq = 4.0;
  g->derefine_poles = 1;
}

phx_status phx_ctx_create(int device, phx_ctx **out) {
  if (!out) return fail(PHX_ERR_INVALID_ARG, "out is NULL");
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return fail(PHX_ERR_NO_DEVICE, "no CUDA device available");
  }
  if (device < 0 || device >= n) return fail(PHX_ERR_INVALID_ARG, "device %d out of range", device);
  if (cudaSetDevice(device) != cudaSuccess) return cuda_status("cudaSetDevice");
  phx_ctx *c = new phx_ctx{};
  c->device = device;
  if (cudaMalloc(&c->stats, sizeof(phx::DevStats)) != cudaSuccess ||
      cudaMalloc(&c->err, sizeof(unsigned int)) != cudaSuccess ||
      cudaMalloc(&c->dt_scr, sizeof(unsigned long long)) != cudaSuccess ||
      cudaMalloc(&c->mlp_w, sizeof(float) * PHX_MLP_NPARAM) != cudaSuccess ||
      cudaMalloc(&c->mlp_grad, sizeof(float) * PHX_MLP_NPARAM) != cudaSuccess ||
      cudaMalloc(&c->mlp_m, sizeof(float) * PHX_MLP_NPARAM) != cudaSuccess ||
      cudaMalloc(&c->mlp_v, sizeof(float) * PHX_MLP_NPARAM) != cudaSuccess ||
      cudaMalloc(&c->mlp_loss, sizeof(float) * PHX_MLP_MAX_EPOCHS) != cudaSuccess ||
      cudaMalloc(&c->mlp_packed, sizeof(phx::MlpPacked)) != cudaSuccess ||
      cudaMalloc(&c->mlp_boxkeys, sizeof(int) * 2 * PHX_MLP_IN) != cudaSuccess ||
      cudaMalloc(&c->red, sizeof(unsigned long long) * 2) != cudaSuccess ||
      cudaMalloc(&c->c2p_mem, c2p_scratch_bytes()) != cudaSuccess) {
    phx_status s = cuda_status("cudaMalloc");
    phx_ctx_destroy(c);
    return s;
  }
  cudaMemset(c->stats, 0, sizeof(phx::DevStats));
  cudaMemset(c->err, 0, sizeof(unsigned int));
  cudaMemset(c->mlp_w, 0, sizeof(float) * PHX_MLP_NPARAM);
  cudaMemset(c->mlp_grad, 0, sizeof(float) * PHX_MLP_NPARAM);
  cudaMemset(c->mlp_m, 0, sizeof(float) * PHX_MLP_NPARAM);
  cudaMemset(c->mlp_v, 0, sizeof(float) * PHX_MLP_NPARAM);
  cudaMemset(c->mlp_packed, 0, sizeof(phx::MlpPacked));
  phx::launch_mlp_box_reset(c->mlp_packed, 0);
  c->c2p = c2p_scratch_carve(c->c2p_mem);
  c->batch = phx::batch_cache_create();
  phx_status s = cuda_status("ctx init");
  if (s != PHX_OK) {
    phx_ctx_destroy(c);
    return s;
  }
  *out = c;
  return PHX_OK;
}

phx_status phx_ctx_destroy(phx_ctx *ctx) {
  if (!ctx) return PHX_OK;
  cudaSetDevice(ctx->device);
  cudaFree(ctx->stats);
  cudaFree(ctx->err);
  cudaFree(ctx->dt_scr);
  cudaFree(ctx->mlp_w);
  cudaFree(ctx->mlp_grad);
  cudaFree(ctx->mlp_m);
  cudaFree(ctx->mlp_v);
  cudaFree(ctx->mlp_loss);
  cudaFree(ctx->mlp_packed);
  cudaFree(ctx->mlp_boxkeys);
  cudaFree(ctx->red);
  cudaFree(ctx->c2p_mem);
  if (ctx->batch) phx::batch_cache_destroy(ctx->batch);
  delete ctx;
  return PHX_OK;
}

phx_status phx_ctx_check(phx_ctx *ctx) {
  phx_status s = ctx_device(ctx);
  if (s != PHX_OK) return s;
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return fail(PHX_ERR_CUDA, "device error: %s", cudaGetErrorString(e));
  unsigned int w = 0;
  cudaMemcpy(&w, ctx->err, sizeof(w), cudaMemcpyDeviceToHost);
  cudaMemset(ctx->err, 0, sizeof(unsigned int));
  if (w & phx::ERR_TIMEOUT) return fail(PHX_ERR_TIMEOUT, "a bounded device wait gave up");
  if (w & phx::ERR_UNBRACKETED) return fail(PHX_ERR_UNBRACKETED, "Aborting with unbracketed root.");
  if (w & phx::ERR_BOUNDS) return fail(PHX_ERR_INVALID_ARG, "device index check failed");
  return cuda_status("phx_ctx_check");
}

phx_status phx_ctx_c2p_stats(phx_ctx *ctx, phx_c2p_stats *out, int reset) {
  phx_status s = ctx_device(ctx);
  if (s != PHX_OK) return s;
  if (!out) return fail(PHX_ERR_INVALID_ARG, "out is NULL");
  static_assert(sizeof(phx::DevStats) == sizeof(phx_c2p_stats), "stats layout");
  if (cudaMemcpy(out, ctx->stats, sizeof(*out), cudaMemcpyDeviceToHost) != cudaSuccess)
    return cuda_status("stats copy");
  if (reset) cudaMemset(ctx->stats, 0, sizeof(phx::DevStats));
  return cuda_status("stats");
}

phx_status phx_prim_to_con(phx_ctx *ctx, const phx_params *p, const phx_block *b, phx_range ib,
                           phx_range jb, phx_range kb, void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx)) || (s = check_params(p))) return s;
  phx::BView v;
  if ((s = make_view(b, v))) return s;
  if (!b->cell_sig) return fail(PHX_ERR_INVALID_ARG, "cell_sig is NULL");
  phx::Range3 r;
  if ((s = check_range(v, ib, jb, kb, r))) return s;
  phx::launch_p2c(make_par(*p), v, r, S(stream));
  return cuda_status("phx_prim_to_con");
}

static phx_status c2p_common(phx_ctx *ctx, const phx_params *p, const phx_block *b, phx_range ib,
                             phx_range jb, phx_range kb, void *stream, bool learned) {
  phx_status s;
  if ((s = ctx_device(ctx)) || (s = check_params(p))) return s;
  phx::BView v;
  if ((s = make_view(b, v))) return s;
  if (!b->fail || !b->cell_sig) return fail(PHX_ERR_INVALID_ARG, "fail/cell_sig is NULL");
  phx::Range3 r;
  if ((s = check_range(v, ib, jb, kb, r))) return s;
  if (learned && !ctx->mlp_loaded) return fail(PHX_ERR_INVALID_ARG, "no learned-guess weights loaded");
  phx::launch_c2p(make_par(*p), v, r, ctx->stats, ctx->err, learned ? ctx->mlp_packed : nullptr, ctx->c2p,
                  S(stream));
  return cuda_status("phx_con_to_prim");
}

phx_status phx_con_to_prim(phx_ctx *ctx, const phx_params *p, const phx_block *b, phx_range ib,
                           phx_range jb, phx_range kb, void *stream) {
  return c2p_common(ctx, p, b, ib, jb, kb, stream, false);
}

phx_status phx_con_to_prim_learned(phx_ctx *ctx, const phx_params *p, const phx_block *b,
                                   phx_range ib, phx_range jb, phx_range kb, void *stream) {
  return c2p_common(ctx, p, b, ib, jb, kb, stream, true);
}

phx_status phx_prim_to_con_zones(phx_ctx *ctx, const phx_params *p, long long n, const double *prim,
                                 const double *geom, double *cons, double *cell_sig, void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx)) || (s = check_params(p))) return s;
  if (n < 0) return fail(PHX_ERR_INVALID_ARG, "n < 0");
  if (n == 0) return PHX_OK;
  if (!cons || !prim) return fail(PHX_ERR_INVALID_ARG, "cons/prim is NULL");
  phx::launch_p2c_zones(make_par(*p), n, prim, geom, cons, cell_sig, S(stream));
  return cuda_status("phx_prim_to_con_zones");
}

phx_status phx_con_to_prim_zones(phx_ctx *ctx, const phx_params *p, long long n, double *cons, double *prim,
                                 const double *geom, double *fail_flag, double *cell_sig, const double *coords,
                                 int learned, void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx)) || (s = check_params(p))) return s;
  if (n < 0) return fail(PHX_ERR_INVALID_ARG, "n < 0");
  if (n == 0) return PHX_OK;
  if (!cons || !prim || !fail_flag) return fail(PHX_ERR_INVALID_ARG, "cons/prim/fail is NULL");
  if (learned && !ctx->mlp_loaded) return fail(PHX_ERR_INVALID_ARG, "no learned-guess weights loaded");
  phx::launch_c2p_zones(make_par(*p), n, cons, prim, geom, fail_flag, cell_sig, coords, ctx->stats, ctx->err,
                        learned ? ctx->mlp_packed : nullptr, ctx->c2p, S(stream));
  return cuda_status("phx_con_to_prim_zones");
}

phx_status phx_geometry_fmks_points(phx_ctx *ctx, const phx_geometry *g, long long n, const double *x1,
                                    const double *x2, double *geom, void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx))) return s;
  if (!g || g->kind != PHX_GEOM_FMKS) return fail(PHX_ERR_INVALID_ARG, "geometry must be FMKS");
  if (n < 0) return fail(PHX_ERR_INVALID_ARG, "n < 0");
  if (n == 0) return PHX_OK;
  if (!x1 || !x2 || !geom) return fail(PHX_ERR_INVALID_ARG, "x1/x2/geom is NULL");
  phx::launch_geom_points(*g, n, x1, x2, geom, S(stream));
  return cuda_status("phx_geometry_fmks_points");
}

phx_status phx_calculate_fluxes(phx_ctx *ctx, const phx_params *p, const phx_block *b, void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx)) || (s = check_params(p))) return s;
  phx::BView v;
  if ((s = make_view(b, v))) return s;
  if (!b->flux || !b->face_sig) return fail(PHX_ERR_INVALID_ARG, "flux/face_sig is NULL");
  phx::launch_fluxes_err(make_par(*p), v, ctx->err, S(stream));
  return cuda_status("phx_calculate_fluxes");
}

phx_status phx_flux_ct(phx_ctx *ctx, const phx_params *p, const phx_block *b, void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx)) || (s = check_params(p))) return s;
  phx::BView v;
  if ((s = make_view(b, v))) return s;
  if (!p->mhd || b->ndim == 1) return PHX_OK;  // fluid.cpp:779-784
  if (!b->flux || !b->emf) return fail(PHX_ERR_INVALID_ARG, "flux/emf is NULL");
  phx::launch_fluxct(v, S(stream));
  return cuda_status("phx_flux_ct");
}

phx_status phx_calculate_fluid_source_terms(phx_ctx *ctx, const phx_params *p, const phx_block *blocks,
                                            int nblocks, void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx)) || (s = check_params(p))) return s;
  if (nblocks < 0 || (nblocks > 0 && !blocks)) return fail(PHX_ERR_INVALID_ARG, "bad block list");
  const phx::Par par = make_par(*p);
  for (int n = 0; n < nblocks; n++) {
    phx::BView v;
    if ((s = make_view(&blocks[n], v))) return s;
    if (!blocks[n].src) return fail(PHX_ERR_INVALID_ARG, "src is NULL");
    phx::launch_sources(par, v, S(stream));
  }
  return cuda_status("phx_calculate_fluid_source_terms");
}

phx_status phx_update_stage(phx_ctx *ctx, const phx_block *b, const double *cons_base, double *cons_out,
                            double beta, double dt, void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx))) return s;
  phx::BView v;
  if ((s = make_view(b, v))) return s;
  if (!b->flux) return fail(PHX_ERR_INVALID_ARG, "flux is NULL");
  if (cons_out && !cons_base) return fail(PHX_ERR_INVALID_ARG, "cons_base is NULL");
  phx::Par par{};
  par.mhd = 1;
  phx::launch_update(par, v, cons_base, cons_out, beta, dt, S(stream));
  return cuda_status("phx_update_stage");
}

phx_status phx_fill_ghosts_periodic(phx_ctx *ctx, const phx_block *b, double *field, int nvar, void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx))) return s;
  phx::BView v;
  if ((s = make_view(b, v))) return s;
  if (!field || nvar < 0) return fail(PHX_ERR_INVALID_ARG, "bad field");
  if (b->nx1 < b->ng || (b->ndim >= 2 && b->nx2 < b->ng) || (b->ndim >= 3 && b->nx3 < b->ng))
    return fail(PHX_ERR_INVALID_ARG, "periodic exchange needs nx >= ng");
  phx::launch_ghost_periodic(v, field, nvar, S(stream));
  return cuda_status("phx_fill_ghosts_periodic");
}

phx_status phx_estimate_timestep(phx_ctx *ctx, const phx_params *p, const phx_block *b, int use_face_speeds,
                                 double *dt_out_device, void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx)) || (s = check_params(p))) return s;
  phx::BView v;
  if ((s = make_view(b, v))) return s;
  if (!dt_out_device || !b->cell_sig || (use_face_speeds && !b->face_sig))
    return fail(PHX_ERR_INVALID_ARG, "dt_out/cell_sig/face_sig is NULL");
  phx::launch_dt(make_par(*p), v, use_face_speeds, ctx->dt_scr, dt_out_device, S(stream));
  return cuda_status("phx_estimate_timestep");
}

phx_status phx_c2p_fixup(phx_ctx *ctx, const phx_params *p, const phx_block *b, void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx)) || (s = check_params(p))) return s;
  phx::BView v;
  if ((s = make_view(b, v))) return s;
  if (!b->fail || !b->cell_sig) return fail(PHX_ERR_INVALID_ARG, "fail/cell_sig is NULL");
  phx::launch_c2p_fixup(make_par(*p), v, S(stream));
  return cuda_status("phx_c2p_fixup");
}

phx_status phx_apply_floors(phx_ctx *ctx, const phx_params *p, const phx_block *b, phx_range ib, phx_range jb,
                            phx_range kb, void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx)) || (s = check_params(p))) return s;
  phx::BView v;
  if ((s = make_view(b, v))) return s;
  if (!b->cell_sig) return fail(PHX_ERR_INVALID_ARG, "cell_sig is NULL");
  phx::Range3 r;
  if ((s = check_range(v, ib, jb, kb, r))) return s;
  phx::launch_floors(make_par(*p), v, r, ctx->stats, ctx->err, S(stream));
  return cuda_status("phx_apply_floors");
}

phx_status phx_geometry_fill_fmks(phx_ctx *ctx, const phx_geometry *g, const phx_block *b, void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx))) return s;
  if (!g || g->kind != PHX_GEOM_FMKS) return fail(PHX_ERR_INVALID_ARG, "geometry must be FMKS");
  if (!g->cent || !g->face1 || !g->face2 || !g->deriv) return fail(PHX_ERR_INVALID_ARG, "tables are NULL");
  phx::BView v;
  phx_block bb = *b;
  bb.geom = nullptr;
  if ((s = make_view(&bb, v))) return s;
  phx::launch_geom_fmks(*g, v, S(stream));
  return cuda_status("phx_geometry_fill_fmks");
}

phx_status phx_stage(phx_ctx *ctx, const phx_params *p, const phx_block *b, const double *cons_base,
                     double *cons_out, double beta, double dt, int use_learned_guess, void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx)) || (s = check_params(p))) return s;
  phx::BView v;
  if ((s = make_view(b, v))) return s;
  if (!b->flux || !b->face_sig || !b->cell_sig || !b->fail || !b->src || !cons_base || !cons_out)
    return fail(PHX_ERR_INVALID_ARG, "stage needs flux, face_sig, cell_sig, fail, src, cons_base, cons_out");
  if (p->mhd && b->ndim > 1 && !b->emf) return fail(PHX_ERR_INVALID_ARG, "emf is NULL");
  if (b->nx1 < b->ng || (b->ndim >= 2 && b->nx2 < b->ng) || (b->ndim >= 3 && b->nx3 < b->ng))
    return fail(PHX_ERR_INVALID_ARG, "periodic exchange needs nx >= ng");
  if (use_learned_guess && !ctx->mlp_loaded) return fail(PHX_ERR_INVALID_ARG, "no learned-guess weights loaded");
  const phx::Par par = make_par(*p);
  cudaStream_t st = S(stream);
  phx::launch_sources(par, v, st);                      // CalculateFluidSourceTerms
  phx::launch_fluxes_err(par, v, ctx->err, st);         // CalculateFluxes
  if (p->mhd && b->ndim > 1) phx::launch_fluxct(v, st);  // FluxCT
  phx::launch_update(par, v, cons_base, cons_out, beta, dt, st);
  phx::BView vo = v;  // the stage result: con2prim reads cons_out
  vo.cons = cons_out;
  const phx::MlpPacked *w = use_learned_guess ? ctx->mlp_packed : nullptr;
  phx::launch_c2p(par, vo, entire(vo), ctx->stats, ctx->err, w, ctx->c2p, st);  // FillDerived (MeshData)
  phx::launch_c2p_fixup(par, vo, st);                                  // ConservedToPrimitiveFixup
  phx::launch_floors(par, vo, entire(vo), ctx->stats, ctx->err, st);    // ApplyFloors
  phx::launch_ghost_periodic(vo, cons_out, p->mhd ? PHX_NCONS : 5, st);  // boundary exchange
  phx::launch_c2p(par, vo, entire(vo), ctx->stats, ctx->err, w, ctx->c2p, st);  // FillDerived (block)
  phx::launch_c2p_fixup(par, vo, st);
  phx::launch_floors(par, vo, entire(vo), ctx->stats, ctx->err, st);
  return cuda_status("phx_stage");
}

phx_status phx_stage_batched(phx_ctx *ctx, const phx_params *p, const phx_block *blocks, int nblocks,
                             const double *const *cons_base, double *const *cons_out, double beta, double dt,
                             int use_learned_guess, void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx)) || (s = check_params(p))) return s;
  if (!blocks || nblocks <= 0 || !cons_base || !cons_out) return fail(PHX_ERR_INVALID_ARG, "no blocks");
  if (use_learned_guess && !ctx->mlp_loaded) return fail(PHX_ERR_INVALID_ARG, "no learned-guess weights loaded");
  std::vector<phx::BView> views(nblocks);
  for (int n = 0; n < nblocks; n++) {
    const phx_block *b = &blocks[n];
    if ((s = make_view(b, views[n]))) return fail(s, "block %d: %s", n, g_last_error.c_str());
    if (!b->flux || !b->face_sig || !b->cell_sig || !b->fail || !b->src || !cons_base[n] || !cons_out[n])
      return fail(PHX_ERR_INVALID_ARG, "block %d: stage needs flux, face_sig, cell_sig, fail, src, cons_base, "
                                       "cons_out", n);
    if (p->mhd && b->ndim > 1 && !b->emf) return fail(PHX_ERR_INVALID_ARG, "block %d: emf is NULL", n);
    if (b->nx1 < b->ng || (b->ndim >= 2 && b->nx2 < b->ng) || (b->ndim >= 3 && b->nx3 < b->ng))
      return fail(PHX_ERR_INVALID_ARG, "block %d: periodic exchange needs nx >= ng", n);
    if (views[n].ndim != views[0].ndim || views[n].fmks != views[0].fmks)
      return fail(PHX_ERR_INVALID_ARG, "blocks must share ndim and geometry kind");
  }
  const char *why = nullptr;
  cudaError_t e = phx::batch_stage(ctx->batch, make_par(*p), blocks, views.data(), nblocks, cons_base, cons_out, beta,
                                   dt, use_learned_guess ? ctx->mlp_packed : nullptr, nullptr, true, phx::BATCH_STAGE,
                                   ctx->stats, ctx->err, S(stream), &why);
  if (e != cudaSuccess) return fail(PHX_ERR_CUDA, "phx_stage_batched: %s", cudaGetErrorString(e));
  return cuda_status("phx_stage_batched");
}

// Validate a tiled mesh against its blocks (3D, ng equal, block extents =
// segment lengths, blocks ordered by segment triple).
static phx_status check_mesh(const phx_mesh *m, const phx_params *p, const phx_block *blocks, int nblocks,
                             std::vector<phx::BView> &views) {
  if (!m || !blocks || nblocks < 1) return fail(PHX_ERR_INVALID_ARG, "mesh/blocks is NULL");
  const int ndim = blocks[0].ndim;
  if (ndim < 1 || ndim > 3) return fail(PHX_ERR_INVALID_ARG, "bad ndim %d", ndim);
  if (m->bc_vars != PHX_BC_VARS_CONSERVED && m->bc_vars != PHX_BC_VARS_PRIMITIVE)
    return fail(PHX_ERR_INVALID_ARG, "\"bc_vars\" must be either \"conserved\" or \"primitive\"!");
  long long nb = 1;
  for (int d = 0; d < 3; d++) {
    if (m->nseg[d] < 1 || m->n[d] < 1 || !m->seg_start[d]) return fail(PHX_ERR_INVALID_ARG, "bad mesh axis %d", d);
    if (m->seg_start[d][0] != 0 || m->seg_start[d][m->nseg[d]] != m->n[d])
      return fail(PHX_ERR_INVALID_ARG, "mesh axis %d: segments must cover [0, n)", d);
    for (int k = 0; k < m->nseg[d]; k++)
      if (m->seg_start[d][k + 1] <= m->seg_start[d][k]) return fail(PHX_ERR_INVALID_ARG, "empty segment");
    if (d >= ndim && (m->n[d] != 1 || m->nseg[d] != 1))
      return fail(PHX_ERR_INVALID_ARG, "mesh axis %d is inactive in %dD: n and nseg must be 1", d, ndim);
    for (int bc : {m->bc_lo[d], m->bc_hi[d]}) {
      if (bc < PHX_BC_PERIODIC || bc > PHX_BC_POLAR) return fail(PHX_ERR_INVALID_ARG, "unknown boundary condition");
      if (bc == PHX_BC_POLAR && d != 1) return fail(PHX_ERR_INVALID_ARG, "polar boundaries are X2 faces only");
      if (bc == PHX_BC_POLAR && m->bc_vars != PHX_BC_VARS_PRIMITIVE)
        return fail(PHX_ERR_INVALID_ARG, "Polar X2 reflecting BCs not supported");  // phoebus_boundaries.cpp:167
    }
    if ((m->bc_lo[d] == PHX_BC_PERIODIC) != (m->bc_hi[d] == PHX_BC_PERIODIC))
      return fail(PHX_ERR_INVALID_ARG, "mesh axis %d: periodic on one face only", d);
    nb *= m->nseg[d];
  }
  if (nb != nblocks) return fail(PHX_ERR_INVALID_ARG, "mesh has %lld blocks, %d given", nb, nblocks);
  views.resize(nblocks);
  phx_status s;
  for (int s3 = 0, b = 0; s3 < m->nseg[2]; s3++)
    for (int s2 = 0; s2 < m->nseg[1]; s2++)
      for (int s1 = 0; s1 < m->nseg[0]; s1++, b++) {
        if ((s = make_view(&blocks[b], views[b]))) return fail(s, "block %d: %s", b, g_last_error.c_str());
        const phx_block &B = blocks[b];
        if (B.ndim != ndim || B.ng != blocks[0].ng)
          return fail(PHX_ERR_INVALID_ARG, "mesh blocks must share ndim and ng");
        if (B.nx1 != m->seg_start[0][s1 + 1] - m->seg_start[0][s1] ||
            B.nx2 != m->seg_start[1][s2 + 1] - m->seg_start[1][s2] ||
            B.nx3 != m->seg_start[2][s3 + 1] - m->seg_start[2][s3])
          return fail(PHX_ERR_INVALID_ARG, "block %d extents differ from its mesh segments", b);
        const int nx[3] = {B.nx1, B.nx2, B.nx3};
        for (int d = 0; d < ndim; d++)  // one neighbour per side; a mirror maps ng ghosts onto ng cells
          if (nx[d] < B.ng) return fail(PHX_ERR_INVALID_ARG, "block %d: ghost exchange needs nx >= ng", b);
        if (views[b].fmks != views[0].fmks) return fail(PHX_ERR_INVALID_ARG, "blocks must share the geometry kind");
      }
  return PHX_OK;
}

phx_status phx_stage_mesh(phx_ctx *ctx, const phx_params *p, const phx_mesh *mesh, const phx_block *blocks,
                          int nblocks, const double *const *cons_base, double *const *cons_out, double beta,
                          double dt, int use_learned_guess, int batched, void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx)) || (s = check_params(p))) return s;
  if (!cons_base || !cons_out) return fail(PHX_ERR_INVALID_ARG, "cons_base/cons_out is NULL");
  if (use_learned_guess && !ctx->mlp_loaded) return fail(PHX_ERR_INVALID_ARG, "no learned-guess weights loaded");
  std::vector<phx::BView> views;
  if ((s = check_mesh(mesh, p, blocks, nblocks, views))) return s;
  for (int n = 0; n < nblocks; n++) {
    const phx_block *b = &blocks[n];
    if (!b->flux || !b->face_sig || !b->cell_sig || !b->fail || !b->src || !cons_base[n] || !cons_out[n])
      return fail(PHX_ERR_INVALID_ARG, "block %d: stage needs flux, face_sig, cell_sig, fail, src, cons_base, "
                                       "cons_out", n);
    if (p->mhd && !b->emf) return fail(PHX_ERR_INVALID_ARG, "block %d: emf is NULL", n);
  }
  const char *why = nullptr;
  cudaError_t e = phx::batch_stage(ctx->batch, make_par(*p), blocks, views.data(), nblocks, cons_base, cons_out, beta,
                                   dt, use_learned_guess ? ctx->mlp_packed : nullptr, mesh, batched != 0, phx::BATCH_STAGE,
                                   ctx->stats, ctx->err, S(stream), &why);
  if (e != cudaSuccess) return fail(PHX_ERR_CUDA, "phx_stage_mesh: %s", cudaGetErrorString(e));
  return cuda_status("phx_stage_mesh");
}

phx_status phx_mesh_exchange(phx_ctx *ctx, const phx_params *p, const phx_mesh *mesh, const phx_block *blocks,
                             int nblocks, void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx)) || (s = check_params(p))) return s;
  std::vector<phx::BView> views;
  if ((s = check_mesh(mesh, p, blocks, nblocks, views))) return s;
  for (int n = 0; n < nblocks; n++)
    if (!blocks[n].cell_sig) return fail(PHX_ERR_INVALID_ARG, "block %d: cell_sig is NULL", n);
  std::vector<const double *> base(nblocks);
  std::vector<double *> out(nblocks);
  for (int n = 0; n < nblocks; n++) {
    base[n] = blocks[n].cons;
    out[n] = blocks[n].cons;
  }
  const char *why = nullptr;
  cudaError_t e = phx::batch_stage(ctx->batch, make_par(*p), blocks, views.data(), nblocks, base.data(), out.data(),
                                   0.0, 0.0, nullptr, mesh, true, phx::BATCH_EXCHANGE, ctx->stats, ctx->err,
                                   S(stream), &why);
  if (e != cudaSuccess) return fail(PHX_ERR_CUDA, "phx_mesh_exchange: %s", cudaGetErrorString(e));
  return cuda_status("phx_mesh_exchange");
}

phx_status phx_fix_fluxes(phx_ctx *ctx, const phx_params *p, const phx_mesh *mesh, const phx_block *blocks,
                          int nblocks, void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx)) || (s = check_params(p))) return s;
  std::vector<phx::BView> views;
  if ((s = check_mesh(mesh, p, blocks, nblocks, views))) return s;
  for (int n = 0; n < nblocks; n++)
    if (!blocks[n].flux) return fail(PHX_ERR_INVALID_ARG, "block %d: flux is NULL", n);
  if (!p->enable_flux_fixup) return PHX_OK;
  std::vector<const double *> base(nblocks);
  std::vector<double *> out(nblocks);
  for (int n = 0; n < nblocks; n++) {
    base[n] = blocks[n].cons;
    out[n] = blocks[n].cons;
  }
  const char *why = nullptr;
  cudaError_t e = phx::batch_stage(ctx->batch, make_par(*p), blocks, views.data(), nblocks, base.data(), out.data(),
                                   0.0, 0.0, nullptr, mesh, true, phx::BATCH_FIXFLUX, ctx->stats, ctx->err,
                                   S(stream), &why);
  if (e != cudaSuccess) return fail(PHX_ERR_CUDA, "phx_fix_fluxes: %s", cudaGetErrorString(e));
  return cuda_status("phx_fix_fluxes");
}

phx_status phx_fix_fluxes_block(phx_ctx *ctx, const phx_params *p, const phx_block *b, const int bc_lo[3],
                                const int bc_hi[3], void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx)) || (s = check_params(p))) return s;
  phx::BView v;
  if ((s = make_view(b, v))) return s;
  if (!b->flux || !bc_lo || !bc_hi) return fail(PHX_ERR_INVALID_ARG, "flux/bc_lo/bc_hi is NULL");
  for (int d = 0; d < 3; d++)
    for (int bc : {bc_lo[d], bc_hi[d]}) {
      if (bc < PHX_BC_PERIODIC || bc > PHX_BC_POLAR) return fail(PHX_ERR_INVALID_ARG, "unknown boundary condition");
      if (bc == PHX_BC_POLAR && d != 1) return fail(PHX_ERR_INVALID_ARG, "polar boundaries are X2 faces only");
    }
  if (!p->enable_flux_fixup) return PHX_OK;
  phx::launch_fix_fluxes_block(make_par(*p), v, bc_lo, bc_hi, S(stream));
  return cuda_status("phx_fix_fluxes_block");
}

phx_status phx_batch_info(phx_ctx *ctx, int *x1_cells, int *sweep_seg, int *graph_nodes) {
  if (!ctx || !x1_cells || !sweep_seg || !graph_nodes) return fail(PHX_ERR_INVALID_ARG, "NULL argument");
  phx::batch_last_tuning(ctx->batch, x1_cells, sweep_seg, graph_nodes);
  return PHX_OK;
}

phx_status phx_mlp_set_weights(phx_ctx *ctx, const float *params_host) {
  phx_status s;
  if ((s = ctx_device(ctx))) return s;
  if (!params_host) return fail(PHX_ERR_INVALID_ARG, "params is NULL");
  if (cudaMemcpy(ctx->mlp_w, params_host, sizeof(float) * PHX_MLP_NPARAM, cudaMemcpyHostToDevice) != cudaSuccess)
    return cuda_status("mlp weights");
  cudaMemset(ctx->mlp_grad, 0, sizeof(float) * PHX_MLP_NPARAM);
  cudaMemset(ctx->mlp_m, 0, sizeof(float) * PHX_MLP_NPARAM);
  cudaMemset(ctx->mlp_v, 0, sizeof(float) * PHX_MLP_NPARAM);
  ctx->mlp_step = 0;
  phx::launch_mlp_pack(ctx->mlp_w, ctx->mlp_packed, 0);
  phx::launch_mlp_box_reset(ctx->mlp_packed, 0);  // weights from elsewhere: no input box until one is set
  if ((s = cuda_status("mlp pack"))) return s;
  if (cudaDeviceSynchronize() != cudaSuccess) return cuda_status("mlp pack");
  ctx->mlp_loaded = 1;
  return PHX_OK;
}

phx_status phx_mlp_set_input_box(phx_ctx *ctx, const float *lo_host, const float *hi_host) {
  phx_status s;
  if ((s = ctx_device(ctx))) return s;
  float lo[8], hi[8];
  for (int c = 0; c < 8; c++) {
    lo[c] = (lo_host && c < PHX_MLP_IN) ? lo_host[c] : -INFINITY;
    hi[c] = (hi_host && c < PHX_MLP_IN) ? hi_host[c] : INFINITY;
    if (!(lo[c] <= hi[c])) return fail(PHX_ERR_INVALID_ARG, "input box: lo > hi (or NaN) in feature %d", c);
  }
  char *base = reinterpret_cast<char *>(ctx->mlp_packed);
  if (cudaMemcpy(base + offsetof(phx::MlpPacked, xlo), lo, sizeof(lo), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(base + offsetof(phx::MlpPacked, xhi), hi, sizeof(hi), cudaMemcpyHostToDevice) != cudaSuccess)
    return cuda_status("phx_mlp_set_input_box");
  return PHX_OK;
}

phx_status phx_mlp_get_input_box(phx_ctx *ctx, float *lo_host, float *hi_host) {
  phx_status s;
  if ((s = ctx_device(ctx))) return s;
  if (!lo_host || !hi_host) return fail(PHX_ERR_INVALID_ARG, "lo/hi is NULL");
  float lo[8], hi[8];
  const char *base = reinterpret_cast<const char *>(ctx->mlp_packed);
  if (cudaMemcpy(lo, base + offsetof(phx::MlpPacked, xlo), sizeof(lo), cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(hi, base + offsetof(phx::MlpPacked, xhi), sizeof(hi), cudaMemcpyDeviceToHost) != cudaSuccess)
    return cuda_status("phx_mlp_get_input_box");
  for (int c = 0; c < PHX_MLP_IN; c++) {
    lo_host[c] = lo[c];
    hi_host[c] = hi[c];
  }
  return PHX_OK;
}

void phx_mlp_train_opts_default(phx_mlp_train_opts *o) {
  o->batch = 4096;
  o->epochs = 10;
  o->lr = 3e-3f;
  o->lr_min = 0.0f;
  o->beta1 = 0.9f;
  o->beta2 = 0.999f;
  o->eps = 1e-8f;
  o->weight_decay = 1e-4f;
}

phx_status phx_mlp_features_zones(phx_ctx *ctx, const phx_params *p, long long n, const double *cons,
                                  const double *geom, const double *coords, float *x, void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx)) || (s = check_params(p))) return s;
  if (n < 0) return fail(PHX_ERR_INVALID_ARG, "n < 0");
  if (n == 0) return PHX_OK;
  if (!cons || !x) return fail(PHX_ERR_INVALID_ARG, "cons/x is NULL");
  phx::launch_mlp_features(make_par(*p), n, cons, geom, coords, x, S(stream));
  return cuda_status("phx_mlp_features_zones");
}

phx_status phx_mlp_forward(phx_ctx *ctx, long long n, const float *x, float *out, void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx))) return s;
  if (n < 0) return fail(PHX_ERR_INVALID_ARG, "n < 0");
  if (n == 0) return PHX_OK;
  if (!x || !out) return fail(PHX_ERR_INVALID_ARG, "x/out is NULL");
  if (!ctx->mlp_loaded) return fail(PHX_ERR_INVALID_ARG, "no learned-guess weights loaded");
  phx::launch_mlp_forward(ctx->mlp_packed, n, x, out, ctx->err, S(stream));
  return cuda_status("phx_mlp_forward");
}

phx_status phx_mlp_bracket_zones(phx_ctx *ctx, const phx_params *p, long long n, const double *cons,
                                 const double *geom, const double *coords, double *bracket, void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx)) || (s = check_params(p))) return s;
  if (n < 0) return fail(PHX_ERR_INVALID_ARG, "n < 0");
  if (n == 0) return PHX_OK;
  if (!cons || !bracket) return fail(PHX_ERR_INVALID_ARG, "cons/bracket is NULL");
  if (!ctx->mlp_loaded) return fail(PHX_ERR_INVALID_ARG, "no learned-guess weights loaded");
  phx::launch_mlp_bracket(make_par(*p), n, cons, geom, coords, ctx->mlp_packed, bracket, ctx->err, S(stream));
  return cuda_status("phx_mlp_bracket_zones");
}

phx_status phx_mlp_loss_grad(phx_ctx *ctx, long long n, const float *x, const float *y, float *grad, float *loss,
                             void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx))) return s;
  if (n <= 0) return fail(PHX_ERR_INVALID_ARG, "n must be positive");
  if (!x || !y || !grad || !loss) return fail(PHX_ERR_INVALID_ARG, "x/y/grad/loss is NULL");
  cudaStream_t st = S(stream);
  cudaMemsetAsync(grad, 0, sizeof(float) * PHX_MLP_NPARAM, st);
  cudaMemsetAsync(loss, 0, sizeof(float), st);
  phx::launch_mlp_grad(ctx->mlp_w, x, y, n, 0, n, (float)(1.0 / (double)n), grad, loss, st);
  return cuda_status("phx_mlp_loss_grad");
}

phx_status phx_mlp_train(phx_ctx *ctx, long long n, const float *x, const float *y, const phx_mlp_train_opts *o,
                         float *epoch_loss, void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx))) return s;
  if (!x || !y || !o) return fail(PHX_ERR_INVALID_ARG, "x/y/opts is NULL");
  if (o->batch <= 0 || o->epochs <= 0) return fail(PHX_ERR_INVALID_ARG, "batch and epochs must be positive");
  if (o->epochs > PHX_MLP_MAX_EPOCHS) return fail(PHX_ERR_CAPACITY, "epochs > PHX_MLP_MAX_EPOCHS");
  const long long steps = n / o->batch;
  if (steps <= 0) return fail(PHX_ERR_INVALID_ARG, "n smaller than one batch");
  cudaStream_t st = S(stream);
  cudaMemsetAsync(ctx->mlp_loss, 0, sizeof(float) * o->epochs, st);
  const long long total = steps * o->epochs;
  const float inv_b = (float)(1.0 / (double)o->batch);
  long long t = 0;
  for (int e = 0; e < o->epochs; e++)
    for (long long k = 0; k < steps; k++, t++) {
      phx::launch_mlp_grad(ctx->mlp_w, x, y, n, k * o->batch, o->batch, inv_b, ctx->mlp_grad, ctx->mlp_loss + e, st);
      const long long step = ++ctx->mlp_step;
      const double lr = o->lr_min + 0.5 * (o->lr - o->lr_min) * (1.0 + cos(M_PI * (double)t / (double)total));
      const double c1 = 1.0 / (1.0 - pow((double)o->beta1, (double)step));
      const double c2 = 1.0 / (1.0 - pow((double)o->beta2, (double)step));
      phx::launch_mlp_adamw(ctx->mlp_w, ctx->mlp_grad, ctx->mlp_m, ctx->mlp_v, (float)lr, o->beta1, o->beta2, o->eps,
                            o->weight_decay, (float)c1, (float)c2, st);
    }
  phx::launch_mlp_pack(ctx->mlp_w, ctx->mlp_packed, st);
  // the learned start only serves zones inside the training set's feature
  // range, widened by 2% of the range on each side
  phx::launch_mlp_box_from(x, n, 0.02f, ctx->mlp_boxkeys, ctx->mlp_packed, st);
  if ((s = cuda_status("phx_mlp_train"))) return s;
  if (cudaStreamSynchronize(st) != cudaSuccess) return cuda_status("phx_mlp_train");
  if (epoch_loss) {
    if (cudaMemcpy(epoch_loss, ctx->mlp_loss, sizeof(float) * o->epochs, cudaMemcpyDeviceToHost) != cudaSuccess)
      return cuda_status("phx_mlp_train");
    for (int e = 0; e < o->epochs; e++) epoch_loss[e] /= (float)steps;
  }
  ctx->mlp_loaded = 1;
  return PHX_OK;
}

phx_status phx_mlp_get_weights(phx_ctx *ctx, float *params_host) {
  phx_status s;
  if ((s = ctx_device(ctx))) return s;
  if (!params_host) return fail(PHX_ERR_INVALID_ARG, "params is NULL");
  if (cudaMemcpy(params_host, ctx->mlp_w, sizeof(float) * PHX_MLP_NPARAM, cudaMemcpyDeviceToHost) != cudaSuccess)
    return cuda_status("mlp weights");
  return PHX_OK;
}

void phx_torus_params_default(phx_torus_params *tp) {
  if (!tp) return;
  tp->rin = 6.0;
  tp->rmax = 12.0;
  tp->kappa = 1.e-2;
  tp->u_jitter = 1.e-2;
  tp->target_beta = 100.;
  tp->magnetized = 1;
  tp->seed = 0;
}

phx_status phx_torus_init(phx_ctx *ctx, const phx_params *p, const phx_torus_params *tp, const phx_block *blocks,
                          int nblocks, double *field_factor, void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx)) || (s = check_params(p))) return s;
  if (!tp || !blocks || nblocks <= 0) return fail(PHX_ERR_INVALID_ARG, "phx_torus_init: params and blocks required");
  if (!(tp->rmax > tp->rin) || !(tp->kappa > 0) || !(tp->target_beta > 0))
    return fail(PHX_ERR_INVALID_ARG, "phx_torus_init: need rmax > rin, kappa > 0, target_beta > 0");
  std::vector<phx::BView> v(nblocks);
  const phx_geometry *g0 = blocks[0].geom;
  for (int q = 0; q < nblocks; q++) {
    if ((s = make_view(&blocks[q], v[q]))) return s;
    const phx_geometry *g = blocks[q].geom;
    if (!v[q].fmks || !g) return fail(PHX_ERR_INVALID_ARG, "phx_torus_init: block %d has no FMKS tables", q);
    if (g->a != g0->a || g->hslope != g0->hslope || g->poly_xt != g0->poly_xt || g->poly_alpha != g0->poly_alpha ||
        g->x0 != g0->x0 || g->smooth != g0->smooth || g->hexp_br != g0->hexp_br || g->hexp_nsq != g0->hexp_nsq ||
        g->hexp_csq != g0->hexp_csq || g->derefine_poles != g0->derefine_poles)
      return fail(PHX_ERR_INVALID_ARG, "phx_torus_init: blocks must share one geometry");
    if ((long long)phx::TORUS_PLANE_VARS * v[q].n1t * v[q].n2t > 3 * phx::C2P_CHUNK)
      return fail(PHX_ERR_CAPACITY, "phx_torus_init: block %d's (j, i) plane is too large for the scratch", q);
    if (!blocks[q].fail) return fail(PHX_ERR_INVALID_ARG, "phx_torus_init: fail field required (ApplyFloors)");
  }
  double fac = 0.0;
  cudaError_t e = phx::torus_init(make_par(*p), *g0, *tp, v.data(), nblocks, ctx->c2p.brk, ctx->red, ctx->stats,
                                  ctx->err, &fac, S(stream));
  if (e != cudaSuccess) return fail(PHX_ERR_CUDA, "phx_torus_init: %s", cudaGetErrorString(e));
  if (field_factor) *field_factor = fac;
  return PHX_OK;
}

phx_status phx_math_eval(int fn, long long n, const double *x, const double *y, double *out, void *stream) {
  if (fn < PHX_MATH_EXP || fn > PHX_MATH_RSQRT)
    return fail(PHX_ERR_INVALID_ARG, "phx_math_eval: unknown function %d", fn);
  if (n < 0) return fail(PHX_ERR_INVALID_ARG, "n < 0");
  if (n == 0) return PHX_OK;
  if (!x || !out || (fn == PHX_MATH_POW && !y)) return fail(PHX_ERR_INVALID_ARG, "x/y/out is NULL");
  phx::launch_math_eval(fn, n, x, y, out, S(stream));
  return cuda_status("phx_math_eval");
}

phx_status phx_probe_bounded_wait(phx_ctx *ctx, long long polls, void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx))) return s;
  if (polls < 1 || polls > phx::MBAR_SPIN_LIMIT)
    return fail(PHX_ERR_INVALID_ARG, "phx_probe_bounded_wait: polls must be in [1, 2^20]");
  phx::launch_wait_probe(polls, ctx->err, S(stream));
  return cuda_status("phx_probe_bounded_wait");
}

phx_status phx_probe_fp64_peak(phx_ctx *ctx, double *flops_out) {
  phx_status s;
  if ((s = ctx_device(ctx))) return s;
  if (!flops_out) return fail(PHX_ERR_INVALID_ARG, "flops_out is NULL");
  double *d = nullptr;
  // the probe's output word lives in the dt scratch (never read back)
  d = reinterpret_cast<double *>(ctx->dt_scr);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int nthreads = 0;
  const int iters = 4096;
  phx::launch_fp64_probe(d, 64, 0, &nthreads);  // warm-up
  cudaEventRecord(e0, 0);
  phx::launch_fp64_probe(d, iters, 0, &nthreads);
  cudaEventRecord(e1, 0);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *flops_out = 2.0 * 8.0 * (double)iters * nthreads / (ms * 1e-3);
  return cuda_status("phx_probe_fp64_peak");
}

}  // extern "C"

// ---------------------------------------------------------------------
// Radiation moments (phx_radiation.h)
// ---------------------------------------------------------------------
namespace {

phx_status check_rad(const phx_rad_params *rp, const phx_params *p, const phx_block *fb) {
  if (!rp) return fail(PHX_ERR_INVALID_ARG, "radiation params is NULL");
  if (rp->method != PHX_RAD_M1 && rp->method != PHX_RAD_EDDINGTON)
    return fail(PHX_ERR_INVALID_ARG, "invalid radiation method %d (choose moment_m1 or moment_eddington)",
                rp->method);
  if (rp->recon < PHX_RECON_CONSTANT || rp->recon > PHX_RECON_MP5)
    return fail(PHX_ERR_INVALID_ARG, "Invalid Reconstruction option.  Choose from [constant,linear,mp5,weno5,weno5z]");
  if (rp->oned_fixup_strategy < PHX_RAD_ONED_FIXUP_NONE || rp->oned_fixup_strategy > PHX_RAD_ONED_FIXUP_IGNORE_ALL)
    return fail(PHX_ERR_INVALID_ARG, "radiation/oned_fixup_strategy has an invalid entry!");
  if (rp->src_rootfind_maxiter < 0) return fail(PHX_ERR_INVALID_ARG, "src_rootfind_maxiter < 0");
  if (rp->src_solver != PHX_RAD_SRC_ONED && rp->src_solver != PHX_RAD_SRC_FOURD)
    return fail(PHX_ERR_INVALID_ARG, "\"radiation/src_solver\" option unrecognized!");
  if (rp->enable_rad_floors && rp->rad_floor_type != PHX_RAD_FLOOR_CONSTANT_J &&
      rp->rad_floor_type != PHX_RAD_FLOOR_EXPX1_J)
    return fail(PHX_ERR_INVALID_ARG, "invalid <fixup>/rad_floor_type input");
  if (p == nullptr) return fail(PHX_ERR_INVALID_ARG, "params is NULL");
  return PHX_OK;
}

phx::rad::RPar make_rpar(const phx_rad_params &rp, const phx_params &p) {
  phx::rad::RPar r;
  std::memset(&r, 0, sizeof(r));
  r.m1 = rp.method == PHX_RAD_M1;
  r.robust = !rp.closure_frail;
  r.bounds = rp.recon_fixup_bounds != 0;
  r.recon = rp.recon;
  r.maxiter = rp.src_rootfind_maxiter;
  r.oned_fixup = rp.oned_fixup_strategy;
  r.update_fluid = rp.update_fluid != 0;
  r.rad_fixup_floors = rp.rad_c2p_failure_floors != 0;
  r.fourd = rp.src_solver == PHX_RAD_SRC_FOURD;
  r.oned_backup = rp.src_use_oned_backup != 0;
  r.fd_eps = rp.src_rootfind_eps;
  r.cfl = rp.cfl;
  r.tol = rp.src_rootfind_tol;
  r.kappa_a = rp.kappa_a;
  r.kappa_s = rp.kappa_s;
  r.jbb = rp.jbb_coeff;
  // RadiationFloors() / RadiationCeilings() / Ceilings() defaults when
  // disabled (fixup.hpp:157-273)
  r.J_floor = rp.enable_rad_floors ? rp.J0_floor : -phx::kDBLMAX;
  r.floor_expx1 = rp.enable_rad_floors && rp.rad_floor_type == PHX_RAD_FLOOR_EXPX1_J;
  r.J_alpha = rp.J_exp_floor;
  r.xi_ceiling = rp.enable_rad_ceilings ? rp.xi0_ceiling : phx::kDBLMAX;
  r.tau_max = rp.enable_rad_ceilings ? rp.tau0_ceiling : phx::kDBLMAX;
  r.W_ceiling = p.enable_ceilings ? p.gam0_ceiling : phx::kDBLMAX;
  r.Cv = p.Cv;
  return r;
}

phx_status make_rview(const phx::BView &v, const phx_rad_block *rb, bool need_flux, phx::rad::RView &r) {
  if (!rb) return fail(PHX_ERR_INVALID_ARG, "radiation block is NULL");
  if (!rb->cons || !rb->prim) return fail(PHX_ERR_INVALID_ARG, "radiation cons/prim pointers are NULL");
  if (need_flux && (!rb->flux || !rb->dudt)) return fail(PHX_ERR_INVALID_ARG, "radiation flux/dudt is NULL");
  const long long N = (long long)v.n1t * v.n2t * v.n3t;
  r.vs = rb->var_stride ? rb->var_stride : N;
  if (r.vs < N) return fail(PHX_ERR_INVALID_ARG, "radiation var_stride smaller than the block");
  r.cons = rb->cons;
  r.prim = rb->prim;
  r.flux = rb->flux;
  r.dudt = rb->dudt;
  return PHX_OK;
}

// fluid block view + radiation view + parameters, validated
// The fluid inversion MomentFluidSourceImpl sets up for update_fluid
// (moments_source.cpp:286-295): the fluid's tolerance, iteration cap and
// floor scale, failing on floors and on ceilings.
phx::Par source_inversion_par(const phx_params &p) {
  phx::Par fp = make_par(p);
  fp.fail_on_floors = 1;
  fp.fail_on_ceilings = 1;
  return fp;
}

// fixup::ApplyFloors with radiation active (fixup.cpp:285-678): the fluid
// part over the range, recording where floors or ceilings acted in the
// radiation scratch dudt, then, with fixup/enable_rad_floors, the radiation
// part (the reference loops over no species otherwise).
void rad_apply_floors(phx_ctx *ctx, const phx::Par &fpar, const phx::rad::RPar &par, const phx_rad_params &rp,
                      const phx::BView &v, const phx::rad::RView &r, phx::Range3 rg, cudaStream_t st) {
  double *flag = rp.enable_rad_floors ? r.dudt : nullptr;
  phx::launch_floors(fpar, v, rg, ctx->stats, ctx->err, st, flag);
  if (rp.enable_rad_floors && fpar.enable_floors) phx::rad::launch_rad_floors(par, v, r, flag, rg, st);
}

phx_status check_rad_fixups(const phx_rad_params *rp, const phx_params *p, const phx_rad_block *rb) {
  if (rp->enable_rad_floors && !p->enable_floors)
    return fail(PHX_ERR_INVALID_ARG, "enable_rad_floors needs fixup/enable_floors (the fixup package forces it on)");
  if (rp->enable_rad_floors && !rb->dudt)
    return fail(PHX_ERR_INVALID_ARG, "the radiation floors use the radiation block's dudt as scratch: it is NULL");
  return PHX_OK;
}

phx_status rad_setup(phx_ctx *ctx, const phx_rad_params *rp, const phx_params *p, const phx_block *fb,
                     const phx_rad_block *rb, bool need_flux, phx::BView &v, phx::rad::RView &r,
                     phx::rad::RPar &par) {
  phx_status s;
  if ((s = ctx_device(ctx)) || (s = check_rad(rp, p, fb))) return s;
  if ((s = make_view(fb, v))) return s;
  if ((s = make_rview(v, rb, need_flux, r))) return s;
  par = make_rpar(*rp, *p);
  return PHX_OK;
}

}  // namespace

extern "C" {

void phx_rad_params_default(phx_rad_params *p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->method = PHX_RAD_M1;
  p->recon = PHX_RECON_LINEAR;  // radiation/recon default "linear" (radiation.cpp:368)
  p->cfl = 0.8;                 // radiation/cfl (radiation.cpp:77)
  p->closure_frail = 0;         // closure_c2p_strategy "robust"
  p->recon_fixup_bounds = 1;    // recon_fixup_strategy "bounds"
  p->src_rootfind_tol = 1.e-12;
  p->src_rootfind_maxiter = 100;
  p->oned_fixup_strategy = PHX_RAD_ONED_FIXUP_NONE;
  p->xi0_ceiling = 0.99;
  p->tau0_ceiling = 1.e3;
  p->src_solver = PHX_RAD_SRC_ONED;  // radiation/src_solver "oned" (radiation.cpp:403-404)
  p->src_rootfind_eps = 1.e-8;       // radiation/src_rootfind_eps (radiation.cpp:421)
  p->src_use_oned_backup = 0;        // radiation/src_use_oned_backup (radiation.cpp:417-418)
  p->rad_floor_type = PHX_RAD_FLOOR_CONSTANT_J;
  p->J_exp_floor = -2.0;             // fixup/J_exp_floor (fixup.cpp:194-195)
}

phx_status phx_rad_prim_to_con(phx_ctx *ctx, const phx_rad_params *rp, const phx_params *p, const phx_block *fb,
                               const phx_rad_block *rb, phx_range ib, phx_range jb, phx_range kb, void *stream) {
  phx::BView v;
  phx::rad::RView r;
  phx::rad::RPar par;
  phx::Range3 rg;
  phx_status s;
  if ((s = rad_setup(ctx, rp, p, fb, rb, false, v, r, par)) || (s = check_range(v, ib, jb, kb, rg))) return s;
  phx::rad::launch_p2c(par, v, r, rg, S(stream));
  return cuda_status("phx_rad_prim_to_con");
}

phx_status phx_rad_con_to_prim(phx_ctx *ctx, const phx_rad_params *rp, const phx_params *p, const phx_block *fb,
                               const phx_rad_block *rb, phx_range ib, phx_range jb, phx_range kb, void *stream) {
  phx::BView v;
  phx::rad::RView r;
  phx::rad::RPar par;
  phx::Range3 rg;
  phx_status s;
  if ((s = rad_setup(ctx, rp, p, fb, rb, false, v, r, par)) || (s = check_range(v, ib, jb, kb, rg))) return s;
  phx::rad::launch_c2p(par, v, r, rg, S(stream));
  return cuda_status("phx_rad_con_to_prim");
}

phx_status phx_rad_calculate_opacities(phx_ctx *ctx, const phx_rad_params *rp, const phx_params *p,
                                       const phx_block *fb, const phx_rad_block *rb, void *stream) {
  phx::BView v;
  phx::rad::RView r;
  phx::rad::RPar par;
  phx_status s;
  if ((s = rad_setup(ctx, rp, p, fb, rb, false, v, r, par))) return s;
  phx::rad::launch_opacities(par, v, r, S(stream));
  return cuda_status("phx_rad_calculate_opacities");
}

phx_status phx_rad_calculate_fluxes(phx_ctx *ctx, const phx_rad_params *rp, const phx_params *p,
                                    const phx_block *fb, const phx_rad_block *rb, void *stream) {
  phx::BView v;
  phx::rad::RView r;
  phx::rad::RPar par;
  phx_status s;
  if ((s = rad_setup(ctx, rp, p, fb, rb, true, v, r, par))) return s;
  if (v.ng < 3) return fail(PHX_ERR_INVALID_ARG, "radiation fluxes need ng >= 3");
  phx::rad::launch_fluxes(par, v, r, S(stream));
  return cuda_status("phx_rad_calculate_fluxes");
}

phx_status phx_rad_update(phx_ctx *ctx, const phx_rad_params *rp, const phx_block *fb, const phx_rad_block *rb,
                          const double *base, double *out, double beta, double dt, void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx))) return s;
  if (!rp) return fail(PHX_ERR_INVALID_ARG, "radiation params is NULL");
  phx::BView v;
  phx::rad::RView r;
  if ((s = make_view(fb, v)) || (s = make_rview(v, rb, true, r))) return s;
  if (!base || !out) return fail(PHX_ERR_INVALID_ARG, "base/out is NULL");
  phx::rad::RPar par;
  std::memset(&par, 0, sizeof(par));
  par.m1 = rp->method == PHX_RAD_M1;  // the geometric source's closure (FMKS blocks)
  phx::rad::launch_update(par, v, r, base, out, beta, dt, S(stream));
  return cuda_status("phx_rad_update");
}

phx_status phx_rad_fluid_source(phx_ctx *ctx, const phx_rad_params *rp, const phx_params *p, const phx_block *fb,
                                const phx_rad_block *rb, double dt, void *stream) {
  phx::BView v;
  phx::rad::RView r;
  phx::rad::RPar par;
  phx_status s;
  if ((s = rad_setup(ctx, rp, p, fb, rb, false, v, r, par))) return s;
  if (par.update_fluid) {
    if ((s = check_params(p))) return s;
    if (!fb->cell_sig) return fail(PHX_ERR_INVALID_ARG, "update_fluid needs the fluid block's cell_sig");
  }
  phx::rad::launch_source(par, source_inversion_par(*p), v, r, dt, S(stream));
  return cuda_status("phx_rad_fluid_source");
}

phx_status phx_rad_fill_ghosts_periodic(phx_ctx *ctx, const phx_block *fb, const phx_rad_block *rb, void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx))) return s;
  phx::BView v;
  phx::rad::RView r;
  if ((s = make_view(fb, v)) || (s = make_rview(v, rb, false, r))) return s;
  phx::rad::launch_ghosts(v, r, S(stream));
  return cuda_status("phx_rad_fill_ghosts_periodic");
}

phx_status phx_rad_mesh_exchange(phx_ctx *ctx, const phx_rad_params *rp, const phx_params *p, const phx_mesh *mesh,
                                 const phx_block *blocks, const phx_rad_block *rblocks, int nblocks, void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx)) || (s = check_params(p))) return s;
  std::vector<phx::BView> views;
  if ((s = check_mesh(mesh, p, blocks, nblocks, views))) return s;
  if (!rblocks) return fail(PHX_ERR_INVALID_ARG, "radiation blocks is NULL");
  std::vector<phx::rad::RView> rviews(nblocks);
  for (int n = 0; n < nblocks; n++) {
    if ((s = check_rad(rp, p, &blocks[n]))) return s;
    if ((s = make_rview(views[n], &rblocks[n], false, rviews[n]))) return fail(s, "block %d: %s", n, g_last_error.c_str());
  }
  const phx::rad::RPar par = make_rpar(*rp, *p);
  // One stream-ordered table: per-axis cell -> segment, block -> origin, the
  // block and radiation views (blocks are ordered by segment triple, so the
  // owner of segment triple s is block s).
  std::vector<int> ints;
  size_t off_seg[3];
  for (int d = 0; d < 3; d++) {
    off_seg[d] = ints.size();
    for (int g = 0; g < mesh->nseg[d]; g++)
      for (int c = mesh->seg_start[d][g]; c < mesh->seg_start[d][g + 1]; c++) ints.push_back(g);
  }
  const size_t off_owner = ints.size();
  for (int b = 0; b < nblocks; b++) ints.push_back(b);
  const size_t off_origin = ints.size();
  for (int s3 = 0; s3 < mesh->nseg[2]; s3++)
    for (int s2 = 0; s2 < mesh->nseg[1]; s2++)
      for (int s1 = 0; s1 < mesh->nseg[0]; s1++) {
        ints.push_back(mesh->seg_start[0][s1]);
        ints.push_back(mesh->seg_start[1][s2]);
        ints.push_back(mesh->seg_start[2][s3]);
      }
  auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t b_views = up(sizeof(phx::BView) * nblocks), b_rviews = up(sizeof(phx::rad::RView) * nblocks);
  const size_t bytes = b_views + b_rviews + sizeof(int) * ints.size();
  std::vector<unsigned char> host(bytes);
  memcpy(host.data(), views.data(), sizeof(phx::BView) * nblocks);
  memcpy(host.data() + b_views, rviews.data(), sizeof(phx::rad::RView) * nblocks);
  memcpy(host.data() + b_views + b_rviews, ints.data(), sizeof(int) * ints.size());
  cudaStream_t st = S(stream);
  unsigned char *dev = nullptr;
  cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&dev), bytes, st);
  if (e != cudaSuccess) return fail(PHX_ERR_CUDA, "phx_rad_mesh_exchange: %s", cudaGetErrorString(e));
  // pageable source: the call returns once the table is staged
  e = cudaMemcpyAsync(dev, host.data(), bytes, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    const phx::BView *dviews = reinterpret_cast<const phx::BView *>(dev);
    const phx::rad::RView *drviews = reinterpret_cast<const phx::rad::RView *>(dev + b_views);
    const int *base = reinterpret_cast<const int *>(dev + b_views + b_rviews);
    phx::MeshDev md{};
    md.bc_vars = mesh->bc_vars;
    for (int d = 0; d < 3; d++) {
      md.n[d] = mesh->n[d];
      md.nseg[d] = mesh->nseg[d];
      md.bc_lo[d] = mesh->bc_lo[d];
      md.bc_hi[d] = mesh->bc_hi[d];
      md.seg_of[d] = base + off_seg[d];
    }
    md.owner = base + off_owner;
    md.origin = base + off_origin;
    const int inflow = p->enable_ox1_fmks_inflow_check ? 1 : 0;
    for (int n = 0; n < nblocks; n++)
      phx::rad::launch_mesh_ghosts(par, !views[n].fmks, views[n], dviews, drviews, md, n, inflow, st);
  }
  const cudaError_t e2 = cudaFreeAsync(dev, st);
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess) return fail(PHX_ERR_CUDA, "phx_rad_mesh_exchange: %s", cudaGetErrorString(e));
  return cuda_status("phx_rad_mesh_exchange");
}

phx_status phx_rad_fix_fluxes(phx_ctx *ctx, const phx_rad_params *rp, const phx_params *p, const phx_mesh *mesh,
                              const phx_block *blocks, const phx_rad_block *rblocks, int nblocks, void *stream) {
  phx_status s;
  if ((s = ctx_device(ctx)) || (s = check_params(p))) return s;
  std::vector<phx::BView> views;
  if ((s = check_mesh(mesh, p, blocks, nblocks, views))) return s;
  if (!rblocks) return fail(PHX_ERR_INVALID_ARG, "radiation blocks is NULL");
  std::vector<phx::rad::RView> rviews(nblocks);
  for (int n = 0; n < nblocks; n++) {
    if ((s = check_rad(rp, p, &blocks[n]))) return s;
    if ((s = make_rview(views[n], &rblocks[n], false, rviews[n]))) return fail(s, "block %d: %s", n, g_last_error.c_str());
    if (!rblocks[n].flux) return fail(PHX_ERR_INVALID_ARG, "block %d: radiation flux is NULL", n);
  }
  if (!p->enable_flux_fixup) return PHX_OK;
  cudaStream_t st = S(stream);
  for (int s3 = 0, b = 0; s3 < mesh->nseg[2]; s3++)
    for (int s2 = 0; s2 < mesh->nseg[1]; s2++)
      for (int s1 = 0; s1 < mesh->nseg[0]; s1++, b++) {
        const int seg[3] = {s1, s2, s3};
        const phx::BView &v = views[b];
        const int nx[3] = {v.nx1, v.nx2, v.nx3};
        for (int d = 0; d < v.ndim; d++)
          for (int outer = 0; outer < 2; outer++) {
            const bool edge = outer ? seg[d] == mesh->nseg[d] - 1 : seg[d] == 0;
            const int bc = outer ? mesh->bc_hi[d] : mesh->bc_lo[d];
            if (!edge || bc == PHX_BC_PERIODIC) continue;
            // reflect: E (X2 faces also F_1, F_3); polar: E, F_1, F_3; gr_outflow: none
            unsigned mask = 0;
            if (bc == PHX_BC_REFLECT) mask = 1u << PHX_RE | (d == 1 ? (1u << PHX_RF | 1u << (PHX_RF + 2)) : 0u);
            if (bc == PHX_BC_POLAR) mask = 1u << PHX_RE | 1u << PHX_RF | 1u << (PHX_RF + 2);
            if (mask) phx::rad::launch_fix_face(v, rviews[b], d, outer ? v.ng + nx[d] : v.ng, mask, st);
          }
      }
  return cuda_status("phx_rad_fix_fluxes");
}

phx_status phx_rad_estimate_timestep(phx_ctx *ctx, const phx_rad_params *rp, const phx_params *p,
                                     const phx_block *fb, const phx_rad_block *rb, double *dt_out_device,
                                     void *stream) {
  phx::BView v;
  phx::rad::RView r;
  phx::rad::RPar par;
  phx_status s;
  if ((s = rad_setup(ctx, rp, p, fb, rb, false, v, r, par))) return s;
  if (!dt_out_device) return fail(PHX_ERR_INVALID_ARG, "dt_out is NULL");
  phx::rad::launch_dt(par, v, r, ctx->dt_scr, dt_out_device, S(stream));
  return cuda_status("phx_rad_estimate_timestep");
}

phx_status phx_rad_stage(phx_ctx *ctx, const phx_rad_params *rp, const phx_params *p, const phx_block *fb,
                         const phx_rad_block *rb, const double *base, double *out, double beta, double dt,
                         void *stream) {
  phx::BView v;
  phx::rad::RView r;
  phx::rad::RPar par;
  phx_status s;
  if ((s = rad_setup(ctx, rp, p, fb, rb, true, v, r, par))) return s;
  if (!base || !out) return fail(PHX_ERR_INVALID_ARG, "base/out is NULL");
  if (v.ng < 3) return fail(PHX_ERR_INVALID_ARG, "radiation fluxes need ng >= 3");
  if ((s = check_rad_fixups(rp, p, rb))) return s;
  if (par.update_fluid)
    return fail(PHX_ERR_INVALID_ARG, "update_fluid = 1 evolves the fluid too: use phx_rad_fluid_stage");
  const phx::Par fpar = make_par(*p);
  cudaStream_t st = S(stream);
  phx::rad::launch_opacities(par, v, r, st);
  phx::rad::launch_fluxes(par, v, r, st);
  phx::rad::launch_update(par, v, r, base, out, beta, dt, st);
  phx::rad::RView ro = r;
  ro.cons = out;
  // hydro off: the fluid's con2prim and its c2p fixup do not run.  Before
  // the exchange only the c2p fixup reads the ghosts' inversion (the
  // exchange overwrites every radiation field there), so without the fixup
  // the first inversion covers the interior alone.
  auto derived = [&](bool first) {
    phx::rad::launch_c2p(par, v, ro, first && !p->enable_c2p_fixup ? interior(v) : entire(v), st);  // FillDerived
    if (p->enable_c2p_fixup) phx::rad::launch_rad_c2p_fixup(par, v, ro, st);  // RadConservedToPrimitiveFixup
    rad_apply_floors(ctx, fpar, par, *rp, v, ro, entire(v), st);               // ApplyFloors
  };
  derived(true);
  phx::rad::launch_source(par, source_inversion_par(*p), v, ro, beta * dt, st);
  rad_apply_floors(ctx, fpar, par, *rp, v, ro, entire(v), st);
  phx::rad::launch_ghosts(v, ro, st);
  derived(false);
  return cuda_status("phx_rad_stage");
}

phx_status phx_rad_c2p_fixup(phx_ctx *ctx, const phx_rad_params *rp, const phx_params *p, const phx_block *fb,
                             const phx_rad_block *rb, void *stream) {
  phx::BView v;
  phx::rad::RView r;
  phx::rad::RPar par;
  phx_status s;
  if ((s = rad_setup(ctx, rp, p, fb, rb, false, v, r, par))) return s;
  if (p->enable_c2p_fixup) phx::rad::launch_rad_c2p_fixup(par, v, r, S(stream));
  return cuda_status("phx_rad_c2p_fixup");
}

phx_status phx_rad_apply_floors(phx_ctx *ctx, const phx_rad_params *rp, const phx_params *p, const phx_block *fb,
                                const phx_rad_block *rb, phx_range ib, phx_range jb, phx_range kb, void *stream) {
  phx::BView v;
  phx::rad::RView r;
  phx::rad::RPar par;
  phx::Range3 rg;
  phx_status s;
  if ((s = rad_setup(ctx, rp, p, fb, rb, false, v, r, par)) || (s = check_range(v, ib, jb, kb, rg)) ||
      (s = check_params(p)) || (s = check_rad_fixups(rp, p, rb)))
    return s;
  r.dudt = rb->dudt;
  rad_apply_floors(ctx, make_par(*p), par, *rp, v, r, rg, S(stream));
  return cuda_status("phx_rad_apply_floors");
}

phx_status phx_rad_fluid_stage(phx_ctx *ctx, const phx_rad_params *rp, const phx_params *p, const phx_block *fb,
                               const phx_rad_block *rb, const double *fluid_base, double *fluid_out,
                               const double *rad_base, double *rad_out, double beta, double dt, void *stream) {
  phx::BView v;
  phx::rad::RView r;
  phx::rad::RPar par;
  phx_status s;
  if ((s = rad_setup(ctx, rp, p, fb, rb, true, v, r, par)) || (s = check_params(p))) return s;
  if (!fluid_base || !fluid_out || !rad_base || !rad_out)
    return fail(PHX_ERR_INVALID_ARG, "fluid_base/fluid_out/rad_base/rad_out is NULL");
  if (!fb->flux || !fb->face_sig || !fb->cell_sig || !fb->fail || !fb->src)
    return fail(PHX_ERR_INVALID_ARG, "stage needs flux, face_sig, cell_sig, fail, src");
  if (p->mhd && fb->ndim > 1 && !fb->emf) return fail(PHX_ERR_INVALID_ARG, "emf is NULL");
  if (v.ng < 3) return fail(PHX_ERR_INVALID_ARG, "radiation fluxes need ng >= 3");
  if (fb->nx1 < fb->ng || (fb->ndim >= 2 && fb->nx2 < fb->ng) || (fb->ndim >= 3 && fb->nx3 < fb->ng))
    return fail(PHX_ERR_INVALID_ARG, "periodic exchange needs nx >= ng");
  if ((s = check_rad_fixups(rp, p, rb))) return s;
  par.update_fluid = 1;  // MomentFluidSource(update_fluid = fluid active)
  const phx::Par fpar = make_par(*p);
  cudaStream_t st = S(stream);
  phx::launch_sources(fpar, v, st);                      // CalculateFluidSourceTerms
  phx::launch_fluxes_err(fpar, v, ctx->err, st);         // fluid CalculateFluxes
  if (p->mhd && fb->ndim > 1) phx::launch_fluxct(v, st);  // FluxCT
  phx::rad::launch_opacities(par, v, r, st);              // MomentCalculateOpacities
  phx::rad::launch_fluxes(par, v, r, st);                 // radiation CalculateFluxes
  phx::launch_update(fpar, v, fluid_base, fluid_out, beta, dt, st);
  phx::rad::launch_update(par, v, r, rad_base, rad_out, beta, dt, st);
  phx::BView vo = v;
  vo.cons = fluid_out;
  phx::rad::RView ro = r;
  ro.cons = rad_out;
  // FillDerived (the fluid's con2prim, then MomentCon2Prim with the new
  // fluid velocity as PostFillDerived), ConservedToPrimitiveFixup,
  // RadConservedToPrimitiveFixup, ApplyFloors
  auto derived = [&] {
    phx::launch_c2p(fpar, vo, entire(vo), ctx->stats, ctx->err, nullptr, ctx->c2p, st);
    phx::rad::launch_c2p(par, vo, ro, entire(vo), st);
    phx::launch_c2p_fixup(fpar, vo, st);
    if (p->enable_c2p_fixup) phx::rad::launch_rad_c2p_fixup(par, vo, ro, st);
    rad_apply_floors(ctx, fpar, par, *rp, vo, ro, entire(vo), st);
  };
  derived();
  phx::rad::launch_source(par, source_inversion_par(*p), vo, ro, beta * dt, st);  // MomentFluidSource
  rad_apply_floors(ctx, fpar, par, *rp, vo, ro, entire(vo), st);                 // ApplyFloors
  phx::launch_ghost_periodic(vo, fluid_out, p->mhd ? PHX_NCONS : 5, st);         // boundary exchange
  phx::rad::launch_ghosts(vo, ro, st);
  derived();
  return cuda_status("phx_rad_fluid_stage");
}

}  // extern "C"
