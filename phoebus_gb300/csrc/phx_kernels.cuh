// phx_kernels.cuh -- kernel declarations shared by the translation units.
#pragma once
#include "phx_c2p.cuh"

namespace phx {

// Sticky error bits (device word in the context).
enum : unsigned int {
  ERR_UNBRACKETED = 1u,
  ERR_NAN_INPUT = 2u,
  ERR_TIMEOUT = 4u,
  ERR_BOUNDS = 8u,
};

struct DevStats {  // mirrors phx_c2p_stats
  unsigned long long zones, iterations, residual_evals, failures, unbracketed, learned_accepted;
  unsigned long long hist[PHX_C2P_HIST];
};

// Optional learned starting bracket: per-zone [lo, hi] computed by the MLP.
struct LearnedBracket {
  const float *w;  // FP32 master parameters (PHX_MLP_NPARAM), or null
  const void *wbf16;  // packed BF16 operand tiles for the tensor-core path
};

struct Range3 {
  int is, ie, js, je, ks, ke;
};

void launch_p2c(const Par &p, const BView &b, Range3 r, cudaStream_t s);
void launch_c2p(const Par &p, const BView &b, Range3 r, DevStats *stats, unsigned int *err,
                const float *mlp_w, cudaStream_t s);
void launch_fluxes(const Par &p, const BView &b, cudaStream_t s);
void launch_fluxct(const BView &b, cudaStream_t s);
void launch_sources(const Par &p, const BView &b, cudaStream_t s);
void launch_update(const Par &p, const BView &b, const double *base, double *out, double beta,
                   double dt, cudaStream_t s);
void launch_ghost_periodic(const BView &b, double *field, int nvar, cudaStream_t s);
void launch_dt(const Par &p, const BView &b, int use_face, unsigned long long *scratch,
               double *dt_out, cudaStream_t s);
void launch_c2p_fixup(const Par &p, const BView &b, cudaStream_t s);
void launch_floors(const Par &p, const BView &b, Range3 r, DevStats *stats, unsigned int *err,
                   cudaStream_t s);
void launch_geom_fmks(const phx_geometry &g, const BView &b, cudaStream_t s);
void launch_fp64_probe(double *out, int iters, cudaStream_t s, int *nthreads_out);

}  // namespace phx
