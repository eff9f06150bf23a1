// Test driver for include/phx_parthenon_shim.hpp: one forward-Euler RK stage of
// a periodic block through the reference's task signatures, in the order of
// PhoebusDriver::RungeKuttaStage (phoebus_driver.cpp:321-668).
//
// usage: shim_stage <in.bin> <out.bin> nx ng recon riemann gamma dt
// in.bin: prims [12][N] (host doubles); out.bin: prims [12][N] then cons [8][N].
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "phx_parthenon_shim.hpp"

#define CK(x)                                                                 \
  do {                                                                        \
    cudaError_t e_ = (x);                                                     \
    if (e_ != cudaSuccess) {                                                  \
      std::fprintf(stderr, "%s: %s\n", #x, cudaGetErrorString(e_));           \
      return 2;                                                               \
    }                                                                         \
  } while (0)

int main(int argc, char **argv) {
  if (argc < 9) {
    std::fprintf(stderr, "usage: shim_stage in out nx ng recon riemann gamma dt\n");
    return 1;
  }
  const int nx = std::atoi(argv[3]), ng = std::atoi(argv[4]);
  const int recon = std::atoi(argv[5]), riemann = std::atoi(argv[6]);
  const double gamma = std::atof(argv[7]), dt = std::atof(argv[8]);
  const int n1 = nx + 2 * ng;
  const long long N = (long long)n1 * n1 * n1;
  std::vector<double> prim((size_t)PHX_NPRIM * N), cons((size_t)PHX_NCONS * N);
  FILE *f = std::fopen(argv[1], "rb");
  if (!f || std::fread(prim.data(), sizeof(double), prim.size(), f) != prim.size()) return 3;
  std::fclose(f);

  double *d_prim, *d_cons, *d_cons1, *d_flux, *d_fsig, *d_csig, *d_fail, *d_src, *d_emf, *d_dt;
  CK(cudaMalloc(&d_prim, sizeof(double) * PHX_NPRIM * N));
  CK(cudaMalloc(&d_cons, sizeof(double) * PHX_NCONS * N));
  CK(cudaMalloc(&d_cons1, sizeof(double) * PHX_NCONS * N));
  CK(cudaMalloc(&d_flux, sizeof(double) * 3 * PHX_NCONS * N));
  CK(cudaMalloc(&d_fsig, sizeof(double) * 3 * N));
  CK(cudaMalloc(&d_csig, sizeof(double) * 3 * N));
  CK(cudaMalloc(&d_fail, sizeof(double) * N));
  CK(cudaMalloc(&d_src, sizeof(double) * PHX_NCONS * N));  // the "geometric source terms" container
  CK(cudaMalloc(&d_emf, sizeof(double) * 3 * N));
  CK(cudaMalloc(&d_dt, sizeof(double)));
  CK(cudaMemcpy(d_prim, prim.data(), sizeof(double) * prim.size(), cudaMemcpyHostToDevice));
  for (double *p : {d_cons, d_cons1, d_flux, d_fsig, d_csig, d_fail, d_src, d_emf})
    CK(cudaMemset(p, 0, sizeof(double) * N));  // first variable; the rest is written before it is read

  parthenon::Mesh mesh;
  phx_params_default(&mesh.params);
  mesh.params.gm1 = gamma - 1.0;
  mesh.params.recon = recon;
  mesh.params.riemann = riemann;
  mesh.params.c2p_tol = 1e-10;
  mesh.params.c2p_max_iter = 100;
  mesh.params.cfl = 0.4;
  phx_geometry_default(&mesh.geometry, PHX_GEOM_MINKOWSKI);
  if (phx_ctx_create(0, &mesh.ctx) != PHX_OK) return 4;
  mesh.dt_device = d_dt;

  phx_block b{};
  b.nx1 = b.nx2 = b.nx3 = nx;
  b.ng = ng;
  b.ndim = 3;
  b.x1min = b.x2min = b.x3min = 0.0;
  b.dx1 = b.dx2 = b.dx3 = 1.0 / nx;
  b.prim = d_prim;
  b.cons = d_cons;
  b.flux = d_flux;
  b.face_sig = d_fsig;
  b.cell_sig = d_csig;
  b.fail = d_fail;
  b.src = d_src + N;  // S_1..3, tau of the source container
  b.emf = d_emf;
  phx_block bsrc = b;
  bsrc.cons = d_src;
  parthenon::MeshBlockData<double> rc(&mesh, b), rc_src(&mesh, bsrc);
  parthenon::MeshData<double> md(&mesh, {&rc}), md_src(&mesh, {&rc_src});

  try {
    // initialisation: pgen's PrimitiveToConserved, boundary exchange, FillDerived
    fluid::PrimitiveToConserved(&rc);
    if (phx_fill_ghosts_periodic(mesh.ctx, &rc.Block(), d_cons, PHX_NCONS, mesh.stream) != PHX_OK) return 5;
    fluid::ConservedToPrimitive(&rc);
    const double dt0 = fluid::EstimateTimestepBlock(&rc);
    std::printf("dt0 %.17g\n", dt0);
    // one stage (beta = 1): sources, fluxes, FluxCT, update into cons1
    fluid::CalculateFluidSourceTerms(&md, &md_src);
    fluid::CalculateFluxes(&rc);
    fluid::FluxCT(&rc);
    if (phx_update_stage(mesh.ctx, &rc.Block(), d_cons, d_cons1, 1.0, dt, mesh.stream) != PHX_OK) return 6;
    // FillDerived on the stage result, boundary exchange, FillDerived again
    phx_block b1 = rc.Block();
    b1.cons = d_cons1;
    parthenon::MeshBlockData<double> rc1(&mesh, b1);
    parthenon::MeshData<double> md1(&mesh, {&rc1});
    fluid::ConservedToPrimitive(&md1);
    if (phx_fill_ghosts_periodic(mesh.ctx, &rc1.Block(), d_cons1, PHX_NCONS, mesh.stream) != PHX_OK) return 7;
    fluid::ConservedToPrimitive(&rc1);
    std::printf("dt1 %.17g\n", fluid::EstimateTimestepBlock(&rc1));
  } catch (const std::exception &e) {
    std::fprintf(stderr, "task failed: %s\n", e.what());
    return 8;
  }
  CK(cudaMemcpy(prim.data(), d_prim, sizeof(double) * prim.size(), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(cons.data(), d_cons1, sizeof(double) * cons.size(), cudaMemcpyDeviceToHost));
  f = std::fopen(argv[2], "wb");
  if (!f) return 9;
  std::fwrite(prim.data(), sizeof(double), prim.size(), f);
  std::fwrite(cons.data(), sizeof(double), cons.size(), f);
  std::fclose(f);
  phx_ctx_destroy(mesh.ctx);
  return 0;
}
