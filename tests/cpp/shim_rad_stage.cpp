// Test driver for the radiation tasks of include/phx_parthenon_shim.hpp: the
// moment initialisation and one forward-Euler stage of a periodic 3D block
// through the reference's task signatures, in the order of
// PhoebusDriver::RungeKuttaStage with the fluid not evolved
// (phoebus_driver.cpp:349-362, 547-620, 640-668).
//
// usage: shim_rad_stage <in.bin> <out.bin> nx ng dt kappa_s kappa_a jbb
// in.bin: fluid prims [12][N] then radiation prims [10][N] (host doubles);
// out.bin: radiation cons [4][N], radiation prims [10][N], then the
// radiation timestep estimate.
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
    std::fprintf(stderr, "usage: shim_rad_stage in out nx ng dt kappa_s kappa_a jbb\n");
    return 1;
  }
  const int nx = std::atoi(argv[3]), ng = std::atoi(argv[4]);
  const double dt = std::atof(argv[5]);
  const int n1 = nx + 2 * ng;
  const long long N = (long long)n1 * n1 * n1;
  std::vector<double> fprim((size_t)PHX_NPRIM * N), rprim((size_t)PHX_RNPRIM * N), rcons((size_t)PHX_RNCONS * N);
  FILE *f = std::fopen(argv[1], "rb");
  if (!f || std::fread(fprim.data(), sizeof(double), fprim.size(), f) != fprim.size() ||
      std::fread(rprim.data(), sizeof(double), rprim.size(), f) != rprim.size())
    return 3;
  std::fclose(f);

  double *d_fprim, *d_fcons, *d_cons0, *d_cons1, *d_rprim, *d_flux, *d_dudt, *d_dt;
  CK(cudaMalloc(&d_fprim, sizeof(double) * PHX_NPRIM * N));
  CK(cudaMalloc(&d_fcons, sizeof(double) * PHX_NCONS * N));
  CK(cudaMalloc(&d_cons0, sizeof(double) * PHX_RNCONS * N));
  CK(cudaMalloc(&d_cons1, sizeof(double) * PHX_RNCONS * N));
  CK(cudaMalloc(&d_rprim, sizeof(double) * PHX_RNPRIM * N));
  CK(cudaMalloc(&d_flux, sizeof(double) * 3 * PHX_RNCONS * N));
  CK(cudaMalloc(&d_dudt, sizeof(double) * PHX_RNCONS * N));
  CK(cudaMalloc(&d_dt, sizeof(double)));
  CK(cudaMemcpy(d_fprim, fprim.data(), sizeof(double) * fprim.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_rprim, rprim.data(), sizeof(double) * rprim.size(), cudaMemcpyHostToDevice));
  CK(cudaMemset(d_cons0, 0, sizeof(double) * PHX_RNCONS * N));
  CK(cudaMemset(d_cons1, 0, sizeof(double) * PHX_RNCONS * N));

  parthenon::Mesh mesh;
  phx_params_default(&mesh.params);
  mesh.params.Cv = 1.0;
  phx_rad_params_default(&mesh.rad_params);
  mesh.rad_params.cfl = 0.5;
  mesh.rad_params.kappa_s = std::atof(argv[6]);
  mesh.rad_params.kappa_a = std::atof(argv[7]);
  mesh.rad_params.jbb_coeff = std::atof(argv[8]);
  phx_geometry_default(&mesh.geometry, PHX_GEOM_MINKOWSKI);
  if (phx_ctx_create(0, &mesh.ctx) != PHX_OK) return 4;
  mesh.dt_device = d_dt;

  phx_block b{};
  b.nx1 = b.nx2 = b.nx3 = nx;
  b.ng = ng;
  b.ndim = 3;
  b.dx1 = b.dx2 = b.dx3 = 1.0 / nx;
  b.prim = d_fprim;
  b.cons = d_fcons;
  parthenon::MeshBlockData<parthenon::Real> rc(&mesh, b);
  phx_rad_block rb{};
  rb.cons = d_cons0;
  rb.prim = d_rprim;
  rb.flux = d_flux;
  rb.dudt = d_dudt;
  rc.SetRadiation(rb);
  using parthenon::IndexDomain;
  try {
    // problem generator's MomentPrim2Con, then Parthenon's initial exchange
    // and FillDerived
    radiation::MomentPrim2Con(&rc, IndexDomain::interior);
    if (phx_rad_fill_ghosts_periodic(mesh.ctx, &rc.Block(), &rc.RadBlock(), mesh.stream) != PHX_OK) return 5;
    radiation::MomentCon2Prim(&rc);
    // one stage, beta = 1
    radiation::MomentCalculateOpacities(&rc);
    radiation::ReconstructEdgeStates(&rc);
    radiation::CalculateFluxes(&rc);
    radiation::CalculateGeometricSource(&rc, &rc);
    if (phx_rad_update(mesh.ctx, &mesh.rad_params, &rc.Block(), &rc.RadBlock(), d_cons0, d_cons1, 1.0, dt,
                       mesh.stream) != PHX_OK)
      return 6;
    rc.RadBlock().cons = d_cons1;  // sc1
    radiation::MomentCon2Prim(&rc);
    radiation::MomentFluidSource(&rc, dt, false);
    if (phx_rad_fill_ghosts_periodic(mesh.ctx, &rc.Block(), &rc.RadBlock(), mesh.stream) != PHX_OK) return 7;
    radiation::MomentCon2Prim(&rc);
    const double dtn = radiation::EstimateTimestepBlock(&rc);
    CK(cudaMemcpy(rcons.data(), d_cons1, sizeof(double) * rcons.size(), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(rprim.data(), d_rprim, sizeof(double) * rprim.size(), cudaMemcpyDeviceToHost));
    FILE *o = std::fopen(argv[2], "wb");
    std::fwrite(rcons.data(), sizeof(double), rcons.size(), o);
    std::fwrite(rprim.data(), sizeof(double), rprim.size(), o);
    std::fwrite(&dtn, sizeof(double), 1, o);
    std::fclose(o);
  } catch (const std::exception &e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 8;
  }
  if (phx_ctx_check(mesh.ctx) != PHX_OK) return 9;
  phx_ctx_destroy(mesh.ctx);
  return 0;
}
