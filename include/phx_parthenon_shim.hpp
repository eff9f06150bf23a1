// phx_parthenon_shim.hpp -- the phoebus fluid task signatures over the C ABI.
//
// Header-only C++17.  It gives the functions phoebus's driver calls
// (fluid.hpp:27-69, paths relative to the phoebus source tree) the same names,
// signatures and error behaviour, and implements them with phx_fluid.h:
//
//   TaskStatus fluid::PrimitiveToConserved(MeshBlockData<Real> *)        fluid.cpp:359
//   TaskStatus fluid::PrimitiveToConservedRegion(MeshBlockData<Real> *,
//                                               ib, jb, kb)              fluid.cpp:368
//   template <T> TaskStatus fluid::ConservedToPrimitive(T *)            fluid.cpp:469
//   template <T> TaskStatus fluid::ConservedToPrimitiveRegion(T *, ...)  fluid.cpp:451
//   template <T> TaskStatus fluid::ConservedToPrimitiveRobust(T *, ...)  fluid.cpp:477
//   TaskStatus fluid::CalculateFluidSourceTerms(MeshData<Real> *,
//                                              MeshData<Real> *)        fluid.cpp:566
//   TaskStatus fluid::CalculateFluxes(MeshBlockData<Real> *)             fluid.cpp:659
//   TaskStatus fluid::FluxCT(MeshBlockData<Real> *)                      fluid.cpp:775
//   TaskStatus fixup::FixFluxes(MeshBlockData<Real> *)                   fixup.cpp:728
//   template <T> TaskStatus radiation::MomentPrim2Con(T *, IndexDomain)  moments.cpp:258
//   template <T> TaskStatus radiation::MomentCon2Prim(T *)               moments.cpp:162
//   template <T> TaskStatus radiation::MomentCalculateOpacities(T *)     moments.cpp:919
//   template <T> TaskStatus radiation::ReconstructEdgeStates(T *)        moments.cpp:280
//   template <T> TaskStatus radiation::CalculateFluxes(T *)              moments.cpp:724
//   template <T> TaskStatus radiation::CalculateGeometricSource(T *, T *) moments.cpp:886
//   template <T> TaskStatus radiation::MomentFluidSource(T *, Real, bool) moments_source.cpp:960
//   TaskStatus fixup::RadConservedToPrimitiveFixup(MeshBlockData<Real> *) fixup_radc2p.cpp:227
//   TaskStatus fixup::ApplyFloors(MeshBlockData<Real> *), radiation on    fixup.cpp:680
//   Real radiation::EstimateTimestepBlock(MeshBlockData<Real> *)         radiation.cpp:585
//   Real fluid::EstimateTimestepBlock(MeshBlockData<Real> *)             fluid.cpp:899
//   template <T> using fluid::c2p_type = TaskStatus (*)(T *, ...)        fluid.hpp:65
//
// Parthenon is not part of this library, so the shim carries the few pieces
// of it these tasks touch (MeshBlockData, MeshData, IndexRange, IndexDomain,
// TaskStatus, the package Params) as small stand-ins in namespace parthenon.
// Inside phoebus the same function bodies are written against the real
// Parthenon types: a pack's variable Views provide the device pointers of
// phx_block (the fluid fields of a block laid out as one [var][k][j][i]
// allocation, or staged into one).
//
// Errors: configuration errors throw std::runtime_error (PARTHENON_THROW);
// an unbracketed con2prim root is detected by phx_ctx_check() at the end of
// ConservedToPrimitive and throws "Aborting with unbracketed root."
// (root_find.hpp:115-118 aborts the run).
#ifndef PHX_PARTHENON_SHIM_HPP_
#define PHX_PARTHENON_SHIM_HPP_

#include <cuda_runtime.h>

#include <stdexcept>
#include <string>
#include <vector>

#include "phx_fluid.h"
#include "phx_radiation.h"

namespace parthenon {
using Real = double;
enum class TaskStatus { fail, complete, incomplete, iterate, skip, waiting };
enum class IndexDomain { entire, interior };
struct IndexRange {
  int s = 0;
  int e = -1;
};

// Package parameters and execution resources the fluid tasks read.
struct Mesh {
  phx_params params{};      // "fluid", "fixup" and "eos" package Params
  phx_geometry geometry{};  // "geometry" package (Minkowski or FMKS tables)
  phx_ctx *ctx = nullptr;   // device context (the execution space)
  void *stream = nullptr;   // CUDA stream the tasks run on
  double *dt_device = nullptr;  // one device double for EstimateTimestepBlock
  bool has_face_speeds = false; // fluid.cpp:911-941 switch
  int ndim = 3;
  phx_rad_params rad_params{};  // "radiation" (+ opacity, fixup) package Params
};

template <typename T>
class MeshBlockData;
template <typename T>
class MeshData;

// One meshblock's fields (device pointers) and its mesh.
template <>
class MeshBlockData<Real> {
 public:
  MeshBlockData(Mesh *mesh, const phx_block &b) : mesh_(mesh), b_(b) { b_.geom = &mesh_->geometry; }
  Mesh *GetMeshPointer() const { return mesh_; }
  phx_block &Block() { return b_; }
  const phx_block &Block() const { return b_; }
  IndexRange GetBoundsI(IndexDomain d) const {
    return d == IndexDomain::entire ? IndexRange{0, b_.nx1 + 2 * b_.ng - 1} : IndexRange{b_.ng, b_.ng + b_.nx1 - 1};
  }
  IndexRange GetBoundsJ(IndexDomain d) const {
    if (b_.ndim < 2) return IndexRange{0, 0};
    return d == IndexDomain::entire ? IndexRange{0, b_.nx2 + 2 * b_.ng - 1} : IndexRange{b_.ng, b_.ng + b_.nx2 - 1};
  }
  IndexRange GetBoundsK(IndexDomain d) const {
    if (b_.ndim < 3) return IndexRange{0, 0};
    return d == IndexDomain::entire ? IndexRange{0, b_.nx3 + 2 * b_.ng - 1} : IndexRange{b_.ng, b_.ng + b_.nx3 - 1};
  }
  // pmb->boundary_flag with the phoebus BC name of each face folded in:
  // PHX_BC_OUTFLOW / REFLECT / POLAR on a physical ("user") boundary,
  // PHX_BC_PERIODIC where the block has a neighbour.
  void SetBoundaries(const int lo[3], const int hi[3]) {
    for (int d = 0; d < 3; d++) {
      bc_lo_[d] = lo[d];
      bc_hi_[d] = hi[d];
    }
  }
  const int *BoundaryLo() const { return bc_lo_; }
  const int *BoundaryHi() const { return bc_hi_; }
  // the radiation fields of the block (E, F_i of this stage container; the
  // OneCopy J, H, xi, phi, c2pfail, kappaJ, kappaH, JBB)
  void SetRadiation(const phx_rad_block &r) { rad_ = r; }
  phx_rad_block &RadBlock() { return rad_; }

 private:
  Mesh *mesh_;
  phx_block b_;
  phx_rad_block rad_{};
  int bc_lo_[3] = {PHX_BC_PERIODIC, PHX_BC_PERIODIC, PHX_BC_PERIODIC};
  int bc_hi_[3] = {PHX_BC_PERIODIC, PHX_BC_PERIODIC, PHX_BC_PERIODIC};
};

// A pack of blocks (a MeshData partition).
template <>
class MeshData<Real> {
 public:
  MeshData(Mesh *mesh, std::vector<MeshBlockData<Real> *> blocks) : mesh_(mesh), blocks_(std::move(blocks)) {}
  Mesh *GetMeshPointer() const { return mesh_; }
  int NumBlocks() const { return static_cast<int>(blocks_.size()); }
  MeshBlockData<Real> *GetBlockData(int n) const { return blocks_.at(n); }

 private:
  Mesh *mesh_;
  std::vector<MeshBlockData<Real> *> blocks_;
};
}  // namespace parthenon

namespace fluid {
using parthenon::IndexDomain;
using parthenon::IndexRange;
using parthenon::Mesh;
using parthenon::MeshBlockData;
using parthenon::MeshData;
using parthenon::Real;
using parthenon::TaskStatus;

template <typename T>
using c2p_type = TaskStatus (*)(T *, const IndexRange &, const IndexRange &, const IndexRange &);
using c2p_meshblock_type = c2p_type<MeshBlockData<Real>>;
using c2p_mesh_type = c2p_type<MeshData<Real>>;

namespace detail {
inline void check(phx_status s, const char *where) {
  if (s != PHX_OK)
    throw std::runtime_error(std::string(where) + ": " + phx_status_string(s) + " (" + phx_last_error() + ")");
}
inline phx_range R(const IndexRange &r) { return phx_range{r.s, r.e}; }
}  // namespace detail

inline TaskStatus PrimitiveToConservedRegion(MeshBlockData<Real> *rc, const IndexRange &ib, const IndexRange &jb,
                                             const IndexRange &kb) {
  Mesh *m = rc->GetMeshPointer();
  detail::check(phx_prim_to_con(m->ctx, &m->params, &rc->Block(), detail::R(ib), detail::R(jb), detail::R(kb),
                                m->stream),
                "PrimitiveToConservedRegion");
  return TaskStatus::complete;
}

inline TaskStatus PrimitiveToConserved(MeshBlockData<Real> *rc) {
  return PrimitiveToConservedRegion(rc, rc->GetBoundsI(IndexDomain::entire), rc->GetBoundsJ(IndexDomain::entire),
                                    rc->GetBoundsK(IndexDomain::entire));
}

// The robust solver (con2prim_robust.hpp) on one block or on every block of
// a pack.  An unbracketed root aborts, as in the reference.
template <typename T>
TaskStatus ConservedToPrimitiveRobust(T *rc, const IndexRange &ib, const IndexRange &jb, const IndexRange &kb);

template <>
inline TaskStatus ConservedToPrimitiveRobust<MeshBlockData<Real>>(MeshBlockData<Real> *rc, const IndexRange &ib,
                                                                  const IndexRange &jb, const IndexRange &kb) {
  Mesh *m = rc->GetMeshPointer();
  detail::check(phx_con_to_prim(m->ctx, &m->params, &rc->Block(), detail::R(ib), detail::R(jb), detail::R(kb),
                                m->stream),
                "ConservedToPrimitiveRobust");
  detail::check(phx_ctx_check(m->ctx), "ConservedToPrimitiveRobust");
  return TaskStatus::complete;
}

template <>
inline TaskStatus ConservedToPrimitiveRobust<MeshData<Real>>(MeshData<Real> *rc, const IndexRange &ib,
                                                             const IndexRange &jb, const IndexRange &kb) {
  Mesh *m = rc->GetMeshPointer();
  for (int n = 0; n < rc->NumBlocks(); n++)
    detail::check(phx_con_to_prim(m->ctx, &m->params, &rc->GetBlockData(n)->Block(), detail::R(ib), detail::R(jb),
                                  detail::R(kb), m->stream),
                  "ConservedToPrimitiveRobust");
  detail::check(phx_ctx_check(m->ctx), "ConservedToPrimitiveRobust");
  return TaskStatus::complete;
}

// fluid.cpp:68-75: the c2p Param is a function pointer; only the robust
// solver is provided (c2p_method = "robust", the default).
template <typename T>
inline c2p_type<T> c2p_func() {
  return ConservedToPrimitiveRobust<T>;
}

template <typename T>
TaskStatus ConservedToPrimitiveRegion(T *rc, const IndexRange &ib, const IndexRange &jb, const IndexRange &kb) {
  auto c2p = c2p_func<T>();
  return c2p(rc, ib, jb, kb);
}

template <typename T>
TaskStatus ConservedToPrimitive(T *rc);

template <>
inline TaskStatus ConservedToPrimitive<MeshBlockData<Real>>(MeshBlockData<Real> *rc) {
  return ConservedToPrimitiveRegion(rc, rc->GetBoundsI(IndexDomain::entire), rc->GetBoundsJ(IndexDomain::entire),
                                    rc->GetBoundsK(IndexDomain::entire));
}

template <>
inline TaskStatus ConservedToPrimitive<MeshData<Real>>(MeshData<Real> *rc) {
  // every block of a pack shares the index ranges of the first
  MeshBlockData<Real> *b0 = rc->GetBlockData(0);
  return ConservedToPrimitiveRegion(rc, b0->GetBoundsI(IndexDomain::entire), b0->GetBoundsJ(IndexDomain::entire),
                                    b0->GetBoundsK(IndexDomain::entire));
}

// Sources go to rc_src's momentum and energy: with the conserved layout
// (D, S_1..3, tau, B) the four source fields are cons + one variable.
inline TaskStatus CalculateFluidSourceTerms(MeshData<Real> *rc, MeshData<Real> *rc_src) {
  Mesh *m = rc->GetMeshPointer();
  std::vector<phx_block> blocks;
  for (int n = 0; n < rc->NumBlocks(); n++) {
    phx_block b = rc->GetBlockData(n)->Block();
    const phx_block &s = rc_src->GetBlockData(n)->Block();
    const long long N = (long long)(b.nx1 + 2 * b.ng) * (b.ndim >= 2 ? b.nx2 + 2 * b.ng : 1) *
                        (b.ndim >= 3 ? b.nx3 + 2 * b.ng : 1);
    const long long vs = s.var_stride ? s.var_stride : N;
    b.src = s.cons + vs;
    blocks.push_back(b);
  }
  detail::check(phx_calculate_fluid_source_terms(m->ctx, &m->params, blocks.data(), (int)blocks.size(), m->stream),
                "CalculateFluidSourceTerms");
  return TaskStatus::complete;
}

inline TaskStatus CalculateFluxes(MeshBlockData<Real> *rc) {
  Mesh *m = rc->GetMeshPointer();
  detail::check(phx_calculate_fluxes(m->ctx, &m->params, &rc->Block(), m->stream), "CalculateFluxes");
  return TaskStatus::complete;
}

inline TaskStatus FluxCT(MeshBlockData<Real> *rc) {
  Mesh *m = rc->GetMeshPointer();
  detail::check(phx_flux_ct(m->ctx, &m->params, &rc->Block(), m->stream), "FluxCT");
  return TaskStatus::complete;
}

inline Real EstimateTimestepBlock(MeshBlockData<Real> *rc) {
  Mesh *m = rc->GetMeshPointer();
  if (!m->dt_device) throw std::runtime_error("EstimateTimestepBlock: Mesh::dt_device is not set");
  detail::check(phx_estimate_timestep(m->ctx, &m->params, &rc->Block(), m->has_face_speeds ? 1 : 0, m->dt_device,
                                      m->stream),
                "EstimateTimestepBlock");
  Real dt = 0.0;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(m->stream);
  if (cudaMemcpyAsync(&dt, m->dt_device, sizeof(Real), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    throw std::runtime_error("EstimateTimestepBlock: copy of dt failed");
  m->has_face_speeds = true;
  return dt;
}

}  // namespace fluid

namespace fixup {
using parthenon::MeshBlockData;
using parthenon::Real;
using parthenon::TaskStatus;

// fixup::FixFluxes (fixup.cpp:728): returns at once unless
// fixup/enable_flux_fixup (Mesh::params.enable_flux_fixup).
inline TaskStatus FixFluxes(MeshBlockData<Real> *rc) {
  parthenon::Mesh *m = rc->GetMeshPointer();
  if (!m->params.enable_flux_fixup) return TaskStatus::complete;
  fluid::detail::check(
      phx_fix_fluxes_block(m->ctx, &m->params, &rc->Block(), rc->BoundaryLo(), rc->BoundaryHi(), m->stream),
      "FixFluxes");
  return TaskStatus::complete;
}
}  // namespace fixup

namespace radiation {
using parthenon::IndexDomain;
using parthenon::IndexRange;
using parthenon::MeshBlockData;
using parthenon::Real;
using parthenon::TaskStatus;

namespace detail {
inline void check(phx_status s, const char *where) {
  if (s != PHX_OK) throw std::runtime_error(std::string(where) + ": " + phx_last_error());
}
inline phx_range R(const IndexRange &r) { return phx_range{r.s, r.e}; }
}  // namespace detail

template <typename T>
TaskStatus MomentPrim2Con(T *rc, IndexDomain domain);
template <>
inline TaskStatus MomentPrim2Con<MeshBlockData<Real>>(MeshBlockData<Real> *rc, IndexDomain domain) {
  parthenon::Mesh *m = rc->GetMeshPointer();
  detail::check(phx_rad_prim_to_con(m->ctx, &m->rad_params, &m->params, &rc->Block(), &rc->RadBlock(),
                                    detail::R(rc->GetBoundsI(domain)), detail::R(rc->GetBoundsJ(domain)),
                                    detail::R(rc->GetBoundsK(domain)), m->stream),
                "MomentPrim2Con");
  return TaskStatus::complete;
}

// the package's PostFillDerivedBlock: the entire block
template <typename T>
TaskStatus MomentCon2Prim(T *rc);
template <>
inline TaskStatus MomentCon2Prim<MeshBlockData<Real>>(MeshBlockData<Real> *rc) {
  parthenon::Mesh *m = rc->GetMeshPointer();
  const IndexDomain e = IndexDomain::entire;
  detail::check(phx_rad_con_to_prim(m->ctx, &m->rad_params, &m->params, &rc->Block(), &rc->RadBlock(),
                                    detail::R(rc->GetBoundsI(e)), detail::R(rc->GetBoundsJ(e)),
                                    detail::R(rc->GetBoundsK(e)), m->stream),
                "MomentCon2Prim");
  return TaskStatus::complete;
}

template <typename T>
TaskStatus MomentCalculateOpacities(T *rc);
template <>
inline TaskStatus MomentCalculateOpacities<MeshBlockData<Real>>(MeshBlockData<Real> *rc) {
  parthenon::Mesh *m = rc->GetMeshPointer();
  detail::check(phx_rad_calculate_opacities(m->ctx, &m->rad_params, &m->params, &rc->Block(), &rc->RadBlock(),
                                            m->stream),
                "MomentCalculateOpacities");
  return TaskStatus::complete;
}

// The reconstruction is fused into CalculateFluxes (no ql/qr/dJ fields).
template <typename T>
TaskStatus ReconstructEdgeStates(T *rc) {
  return TaskStatus::complete;
}

template <typename T>
TaskStatus CalculateFluxes(T *rc);
template <>
inline TaskStatus CalculateFluxes<MeshBlockData<Real>>(MeshBlockData<Real> *rc) {
  parthenon::Mesh *m = rc->GetMeshPointer();
  detail::check(phx_rad_calculate_fluxes(m->ctx, &m->rad_params, &m->params, &rc->Block(), &rc->RadBlock(),
                                         m->stream),
                "radiation::CalculateFluxes");
  return TaskStatus::complete;
}

// The geometric source is computed inside phx_rad_update (zero on
// Minkowski; on FMKS per zone from the stage input), so the task itself has
// nothing left to do.
template <typename T>
TaskStatus CalculateGeometricSource(T *rc, T *rc_src) {
  return TaskStatus::complete;
}

template <typename T>
TaskStatus MomentFluidSource(T *rc, Real dt, bool update_fluid);
template <>
inline TaskStatus MomentFluidSource<MeshBlockData<Real>>(MeshBlockData<Real> *rc, Real dt, bool update_fluid) {
  parthenon::Mesh *m = rc->GetMeshPointer();
  phx_rad_params rp = m->rad_params;
  rp.update_fluid = update_fluid ? 1 : 0;
  detail::check(phx_rad_fluid_source(m->ctx, &rp, &m->params, &rc->Block(), &rc->RadBlock(), dt, m->stream),
                "MomentFluidSource");
  return TaskStatus::complete;
}

inline Real EstimateTimestepBlock(MeshBlockData<Real> *rc) {
  parthenon::Mesh *m = rc->GetMeshPointer();
  if (!m->dt_device) throw std::runtime_error("EstimateTimestepBlock: Mesh::dt_device is not set");
  detail::check(phx_rad_estimate_timestep(m->ctx, &m->rad_params, &m->params, &rc->Block(), &rc->RadBlock(),
                                          m->dt_device, m->stream),
                "radiation::EstimateTimestepBlock");
  Real dt = 0.0;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(m->stream);
  if (cudaMemcpyAsync(&dt, m->dt_device, sizeof(Real), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    throw std::runtime_error("radiation::EstimateTimestepBlock: copy of dt failed");
  return dt;
}
}  // namespace radiation

namespace fixup {
// fixup::RadConservedToPrimitiveFixup (fixup_radc2p.cpp:227): a no-op unless
// fixup/enable_c2p_fixup.
inline TaskStatus RadConservedToPrimitiveFixup(MeshBlockData<Real> *rc) {
  parthenon::Mesh *m = rc->GetMeshPointer();
  radiation::detail::check(
      phx_rad_c2p_fixup(m->ctx, &m->rad_params, &m->params, &rc->Block(), &rc->RadBlock(), m->stream),
      "RadConservedToPrimitiveFixup");
  return TaskStatus::complete;
}

// fixup::ApplyFloors (fixup.cpp:680) with the radiation package active, over
// the entire block: the fluid floors, then the radiation floors and ceilings.
inline TaskStatus ApplyFloorsWithRadiation(MeshBlockData<Real> *rc) {
  parthenon::Mesh *m = rc->GetMeshPointer();
  const parthenon::IndexDomain e = parthenon::IndexDomain::entire;
  radiation::detail::check(
      phx_rad_apply_floors(m->ctx, &m->rad_params, &m->params, &rc->Block(), &rc->RadBlock(),
                           radiation::detail::R(rc->GetBoundsI(e)), radiation::detail::R(rc->GetBoundsJ(e)),
                           radiation::detail::R(rc->GetBoundsK(e)), m->stream),
      "ApplyFloors");
  return TaskStatus::complete;
}
}  // namespace fixup

#endif  // PHX_PARTHENON_SHIM_HPP_
