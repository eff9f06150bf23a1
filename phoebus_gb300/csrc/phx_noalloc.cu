// phx_noalloc.cu -- timestep estimate that allocates nothing.
//
// phx_estimate_timestep needs a phx_ctx, and creating one calls cudaMalloc.
// Some callers of this library cannot allocate device memory at the point
// where they need a timestep: a host code that owns every device buffer
// through its own memory pool (a Kokkos/Parthenon memory space, a fixed
// arena set up at start-up) and forbids libraries from allocating, or a
// driver loop that must not risk the implicit device synchronisation an
// allocation can cause in the middle of a step.  phx_estimate_timestep_static
// serves them: the caller passes the block (inputs) and the device word for
// the result (output); the only other memory it touches is the file-scope
// array below, which every device that loads this library holds until the
// process exits.
//
// Scratch: g_dt_partials, PHX_DT_STATIC_MAX_PARTIALS doubles (512 KiB).  Each
// call writes one partial minimum per thread block of the first kernel and
// reads them back in the second, so blocks of more than
// PHX_DT_STATIC_MAX_ZONES interior zones are rejected.  Every call shares the
// array: calls whose kernels overlap on the GPU (e.g. on two streams) race on
// it.  Nothing needs clearing: each call writes every partial it reads.
#include <cuda.h>

#include <mutex>

#include "phx_kernels.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kMaxPartials = PHX_DT_STATIC_MAX_PARTIALS;
static_assert((long long)kMaxPartials * kThreads == PHX_DT_STATIC_MAX_ZONES, "capacity");

static __device__ __align__(256) double g_dt_partials[kMaxPartials];

// Device address of g_dt_partials per device, looked up on the first call
// with that device current.  The address belongs to the context the module
// was loaded into: it is kept with that context's unique id and looked up
// again when the current context differs (after cudaDeviceReset the primary
// context is a new one, and the module may sit at another address).
constexpr int kMaxDevices = 64;
std::mutex g_mu;
double *g_addr[kMaxDevices] = {};
unsigned long long g_ctx_id[kMaxDevices] = {};

// Errors go to phx_last_error() like every other entry point's.
phx_status reject(phx_status s, const char *msg) {
  phx::set_last_error(msg);
  return s;
}

// Same per-zone estimate as fluid.cpp:913-939: 1 / (sum_d max signal speed /
// dx_d + 1e-50); one partial minimum per thread block.
__global__ void __launch_bounds__(kThreads)
    k_dt_partials(phx::BView b, int use_face, double *partials, long long n) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double v = 1.7976931348623157e308;
  if (t < n) {
    const int ni = b.nx1, nj = b.ndim >= 2 ? b.nx2 : 1;
    const int i = b.ng + (int)(t % ni);
    const int j = (b.ndim >= 2 ? b.ng : 0) + (int)((t / ni) % nj);
    const int k = (b.ndim >= 3 ? b.ng : 0) + (int)(t / ((long long)ni * nj));
    const long long id = b.idx(k, j, i);
    double ldt = 0.0;
    for (int d = 0; d < b.ndim; d++) {
      double ms = b.cell_sig[d * b.vs + id];
      if (use_face) {
        const long long off = d == 0 ? 1 : (d == 1 ? (long long)b.n1t : (long long)b.n1t * b.n2t);
        ms = fmax(ms, fmax(b.face_sig[d * b.vs + id], b.face_sig[d * b.vs + id + off]));
      }
      ldt += ms / b.dx[d];
    }
    v = 1.0 / (ldt + 1.e-50);
  }
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  __shared__ double sm[kThreads / 32];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < kThreads / 32; w++) v = fmin(v, sm[w]);
    if (!(v >= 0.0)) v = 1.7976931348623157e308;  // a block of NaN speeds is skipped
    partials[blockIdx.x] = v;
  }
}

__global__ void __launch_bounds__(1024) k_dt_finish(const double *partials, int nparts, double cfl, double *out) {
  double v = 1.7976931348623157e308;
  for (int q = threadIdx.x; q < nparts; q += blockDim.x) v = fmin(v, partials[q]);
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  __shared__ double sm[32];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) v = fmin(v, sm[w]);
    *out = cfl * v;
  }
}

// Set-up, once per device (and again after the device's context was
// replaced), with that device current: the host-side name of a __device__
// array is not a device address, so look the address up.
phx_status scratch_address(double **out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0)
    return reject(PHX_ERR_NO_DEVICE, "phx_estimate_timestep_static: no current CUDA device");
  if (dev >= kMaxDevices) return reject(PHX_ERR_CAPACITY, "phx_estimate_timestep_static: device index >= 64");
  std::lock_guard<std::mutex> lock(g_mu);
  // The driver calls are resolved through the runtime, so the library keeps
  // loading on hosts without a driver (the CPU test suite).
  using GetCurrentFn = CUresult (*)(CUcontext *);
  using GetIdFn = CUresult (*)(CUcontext, unsigned long long *);
  static GetCurrentFn get_current = nullptr;
  static GetIdFn get_id = nullptr;
  if (!get_current || !get_id) {
    void *f0 = nullptr, *f1 = nullptr;
    cudaDriverEntryPointQueryResult q0, q1;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 4000, cudaEnableDefault, &q0) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
        q0 != cudaDriverEntryPointSuccess || q1 != cudaDriverEntryPointSuccess || !f0 || !f1) {
      cudaGetLastError();
      return reject(PHX_ERR_CUDA, "phx_estimate_timestep_static: driver entry points not found");
    }
    get_current = reinterpret_cast<GetCurrentFn>(f0);
    get_id = reinterpret_cast<GetIdFn>(f1);
  }
  // The id of the current context (0 when the runtime has not made one current
  // yet; the lookup below does, and the id is read again after it).
  auto ctx_id = [&]() -> unsigned long long {
    CUcontext cu = nullptr;
    unsigned long long id = 0;
    if (get_current(&cu) != CUDA_SUCCESS || cu == nullptr || get_id(cu, &id) != CUDA_SUCCESS) return 0;
    return id;
  };
  const unsigned long long id = ctx_id();
  if (!g_addr[dev] || id == 0 || g_ctx_id[dev] != id) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_dt_partials);
    if (e != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      return reject(PHX_ERR_CUDA, "phx_estimate_timestep_static: cudaGetSymbolAddress failed");
    }
    g_addr[dev] = static_cast<double *>(p);
    g_ctx_id[dev] = ctx_id();
  }
  *out = g_addr[dev];
  return PHX_OK;
}

}  // namespace

extern "C" {

phx_status phx_estimate_timestep_static(const phx_params *p, const phx_block *blk, int use_face_speeds,
                                        double *dt_out_device, void *stream) {
  if (!p || !blk || !dt_out_device)
    return reject(PHX_ERR_INVALID_ARG, "phx_estimate_timestep_static: params, block and dt_out are required");
  // the block checks of phx_estimate_timestep that do not involve prim/cons
  if (blk->ndim < 1 || blk->ndim > 3 || blk->nx1 < 1 || blk->nx2 < 1 || blk->nx3 < 1 ||
      (blk->ndim < 2 && blk->nx2 != 1) || (blk->ndim < 3 && blk->nx3 != 1))
    return reject(PHX_ERR_INVALID_ARG, "phx_estimate_timestep_static: invalid block shape");
  if (blk->ng < 3) return reject(PHX_ERR_INVALID_ARG, "phx_estimate_timestep_static: ng must be >= 3");
  if (!blk->cell_sig || (use_face_speeds && !blk->face_sig))
    return reject(PHX_ERR_INVALID_ARG,
                  "phx_estimate_timestep_static: cell_sig (and face_sig with use_face_speeds) are required");
  {
    const long long N = (long long)(blk->nx1 + 2 * blk->ng) * (blk->ndim >= 2 ? blk->nx2 + 2 * blk->ng : 1) *
                        (blk->ndim >= 3 ? blk->nx3 + 2 * blk->ng : 1);
    if (blk->var_stride != 0 && blk->var_stride < N)
      return reject(PHX_ERR_INVALID_ARG, "phx_estimate_timestep_static: var_stride smaller than the block");
  }
  const long long n = (long long)blk->nx1 * (blk->ndim >= 2 ? blk->nx2 : 1) * (blk->ndim >= 3 ? blk->nx3 : 1);
  if (n > PHX_DT_STATIC_MAX_ZONES)
    return reject(PHX_ERR_CAPACITY,
                  "phx_estimate_timestep_static: block has more than PHX_DT_STATIC_MAX_ZONES (16777216) interior "
                  "zones; use phx_estimate_timestep");
  double *scratch = nullptr;
  phx_status s = scratch_address(&scratch);
  if (s != PHX_OK) return s;
  phx::BView v{};
  v.ndim = blk->ndim;
  v.ng = blk->ng;
  v.nx1 = blk->nx1;
  v.nx2 = blk->nx2;
  v.nx3 = blk->nx3;
  v.n1t = blk->nx1 + 2 * blk->ng;
  v.n2t = blk->ndim >= 2 ? blk->nx2 + 2 * blk->ng : 1;
  v.n3t = blk->ndim >= 3 ? blk->nx3 + 2 * blk->ng : 1;
  const long long N = (long long)v.n1t * v.n2t * v.n3t;
  v.vs = blk->var_stride ? blk->var_stride : N;
  v.dx[0] = blk->dx1;
  v.dx[1] = blk->dx2;
  v.dx[2] = blk->dx3;
  v.cell_sig = blk->cell_sig;
  v.face_sig = blk->face_sig;
  const int nparts = (int)((n + kThreads - 1) / kThreads);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  k_dt_partials<<<nparts, kThreads, 0, st>>>(v, use_face_speeds, scratch, n);
  k_dt_finish<<<1, 1024, 0, st>>>(scratch, nparts, p->cfl, dt_out_device);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return reject(PHX_ERR_CUDA, "phx_estimate_timestep_static: launch failed");
  return PHX_OK;
}

}  // extern "C"
