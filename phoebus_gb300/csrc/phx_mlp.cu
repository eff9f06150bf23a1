// phx_mlp.cu -- learned con2prim starting bracket (placeholder translation
// unit; the network kernels are added here).
#include "phx_kernels.cuh"
namespace phx {}
