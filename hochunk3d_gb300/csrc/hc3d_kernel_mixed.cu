// Mixed-precision instantiation of the transport kernel (FP32 walk, scatter,
// peel and Stokes; FP64 position, radial quadratic, peel escape tau and the
// per-event table lookups).
#include "hc3d_transport.cuh"

namespace hc3d {

cudaError_t launch_transport_mixed(const DevModel& m, const DevTallies& t, const TallyDims& d, const RunArgs& a,
                                   const LaunchCfg& cfg) {
  dev::k_transport<float><<<cfg.blocks, cfg.threads, 0, cfg.stream>>>(m, t, d, a);
  return cudaGetLastError();
}

int transport_regs_mixed() {
  cudaFuncAttributes attr;
  if (cudaFuncGetAttributes(&attr, dev::k_transport<float>) != cudaSuccess) return -1;
  return attr.numRegs;
}

const void* transport_fn_mixed() { return (const void*)dev::k_transport<float>; }

}  // namespace hc3d
