// All-FP64 instantiation of the transport kernel.  This translation unit is
// compiled with --fmad=false: multiplies and adds round separately, as in the
// CPU restatement, so the two can be compared packet by packet.
#include "hc3d_transport.cuh"

namespace hc3d {

cudaError_t launch_transport_fp64(const DevModel& m, const DevTallies& t, const TallyDims& d, const RunArgs& a,
                                  const LaunchCfg& cfg) {
  dev::k_transport<double><<<cfg.blocks, cfg.threads, 0, cfg.stream>>>(m, t, d, a);
  return cudaGetLastError();
}

int transport_regs_fp64() {
  cudaFuncAttributes attr;
  if (cudaFuncGetAttributes(&attr, dev::k_transport<double>) != cudaSuccess) return -1;
  return attr.numRegs;
}

const void* transport_fn_fp64() { return (const void*)dev::k_transport<double>; }

}  // namespace hc3d
