// All-FP64 instantiation of the transport kernel.  This translation unit is
// compiled with --fmad=false: multiplies and adds round separately, as in the
// CPU restatement, so the two can be compared packet by packet.
#include "hc3d_transport.cuh"

namespace hc3d {

cudaError_t launch_transport_fp64(const DevModel& m, const DevTallies& t, const TallyDims& d, const RunArgs& a,
                                  const LaunchCfg& cfg) {
  dev::k_transport<double><<<cfg.blocks, cfg.threads, m.dust_smem, cfg.stream>>>(m, t, d, a);
  return cudaGetLastError();
}

int transport_regs_fp64() {
  cudaFuncAttributes attr;
  if (cudaFuncGetAttributes(&attr, dev::k_transport<double>) != cudaSuccess) return -1;
  return attr.numRegs;
}

const void* transport_fn_fp64() { return (const void*)dev::k_transport<double>; }

cudaError_t launch_transport_batch_fp64(const BatchItem* items, const int64_t* first, int n, unsigned long long* work,
                                         int64_t total, const LaunchCfg& cfg) {
  dev::k_transport_batch<double><<<cfg.blocks, cfg.threads, 0, cfg.stream>>>(items, first, n, work, total);
  return cudaGetLastError();
}

const void* transport_batch_fn_fp64() { return (const void*)dev::k_transport_batch<double>; }

}  // namespace hc3d

namespace hc3d {

cudaError_t launch_wave_transport_fp64(const DevModel& m, const DevTallies& t, const TallyDims& d, const RunArgs& a,
                                        const WaveBufs& w, int q, int E, const LaunchCfg& cfg) {
  dev::k_wave<double><<<cfg.blocks, cfg.threads, m.dust_smem, cfg.stream>>>(
      m, t, d, a, static_cast<dev::Slot<double>*>(w.pool), static_cast<dev::PeelRec<double>*>(w.queue[q]), w.qcount[q], E,
      w.alive);
  return cudaGetLastError();
}

cudaError_t launch_wave_peel_fp64(const DevModel& m, const DevTallies& t, const TallyDims& d, const RunArgs& a,
                                   const WaveBufs& w, int q, const LaunchCfg& cfg) {
  dev::k_peel<double><<<cfg.blocks, cfg.threads, 0, cfg.stream>>>(
      m, t, d, a, static_cast<const dev::PeelRec<double>*>(w.queue[q]), w.qcount[q], w.next_ray[q]);
  return cudaGetLastError();
}

size_t slot_bytes_fp64() { return sizeof(dev::Slot<double>); }
size_t rec_bytes_fp64() { return sizeof(dev::PeelRec<double>); }
const void* wave_fn_fp64() { return (const void*)dev::k_wave<double>; }
const void* peel_fn_fp64() { return (const void*)dev::k_peel<double>; }

}  // namespace hc3d
