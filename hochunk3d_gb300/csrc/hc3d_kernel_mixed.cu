// Mixed-precision instantiation of the transport kernel (FP32 walk, scatter,
// peel and Stokes; FP64 position, radial quadratic, peel escape tau and the
// per-event table lookups).
#include "hc3d_transport.cuh"

namespace hc3d {

cudaError_t launch_transport_mixed(const DevModel& m, const DevTallies& t, const TallyDims& d, const RunArgs& a,
                                   const LaunchCfg& cfg) {
  dev::k_transport<float><<<cfg.blocks, cfg.threads, m.dust_smem, cfg.stream>>>(m, t, d, a);
  return cudaGetLastError();
}

int transport_regs_mixed() {
  cudaFuncAttributes attr;
  if (cudaFuncGetAttributes(&attr, dev::k_transport<float>) != cudaSuccess) return -1;
  return attr.numRegs;
}

const void* transport_fn_mixed() { return (const void*)dev::k_transport<float>; }

cudaError_t launch_transport_batch_mixed(const BatchItem* items, const int64_t* first, int n, unsigned long long* work,
                                         int64_t total, const LaunchCfg& cfg) {
  dev::k_transport_batch<float><<<cfg.blocks, cfg.threads, 0, cfg.stream>>>(items, first, n, work, total);
  return cudaGetLastError();
}

const void* transport_batch_fn_mixed() { return (const void*)dev::k_transport_batch<float>; }

}  // namespace hc3d

namespace hc3d {

cudaError_t launch_wave_transport_mixed(const DevModel& m, const DevTallies& t, const TallyDims& d, const RunArgs& a,
                                        const WaveBufs& w, int q, int E, const LaunchCfg& cfg) {
  dev::k_wave<float><<<cfg.blocks, cfg.threads, m.dust_smem, cfg.stream>>>(
      m, t, d, a, static_cast<dev::Slot<float>*>(w.pool), static_cast<dev::PeelRec<float>*>(w.queue[q]), w.qcount[q], E,
      w.alive);
  return cudaGetLastError();
}

// the block shapes of k_peel_mixed: (threads, blocks per SM at launch bounds)
constexpr int kPeelShapes[kPeelVariants][2] = {{128, 5}, {192, 3}};

cudaError_t launch_wave_peel_mixed(const DevModel& m, const DevTallies& t, const TallyDims& d, const RunArgs& a,
                                   const WaveBufs& w, int q, const LaunchCfg& cfg) {
  const auto* qu = static_cast<const dev::PeelRec<float>*>(w.queue[q]);
  switch (cfg.variant) {
    case 1:
      dev::k_peel_mixed<float, 192, 3><<<cfg.blocks, 192, 0, cfg.stream>>>(m, t, d, a, qu, w.qcount[q], w.next_ray[q]);
      break;
    default:
      dev::k_peel_mixed<float, 128, 5><<<cfg.blocks, 128, 0, cfg.stream>>>(m, t, d, a, qu, w.qcount[q], w.next_ray[q]);
  }
  return cudaGetLastError();
}

int peel_threads_mixed(int variant) { return kPeelShapes[variant < 0 || variant >= kPeelVariants ? 0 : variant][0]; }

size_t slot_bytes_mixed() { return sizeof(dev::Slot<float>); }
size_t rec_bytes_mixed() { return sizeof(dev::PeelRec<float>); }
const void* wave_fn_mixed() { return (const void*)dev::k_wave<float>; }
const void* peel_fn_mixed(int variant) {
  switch (variant) {
    case 1: return (const void*)dev::k_peel_mixed<float, 192, 3>;
    default: return (const void*)dev::k_peel_mixed<float, 128, 5>;
  }
}

}  // namespace hc3d
