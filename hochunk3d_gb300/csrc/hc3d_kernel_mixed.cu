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

cudaError_t launch_wave_mixed(const DevModel& m, const DevTallies& t, const TallyDims& d, const RunArgs& a,
                              const WaveBufs& w, int E, const LaunchCfg& wave, const LaunchCfg& peel,
                              cudaEvent_t ev[3]) {
  cudaError_t e;
  if (ev && (e = cudaEventRecord(ev[0], wave.stream)) != cudaSuccess) return e;
  dev::k_wave<float><<<wave.blocks, wave.threads, m.dust_smem, wave.stream>>>(
      m, t, d, a, static_cast<dev::Slot<float>*>(w.pool), static_cast<dev::PeelRec<float>*>(w.queue), w.qcount, E, w.alive);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (ev && (e = cudaEventRecord(ev[1], wave.stream)) != cudaSuccess) return e;
  dev::k_peel_mixed<float><<<peel.blocks, dev::kPeelThreads, 0, peel.stream>>>(
      m, t, d, a, static_cast<const dev::PeelRec<float>*>(w.queue), w.qcount, w.next_ray);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (ev && (e = cudaEventRecord(ev[2], wave.stream)) != cudaSuccess) return e;
  return cudaSuccess;
}

size_t slot_bytes_mixed() { return sizeof(dev::Slot<float>); }
size_t rec_bytes_mixed() { return sizeof(dev::PeelRec<float>); }
const void* wave_fn_mixed() { return (const void*)dev::k_wave<float>; }
const void* peel_fn_mixed() { return (const void*)dev::k_peel_mixed<float>; }

}  // namespace hc3d
