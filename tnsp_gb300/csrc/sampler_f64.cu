// float64 instantiation of the sampler kernels and its host launch wrappers.
#include <mutex>

#include "launch.h"

namespace tnsp {

void launch_sweep_f64(int grid, size_t smem, cudaStream_t st, const Model& md, const Chains& ch, const Slots& sl,
                      void* scratch, const void* ones, int nsweeps, int observe, int rec_base) {
  sweep_kernel<double, double><<<grid, kThreads, smem, st>>>(md, ch, sl, (unsigned char*)scratch, (const double*)ones,
                                                             nsweeps, observe, rec_base);
}

void launch_amplitude_f64(int grid, size_t smem, cudaStream_t st, const Model& md, const Slots& sl, void* scratch,
                          const void* ones, int B, const int32_t* confs, double* out_m, int32_t* out_e,
                          int32_t* status) {
  amplitude_kernel<double, double><<<grid, kThreads, smem, st>>>(md, sl, (unsigned char*)scratch, (const double*)ones,
                                                                 B, confs, out_m, out_e, status);
}

// The limit is a property of the kernel function, shared by every context of the process: it is only
// ever raised, so a context planned with less dynamic shared memory never lowers it under another
// context that launches with more.
cudaError_t set_smem_limit_f64(int bytes) {
  static std::mutex mu;
  static int current = -1;
  std::lock_guard<std::mutex> lock(mu);
  if (bytes <= current) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(sweep_kernel<double, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(sweep_kernel<double, double>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(amplitude_kernel<double, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(amplitude_kernel<double, double>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
  if (e == cudaSuccess) current = bytes;
  return e;
}

cudaError_t occupancy_f64(int smem_bytes, int* blocks_per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, sweep_kernel<double, double>, kThreads, smem_bytes);
}

}  // namespace tnsp
