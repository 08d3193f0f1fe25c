// Host launch wrappers of the sampler kernels.  The float64, double-float, float32 and mixed
// instantiations are compiled in separate translation units (sampler_f64.cu, sampler_dd.cu,
// sampler_f32.cu, sampler_mixed.cu) so they build in parallel; the host API (tnsp_capi.cu) and the allocation-free
// entry point (noalloc.cu) call them through these declarations.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "sampler_kernels.cuh"

namespace tnsp {

void launch_sweep_f64(int grid, size_t smem, cudaStream_t st, const Model& md, const Chains& ch, const Slots& sl,
                      void* scratch, const void* ones, int nsweeps, int observe, int rec_base);
void launch_sweep_f32(int grid, size_t smem, cudaStream_t st, const Model& md, const Chains& ch, const Slots& sl,
                      void* scratch, const void* ones, int nsweeps, int observe, int rec_base);
void launch_amplitude_f64(int grid, size_t smem, cudaStream_t st, const Model& md, const Slots& sl, void* scratch,
                          const void* ones, int B, const int32_t* confs, double* out_m, int32_t* out_e,
                          int32_t* status);
void launch_amplitude_f32(int grid, size_t smem, cudaStream_t st, const Model& md, const Slots& sl, void* scratch,
                          const void* ones, int B, const int32_t* confs, double* out_m, int32_t* out_e,
                          int32_t* status);
void launch_sweep_dd(int grid, size_t smem, cudaStream_t st, const Model& md, const Chains& ch, const Slots& sl,
                     void* scratch, const void* ones, int nsweeps, int observe, int rec_base);
void launch_amplitude_dd(int grid, size_t smem, cudaStream_t st, const Model& md, const Slots& sl, void* scratch,
                         const void* ones, int B, const int32_t* confs, double* out_m, int32_t* out_e,
                         int32_t* status);
void launch_sweep_mx(int grid, size_t smem, cudaStream_t st, const Model& md, const Chains& ch, const Slots& sl,
                     void* scratch, const void* ones, int nsweeps, int observe, int rec_base);
void launch_amplitude_mx(int grid, size_t smem, cudaStream_t st, const Model& md, const Slots& sl, void* scratch,
                         const void* ones, int B, const int32_t* confs, double* out_m, int32_t* out_e,
                         int32_t* status);
cudaError_t set_smem_limit_f64(int bytes);
cudaError_t set_smem_limit_mx(int bytes);
cudaError_t set_smem_limit_dd(int bytes);
cudaError_t set_smem_limit_f32(int bytes);
cudaError_t occupancy_f64(int smem_bytes, int* blocks_per_sm);
cudaError_t occupancy_dd(int smem_bytes, int* blocks_per_sm);
cudaError_t occupancy_f32(int smem_bytes, int* blocks_per_sm);
cudaError_t occupancy_mx(int smem_bytes, int* blocks_per_sm);

}  // namespace tnsp
