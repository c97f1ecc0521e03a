// step_hllc.cu -- instantiations of the fused FP64 step for the HLLC solver
// (one translation unit per solver so that they compile in parallel).
#include "step_kernel.cuh"

namespace fv2d {

cudaError_t set_step_attrs_hllc() {
  cudaError_t e = cudaFuncSetAttribute(step_kernel<RECON_PCM, RS_HLLC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)Smem<RECON_PCM>::BYTES);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(step_kernel<RECON_PLM, RS_HLLC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)Smem<RECON_PLM>::BYTES);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(step_kernel<RECON_MH, RS_HLLC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)Smem<RECON_MH>::BYTES);
  return e;
}

cudaError_t launch_step_hllc(int recon, dim3 grid, cudaStream_t s, const CUtensorMap &t0, const CUtensorMap &t1,
                            const StepArgs &a) {
  switch (recon) {
    case RECON_PLM:
      step_kernel<RECON_PLM, RS_HLLC><<<grid, NT, Smem<RECON_PLM>::BYTES, s>>>(t0, t1, a);
      break;
    case RECON_MH:
      step_kernel<RECON_MH, RS_HLLC><<<grid, NT, Smem<RECON_MH>::BYTES, s>>>(t0, t1, a);
      break;
    default:
      step_kernel<RECON_PCM, RS_HLLC><<<grid, NT, Smem<RECON_PCM>::BYTES, s>>>(t0, t1, a);
      break;
  }
  return cudaGetLastError();
}

}  // namespace fv2d
