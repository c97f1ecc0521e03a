// step_fslp.cu -- instantiations of the fused FP64 step for the FSLP solver
// (one translation unit per solver so that they compile in parallel).
#include "step_kernel.cuh"

namespace fv2d {

namespace {
template <int RECON, bool VISC>
cudaError_t attr() {
  return cudaFuncSetAttribute(step_kernel<RECON, RS_FSLP, VISC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)Smem<RECON, VISC>::BYTES);
}
template <bool VISC>
void launch(int recon, dim3 grid, cudaStream_t s, const CUtensorMap &t0, const CUtensorMap &t1, const StepArgs &a) {
  switch (recon) {
    case RECON_PLM:
      step_kernel<RECON_PLM, RS_FSLP, VISC><<<grid, NT, Smem<RECON_PLM, VISC>::BYTES, s>>>(t0, t1, a);
      break;
    case RECON_MH:
      step_kernel<RECON_MH, RS_FSLP, VISC><<<grid, NT, Smem<RECON_MH, VISC>::BYTES, s>>>(t0, t1, a);
      break;
    default:
      step_kernel<RECON_PCM, RS_FSLP, VISC><<<grid, NT, Smem<RECON_PCM, VISC>::BYTES, s>>>(t0, t1, a);
      break;
  }
}
}  // namespace

cudaError_t set_step_attrs_fslp() {
  cudaError_t e = attr<RECON_PCM, false>();
  if (e == cudaSuccess) e = attr<RECON_PLM, false>();
  if (e == cudaSuccess) e = attr<RECON_MH, false>();
  if (e == cudaSuccess) e = attr<RECON_PCM, true>();
  if (e == cudaSuccess) e = attr<RECON_PLM, true>();
  if (e == cudaSuccess) e = attr<RECON_MH, true>();
  return e;
}

// the viscous terms are a separate instantiation: kernels without them keep
// their registers and shared memory
cudaError_t launch_step_fslp(int recon, dim3 grid, cudaStream_t s, const CUtensorMap &t0, const CUtensorMap &t1,
                            const StepArgs &a) {
  if (a.visc)
    launch<true>(recon, grid, s, t0, t1, a);
  else
    launch<false>(recon, grid, s, t0, t1, a);
  return cudaGetLastError();
}

}  // namespace fv2d
