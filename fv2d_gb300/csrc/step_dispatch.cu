// step_dispatch.cu -- selects the fused-step instantiation for a
// (Riemann solver, reconstruction) pair.
#include "step_kernel.cuh"

namespace fv2d {

cudaError_t set_step_attrs_hll();
cudaError_t set_step_attrs_hllc();
cudaError_t set_step_attrs_fslp();
cudaError_t launch_step_hll(int, dim3, cudaStream_t, const CUtensorMap &, const CUtensorMap &, const StepArgs &);
cudaError_t launch_step_hllc(int, dim3, cudaStream_t, const CUtensorMap &, const CUtensorMap &, const StepArgs &);
cudaError_t launch_step_fslp(int, dim3, cudaStream_t, const CUtensorMap &, const CUtensorMap &, const StepArgs &);

cudaError_t init_step_kernels() {
  static cudaError_t done = cudaErrorNotReady;
  if (done == cudaErrorNotReady) {
    cudaError_t e = set_step_attrs_hll();
    if (e == cudaSuccess) e = set_step_attrs_hllc();
    if (e == cudaSuccess) e = set_step_attrs_fslp();
    done = e;
  }
  return done;
}

cudaError_t launch_step(int rs, int recon, dim3 grid, cudaStream_t s, const CUtensorMap &t0, const CUtensorMap &t1,
                        const StepArgs &a) {
  switch (rs) {
    case 0: return launch_step_hll(recon, grid, s, t0, t1, a);
    case 2: return launch_step_fslp(recon, grid, s, t0, t1, a);
    default: return launch_step_hllc(recon, grid, s, t0, t1, a);
  }
}

cudaError_t launch_commit(cudaStream_t s, const StepArgs &a) {
  commit_kernel<<<1, 1, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace fv2d
