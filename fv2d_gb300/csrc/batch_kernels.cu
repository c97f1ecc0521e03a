// batch_kernels.cu -- the launch configurations of the batched FP32 step that
// the autotuner chooses from (tile shape, threads per CTA, halo staging),
// and their launch.
// Compiled with fast single-precision math: the service's tolerance is set
// against the binary64 path, not bit parity.
#include <vector>

#include "batch_cfg.h"
#include "batch_kernel.cuh"
#include "batch_march.cuh"

namespace fv2d {

constexpr int kCommon = (1 << FAM_PLAIN) | (1 << FAM_DIFF);

#define FV2D_CFG(TX, TY, NT, ST, NAME) \
  {TX, TY, NT, ST, kCommon, NAME, BatchSmem<TX, TY>::BYTES, (const void *)batch_step_kernel<TX, TY, NT, ST>}

// Column-marching configurations (batch_march.cuh): 28 interior columns per
// warp, no shared memory (staging code 2).  H is the default band height (the
// service sets each lane's band); MINB caps the registers so that MINB CTAs
// fit on an SM.
#define FV2D_MARCH(H, NT, MINB, NAME) \
  {bm::STRIP, H, NT, 2, kCommon, NAME, 0, (const void *)batch_march_kernel<NT, MINB>}
// The extended family (FSLP, MUSCL-Hancock, per-row tables, boundary fluxes).
#define FV2D_MARCH_EXT(H, NT, MINB, NAME) \
  {bm::STRIP, H, NT, 2, 1 << FAM_EXT, NAME, 0, (const void *)batch_march_ext_kernel<NT, MINB>}

static const BatchCfg kCfgs[] = {
    FV2D_CFG(32, 8, 128, 0, "32x8/128/ldg"),
    FV2D_CFG(32, 16, 256, 0, "32x16/256/ldg"),
    FV2D_CFG(32, 16, 256, 1, "32x16/256/tma"),
    FV2D_CFG(32, 32, 256, 1, "32x32/256/tma"),
    FV2D_CFG(32, 32, 512, 0, "32x32/512/ldg"),
    FV2D_CFG(64, 16, 256, 1, "64x16/256/tma"),
    // named <strip columns>/<threads per CTA>x<CTAs per SM>/march
    FV2D_MARCH(32, 128, 4, "28/128x4/march"),
    FV2D_MARCH(32, 128, 5, "28/128x5/march"),
    FV2D_MARCH(32, 96, 5, "28/96x5/march"),
    FV2D_MARCH(32, 64, 8, "28/64x8/march"),
    FV2D_MARCH(32, 64, 10, "28/64x10/march"),
    FV2D_MARCH(32, 32, 16, "28/32x16/march"),
    FV2D_MARCH(32, 32, 20, "28/32x20/march"),
    FV2D_MARCH_EXT(32, 64, 8, "28/64x8/march-ext"),
};

// Every configuration: the table above, then the two-column march's.
static const std::vector<BatchCfg> &all_cfgs() {
  static const std::vector<BatchCfg> v = [] {
    std::vector<BatchCfg> c(kCfgs, kCfgs + sizeof(kCfgs) / sizeof(kCfgs[0]));
    int n = 0;
    const BatchCfg *m2 = batch_march2_cfgs(&n);
    c.insert(c.end(), m2, m2 + n);
    return c;
  }();
  return v;
}

int batch_num_cfgs() { return (int)all_cfgs().size(); }

void batch_cfg_info(int i, int *tx, int *ty, int *nt, int *staging, size_t *smem, const char **name, int *fams) {
  const BatchCfg &c = all_cfgs()[i];
  if (fams) *fams = c.fams;
  if (tx) *tx = c.tx;
  if (ty) *ty = c.ty;
  if (nt) *nt = c.nt;
  if (staging) *staging = c.staging;
  if (smem) *smem = c.smem;
  if (name) *name = c.name;
}

// Sets the shared-memory limit and returns resident CTAs per SM.
cudaError_t batch_setup(int i, int *ctas_per_sm) {
  const BatchCfg &c = all_cfgs()[i];
  cudaError_t e = cudaFuncSetAttribute(c.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c.smem);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, c.fn, c.nt, c.smem);
}

cudaError_t batch_launch(int i, int grid, cudaStream_t s, const BatchArgs &a) {
  const BatchCfg &c = all_cfgs()[i];
  void *args[] = {(void *)&a};
  return cudaLaunchKernel(c.fn, dim3(grid), dim3(c.nt), args, c.smem, s);
}

}  // namespace fv2d
