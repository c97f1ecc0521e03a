// batch_kernels.cu -- the tile configurations of the batched FP32 step that
// the autotuner chooses from (tile shape, threads per CTA, halo staging).
// Compiled with fast single-precision math: the service's tolerance is set
// against the binary64 path, not bit parity.
#include "batch_kernel.cuh"
#include "batch_march.cuh"

namespace fv2d {

struct BatchCfg {
  int tx, ty, nt, staging;
  int ext;  // 1: the extended family (batch_march_ext_kernel)
  const char *name;
  size_t smem;
  const void *fn;
};

#define FV2D_CFG(TX, TY, NT, ST, NAME) \
  {TX, TY, NT, ST, 0, NAME, BatchSmem<TX, TY>::BYTES, (const void *)batch_step_kernel<TX, TY, NT, ST>}

// Column-marching configurations (batch_march.cuh): 28 interior columns per
// warp, H rows per work item, no shared memory (staging code 2).
// MINB caps the registers so that MINB CTAs fit on an SM.
#define FV2D_MARCH(H, NT, MINB, NAME) \
  {bm::STRIP, H, NT, 2, 0, NAME, 0, (const void *)batch_march_kernel<H, NT, MINB>}
// The extended family (FSLP, MUSCL-Hancock, per-row tables, boundary fluxes).
#define FV2D_MARCH_EXT(H, NT, MINB, NAME) \
  {bm::STRIP, H, NT, 2, 1, NAME, 0, (const void *)batch_march_ext_kernel<H, NT, MINB>}

static const BatchCfg kCfgs[] = {
    FV2D_CFG(32, 8, 128, 0, "32x8/128/ldg"),
    FV2D_CFG(32, 16, 256, 0, "32x16/256/ldg"),
    FV2D_CFG(32, 16, 256, 1, "32x16/256/tma"),
    FV2D_CFG(32, 32, 256, 1, "32x32/256/tma"),
    FV2D_CFG(32, 32, 512, 0, "32x32/512/ldg"),
    FV2D_CFG(64, 16, 256, 1, "64x16/256/tma"),
    FV2D_MARCH(32, 128, 4, "28x32/128/march"),
    FV2D_MARCH(64, 128, 4, "28x64/128/march"),
    FV2D_MARCH(32, 128, 5, "28x32/128x5/march"),
    FV2D_MARCH(64, 128, 5, "28x64/128x5/march"),
    FV2D_MARCH(32, 64, 8, "28x32/64/march"),
    FV2D_MARCH(64, 64, 8, "28x64/64/march"),
    FV2D_MARCH(64, 96, 5, "28x64/96/march"),
    FV2D_MARCH(16, 64, 8, "28x16/64/march"),
    FV2D_MARCH(16, 128, 4, "28x16/128/march"),
    FV2D_MARCH(32, 32, 16, "28x32/32/march"),
    FV2D_MARCH(32, 64, 10, "28x32/64x10/march"),
    FV2D_MARCH(32, 32, 20, "28x32/32x20/march"),
    FV2D_MARCH_EXT(32, 64, 8, "28x32/64/march-ext"),
    FV2D_MARCH_EXT(16, 64, 8, "28x16/64/march-ext"),
};

// the service sizes its per-configuration tables for at most 32 entries
static_assert(sizeof(kCfgs) / sizeof(kCfgs[0]) <= 32, "more tile configurations than the service's tables hold");

int batch_num_cfgs() { return (int)(sizeof(kCfgs) / sizeof(kCfgs[0])); }

void batch_cfg_info(int i, int *tx, int *ty, int *nt, int *staging, size_t *smem, const char **name, int *ext) {
  const BatchCfg &c = kCfgs[i];
  if (ext) *ext = c.ext;
  if (tx) *tx = c.tx;
  if (ty) *ty = c.ty;
  if (nt) *nt = c.nt;
  if (staging) *staging = c.staging;
  if (smem) *smem = c.smem;
  if (name) *name = c.name;
}

// Sets the shared-memory limit and returns resident CTAs per SM.
cudaError_t batch_setup(int i, int *ctas_per_sm) {
  const BatchCfg &c = kCfgs[i];
  cudaError_t e = cudaFuncSetAttribute(c.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c.smem);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, c.fn, c.nt, c.smem);
}

cudaError_t batch_launch(int i, int grid, cudaStream_t s, const BatchArgs &a) {
  const BatchCfg &c = kCfgs[i];
  void *args[] = {(void *)&a};
  return cudaLaunchKernel(c.fn, dim3(grid), dim3(c.nt), args, c.smem, s);
}

}  // namespace fv2d
