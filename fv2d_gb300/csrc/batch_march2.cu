// batch_march2.cu -- launch configurations of the two-column march
// (batch_march2.cuh), compiled apart from the other batch kernels so that
// the two build in parallel.  Fast single-precision math, like them.
#include "batch_cfg.h"
#include "batch_march2.cuh"

namespace fv2d {

// 60 interior columns per warp, no shared memory (staging code 2); H is the
// default band height (the service sets each lane's band), MINB caps the
// registers so that MINB CTAs fit on an SM.
#define FV2D_MARCH2(H, NT, MINB, NAME) \
  {bm2::STRIP, H, NT, 2, 1 << FAM_PLAIN, NAME, 0, (const void *)batch_march2_kernel<NT, MINB, false>}
#define FV2D_MARCH2_DIFF(H, NT, MINB, NAME) \
  {bm2::STRIP, H, NT, 2, 1 << FAM_DIFF, NAME, 0, (const void *)batch_march2_kernel<NT, MINB, true>}

static const BatchCfg kMarch2[] = {
    // named <strip columns>/<threads per CTA>x<CTAs per SM>/march2[-diff]
    FV2D_MARCH2(32, 32, 16, "60/32x16/march2"),
    FV2D_MARCH2(32, 32, 12, "60/32x12/march2"),
    // the diffusive body measured slower than the one-column march on the
    // Rayleigh-Taylor set-up (31.8 against 37.2 G cell-updates/s at
    // 1024 x 3072); kept as a candidate for other devices and mixes
    FV2D_MARCH2_DIFF(32, 32, 10, "60/32x10/march2-diff"),
};

const BatchCfg *batch_march2_cfgs(int *n) {
  *n = (int)(sizeof(kMarch2) / sizeof(kMarch2[0]));
  return kMarch2;
}

}  // namespace fv2d
