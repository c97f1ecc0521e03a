// batch_cfg.h -- one launch configuration of the batched FP32 step (the
// autotuner's candidates).
#pragma once

#include <stddef.h>

namespace fv2d {

struct BatchCfg {
  int tx, ty, nt, staging;  // work item columns x rows, threads per CTA, staging (0 ldg, 1 TMA, 2 march)
  int fams;                 // kernel families it runs (bit FAM_*)
  const char *name;
  size_t smem;
  const void *fn;
};

// The two-column march configurations (batch_march2.cu).
const BatchCfg *batch_march2_cfgs(int *n);

}  // namespace fv2d
