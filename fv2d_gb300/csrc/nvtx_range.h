// nvtx_range.h -- NVTX ranges around the library's host-side stages
// (set-up, dt, update, device-driven loop, server replays), visible to
// profilers; the header-only NVTX3 API costs nothing without one attached.
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace fv2d {

struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

}  // namespace fv2d
