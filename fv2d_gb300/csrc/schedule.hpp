// schedule.hpp -- the service's scheduling choices: which resident requests
// advance at the next steps (shortest remaining work first), and how tall the
// march kernels' work items of a lane are.
#pragma once

#include <algorithm>
#include <vector>

namespace fv2d {

struct Candidate {
  int slot;          // simulation-table slot
  double remaining;  // remaining cell-updates (remaining steps x cells)
  double cells;      // cells advanced per step
};

// With cap <= 0 every candidate advances.  Otherwise the candidates are taken
// in order of least remaining work (ties: lower slot first) while the cells
// already taken are below `cap`: at least one advances, and the total exceeds
// the cap by less than the last one taken.  Returns the chosen slots in
// increasing order.
inline std::vector<int> select_active(std::vector<Candidate> c, double cap) {
  std::vector<int> run;
  run.reserve(c.size());
  if (cap > 0) {
    std::sort(c.begin(), c.end(), [](const Candidate &a, const Candidate &b) {
      return a.remaining < b.remaining || (a.remaining == b.remaining && a.slot < b.slot);
    });
    double cells = 0;
    for (const Candidate &x : c) {
      if (!run.empty() && cells >= cap) break;
      run.push_back(x.slot);
      cells += x.cells;
    }
  } else {
    for (const Candidate &x : c) run.push_back(x.slot);
  }
  std::sort(run.begin(), run.end());
  return run;
}

// Band heights the march lanes choose from (rows per work item), tallest
// first, and the work items per resident warp a lane's launch should have.
constexpr int kBands[] = {32, 24, 16, 12, 8};
constexpr int kMinBand = 8;
constexpr double kItemsPerWarp = 2.0;

// One simulation of a lane: its strips of columns and its interior rows.
struct BandGrid {
  int strips;
  int Ny;
};

// Band height of a march lane for the simulations it is about to run: the
// tallest of kBands that gives the launch at least kItemsPerWarp work items
// per resident warp, else the shortest.  Measured on single grids (one
// simulation in the lane; KH 4096^2 and RT 1024 x 3072, bands 12..64) and on
// batches of 12 and 40 Sedov 768^2 grids: the rate falls by 10-20 % when the
// items end within one or a little over one wave of the resident warps (the
// last warps run alone, or every warp runs its one item in step with the
// others), by a few per cent still at 1.5 items per warp, while the extra
// window fill of a shorter band costs a few per cent; bands taller than 32
// rows gained nothing where the items were plentiful and lost 9 % at 64.
inline int choose_band(const std::vector<BandGrid> &grids, double resident_warps) {
  for (int H : kBands) {
    double items = 0;
    for (const BandGrid &g : grids) items += (double)g.strips * ((g.Ny + H - 1) / H);
    if (items >= kItemsPerWarp * resident_warps) return H;
  }
  return kMinBand;
}

}  // namespace fv2d
