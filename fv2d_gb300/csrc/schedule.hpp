// schedule.hpp -- which resident requests of the service advance at the next
// steps: shortest remaining work first.
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

}  // namespace fv2d
