// Runs the service's scheduling choice (fv2d_gb300/csrc/schedule.hpp) on
// cases read from stdin: per case a line "n cap" then n lines "slot remaining
// cells"; prints the chosen slots of each case on one line.
#include <cstdio>
#include <vector>

#include "../fv2d_gb300/csrc/schedule.hpp"

int main() {
  int n;
  double cap;
  while (std::scanf("%d %lf", &n, &cap) == 2) {
    std::vector<fv2d::Candidate> c(n);
    for (auto &x : c)
      if (std::scanf("%d %lf %lf", &x.slot, &x.remaining, &x.cells) != 3) return 2;
    const std::vector<int> run = fv2d::select_active(c, cap);
    for (size_t k = 0; k < run.size(); ++k) std::printf(k ? " %d" : "%d", run[k]);
    std::printf("\n");
  }
  return 0;
}
