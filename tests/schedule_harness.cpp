// Runs the service's scheduling choices (fv2d_gb300/csrc/schedule.hpp) on
// cases read from stdin.
//   schedule_harness         per case a line "n cap" then n lines "slot
//                            remaining cells"; prints the chosen slots of each
//                            case on one line (select_active).
//   schedule_harness band    per case a line "n warps" then n lines "strips
//                            Ny"; prints the band height of each case
//                            (choose_band).
#include <cstdio>
#include <cstring>
#include <vector>

#include "../fv2d_gb300/csrc/schedule.hpp"

int main(int argc, char **argv) {
  if (argc > 1 && !std::strcmp(argv[1], "band")) {
    int n;
    double warps;
    while (std::scanf("%d %lf", &n, &warps) == 2) {
      std::vector<fv2d::BandGrid> g(n);
      for (auto &x : g)
        if (std::scanf("%d %d", &x.strips, &x.Ny) != 2) return 2;
      std::printf("%d\n", fv2d::choose_band(g, warps));
    }
    return 0;
  }
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
