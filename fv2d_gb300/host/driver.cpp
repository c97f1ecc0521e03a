// driver.cpp -- fv2d_gpu <file.ini> [--device N] [--metrics FILE]
//
// The reference's executable (main.cpp:13-101) on the GB300 path: read the
// .ini, echo it, initialise or restart, then run the main loop
//   while (t + eps < tend) { save if due; dt = computeDt; update; t += dt; }
// with the iterations between snapshots executed on the device
// (fv2d_advance) and the console lines of the reference (dt log every
// log_frequency + 1 iterations, negative-value messages, save notices)
// printed from the per-iteration device log.  --metrics writes the same log
// as JSON lines (one per iteration: t, dt, inverse dts, checkNegatives counts)
// plus one line per device-driven batch with its wall time and throughput.
#include <chrono>
#include <climits>
#include <fstream>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <iostream>
#include <string>
#include <vector>

#include "../../include/fv2d_gpu.h"
#include "../../include/fv2d_io.h"

namespace {

struct Run {
  fv2d_params p;
  fv2d_run_config cfg;
  fv2d_ctx *ctx = nullptr;
  bool force_truncation = false;
  std::vector<double> q;
};

int die(const std::string &msg) {
  std::cerr << msg << std::endl;
  return 1;
}

// IOManager::saveSolution: truncate on the first snapshot of a run or after a
// restart into another file.
bool save(Run &r, int number, double t) {
  if (fv2d_get_prim(r.ctx, r.q.data()) != FV2D_OK) return false;
  const bool truncate = r.force_truncation || number == 0;
  char err[512];
  if (fv2d_snapshot_write(r.cfg.output_path, r.cfg.output_filename, r.cfg.multiple_outputs, truncate ? 1 : 0, &r.p,
                          r.cfg.problem, number, t, r.q.data(), err, sizeof err) != FV2D_OK) {
    std::cerr << err << std::endl;
    return false;
  }
  if (truncate) r.force_truncation = false;
  return true;
}

void print_dt(const Run &r, double t, double inv_hyp, double inv_tc, double inv_visc) {
  std::cout << "Computing dts at (t=" << t << ") : dt_hyp=" << 1.0 / inv_hyp;
  if (r.p.thermal_conductivity_active) std::cout << "; dt_TC=" << 1.0 / inv_tc;
  if (r.p.viscosity_active) std::cout << "; dt_visc=" << 1.0 / inv_visc;
  std::cout << std::endl;
}

void print_counters(double nd, double np, double nn) {
  if (nd > 0) std::cout << "--> negative density: " << (unsigned long long)nd << std::endl;
  if (np > 0) std::cout << "--> negative pressure: " << (unsigned long long)np << std::endl;
  if (nn > 0) std::cout << "--> NaN detected." << std::endl;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc < 2) return die("usage: fv2d_gpu <file.ini> [--device N] [--metrics FILE]");
  int device = 0;
  std::ofstream metrics;
  for (int k = 2; k + 1 < argc; ++k) {
    if (std::string(argv[k]) == "--device") device = std::atoi(argv[k + 1]);
    if (std::string(argv[k]) == "--metrics") {
      metrics.open(argv[k + 1]);
      if (!metrics) return die(std::string("cannot write ") + argv[k + 1]);
      metrics.precision(17);
    }
  }
  std::cout << "fv2d on GB300 (binary64, bit-identical to the reference step)" << std::endl;

  Run r;
  char err[1024];
  if (fv2d_read_ini(argv[1], &r.p, &r.cfg, err, sizeof err) != FV2D_OK) return die(err);
  if (r.cfg.problem_id < 0) return die(std::string("Error unknown problem ") + r.cfg.problem);  // Init.h:303-304

  namespace fs = std::filesystem;
  std::error_code fs_ec;
  if (!fs::exists(r.cfg.output_path, fs_ec)) {  // IOManager.h:84-88
    std::cout << "Output path does not exist, creating directory `" << r.cfg.output_path << "`." << std::endl;
    if (!fs::create_directory(r.cfg.output_path, fs_ec) && fs_ec)
      return die(std::string("cannot create ") + r.cfg.output_path + ": " + fs_ec.message());
  }
  fv2d_write_ini_echo(argv[1], "last.ini");
  fv2d_write_ini_echo(argv[1], (std::string(r.cfg.output_path) + "/" + r.cfg.output_filename + ".ini").c_str());

  if (fv2d_create(&r.p, device, &r.ctx) != FV2D_OK) return die(fv2d_last_error(nullptr));
  r.q.resize((size_t)r.p.Nx * r.p.Ny * 4);
  double t = 0.0, next_save = 0.0;
  int ite = 0;
  const double eps = r.p.epsilon;

  if (r.cfg.restart_file[0]) {  // main.cpp:45-55, IOManager.h:284-398
    std::string file(r.cfg.restart_file);
    const size_t d = file.find(".h5:/");
    const std::string path = d == std::string::npos ? file : file.substr(0, d + 3);
    const std::string out = std::string(r.cfg.output_path) + "/" + r.cfg.output_filename + ".h5";
    std::error_code ec;
    if (!r.cfg.multiple_outputs && fs::exists(out, ec) && fs::equivalent(path, out, ec)) {
      if (d != std::string::npos)
        return die(
            "Invalid restart file : if your restart file and output file are the same, you can only start from the "
            "last iteration.\n\nERROR : Invalid restart_file.");
    } else {
      r.force_truncation = true;
    }
    double time;
    int iteration;
    std::cout << "Loading restart data from hdf5" << std::endl;
    if (fv2d_snapshot_read(r.cfg.restart_file, r.p.Nx, r.p.Ny, r.q.data(), &time, &iteration, err, sizeof err) !=
        FV2D_OK)
      return die(std::string(err) + "\nERROR : Trying to restart from a file with a different resolution !");
    if (fv2d_set_prim(r.ctx, r.q.data()) != FV2D_OK) return die(fv2d_last_error(r.ctx));
    if (time + eps > r.p.tend) {
      std::cerr << "Restart time is greater than end time : " << std::endl
                << "  time: " << time << "\ttend: " << r.p.tend << std::endl
                << std::endl;
      return die("ERROR : restart time is greater than the end time.");
    }
    std::cout << "Restart finished !" << std::endl;
    if (r.force_truncation && !save(r, iteration, time)) return 1;
    t = time;
    ite = iteration;
    std::cout << "Restart at iteration " << ite << " and time " << t << std::endl;
    next_save = t + r.p.save_freq;
    ite++;
    fv2d_set_time(r.ctx, t, 0);
  } else if (fv2d_init_problem(r.ctx, r.cfg.problem_id) != FV2D_OK) {
    return die(fv2d_last_error(r.ctx));
  }

  int next_log = 0;
  bool resumed_after_save = false;
  std::vector<double> rec(6 * 4096);
  long long step_no = 0;
  for (;;) {
    double td = t;  // outputs of fv2d_advance, kept defined when it fails before writing them
    int n = 0, status = FV2D_RUN_NUMERIC;
    const auto w0 = std::chrono::steady_clock::now();
    const int rc = fv2d_advance(r.ctx, 4096, r.p.tend, next_save, resumed_after_save ? 1 : 0, &td, &n, &status);
    const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - w0).count();
    int got = 0;
    fv2d_get_step_log(r.ctx, rec.data(), 4096, &got);
    double itc = 0, iv = 0;
    fv2d_compute_dt(r.ctx, nullptr, nullptr, &itc, &iv);
    if (metrics.is_open()) {
      for (int k = 0; k < got; ++k, ++step_no) {
        const double *e = &rec[6 * k];
        metrics << "{\"step\": " << step_no << ", \"t\": " << e[0] << ", \"dt\": " << e[1] << ", \"inv_dt_hyp\": " << e[2]
                << ", \"inv_dt_tc\": " << itc << ", \"inv_dt_visc\": " << iv << ", \"neg_rho\": " << (long long)e[3]
                << ", \"neg_p\": " << (long long)e[4] << ", \"nan\": " << (long long)e[5] << "}\n";
      }
      const double cells = (double)r.p.Nx * r.p.Ny * got;
      metrics << "{\"batch_steps\": " << got << ", \"wall_s\": " << wall
              << ", \"cell_updates_per_s\": " << (wall > 0 ? cells / wall : 0.0) << "}\n";
      metrics.flush();
    }
    for (int k = 0; k < got; ++k) {
      const double *e = &rec[6 * k];
      if (!(k == 0 && resumed_after_save)) {  // that iteration's dt line preceded the save notice
        if (next_log == 0) print_dt(r, e[0], e[2], itc, iv);
        next_log = next_log == 0 ? r.p.log_frequency : next_log - 1;
      }
      print_counters(e[3], e[4], e[5]);
    }
    resumed_after_save = false;
    t = td;
    if (status == FV2D_RUN_NUMERIC || rc != FV2D_OK) {  // also a device error reported with a save stop
      std::cerr << "stopping: " << fv2d_last_error(r.ctx) << std::endl;
      break;
    }
    if (status == FV2D_RUN_SAVE) {  // main.cpp:64-77: dt line, save, then the update
      double dt = 0, ih = 0, itc_s = 0, iv_s = 0;
      fv2d_compute_dt(r.ctx, &dt, &ih, &itc_s, &iv_s);
      if (next_log == 0) print_dt(r, t, ih, itc_s, iv_s);
      next_log = next_log == 0 ? r.p.log_frequency : next_log - 1;
      std::cout << " - Saving at time " << t << std::endl;
      if (!save(r, ite++, t)) return 1;
      next_save += r.p.save_freq;
      resumed_after_save = true;
      continue;
    }
    if (status == FV2D_RUN_DONE) break;
  }
  std::cout << "Time at end is " << t << std::endl;
  const bool ok = save(r, ite++, t);
  fv2d_destroy(r.ctx);
  return ok ? 0 : 1;
}
