// io_api.cpp -- C-ABI of the .ini and snapshot functions (include/fv2d_io.h).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <new>
#include <string>
#include <vector>

#include "../../include/fv2d_io.h"
#include "h5.hpp"
#include "ini.hpp"

using namespace fv2d;

namespace {
void set_err(char *err, int len, const std::string &m) {
  if (err && len > 0) {
    std::strncpy(err, m.c_str(), (size_t)len - 1);
    err[len - 1] = '\0';
  }
}
// Runs f and turns any exception into a status code: none crosses the C ABI.
template <class F>
int guarded(char *err, int errlen, F &&f) {
  try {
    return f();
  } catch (const std::bad_alloc &) {
    set_err(err, errlen, "out of host memory");
    return FV2D_ERR_NOMEM;
  } catch (const std::exception &e) {
    set_err(err, errlen, e.what());
    return FV2D_ERR_INVALID;
  }
}

void copy_str(char *dst, size_t cap, const std::string &s) {
  std::strncpy(dst, s.c_str(), cap - 1);
  dst[cap - 1] = '\0';
}
h5::RootInfo root_info(const fv2d_params &p, const char *problem) {
  h5::RootInfo r;
  const int Ng = p.Nghosts;
  r.Nx = p.Nx;
  r.Ny = p.Ny;
  r.Ntx = p.Nx + 2 * Ng;
  r.Nty = p.Ny + 2 * Ng;
  r.ibeg = Ng;
  r.iend = Ng + p.Nx;
  r.jbeg = Ng;
  r.jend = Ng + p.Ny;
  r.problem = problem ? problem : "";
  r.xmin = p.xmin;
  r.ymin = p.ymin;
  r.dx = (p.xmax - p.xmin) / p.Nx;
  r.dy = (p.ymax - p.ymin) / p.Ny;
  return r;
}
}  // namespace

extern "C" {

int fv2d_read_ini(const char *path, fv2d_params *p, fv2d_run_config *run, char *err, int errlen) {
  if (!path || !p || !run) return FV2D_ERR_INVALID;
  return guarded(err, errlen, [&]() -> int {
    IniFile ini(path);
    if (ini.error() < 0) {
      set_err(err, errlen, std::string("cannot open ") + path);
      return FV2D_ERR_INVALID;
    }
    ParamReader reader(std::move(ini));
    RunConfig rc;
    read_ini(reader, p, &rc);
    reader.check_validity(std::cerr);
    // a string that does not fit its fixed field is refused, never cut short
    // (a shortened output path would write somewhere else)
    const struct {
      char *dst;
      size_t cap;
      const std::string *src;
      const char *key;
    } fields[] = {{run->problem, sizeof run->problem, &rc.problem, "[physics] problem"},
                  {run->output_filename, sizeof run->output_filename, &rc.filename_out, "[run] output_filename"},
                  {run->output_path, sizeof run->output_path, &rc.output_path, "[run] output_path"},
                  {run->restart_file, sizeof run->restart_file, &rc.restart_file, "[run] restart_file"}};
    for (const auto &f : fields)
      if (f.src->size() >= f.cap) {
        set_err(err, errlen, std::string(f.key) + " is longer than " + std::to_string(f.cap - 1) + " bytes");
        return FV2D_ERR_SIZE;
      }
    std::memset(run, 0, sizeof(*run));
    for (const auto &f : fields) copy_str(f.dst, f.cap, *f.src);
    run->multiple_outputs = rc.multiple_outputs ? 1 : 0;
    run->problem_id = problem_id(rc.problem);
    return FV2D_OK;
  });
}

int fv2d_write_ini_echo(const char *ini_path, const char *out_path) {
  if (!ini_path || !out_path) return FV2D_ERR_INVALID;
  return guarded(nullptr, 0, [&]() -> int {
    IniFile ini(ini_path);
    if (ini.error() < 0) return FV2D_ERR_INVALID;
    ParamReader reader(std::move(ini));
    fv2d_params p;
    RunConfig rc;
    read_ini(reader, &p, &rc);
    std::ofstream out(out_path);
    if (!out) return FV2D_ERR_INVALID;
    reader.write_echo(out);
    return FV2D_OK;
  });
}

int fv2d_snapshot_write(const char *dir, const char *name, int multiple_outputs, int truncate, const fv2d_params *p,
                        const char *problem, int iteration, double t, const double *q, char *err, int errlen) {
  if (!dir || !name || !p || !q) return FV2D_ERR_INVALID;
  return guarded(err, errlen, [&]() -> int {
    const h5::RootInfo r = root_info(*p, problem);
    std::string e;
    const std::string base = std::string(dir) + "/";
    if (multiple_outputs) {
      char stem[512];
      std::snprintf(stem, sizeof stem, "%s_%04d", name, iteration);
      const std::string h5name = std::string(stem) + ".h5";
      if (!h5::write_multiple(base + h5name, r, iteration, t, q, &e) ||
          !h5::write_xdmf(base + stem + ".xmf", h5name, r, true, false, stem, t, "", &e)) {
        set_err(err, errlen, e);
        return FV2D_ERR_INVALID;
      }
      return FV2D_OK;
    }
    char gname[32];
    std::snprintf(gname, sizeof gname, "ite_%04d", iteration);
    const std::string h5name = std::string(name) + ".h5";
    if (!h5::write_unique(base + h5name, truncate != 0, r, iteration, t, q, &e) ||
        !h5::write_xdmf(base + name + ".xmf", h5name, r, truncate != 0, true, gname, t, std::string(gname) + "/",
                        &e)) {
      set_err(err, errlen, e);
      return FV2D_ERR_INVALID;
    }
    return FV2D_OK;
  });
}

int fv2d_snapshot_read(const char *file, int nx, int ny, double *q, double *t, int *iteration, char *err,
                       int errlen) {
  if (!file || !q || !t || !iteration) return FV2D_ERR_INVALID;
  return guarded(err, errlen, [&]() -> int {
    std::string path(file), group;
    const size_t d = path.find(".h5:/");  // IOManager.h:292-298
    if (d != std::string::npos) {
      group = path.substr(d + 5);
      path.resize(d + 3);
    }
    std::vector<double> v;
    std::string e;
    if (!h5::read_snapshot(path, group, nx, ny, &v, t, iteration, &e)) {
      set_err(err, errlen, e);
      return FV2D_ERR_INVALID;
    }
    std::memcpy(q, v.data(), sizeof(double) * v.size());  // read_snapshot checked nx * ny * 4
    return FV2D_OK;
  });
}

int fv2d_h5_read_doubles(const char *file, const char *dataset, double *out, int64_t max, int64_t *n) {
  if (!file || !dataset || !n || max < 0) return FV2D_ERR_INVALID;
  return guarded(nullptr, 0, [&]() -> int {
    h5::File f;
    std::string e;
    std::vector<double> v;
    std::vector<uint64_t> dims;
    if (!f.open(file, &e) || !f.read_doubles(dataset, &v, &dims, &e)) return FV2D_ERR_INVALID;
    *n = (int64_t)v.size();
    if (out) std::memcpy(out, v.data(), sizeof(double) * (size_t)std::min<int64_t>(max, *n));
    return FV2D_OK;
  });
}

int fv2d_h5_read_attr(const char *file, const char *object, const char *name, double *value) {
  if (!file || !object || !name || !value) return FV2D_ERR_INVALID;
  return guarded(nullptr, 0, [&]() -> int {
    h5::File f;
    std::string e;
    if (!f.open(file, &e) || !f.attr_double(object, name, value, &e)) return FV2D_ERR_INVALID;
    return FV2D_OK;
  });
}

}  // extern "C"
