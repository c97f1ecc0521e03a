// h5.hpp -- the reference's HDF5 snapshot layout (IOManager.h:107-282) and
// restart reading (IOManager.h:284-398), written and read without libhdf5
// (the library is not a dependency here) from the published HDF5 file-format
// specification.
//
// Files written here use the classic format every HDF5 reader accepts:
// superblock version 0, version-1 object headers, groups as symbol tables
// (version-1 B-tree + local heap + symbol-table node), contiguous binary64 /
// int32 datasets, attributes in the object header.  One-file runs
// ("run.h5") hold root attributes Ntx..jend (int32) and problem (string), the
// vertex coordinates x, y, and one group "ite_%04d" per snapshot with rho, u,
// v, prs (Nx*Ny values, j outer) and attributes time (binary64), iteration
// (int32).  Multiple-output runs write the fields and time/iteration at the
// root of "<name>_%04d.h5".  The "problem" attribute is a fixed-length string
// (the reference's HighFive writes a variable-length one; readers see the
// same text).
//
// The reader follows what a restart needs: superblock versions 0-3 (with or
// without a user block), version-1 and version-2 object headers with
// continuation blocks, symbol-table groups (any B-tree depth) and compact
// link messages, contiguous and compact layouts of binary64/binary32 data,
// attribute messages versions 1-3.
#pragma once

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

namespace fv2d {
namespace h5 {

struct RootInfo {
  int Ntx, Nty, Nx, Ny, ibeg, iend, jbeg, jend;
  std::string problem;
  double xmin, ymin, dx, dy;
};

// IOManager.h:191-282: create (truncate == true) or extend run.h5 with group
// ite_%04d holding the interior primitives q (Ny x Nx x {rho,u,v,p}).
bool write_unique(const std::string &path, bool truncate, const RootInfo &root, int iteration, double t,
                  const double *q, std::string *err);

// IOManager.h:107-189: one file per snapshot.
bool write_multiple(const std::string &path, const RootInfo &root, int iteration, double t, const double *q,
                    std::string *err);

// IOManager.h:284-351: restart data.  group == "" selects, for one-file runs,
// the last object before x and y (the latest ite group); multiple-output files
// carry time/iteration at the root.  q receives Ny x Nx x {rho,u,v,p}.
bool read_snapshot(const std::string &path, const std::string &group, int nx, int ny, std::vector<double> *q,
                   double *time, int *iteration, std::string *err);

// XDMF sidecar (IOManager.h:22-73, 181-188, 238-240, 274-280): a new file
// (truncate) or the previous text with one more grid before the footer.
// unique: the one-file-per-run layout, where the reference rewinds
// sizeof(footer) bytes -- the footer and the character before it -- before
// each grid (IOManager.h:238-240, 274); the file is byte-identical to its.
bool write_xdmf(const std::string &xmf_path, const std::string &h5name, const RootInfo &root, bool truncate,
                bool unique, const std::string &grid_name, double t, const std::string &group, std::string *err);

// General access used by tests and tools.
class File {
 public:
  bool open(const std::string &path, std::string *err);
  // names of the links of a group ("/" = root), sorted
  bool list(const std::string &group, std::vector<std::string> *names, std::string *err);
  bool read_doubles(const std::string &dataset, std::vector<double> *out, std::vector<uint64_t> *dims,
                    std::string *err);
  bool attr_double(const std::string &object, const std::string &name, double *v, std::string *err);
  bool attr_int(const std::string &object, const std::string &name, long long *v, std::string *err);
  bool attr_string(const std::string &object, const std::string &name, std::string *v, std::string *err);
  bool has_attr(const std::string &object, const std::string &name);

  struct Impl;

 private:
  std::shared_ptr<Impl> impl_;
};

}  // namespace h5
}  // namespace fv2d
