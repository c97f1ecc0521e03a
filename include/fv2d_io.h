/*
 * fv2d_io.h -- the reference's .ini parameters and HDF5 snapshot layout,
 * host-side, in libfv2d_gpu.so (no libhdf5 needed).
 *
 *   fv2d_read_ini          <- readInifile (SimInfo.h:529-568) +
 *                             DeviceParams::init_from_inifile (SimInfo.h:356-459);
 *                             real values float-rounded like INIReader::GetFloat
 *   fv2d_write_ini_echo    <- Reader::outputValues (SimInfo.h:224-262), the
 *                             "last.ini" / "<output>.ini" echo (IOManager.h:90-94)
 *   fv2d_snapshot_write    <- IOManager::saveSolutionUnique / saveSolutionMultiple
 *                             (IOManager.h:107-282), XDMF sidecar included
 *   fv2d_snapshot_read     <- IOManager::loadSnapshot data part (IOManager.h:284-376)
 */
#ifndef FV2D_IO_H
#define FV2D_IO_H

#include "fv2d_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Run-level settings of the reference's Params that fv2d_params does not
 * carry (SimInfo.h:463-492). */
typedef struct fv2d_run_config {
  char problem[64];
  char output_filename[256];
  char output_path[512];
  char restart_file[512];
  int32_t multiple_outputs;
  int32_t problem_id; /* FV2D_PB_*, -1 if the name is unknown */
} fv2d_run_config;

/* Parses an .ini file.  FV2D_ERR_INVALID with a message in err (the
 * reference's exception text) on a bad map-valued parameter or an unreadable
 * file; FV2D_ERR_SIZE when a string value does not fit its field of
 * fv2d_run_config (it is never cut short); warnings for unknown sections/keys
 * go to stderr like checkValidityIni (SimInfo.h:501-527). */
int fv2d_read_ini(const char *path, fv2d_params *p, fv2d_run_config *run, char *err, int errlen);

/* Writes the parameter echo of the .ini at ini_path to out_path. */
int fv2d_write_ini_echo(const char *ini_path, const char *out_path);

/* Writes snapshot number `iteration` at time t of the interior primitives q
 * (Ny x Nx x {rho,u,v,p}).  multiple_outputs == 0: group ite_%04d of
 * <dir>/<name>.h5 (created when truncate != 0, else extended) and
 * <dir>/<name>.xmf; otherwise <dir>/<name>_%04d.h5 / .xmf. */
int fv2d_snapshot_write(const char *dir, const char *name, int multiple_outputs, int truncate, const fv2d_params *p,
                        const char *problem, int iteration, double t, const double *q, char *err, int errlen);

/* Reads a restart: `file` may be "path.h5" (latest ite group, or the root of
 * a multiple-output file) or "path.h5:/ite_XXXX".  Fills q (Ny x Nx x 4),
 * *t and *iteration; FV2D_ERR_INVALID with the reference's message when the
 * resolution differs. */
int fv2d_snapshot_read(const char *file, int nx, int ny, double *q, double *t, int *iteration, char *err,
                       int errlen);

/* Generic access to an HDF5 file: the float dataset at `dataset` ("/ite_0003/rho")
 * as binary64 (at most max values; *n receives the element count), and a
 * numeric attribute of an object ("/" = root).  Used to inspect snapshots. */
int fv2d_h5_read_doubles(const char *file, const char *dataset, double *out, int64_t max, int64_t *n);
int fv2d_h5_read_attr(const char *file, const char *object, const char *name, double *value);

#ifdef __cplusplus
}
#endif
#endif /* FV2D_IO_H */
