"""ctypes mirror of include/fv2d_types.h (the parameter block shared by the
GB300 library, its C++ driver and the CPU oracle).

Field order and types must match the C header exactly; ``tests/test_abi.py``
checks this against the header text and against ``sizeof`` reported by the
compiled library.
"""
import ctypes as C

_FIELDS = [
    ("struct_size", C.c_uint32),
    # [mesh]
    ("Nx", C.c_int32), ("Ny", C.c_int32), ("Nghosts", C.c_int32),
    ("xmin", C.c_double), ("xmax", C.c_double), ("ymin", C.c_double), ("ymax", C.c_double),
    # [run] / [solvers]
    ("CFL", C.c_double),
    ("boundary_x", C.c_int32), ("boundary_y", C.c_int32),
    ("reconstruction", C.c_int32),
    ("riemann_solver", C.c_int32),
    ("time_stepping", C.c_int32),
    ("tend", C.c_double), ("save_freq", C.c_double),
    # [physics] / [misc]
    ("gamma0", C.c_double),
    ("epsilon", C.c_double),
    ("epsilon_reset_negative", C.c_double),
    ("well_balanced_flux_at_y_bc", C.c_int32),
    ("fslp_K", C.c_double),
    ("seed", C.c_int32),
    ("log_frequency", C.c_int32),
    # [gravity]
    ("gravity_mode", C.c_int32),
    ("analytical_gravity_mode", C.c_int32),
    ("gx", C.c_double), ("gy", C.c_double),
    ("hot_bubble_g0", C.c_double),
    # [thermal_conduction]
    ("thermal_conductivity_active", C.c_int32),
    ("thermal_conductivity_mode", C.c_int32),
    ("kappa", C.c_double),
    ("bctc_ymin", C.c_int32), ("bctc_ymax", C.c_int32),
    ("bctc_ymin_value", C.c_double), ("bctc_ymax_value", C.c_double),
    ("b02_ymid", C.c_double), ("b02_kappa1", C.c_double), ("b02_kappa2", C.c_double),
    ("b02_thickness", C.c_double),
    # [viscosity]
    ("viscosity_active", C.c_int32),
    ("viscosity_mode", C.c_int32),
    ("mu", C.c_double),
    # problem parameters
    ("m1", C.c_double), ("theta1", C.c_double), ("m2", C.c_double), ("theta2", C.c_double),
    ("h84_pert", C.c_double), ("c91_pert", C.c_double),
    ("kh_a", C.c_double), ("kh_amp", C.c_double), ("kh_P0", C.c_double), ("kh_rho_fac", C.c_double),
    ("kh_sigma", C.c_double), ("kh_uflow", C.c_double), ("kh_y1", C.c_double), ("kh_y2", C.c_double),
    ("gresho_density", C.c_double), ("gresho_Mach", C.c_double),
    # extension problems
    ("sod_rho_left", C.c_double), ("sod_p_left", C.c_double),
    ("sod_rho_right", C.c_double), ("sod_p_right", C.c_double),
    ("sedov_E0", C.c_double), ("sedov_r0", C.c_double), ("sedov_p_ambient", C.c_double),
    ("sedov_rho", C.c_double),
    ("khs_rho_in", C.c_double), ("khs_rho_out", C.c_double), ("khs_u", C.c_double),
    ("khs_p0", C.c_double), ("khs_amp", C.c_double), ("khs_noise", C.c_double),
    ("rt_rho_top", C.c_double), ("rt_rho_bottom", C.c_double), ("rt_p_interface", C.c_double),
    ("rt_y_interface", C.c_double), ("rt_amp", C.c_double),
]


class Params(C.Structure):
    """fv2d_params (include/fv2d_types.h)."""
    _fields_ = _FIELDS

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in _FIELDS}

    def update(self, **kw):
        for k, v in kw.items():
            if not hasattr(self, k):
                raise KeyError(f"unknown fv2d_params field {k!r}")
            setattr(self, k, v)
        return self

    def copy(self):
        c = Params()
        C.memmove(C.byref(c), C.byref(self), C.sizeof(Params))
        return c


# Enumerations (include/fv2d_types.h, reference SimInfo.h:26-97, Init.h:271-282)
HLL, HLLC, FSLP = 0, 1, 2
BC_ABSORBING, BC_REFLECTING, BC_PERIODIC = 0, 1, 2
TS_EULER, TS_RK2 = 0, 1
PCM, PCM_WB, PLM, MUSCL_HANCOCK = 0, 1, 2, 3
TCM_CONSTANT, TCM_B02 = 0, 1
BCTC_NONE, BCTC_FIXED_TEMPERATURE, BCTC_FIXED_GRADIENT = 0, 1, 2
GRAV_NONE, GRAV_CONSTANT, GRAV_ANALYTICAL = 0, 1, 2

PROBLEMS = {
    "sod_x": 0, "sod_y": 1, "blast": 2, "rayleigh-taylor": 3, "diffusion": 4,
    "H84": 5, "C91": 6, "kelvin_helmholtz": 7, "gresho_vortex": 8,
    "sedov": 100, "kh_step": 101, "rt_hydrostatic": 102,
}

OK, ERR_INVALID, ERR_CUDA, ERR_NOMEM, ERR_STATE, ERR_NUMERIC, ERR_UNSUPPORTED, ERR_SIZE = range(8)
ERROR_NAMES = {0: "OK", 1: "INVALID", 2: "CUDA", 3: "NOMEM", 4: "STATE", 5: "NUMERIC", 6: "UNSUPPORTED",
               7: "SIZE"}


def as_float32(x):
    """Value of x after the reference's parameter reading: INIReader::GetFloat
    parses with strtof and returns float (jtilly/inih), so every real-valued
    .ini parameter the reference sees is float-rounded (SimInfo.h:195-200)."""
    return float(C.c_float(x).value)
