"""ctypes view of the C ABI declared in include/horses3d_gb300.h.

The structures mirror the header field for field; every call goes through the shared library
``horses3d_gb300/lib/libhorses3d_gb300.so`` that ``horses3d_gb300.build`` compiles for sm_103a.
There is no Python fallback: a missing library raises ``LibraryNotBuilt``.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
LIB_DIR = PKG_DIR / "lib"
LIB_NAME = "libhorses3d_gb300.so"

DG_OK = 0
DG_ERR_INVALID = -1
DG_ERR_UNSUPPORTED = -2
DG_ERR_CUDA = -3
DG_ERR_NAN = -4
DG_ERR_TIMEOUT = -5
DG_ERR_NOMEM = -6
DG_ERR_NODEVICE = -7
DG_ERR_IO = -8
DG_FAULT_NONE, DG_FAULT_TMA_WAIT = 0, 1

DG_NODES_GAUSS, DG_NODES_GAUSS_LOBATTO = 0, 1
DG_INVISCID_STANDARD, DG_INVISCID_SPLIT = 0, 1
DG_RIEMANN_ROE, DG_RIEMANN_LXF, DG_RIEMANN_CENTRAL, DG_RIEMANN_RUSANOV = 0, 1, 2, 3
DG_RIEMANN_STD_ROE, DG_RIEMANN_ROE_PIKE, DG_RIEMANN_LOW_DISS_ROE = 4, 5, 6
DG_RIEMANN_MATRIX_DISS, DG_RIEMANN_VISCOUS_NS, DG_RIEMANN_U_DISS = 7, 8, 9
DG_AVG_STANDARD, DG_AVG_PIROZZOLI, DG_AVG_DUCROS, DG_AVG_MORINISHI, DG_AVG_KENNEDY_GRUBER = 0, 1, 2, 3, 4
DG_AVG_ENTROPY_CONSERVING, DG_AVG_CHANDRASEKAR = 5, 6
DG_PRECISION_FP64, DG_PRECISION_MIXED, DG_PRECISION_MIXED_TC = 0, 1, 2
DG_SOURCE_NONE, DG_SOURCE_MMS_CONVERGENCE, DG_SOURCE_MMS_LAMB_VECTOR = 0, 1, 2
DG_GRADVARS_STATE, DG_GRADVARS_ENTROPY, DG_GRADVARS_ENERGY = 0, 1, 2
DG_BC_NO_SLIP_WALL, DG_BC_FREE_SLIP_WALL, DG_BC_INFLOW, DG_BC_OUTFLOW = 1, 2, 3, 4
DG_FIELD_Q, DG_FIELD_QDOT, DG_FIELD_G, DG_FIELD_UX, DG_FIELD_UY, DG_FIELD_UZ = range(6)
DG_HALO_Q_TRACES, DG_HALO_VISCOUS_FLUX = 0, 1

_i32p = C.POINTER(C.c_int32)
_f64p = C.POINTER(C.c_double)


class DgBoundary(C.Structure):
    _fields_ = [
        ("type", C.c_int32),
        ("isothermal", C.c_int32),
        ("wall_temperature", C.c_double),
        ("wall_velocity", C.c_double * 3),
        ("rho", C.c_double),
        ("u", C.c_double),
        ("v", C.c_double),
        ("w", C.c_double),
        ("p", C.c_double),
        ("pressure", C.c_double),
    ]


class DgMeshDesc(C.Structure):
    _fields_ = [
        ("n_elements", C.c_int32),
        ("node_type", C.c_int32),
        ("order", _i32p),
        ("x", _f64p),
        ("ja_xi", _f64p),
        ("ja_eta", _f64p),
        ("ja_zeta", _f64p),
        ("jacobian", _f64p),
        ("inv_jacobian", _f64p),
        ("n_faces", C.c_int32),
        ("face_elem", _i32p),
        ("face_side", _i32p),
        ("face_rotation", _i32p),
        ("face_nf", _i32p),
        ("face_normal", _f64p),
        ("face_t1", _f64p),
        ("face_t2", _f64p),
        ("face_jacobian", _f64p),
        ("face_boundary", _i32p),
        ("n_boundaries", C.c_int32),
        ("boundaries", C.POINTER(DgBoundary)),
    ]


class DgPhysics(C.Structure):
    _fields_ = [
        ("mach", C.c_double),
        ("reynolds", C.c_double),
        ("prandtl", C.c_double),
        ("navier_stokes", C.c_int32),
    ]


class DgOptions(C.Structure):
    _fields_ = [
        ("inviscid", C.c_int32),
        ("riemann", C.c_int32),
        ("averaging", C.c_int32),
        ("lambda_stab", C.c_double),
        ("precision", C.c_int32),
        ("source", C.c_int32),
        ("gradient_variables", C.c_int32),
    ]


# (name, restype, argtypes) of every entry point in include/horses3d_gb300.h
class SolutionHeader(C.Structure):
    """h3d_solution_header: the .hsol header (io/SolutionFile.f90)."""
    _fields_ = [("name", C.c_char * 128), ("file_type", C.c_int32), ("node_type", C.c_int32),
                ("n_elements", C.c_int32), ("iteration", C.c_int32), ("time", C.c_double), ("refs", C.c_double * 6)]


SIGNATURES = [
    ("dg_version", C.c_char_p, []),
    ("dg_strerror", C.c_char_p, [C.c_int]),
    ("dg_last_error", C.c_char_p, []),
    ("dg_device_count", C.c_int, [C.POINTER(C.c_int)]),
    ("dg_create", C.c_int, [C.POINTER(DgMeshDesc), C.POINTER(DgPhysics), C.POINTER(DgOptions), C.POINTER(C.c_void_p)]),
    ("dg_destroy", None, [C.c_void_p]),
    ("dg_upload_state", C.c_int, [C.c_void_p, _f64p]),
    ("dg_download", C.c_int, [C.c_void_p, C.c_int, _f64p]),
    ("dg_ndof", C.c_int64, [C.c_void_p]),
    ("dg_rhs", C.c_int, [C.c_void_p, C.c_double]),
    ("dg_rk3_step", C.c_int, [C.c_void_p, C.c_double, C.c_double]),
    ("dg_run_steps", C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, _f64p]),
    ("dg_time_steps", C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, _f64p]),
    ("dg_kernel_times", C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_double, _f64p]),
    ("dg_max_dt", C.c_int, [C.c_void_p, C.c_double, C.c_double, _f64p]),
    ("dg_max_dt_noalloc", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int,
                                    C.c_int, C.POINTER(DgPhysics), C.c_double, C.c_double, C.c_void_p, _f64p]),
    ("dg_max_dt_noalloc_max_dof", C.c_int64, []),
    ("dg_measure_fp64_peak", C.c_int, [_f64p]),
    ("dg_keep_gradients", C.c_int, [C.c_void_p, C.c_int]),
    ("dg_tc_selftest", C.c_int, [C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int]),
    ("dg_create_partition", C.c_int, [C.POINTER(DgMeshDesc), C.c_int32, C.POINTER(DgPhysics), C.POINTER(DgOptions),
                                      C.POINTER(C.c_void_p)]),
    ("dg_halo_set_slots", C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.c_int32, C.POINTER(C.c_int32)]),
    ("dg_halo_slot_bytes", C.c_int64, [C.c_void_p]),
    ("dg_halo_pack", C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    ("dg_halo_unpack", C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    ("dg_partition_stage", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double]),
    ("dg_set_energy_reference", C.c_int, [C.c_void_p, C.c_double]),
    ("dg_residuals", C.c_int, [C.c_void_p, _f64p, C.POINTER(C.c_int)]),
    ("dg_synchronize", C.c_int, [C.c_void_p]),
    ("dg_create_batch", C.c_int, [C.c_int, C.POINTER(DgMeshDesc), C.POINTER(DgPhysics), C.POINTER(DgOptions),
                                  C.POINTER(C.c_void_p)]),
    ("dg_batch_size", C.c_int, [C.c_void_p]),
    ("dg_case_offset", C.c_int64, [C.c_void_p, C.c_int]),
    ("dg_batch_set_clock", C.c_int, [C.c_void_p, _f64p, _f64p]),
    ("dg_batch_get_clock", C.c_int, [C.c_void_p, _f64p, _f64p]),
    ("dg_batch_max_dt", C.c_int, [C.c_void_p, C.c_double, C.c_double, _f64p]),
    ("dg_batch_residuals", C.c_int, [C.c_void_p, _f64p, C.POINTER(C.c_int)]),
    ("dg_batch_run_steps", C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_double, _f64p]),
    ("dg_autotune", C.c_int, [C.c_void_p, C.c_int]),
    ("dg_inject_fault", C.c_int, [C.c_void_p, C.c_int]),
    ("h3d_read_solution_header", C.c_int, [C.c_char_p, C.POINTER(SolutionHeader)]),
    ("h3d_read_solution", C.c_int, [C.c_char_p, C.c_int32, _i32p, _f64p, _f64p]),
    ("h3d_write_solution", C.c_int, [C.c_char_p, C.POINTER(SolutionHeader), _i32p, _f64p, _f64p]),
    ("dg_batch_integrate", C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_double, _f64p, C.POINTER(C.c_int)]),
    ("dg_integrate", C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                               C.POINTER(C.c_double), _f64p, C.POINTER(C.c_int)]),
    ("dg_save_solution", C.c_int, [C.c_void_p, C.c_int, C.c_char_p, C.c_int, C.c_double, C.c_int]),
    ("dg_load_solution", C.c_int, [C.c_void_p, C.c_int, C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    ("h3d_mesh_read_specmesh", C.c_int, [C.c_char_p, C.c_int, C.c_int, _i32p, C.c_char_p, C.POINTER(C.c_void_p)]),
    ("h3d_mesh_box", C.c_int, [C.c_int, C.c_int, C.c_int, _f64p, _f64p, C.c_double, C.c_int, C.c_int, C.c_int,
                               _i32p, C.POINTER(C.c_void_p)]),
    ("h3d_mesh_box_zones", C.c_int, [C.c_int, C.c_int, C.c_int, _f64p, _f64p, C.c_double, C.c_int, C.c_int,
                                     C.c_int, _i32p, C.c_char_p, C.POINTER(C.c_void_p)]),
    ("h3d_mesh_describe", C.c_int, [C.c_void_p, C.POINTER(DgMeshDesc)]),
    ("h3d_mesh_zone_count", C.c_int, [C.c_void_p]),
    ("h3d_mesh_zone_name", C.c_char_p, [C.c_void_p, C.c_int]),
    ("h3d_mesh_volume", C.c_double, [C.c_void_p]),
    ("h3d_mesh_free", None, [C.c_void_p]),
    ("h3d_nodal_storage", C.c_int, [C.c_int, C.c_int, _f64p, _f64p, _f64p]),
]


class LibraryNotBuilt(RuntimeError):
    pass


class DgError(RuntimeError):
    def __init__(self, code: int, where: str, detail: str):
        super().__init__(f"{where} failed: {code} ({detail})")
        self.code = code


_lib = None


def library_path() -> Path:
    override = os.environ.get("HORSES3D_GB300_LIB")
    return Path(override) if override else LIB_DIR / LIB_NAME


def lib():
    """Loads the C ABI library once; raises LibraryNotBuilt when it has not been compiled."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not path.exists():
        raise LibraryNotBuilt(f"{path} is missing: run horses3d_gb300.build.build() (nvcc, sm_103a)")
    handle = C.CDLL(str(path))
    for name, res, args in SIGNATURES:
        fn = getattr(handle, name)
        fn.restype = res
        fn.argtypes = args
    _lib = handle
    return _lib


def check(code: int, where: str) -> None:
    if code != DG_OK:
        L = lib()
        raise DgError(code, where, f"{L.dg_strerror(code).decode()}: {L.dg_last_error().decode()}")


def f64ptr(arr):
    return arr.ctypes.data_as(_f64p)


def i32ptr(arr):
    return arr.ctypes.data_as(_i32p)
