"""ORACLE -- test infrastructure only (tests/, __graft_entry__.smoke(), bench.py cpu_baseline).

ctypes front end of oracle/dg_oracle.cpp, the CPU FP64 restatement of HORSES3D's
ComputeTimeDerivative / TakeRK3Step / MaxTimeStep / ComputeMaxResiduals. The product never imports
this module. ``build()`` compiles the library with oracle/Makefile.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
LIB = ORACLE_DIR / "_build" / "libh3d_oracle.so"

_f64p = C.POINTER(C.c_double)
_lib = None


def build(quiet: bool = True) -> Path:
    out = subprocess.run(["make", "-C", str(ORACLE_DIR)], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{out.stdout}\n{out.stderr}")
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_ndof.restype = C.c_int64
        L.orc_ndof.argtypes = [C.c_void_p]
        L.orc_set_state.argtypes = [C.c_void_p, _f64p]
        L.orc_get.argtypes = [C.c_void_p, C.c_int, _f64p]
        L.orc_rhs.argtypes = [C.c_void_p, C.c_double]
        L.orc_rk3_step.argtypes = [C.c_void_p, C.c_double, C.c_double]
        L.orc_max_dt.restype = C.c_double
        L.orc_max_dt.argtypes = [C.c_void_p, C.c_double, C.c_double]
        L.orc_residuals.restype = C.c_int
        L.orc_residuals.argtypes = [C.c_void_p, _f64p]
        L.orc_mms_state.argtypes = [C.c_void_p, C.c_double, _f64p, _f64p]
        L.orc_box_mesh_create.restype = C.c_void_p
        L.orc_box_mesh_create.argtypes = [C.c_int, C.c_int, C.c_int, _f64p, _f64p, C.c_double, C.c_int, C.c_int,
                                          C.c_int]
        L.orc_box_mesh_describe.restype = C.c_int
        L.orc_box_mesh_describe.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_box_mesh_free.argtypes = [C.c_void_p]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_create_partition.restype = C.c_void_p
        L.orc_create_partition.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        L.orc_rhs_phase.argtypes = [C.c_void_p, C.c_double, C.c_int]
        L.orc_face_trace.restype = C.c_int64
        L.orc_face_trace.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, _f64p, C.c_int]
        L.orc_rk3_update.argtypes = [C.c_void_p, C.c_int, C.c_double]
        _lib = L
    return _lib


def set_threads(n: int) -> None:
    """OpenMP threads of the oracle's later parallel regions."""
    os.environ["OMP_NUM_THREADS"] = str(n)
    lib().orc_set_threads(int(n))


class Oracle:
    """One oracle solver on a mesh (a HexMesh or anything with a ``desc`` dg_mesh_desc)."""

    def __init__(self, mesh, physics, options, boundaries=None):
        """boundaries: one DgBoundary per mesh zone (Config.boundary_table), required when the mesh
        has non-periodic boundary faces."""
        self.mesh = mesh
        self.physics = physics
        self.options = options
        desc = mesh.desc
        if getattr(mesh, "n_boundary_faces", 0):
            if boundaries is None:
                raise ValueError("the mesh has boundary faces: pass the boundary conditions")
            self._bc = boundaries
            desc = mesh.with_boundaries(boundaries)
        self._desc = desc
        self._h = lib().orc_create(C.byref(desc), C.byref(physics), C.byref(options))
        self.ndof = int(lib().orc_ndof(self._h))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_destroy(self._h)
            self._h = None

    def set_state(self, q: np.ndarray) -> None:
        q = np.ascontiguousarray(q, dtype=np.float64)
        assert q.size == 5 * self.ndof
        lib().orc_set_state(self._h, q.ctypes.data_as(_f64p))

    def get(self, field: int) -> np.ndarray:
        out = np.empty(5 * self.ndof)
        lib().orc_get(self._h, field, out.ctypes.data_as(_f64p))
        return out

    def rhs(self, t: float) -> np.ndarray:
        lib().orc_rhs(self._h, t)
        return self.get(1)

    def rk3_step(self, t: float, dt: float) -> None:
        lib().orc_rk3_step(self._h, t, dt)

    def max_dt(self, cfl: float, dcfl: float) -> float:
        return float(lib().orc_max_dt(self._h, cfl, dcfl))

    def residuals(self):
        r = np.zeros(5)
        nan = lib().orc_residuals(self._h, r.ctypes.data_as(_f64p))
        return r, bool(nan)

    def mms_state(self, t: float):
        q = np.empty(5 * self.ndof)
        qd = np.empty(5 * self.ndof)
        lib().orc_mms_state(self._h, t, q.ctypes.data_as(_f64p), qd.ctypes.data_as(_f64p))
        return q, qd


class BoxMesh:
    """The oracle's own periodic box mesh (oracle/geometry.cpp): [lo,hi]^3 in n^3 hexahedra of
    uniform order N, optionally warped by warp*sin(x)sin(y)sin(z) with curved faces given as
    patches of order patch_order. It carries what the Oracle and the benchmark's CPU reference
    timing need (``desc``, ``x``, ``ndof``) without the product library."""

    def __init__(self, n, lo, hi, order, node_type=0, warp=0.0, patch_order=0):
        from horses3d_gb300 import _abi  # ctypes declarations of the C ABI structures only

        lo = np.ascontiguousarray(lo, dtype=np.float64)
        hi = np.ascontiguousarray(hi, dtype=np.float64)
        self._h = lib().orc_box_mesh_create(n, n, n, lo.ctypes.data_as(_f64p), hi.ctypes.data_as(_f64p), warp,
                                            patch_order, node_type, order)
        if not self._h:
            raise ValueError("invalid box mesh arguments")
        self.desc = _abi.DgMeshDesc()
        if lib().orc_box_mesh_describe(self._h, C.byref(self.desc)) != 0:
            raise RuntimeError("orc_box_mesh_describe failed")
        self.n_elements = n ** 3
        self.order = order
        self.ndof = self.n_elements * (order + 1) ** 3
        self.n_faces = int(self.desc.n_faces)
        self.n_boundary_faces = 0
        self.x = np.ctypeslib.as_array(self.desc.x, shape=(3 * self.ndof,))

    def array(self, name, count):
        return np.ctypeslib.as_array(getattr(self.desc, name), shape=(count,))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_box_mesh_free(self._h)
            self._h = None


class OraclePartition:
    """The oracle on one element partition (orc_create_partition; ``part`` from
    horses3d_gb300.partition.partition_mesh): the right-hand side in its three phases with the
    reference's MPI-face exchanges between them (the face Q after phase 0, the face gradients after
    phase 1; MPI_Face.f90:203-383). Payloads are numpy arrays, one per neighbour: the faces shared
    with it in ascending global order, each side's face-frame trace."""

    Q, GRADIENTS = 0, 1

    def __init__(self, part, physics, options):
        self.part = part
        self.ns = physics.navier_stokes != 0
        self._h = lib().orc_create_partition(C.byref(part.desc), part.n_ghost, C.byref(physics), C.byref(options))
        if not self._h:
            raise ValueError("orc_create_partition failed")
        self.ndof = int(lib().orc_ndof(self._h))
        self._np = {}
        nf = np.ctypeslib.as_array(part.desc.face_nf, shape=(2 * part.desc.n_faces,)).reshape(-1, 2)
        for n in part.neighbours:
            self._np[n.rank] = [(int(nf[f, 0]) + 1) * (int(nf[f, 1]) + 1) for f in n.faces]

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_destroy(self._h)
            self._h = None

    def set_state(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64)
        assert q.size == 5 * self.ndof
        lib().orc_set_state(self._h, q.ctypes.data_as(_f64p))

    def get(self, field: int) -> np.ndarray:
        out = np.empty(5 * self.ndof)
        lib().orc_get(self._h, field, out.ctypes.data_as(_f64p))
        return out

    def phase(self, t: float, k: int) -> None:
        lib().orc_rhs_phase(self._h, t, k)

    def update(self, k: int, dt: float) -> None:
        lib().orc_rk3_update(self._h, k, dt)

    def max_dt(self, cfl: float, dcfl: float) -> float:
        return float(lib().orc_max_dt(self._h, cfl, dcfl))

    def _size(self, what: int, q: int) -> int:
        return sum(self._np[q]) * (5 if what == self.Q else 15)

    def pack(self, what: int) -> dict:
        out = {}
        for n in self.part.neighbours:
            buf = np.empty(self._size(what, n.rank))
            a = 0
            for f, side, npts in zip(n.faces, n.own_side, self._np[n.rank]):
                m = npts * (5 if what == self.Q else 15)
                got = lib().orc_face_trace(self._h, int(f), int(side), what, buf[a:a + m].ctypes.data_as(_f64p), 0)
                assert got == m, (f, side, got, m)
                a += m
            out[(self.part.rank, n.rank)] = buf
        return out

    def recv_like(self, what: int) -> dict:
        return {(self.part.rank, n.rank): np.empty(self._size(what, n.rank)) for n in self.part.neighbours}

    def unpack(self, what: int, recvs: dict) -> None:
        for n in self.part.neighbours:
            buf = np.ascontiguousarray(recvs[(self.part.rank, n.rank)], dtype=np.float64)
            a = 0
            for f, side, npts in zip(n.faces, n.own_side, self._np[n.rank]):
                m = npts * (5 if what == self.Q else 15)
                lib().orc_face_trace(self._h, int(f), int(3 - side), what, buf[a:a + m].ctypes.data_as(_f64p), 1)
                a += m


def partition_rhs(parts, t: float, exchange) -> None:
    """ComputeTimeDerivative over OraclePartitions; exchange(sends, recv_like) -> recvs moves the
    per-neighbour numpy payloads (keys (this rank, neighbour))."""
    def move(what):
        sends, like = {}, {}
        for p in parts:
            sends.update(p.pack(what))
            like.update(p.recv_like(what))
        recvs = exchange(sends, like)
        for p in parts:
            p.unpack(what, recvs)

    for p in parts:
        p.phase(t, 0)
    move(OraclePartition.Q)
    if parts and parts[0].ns:
        for p in parts:
            p.phase(t, 1)
        move(OraclePartition.GRADIENTS)
    for p in parts:
        p.phase(t, 2)


def partition_rk3_step(parts, t: float, dt: float, exchange) -> None:
    """TakeRK3Step over OraclePartitions (ExplicitMethods.f90:748-779)."""
    b = (0.0, 1.0 / 3.0, 3.0 / 4.0)
    for k in range(3):
        partition_rhs(parts, t + b[k] * dt, exchange)
        for p in parts:
            p.update(k, dt)
