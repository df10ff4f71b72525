"""Batches of independent cases on one GPU context (``dg_create_batch``).

Every case keeps its own mesh (any per-element orders), Mach/Reynolds numbers, time and dt; the
numerical options (nodes, Riemann solver, precision) are shared. One RK3 step of the batch is one
sequence of kernel launches over all cases, bucketed by element order triple. The reference has no
counterpart (it runs one case per process); each case's results equal what ``NavierStokesDG`` gives
for that case alone.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from .control import Config


class CaseBatch:
    def __init__(self, meshes, configs: list[Config]):
        if len(meshes) != len(configs) or not meshes:
            raise ValueError("one configuration per mesh, at least one case")
        self.meshes = list(meshes)
        self.configs = list(configs)
        self.n_cases = len(meshes)
        self._bcs = [c.boundary_table(m.zone_names) if m.n_boundary_faces else None for m, c in zip(meshes, configs)]
        descs = (_abi.DgMeshDesc * self.n_cases)(*[m.with_boundaries(b) if b is not None else m.desc
                                                   for m, b in zip(meshes, self._bcs)])
        phys = (_abi.DgPhysics * self.n_cases)(*[c.physics() for c in configs])
        self._keep = (descs, phys)
        opts = configs[0].options()
        h = C.c_void_p()
        _abi.check(_abi.lib().dg_create_batch(self.n_cases, descs, phys, C.byref(opts), C.byref(h)), "dg_create_batch")
        self._h = h
        L = _abi.lib()
        self.offsets = np.array([L.dg_case_offset(self._h, k) for k in range(self.n_cases + 1)], dtype=np.int64)
        self.ndof = int(self.offsets[-1])

    def close(self):
        if getattr(self, "_h", None):
            _abi.lib().dg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- state ------------------------------------------------------------------------------------
    def set_state(self, qs) -> None:
        q = np.concatenate([np.ascontiguousarray(x, dtype=np.float64).reshape(-1) for x in qs])
        if q.size != 5 * self.ndof:
            raise ValueError(f"states hold {q.size} values, expected {5 * self.ndof}")
        _abi.check(_abi.lib().dg_upload_state(self._h, _abi.f64ptr(q)), "dg_upload_state")

    def get(self, field: int = _abi.DG_FIELD_Q) -> list[np.ndarray]:
        out = np.empty(5 * self.ndof)
        _abi.check(_abi.lib().dg_download(self._h, field, _abi.f64ptr(out)), "dg_download")
        return [out[5 * self.offsets[k]:5 * self.offsets[k + 1]] for k in range(self.n_cases)]

    # -- clocks and steps -------------------------------------------------------------------------
    def set_clock(self, t, dt) -> None:
        t = np.ascontiguousarray(np.broadcast_to(t, (self.n_cases,)), dtype=np.float64)
        dt = np.ascontiguousarray(np.broadcast_to(dt, (self.n_cases,)), dtype=np.float64)
        _abi.check(_abi.lib().dg_batch_set_clock(self._h, _abi.f64ptr(t), _abi.f64ptr(dt)), "dg_batch_set_clock")

    def clock(self):
        t = np.empty(self.n_cases)
        dt = np.empty(self.n_cases)
        _abi.check(_abi.lib().dg_batch_get_clock(self._h, _abi.f64ptr(t), _abi.f64ptr(dt)), "dg_batch_get_clock")
        return t, dt

    def max_time_steps(self, cfl: float, dcfl: float) -> np.ndarray:
        dt = np.empty(self.n_cases)
        _abi.check(_abi.lib().dg_batch_max_dt(self._h, float(cfl), float(dcfl), _abi.f64ptr(dt)), "dg_batch_max_dt")
        return dt

    def run_steps(self, n: int, cfl: float = 0.0, dcfl: float = 0.0) -> float:
        """n RK3 steps of every case from its clock; returns the device time in ms."""
        ms = C.c_double()
        _abi.check(_abi.lib().dg_batch_run_steps(self._h, int(n), float(cfl), float(dcfl), C.byref(ms)),
                   "dg_batch_run_steps")
        return ms.value

    def integrate_on_device(self, n: int, cfl: float = 0.0, dcfl: float = 0.0) -> np.ndarray:
        """n steps of every case from its clock with the residual monitor (dg_batch_integrate); returns
        the residual history [n, n_cases, 5]."""
        hist = np.zeros((max(1, n), self.n_cases, 5))
        nan_step = C.c_int()
        rc = _abi.lib().dg_batch_integrate(self._h, int(n), float(cfl), float(dcfl), _abi.f64ptr(hist),
                                           C.byref(nan_step))
        if rc == _abi.DG_ERR_NAN:
            raise FloatingPointError(f"NaN or Inf after step {nan_step.value}")
        _abi.check(rc, "dg_batch_integrate")
        return hist[:n]

    def compute_max_residuals(self):
        r = np.zeros(5 * self.n_cases)
        nan = np.zeros(self.n_cases, dtype=np.int32)
        rc = _abi.lib().dg_batch_residuals(self._h, _abi.f64ptr(r), nan.ctypes.data_as(C.POINTER(C.c_int)))
        if rc not in (_abi.DG_OK, _abi.DG_ERR_NAN):
            _abi.check(rc, "dg_batch_residuals")
        return r.reshape(self.n_cases, 5), nan.astype(bool)

    def synchronize(self):
        _abi.check(_abi.lib().dg_synchronize(self._h), "dg_synchronize")

    def save_solution(self, case: int, path, iteration: int, time: float, gradients: bool = False) -> None:
        """One case's state (and gradients) as a HORSES3D solution file (HexMesh_SaveSolution)."""
        _abi.check(_abi.lib().dg_save_solution(self._h, int(case), str(path).encode(), int(iteration), float(time),
                                               1 if gradients else 0), "dg_save_solution")

    def load_solution(self, case: int, path):
        """Restarts one case from a solution file; the other cases keep their state. Returns
        (iteration, time) from the file's header."""
        it = C.c_int()
        t = C.c_double()
        _abi.check(_abi.lib().dg_load_solution(self._h, int(case), str(path).encode(), C.byref(it), C.byref(t)),
                   "dg_load_solution")
        return it.value, t.value

    def autotune(self, reps: int = 5) -> None:
        """Elements per CTA of every order triple, timed on this batch and cached for the process."""
        _abi.check(_abi.lib().dg_autotune(self._h, int(reps)), "dg_autotune")
