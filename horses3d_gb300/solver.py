"""Reference-shaped host driver over the C ABI.

``NavierStokesDG`` mirrors the calls HORSES3D's time integrator makes on the spatial operator:
``compute_time_derivative`` (ComputeTimeDerivative, SpatialDiscretization.f90:227-320),
``take_rk3_step`` (TakeRK3Step, ExplicitMethods.f90:667-788), ``max_time_step`` (MaxTimeStep,
DGSEMClass.f90:870-1038), ``compute_max_residuals`` (ComputeMaxResiduals, DGSEMClass.f90:770-868)
and ``integrate_in_time`` (the explicit branch of IntegrateInTime, TimeIntegrator.f90:737-890, with
CorrectDt's final-time clip, TimeIntegrator.f90:1100-1133). Every operation runs on the GPU through
libhorses3d_gb300.so; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _abi
from .control import Config


@dataclass
class StepReport:
    iterations: int
    time: float
    residuals: np.ndarray


class NavierStokesDG:
    def __init__(self, mesh, config: Config):
        self.mesh = mesh
        self.config = config
        self.physics = config.physics()
        self.options = config.options()
        desc = mesh.desc
        if mesh.n_boundary_faces:  # the zones' boundary conditions from the configuration
            self._bc = config.boundary_table(mesh.zone_names)
            desc = mesh.with_boundaries(self._bc)
        self._desc = desc
        h = C.c_void_p()
        _abi.check(_abi.lib().dg_create(C.byref(desc), C.byref(self.physics), C.byref(self.options), C.byref(h)),
                   "dg_create")
        self._h = h
        self.ndof = int(_abi.lib().dg_ndof(self._h))

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

    # -- state -----------------------------------------------------------------------------------
    def set_state(self, q: np.ndarray) -> None:
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(-1)
        if q.size != 5 * self.ndof:
            raise ValueError(f"state has {q.size} values, expected {5 * self.ndof}")
        _abi.check(_abi.lib().dg_upload_state(self._h, _abi.f64ptr(q)), "dg_upload_state")

    def get(self, field: int = _abi.DG_FIELD_Q) -> np.ndarray:
        out = np.empty(5 * self.ndof)
        _abi.check(_abi.lib().dg_download(self._h, field, _abi.f64ptr(out)), "dg_download")
        return out

    @property
    def Q(self):
        return self.get(_abi.DG_FIELD_Q)

    @property
    def QDot(self):
        return self.get(_abi.DG_FIELD_QDOT)

    # -- the reference's operator interface --------------------------------------------------------
    def keep_gradients(self, on: bool = True) -> None:
        """Keep the last stage's lifted gradients of every step (get(DG_FIELD_UX..UZ)) for monitors."""
        _abi.check(_abi.lib().dg_keep_gradients(self._h, int(on)), "dg_keep_gradients")

    def compute_time_derivative(self, t: float) -> None:
        _abi.check(_abi.lib().dg_rhs(self._h, float(t)), "dg_rhs")

    def take_rk3_step(self, t: float, dt: float) -> None:
        _abi.check(_abi.lib().dg_rk3_step(self._h, float(t), float(dt)), "dg_rk3_step")

    def max_time_step(self, cfl: float, dcfl: float) -> float:
        dt = C.c_double()
        _abi.check(_abi.lib().dg_max_dt(self._h, float(cfl), float(dcfl), C.byref(dt)), "dg_max_dt")
        return dt.value

    def compute_max_residuals(self):
        r = np.zeros(5)
        nan = C.c_int(0)
        rc = _abi.lib().dg_residuals(self._h, _abi.f64ptr(r), C.byref(nan))
        if rc not in (_abi.DG_OK, _abi.DG_ERR_NAN):
            _abi.check(rc, "dg_residuals")
        return r, bool(nan.value)

    def run_steps(self, n: int, t0: float, dt: float = 0.0, cfl: float = 0.0, dcfl: float = 0.0) -> float:
        t_end = C.c_double()
        _abi.check(_abi.lib().dg_run_steps(self._h, int(n), float(t0), float(dt), float(cfl), float(dcfl),
                                           C.byref(t_end)), "dg_run_steps")
        return t_end.value

    def integrate_on_device(self, n_steps: int, t0: float = 0.0, dt: float = 0.0, cfl: float = 0.0,
                            dcfl: float = 0.0):
        """IntegrateInTime's explicit loop in one call (dg_integrate): n steps of MaxTimeStep (when
        dt is 0) + TakeRK3Step + ComputeMaxResiduals from one CUDA graph. Returns (t_end, residual
        history [n_steps, 5]); raises FloatingPointError naming the first step with a NaN/Inf."""
        t_end = C.c_double()
        hist = np.zeros((max(1, n_steps), 5))
        nan_step = C.c_int()
        rc = _abi.lib().dg_integrate(self._h, int(n_steps), float(t0), float(dt), float(cfl), float(dcfl),
                                     C.byref(t_end), _abi.f64ptr(hist), C.byref(nan_step))
        if rc == _abi.DG_ERR_NAN:
            raise FloatingPointError(f"NaN or Inf in the solution after step {nan_step.value} (checkForNan)")
        _abi.check(rc, "dg_integrate")
        return t_end.value, hist[:n_steps]

    def synchronize(self):
        _abi.check(_abi.lib().dg_synchronize(self._h), "dg_synchronize")

    def save_solution(self, path, iteration: int, time: float, gradients: bool = False) -> None:
        """HexMesh_SaveSolution (HexMesh.f90:3376-3555) from the device state."""
        _abi.check(_abi.lib().dg_save_solution(self._h, 0, str(path).encode(), int(iteration), float(time),
                                               1 if gradients else 0), "dg_save_solution")

    def load_solution(self, path):
        """Restart (HexMesh_LoadSolution, HexMesh.f90:4708-): uploads Q; returns (iteration, time)."""
        it = C.c_int()
        t = C.c_double()
        _abi.check(_abi.lib().dg_load_solution(self._h, 0, str(path).encode(), C.byref(it), C.byref(t)),
                   "dg_load_solution")
        return it.value, t.value

    def autotune(self, reps: int = 5) -> None:
        """Per-order-triple item sizes of the variable-order kernels (a no-op for uniform orders)."""
        _abi.check(_abi.lib().dg_autotune(self._h, int(reps)), "dg_autotune")

    def integrate_in_time(self, t0: float = 0.0, n_steps: int | None = None, t_final: float | None = None,
                          cfl: float | None = None, dcfl: float | None = None, dt: float | None = None,
                          compute_after_steps: bool = False) -> StepReport:
        """IntegrateInTime's explicit loop: MaxTimeStep (when cfl is given), CorrectDt, RKStep,
        t += dt, ComputeMaxResiduals, stop at the final time or after n_steps; without a final time
        (a steady-state run) also at the first step whose maximum residual is at most the
        convergence tolerance (TimeIntegrator.f90:820-828)."""
        cfg = self.config
        cfl = cfg.cfl if cfl is None else cfl
        dcfl = cfg.dcfl if dcfl is None else dcfl
        dt_fixed = cfg.dt if dt is None else dt
        n_steps = cfg.n_steps if n_steps is None else n_steps
        t_final = cfg.t_final if t_final is None else t_final
        tol = cfg.convergence_tolerance if t_final is None else None
        t = float(t0)
        it = 0
        eps = np.finfo(float).eps
        res = np.zeros(5)
        while it < n_steps:
            step = self.max_time_step(cfl, dcfl) if (cfl and not dt_fixed) else dt_fixed
            if t_final is not None and t + step > t_final:
                step = t_final - t
            self.take_rk3_step(t, step)
            if compute_after_steps:
                self.compute_time_derivative(t + step)
            t += step
            it += 1
            res, nan = self.compute_max_residuals()
            if nan:
                raise FloatingPointError(f"NaN or Inf in the solution at t={t} (checkForNan)")
            if t_final is not None and (t >= t_final or abs(t - t_final) <= 100.0 * eps):
                break
            if tol is not None and np.max(res) <= tol:
                break
        return StepReport(it, t, res)
