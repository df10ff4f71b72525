"""Initial conditions of the benchmark and test cases (the reference keeps these in ProblemFile
plugins, libs/problemfile/ProblemFile.f90:26-235). States are returned in the reference layout
Q(1:5,i,j,k) element after element, as one flat float64 array.
"""
from __future__ import annotations

import numpy as np

GAMMA = 1.4


def _splitmix64(x: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser on uint64 (public-domain generator by S. Vigna)."""
    with np.errstate(over="ignore"):
        z = (x + np.uint64(0x9E3779B97F4A7C15)).astype(np.uint64)
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)).astype(np.uint64)
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)).astype(np.uint64)
        return z ^ (z >> np.uint64(31))


def uniform_pm1(seed: int, index: np.ndarray) -> np.ndarray:
    """Deterministic U[-1,1) numbers: splitmix64(seed * 2^32 + index), top 53 bits."""
    key = (np.uint64(seed) << np.uint64(32)) + index.astype(np.uint64)
    bits = _splitmix64(key) >> np.uint64(11)
    return bits.astype(np.float64) * (2.0 / 9007199254740992.0) - 1.0


def taylor_green(x: np.ndarray, mach: float, p0: float | None = None, perturbation: float = 0.0,
                 seed: int = 0) -> np.ndarray:
    """Taylor-Green vortex of the reference's TaylorGreen case (test/NavierStokes/TaylorGreen/SETUP/
    ProblemFile.f90:100-146) with rho0 = u0 = L = 1 and p0 = 1/(gamma M^2) unless given. With
    perturbation > 0 each velocity component of each node gets + perturbation * U[-1,1) from
    splitmix64(seed, 3 * node + component)."""
    x = np.asarray(x).reshape(-1, 3)
    p0 = 1.0 / (GAMMA * mach * mach) if p0 is None else p0
    X, Y, Z = x[:, 0], x[:, 1], x[:, 2]
    rho = np.ones_like(X)
    u = np.sin(X) * np.cos(Y) * np.cos(Z)
    v = -np.cos(X) * np.sin(Y) * np.cos(Z)
    w = np.zeros_like(X)
    if perturbation:
        idx = np.arange(X.size, dtype=np.uint64) * np.uint64(3)
        u = u + perturbation * uniform_pm1(seed, idx)
        v = v + perturbation * uniform_pm1(seed, idx + np.uint64(1))
        w = w + perturbation * uniform_pm1(seed, idx + np.uint64(2))
    p = p0 + 1.0 / 16.0 * (np.cos(2 * X) * np.cos(2 * Z) + 2 * np.cos(2 * Y) + 2 * np.cos(2 * X) +
                           np.cos(2 * Y) * np.cos(2 * Z))
    q = np.empty((X.size, 5))
    q[:, 0] = rho
    q[:, 1] = rho * u
    q[:, 2] = rho * v
    q[:, 3] = rho * w
    q[:, 4] = p / (GAMMA - 1.0) + 0.5 * rho * (u * u + v * v + w * w)
    return q.reshape(-1)


def isentropic_vortex(x: np.ndarray, mach: float, strength: float = 5.0, center=(0.0, 0.0, 0.0),
                      period: float | None = None) -> np.ndarray:
    """Isentropic vortex about the z axis through ``center`` advected along (1,1,1)/sqrt(3) with
    Mach number ``mach`` (free stream rho=1, p=1/(gamma M^2), |u|=1). The vortex of strength beta has
    du = beta/(2 pi) exp((1-r^2)/2) (-y', x'), dT = -(gamma-1) beta^2/(8 gamma pi^2) exp(1-r^2) in units
    of the standard (rho = p = 1) vortex, rescaled to p_inf by the velocity scale sqrt(p_inf) so that
    it stays an exact steady solution; with ``period`` the nearest periodic image is used."""
    x = np.asarray(x).reshape(-1, 3)
    p_inf = 1.0 / (GAMMA * mach * mach)
    scale = np.sqrt(p_inf)
    dx = x[:, 0] - center[0]
    dy = x[:, 1] - center[1]
    if period is not None:
        dx = dx - period * np.round(dx / period)
        dy = dy - period * np.round(dy / period)
    r2 = dx * dx + dy * dy
    f = np.exp(0.5 * (1.0 - r2))
    du = strength / (2 * np.pi) * f * (-dy) * scale
    dv = strength / (2 * np.pi) * f * dx * scale
    dT = -(GAMMA - 1.0) * strength ** 2 / (8 * GAMMA * np.pi ** 2) * f * f
    T = 1.0 + dT  # T / T_inf
    rho = T ** (1.0 / (GAMMA - 1.0))
    p = p_inf * rho ** GAMMA
    ub = 1.0 / np.sqrt(3.0)
    u = ub + du
    v = ub + dv
    w = np.full_like(u, ub)
    q = np.empty((x.shape[0], 5))
    q[:, 0] = rho
    q[:, 1] = rho * u
    q[:, 2] = rho * v
    q[:, 3] = rho * w
    q[:, 4] = p / (GAMMA - 1.0) + 0.5 * rho * (u * u + v * v + w * w)
    return q.reshape(-1)


def mms_convergence_state(x: np.ndarray, t: float):
    """State and exact time derivative of the manufactured solution of the reference's Convergence
    case (test/NavierStokes/Convergence/SETUP/ProblemFile.f90:31-133)."""
    x = np.asarray(x).reshape(-1, 3)
    arg = np.pi * (x[:, 0] + x[:, 1] + x[:, 2] - 2.0 * t)
    rho = 2.0 + 0.1 * np.sin(arg)
    u, v, w, e = 1.0 * rho - 1.0, 2.0 * rho - 4.0, -3.0 * rho + 5.0, rho
    q = np.stack([rho, rho * u, rho * v, rho * w, rho * e], axis=1)
    rho_t = 0.1 * (-2.0 * np.pi) * np.cos(arg)
    u_t, v_t, w_t, e_t = 1.0 * rho_t, 2.0 * rho_t, -3.0 * rho_t, rho_t
    qd = np.stack([rho_t, rho_t * u + rho * u_t, rho_t * v + rho * v_t, rho_t * w + rho * w_t,
                   rho_t * e + rho * e_t], axis=1)
    return q.reshape(-1), qd.reshape(-1)


def mms_lamb_vector_state(x: np.ndarray, t: float) -> np.ndarray:
    """Manufactured state of the reference's NavierStokes/LambVector case
    (test/NavierStokes/LambVector/SETUP/ProblemFile.f90:8-27): rho = 3 + sin(phi) e^t,
    (u, v, w) = (cos phi, sin phi, cos phi) e^-t, E = rho |u|^2 / 2 + 1, phi = x + y + z."""
    x = np.asarray(x).reshape(-1, 3)
    phi = x[:, 0] + x[:, 1] + x[:, 2]
    rho = 3.0 + np.sin(phi) * np.exp(t)
    u = np.cos(phi) * np.exp(-t)
    v = np.sin(phi) * np.exp(-t)
    w = np.cos(phi) * np.exp(-t)
    e = rho * (u ** 2 + v ** 2 + w ** 2) / 2.0 + 1.0
    return np.stack([rho, rho * u, rho * v, rho * w, rho * e], axis=1).reshape(-1)


def rel_l2(a: np.ndarray, b: np.ndarray, weights: np.ndarray | None = None) -> np.ndarray:
    """Relative L2 difference per conserved variable: sqrt(sum w (a-b)^2) / sqrt(sum w b^2).

    The three momentum components share one denominator, the L2 norm of the momentum vector
    sqrt(sum w |rho u|^2): a single component can vanish identically (w = 0 in the Taylor-Green
    vortex), which would turn its own norm into a division by ~0."""
    a = np.asarray(a).reshape(-1, 5)
    b = np.asarray(b).reshape(-1, 5)
    w = np.ones(a.shape[0]) if weights is None else np.asarray(weights).reshape(-1)
    num = np.sqrt(np.einsum("n,nv->v", w, (a - b) ** 2))
    den = np.sqrt(np.einsum("n,nv->v", w, b ** 2))
    den[1:4] = np.sqrt(np.sum(den[1:4] ** 2))
    return num / np.where(den > 0, den, 1.0)
