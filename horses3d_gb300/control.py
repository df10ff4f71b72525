"""The .control keys that select the hot path, read the way the reference reads them.

``read_control`` follows ReadControlFile (io/ReadInputFile.f90:20-130): ``key = value`` lines,
keys case-insensitive, ``!`` comments, ``#define boundary <name>`` ... ``#end`` blocks (only the
periodic ``coupled boundary`` pairs matter here). Defaults are the reference's:
Gauss nodes (main.f90:239-324), Roe (RiemannSolvers_NS.f90:201-204), standard averaging, lambda 1,
standard inviscid form, BR1, Prandtl 0.72, RK3. The extra key ``gpu precision = fp64 | mixed``
selects the plain or the mixed-precision form. Options outside the GPU path raise
``UnsupportedOption`` so the caller keeps the reference's CPU path for them.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import _abi


class UnsupportedOption(ValueError):
    pass


@dataclass
class Config:
    mesh_file: str | None = None
    order: int = 3
    nodes: int = _abi.DG_NODES_GAUSS
    flow: str = "ns"
    mach: float = 0.1
    reynolds: float = 1600.0
    prandtl: float = 0.72
    riemann: int = _abi.DG_RIEMANN_ROE
    averaging: int = _abi.DG_AVG_STANDARD
    inviscid: int = _abi.DG_INVISCID_STANDARD
    lambda_stab: float = 1.0
    precision: int = _abi.DG_PRECISION_FP64
    source: int = _abi.DG_SOURCE_NONE
    gradient_variables: int = _abi.DG_GRADVARS_STATE
    cfl: float | None = None
    dcfl: float | None = None
    dt: float | None = None
    n_steps: int = 1
    t_final: float | None = None
    # steady-state runs stop when the maximum residual reaches it ("convergence tolerance",
    # TimeIntegrator.f90:214,820-828); None runs the step count
    convergence_tolerance: float | None = None
    periodic: list = field(default_factory=list)
    order_file: str | None = None
    aoa_theta: float = 0.0  # degrees ("AOA theta", PhysicsStorage_NS.f90)
    aoa_phi: float = 0.0    # degrees ("AOA phi")
    boundaries: dict = field(default_factory=dict)  # zone name -> {"type": ..., block keys}

    def element_orders(self, base_dir=None):
        """(Nx, Ny, Nz) per element from "polynomial order file" (ReadInputFile.f90:132-153: the element
        count, then one "Nx Ny Nz" line per element), else the scalar or (i, j, k) order."""
        if self.order_file is None:
            return self.order
        path = Path(self.order_file)
        if base_dir is not None and not path.is_absolute():
            path = Path(base_dir) / path
        return read_order_file(path)

    def physics(self) -> _abi.DgPhysics:
        return _abi.DgPhysics(self.mach, self.reynolds, self.prandtl, 1 if self.flow == "ns" else 0)

    def options(self) -> _abi.DgOptions:
        return _abi.DgOptions(self.inviscid, self.riemann, self.averaging, self.lambda_stab, self.precision,
                              self.source, self.gradient_variables)

    def periodic_spec(self) -> str:
        return ",".join(f"{a}:{b}" for a, b in self.periodic)

    # -- reference values (PhysicsStorage_NS.f90:284-318; air, T_ref = 520*5/9 K, p_ref = 101325 Pa) --
    def _ref(self):
        R, gamma = 287.15, 1.4
        T = 520.0 * 5.0 / 9.0
        rho = 101325.0 / (R * T)
        V = self.mach * np.sqrt(gamma * R * T)
        return {"T": T, "rho": rho, "V": V, "p": rho * V * V}

    def free_stream(self):
        """(rho, u, v, w, p) of the free stream: unit density and speed along the angles of attack,
        p = 1/(gamma M^2) (the reference's uniform initial state and inflow defaults)."""
        th, ph = np.radians(self.aoa_theta), np.radians(self.aoa_phi)
        return (1.0, np.cos(th) * np.cos(ph), np.sin(th) * np.cos(ph), np.sin(ph), 1.0 / (1.4 * self.mach ** 2))

    def boundary(self, zone: str) -> _abi.DgBoundary:
        """The DgBoundary of a zone from its "#define boundary" block (NoSlipWallBC.f90:80-216,
        FreeSlipWallBC.f90:80-200, InflowBC.f90:112-290, OutflowBC.f90:85-188), dimensionless."""
        spec = self.boundaries.get(zone.lower())
        if spec is None:
            raise ValueError(f"no boundary condition for zone '{zone}'")
        kind = spec["type"].replace(" ", "").lower()
        b = _abi.DgBoundary()
        ref = self._ref()
        gM2 = 1.4 * self.mach ** 2
        if kind in ("noslipwall", "freeslipwall"):
            b.type = _abi.DG_BC_NO_SLIP_WALL if kind == "noslipwall" else _abi.DG_BC_FREE_SLIP_WALL
            wt = str(spec.get("wall type (adiabatic/isothermal)", "adiabatic")).lower()
            b.isothermal = 1 if wt == "isothermal" else 0
            b.wall_temperature = float(spec.get("wall temperature", ref["T"])) / ref["T"]
            if kind == "noslipwall" and "wall velocity" in spec:
                vw = [float(x) for x in str(spec["wall velocity"]).strip("[]() ").replace(",", " ").split()]
                for c in range(3):
                    b.wall_velocity[c] = vw[c]
        elif kind == "inflow":
            b.type = _abi.DG_BC_INFLOW
            if float(spec.get("turbintensity", 0.0)) != 0.0:
                raise UnsupportedOption("inflow turbulence intensity (random fluctuations)")
            p = float(spec.get("pressure", ref["p"] / gM2)) / ref["p"]
            rho = float(spec.get("density", ref["rho"])) / ref["rho"]
            v = float(spec.get("mach", self.mach)) * np.sqrt(1.4 * p / rho)
            th = np.radians(float(spec.get("aoatheta", self.aoa_theta)))
            ph = np.radians(float(spec.get("aoaphi", self.aoa_phi)))
            b.rho, b.p = rho, p
            b.u, b.v, b.w = v * np.cos(th) * np.cos(ph), v * np.sin(th) * np.cos(ph), v * np.sin(ph)
        elif kind == "outflow":
            b.type = _abi.DG_BC_OUTFLOW
            if "pressure" in spec:
                pext = float(spec["pressure"])
            elif "dp" in spec:
                pext = ref["p"] / gM2 - float(spec["dp"])
            else:
                pext = ref["p"] / gM2
            b.pressure = pext / ref["p"]
        else:
            raise UnsupportedOption(f"boundary '{zone}' of type '{spec['type']}'")
        return b

    def boundary_table(self, zone_names):
        """One DgBoundary per mesh zone, in the mesh's zone order (a ctypes array)."""
        arr = (_abi.DgBoundary * max(1, len(zone_names)))()
        for z, name in enumerate(zone_names):
            arr[z] = self.boundary(name)
        return arr


# SpatialDiscretization.f90:106-148 "gradient variables"
_GRADVARS = {"state": _abi.DG_GRADVARS_STATE, "entropy": _abi.DG_GRADVARS_ENTROPY, "energy": _abi.DG_GRADVARS_ENERGY}

# RiemannSolvers_NS.f90:5-40 keyword values
_RIEMANN = {"roe": _abi.DG_RIEMANN_ROE, "lax-friedrichs": _abi.DG_RIEMANN_LXF, "central": _abi.DG_RIEMANN_CENTRAL,
            "rusanov": _abi.DG_RIEMANN_RUSANOV, "standard roe": _abi.DG_RIEMANN_STD_ROE,
            "roe-pike": _abi.DG_RIEMANN_ROE_PIKE, "low dissipation roe": _abi.DG_RIEMANN_LOW_DISS_ROE,
            "matrix dissipation": _abi.DG_RIEMANN_MATRIX_DISS, "viscous ns": _abi.DG_RIEMANN_VISCOUS_NS,
            "u-diss": _abi.DG_RIEMANN_U_DISS}
_AVERAGING = {"standard": _abi.DG_AVG_STANDARD, "pirozzoli": _abi.DG_AVG_PIROZZOLI, "ducros": _abi.DG_AVG_DUCROS,
              "morinishi": _abi.DG_AVG_MORINISHI, "kennedy-gruber": _abi.DG_AVG_KENNEDY_GRUBER,
              "entropy conserving": _abi.DG_AVG_ENTROPY_CONSERVING, "chandrasekar": _abi.DG_AVG_CHANDRASEKAR}


def _value(v: str) -> str:
    v = v.split("!")[0].strip()
    if len(v) >= 2 and v[0] == v[-1] and v[0] in "\"'":
        v = v[1:-1]
    return v.strip()


def _fortran_real(v: str) -> float:
    """A real in Fortran list-directed form (1.d-10, 1.0D0, 2.5e-3)."""
    return float(v.strip().lower().replace("d", "e"))


def parse_control(text: str) -> Config:
    cfg = Config()
    keys: dict[str, str] = {}
    blocks = []
    block = None
    for raw in text.splitlines():
        line = raw.split("!")[0].strip() if not raw.strip().startswith("#") else raw.strip()
        if not line:
            continue
        low = line.lower()
        if low.startswith("#define"):
            block = {"kind": low.split()[1] if len(low.split()) > 1 else "", "name": " ".join(low.split()[2:])}
            continue
        if low.startswith("#end"):
            if block is not None:
                blocks.append(block)
            block = None
            continue
        if "=" not in line:
            continue
        k, v = line.split("=", 1)
        k = " ".join(k.strip().lower().split())
        if block is not None:
            block[k] = _value(v)
        else:
            keys[k] = _value(v)

    def get(k, default=None):
        return keys.get(k, default)

    cfg.mesh_file = get("mesh file name")
    # pAdaptationClass.f90:218-239: an order file wins over "polynomial order", which wins over i/j/k
    if "polynomial order file" in keys:
        cfg.order_file = keys["polynomial order file"]
    elif "polynomial order" in keys:
        cfg.order = int(float(keys["polynomial order"]))
    elif all(f"polynomial order {a}" in keys for a in "ijk"):
        cfg.order = tuple(int(float(keys[f"polynomial order {a}"])) for a in "ijk")
    elif any(f"polynomial order {a}" in keys for a in "ijk"):
        raise ValueError("The polynomial order(s) must be specified")
    nodes = (get("discretization nodes", "gauss") or "gauss").lower()
    cfg.nodes = _abi.DG_NODES_GAUSS_LOBATTO if nodes.replace("_", "-") == "gauss-lobatto" else _abi.DG_NODES_GAUSS
    flow = (get("flow equations", "ns") or "ns").lower()
    if flow not in ("ns", "euler"):
        raise UnsupportedOption(f"flow equations '{flow}'")
    cfg.flow = flow
    cfg.mach = float(get("mach number", cfg.mach))
    if flow == "ns":
        if "reynolds number" not in keys:
            raise ValueError("Input file is missing entry for keyword: reynolds number")
        cfg.reynolds = float(keys["reynolds number"])
    cfg.prandtl = float(get("prandtl number", 0.72))
    rs = (get("riemann solver", "roe") or "roe").lower()
    if rs not in _RIEMANN:
        raise UnsupportedOption(f"riemann solver '{rs}'")
    cfg.riemann = _RIEMANN[rs]
    av = (get("averaging", "standard") or "standard").lower()
    if av not in _AVERAGING:
        raise UnsupportedOption(f"averaging '{av}'")
    cfg.averaging = _AVERAGING[av]
    inv = (get("inviscid discretization", "standard") or "standard").lower()
    if inv not in ("standard", "split-form"):
        raise UnsupportedOption(f"inviscid discretization '{inv}'")
    cfg.inviscid = _abi.DG_INVISCID_SPLIT if inv == "split-form" else _abi.DG_INVISCID_STANDARD
    if cfg.inviscid == _abi.DG_INVISCID_SPLIT:
        cfg.nodes = _abi.DG_NODES_GAUSS_LOBATTO  # main.f90:306-313 forces Gauss-Lobatto for split form
    vd = (get("viscous discretization", "br1") or "br1").lower()
    if vd != "br1":
        raise UnsupportedOption(f"viscous discretization '{vd}'")
    gv = (get("gradient variables", "state") or "state").lower()
    if gv not in _GRADVARS:
        raise UnsupportedOption(f"gradient variables '{gv}'")
    cfg.gradient_variables = _GRADVARS[gv]
    em = (get("explicit method", "rk3") or "rk3").lower()
    if em not in ("rk3", "williamson rk3"):
        raise UnsupportedOption(f"explicit method '{em}'")
    for k in ("les model", "shock-capturing", "enable particles"):
        if k in keys and keys[k].lower() not in ("none", ".false.", "false"):
            raise UnsupportedOption(k)
    cfg.lambda_stab = float(get("lambda stabilization", 1.0))
    prec = (get("gpu precision", "fp64") or "fp64").lower()
    cfg.precision = _abi.DG_PRECISION_MIXED if prec == "mixed" else _abi.DG_PRECISION_FP64
    if "cfl" in keys:
        cfg.cfl = float(keys["cfl"])
        cfg.dcfl = float(keys.get("dcfl", keys["cfl"]))
    if "dt" in keys:
        cfg.dt = float(keys["dt"])
    cfg.n_steps = int(float(get("number of time steps", 1)))
    if "convergence tolerance" in keys:
        cfg.convergence_tolerance = _fortran_real(keys["convergence tolerance"])
    if "final time" in keys:
        cfg.t_final = float(keys["final time"])
    cfg.aoa_theta = float(get("aoa theta", 0.0))
    cfg.aoa_phi = float(get("aoa phi", 0.0))
    pairs = []
    for b in blocks:
        if b.get("kind") != "boundary":
            continue
        kind = str(b.get("type", "")).replace(" ", "").lower()
        # the names of a "#define boundary" line are joined by "__"
        # (GenericBoundaryConditionClass.f90:400-456, CheckIfBoundaryNameIsContained)
        names = [n for part in b["name"].split("__") for n in part.split()]
        if kind == "periodic":
            pairs.append((b["name"].strip(), str(b.get("coupled boundary", "")).lower().strip()))
        elif kind in ("noslipwall", "freeslipwall", "inflow", "outflow"):
            for nm in names:
                cfg.boundaries[nm.lower()] = dict(b, type=kind)
        else:
            raise UnsupportedOption(f"boundary '{b.get('name')}' of type '{b.get('type')}'")
    seen = set()
    for a, b in pairs:
        if (b, a) in seen:
            continue
        seen.add((a, b))
        cfg.periodic.append((a, b))
    return cfg


def read_order_file(path) -> np.ndarray:
    tokens = Path(path).read_text().split()
    n = int(tokens[0])
    vals = np.array([int(t) for t in tokens[1:1 + 3 * n]], dtype=np.int32)
    if vals.size != 3 * n:
        raise ValueError(f"{path}: expected {n} order triples")
    return vals.reshape(n, 3)


def read_control(path) -> Config:
    return parse_control(Path(path).read_text())
