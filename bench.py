"""Benchmark: DOF x RK-stage updates per second of the DGSEM Navier-Stokes RHS + Williamson RK3.

Workload: the curvilinear Taylor-Green case, 32^3 hexahedra on [0,2pi]^3 warped by
x_i += 0.1 sin x sin y sin z, order N=5 on Gauss nodes (7,077,888 DOF), Lax-Friedrichs, BR1,
M=0.1, Re=1600, Pr=0.72, fixed dt from CFL 0.4 at t=0. One bench step = one RK3 time step of the
whole mesh (3 RHS evaluations + 3 low-storage updates) = 3*NDOF DOF-stage updates.

value    : mixed form (FP32 fluxes/contractions, FP64 state and RK accumulation), state resident in
           HBM, K steps replayed from a CUDA graph, timed with CUDA events on the solver's stream.
plain    : the plain FP64 form timed the same way (the mixed-over-plain ratio is value/plain).
e2e      : the reference-facing C ABI driven like IntegrateInTime with host buffers: upload Q from
           pinned host memory, dg_integrate (per step MaxTimeStep + TakeRK3Step + ComputeMaxResiduals /
           checkForNan on the device), download Q and the per-step residuals; all inside the timed
           region.
roofline : the dominant kernel's algorithmic bytes per launch over its CUDA-event launch time,
           against the measured HBM copy bandwidth (MEASURED_PEAKS.json).
cpu_baseline: the CPU FP64 oracle (port of the reference loops) on the host cores.

--impl reference times the reference's CPU implementation of this path. The Fortran reference does
not build on this image (no Fortran compiler), so the reference arm runs the oracle port with all
host threads: W untimed and K timed RK3 steps of the same workload, on a mesh and geometry the
oracle builds itself (oracle/geometry.cpp), so that arm loads no product library.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_ELEM = 32
ORDER = 5
MACH, RE = 0.1, 1600.0
WARP = 0.1
CFL = 0.4
WORKLOAD = "tgv_curvilinear_32^3_N5_gauss_lxf_br1"


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def _barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def _allreduce_max(x, world):
    """Maximum of x over the ranks (NCCL reduces device tensors, gloo host tensors)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        self.file.flush()
        rows = [r.split(",") for r in Path(self.file.name).read_text().splitlines() if r.strip()]
        sm = [float(r[1]) for r in rows if len(r) > 2 and r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) > 2 and r[2].strip().replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for name, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def build_case(n_elem: int = N_ELEM):
    from horses3d_gb300 import _abi, problems
    from horses3d_gb300.mesh import HexMesh

    mesh = HexMesh.box(n_elem, [0, 0, 0], [2 * np.pi] * 3, ORDER, node_type=_abi.DG_NODES_GAUSS, warp=WARP,
                       patch_order=ORDER)
    q0 = problems.taylor_green(mesh.x, MACH)
    base = dict(order=ORDER, nodes=_abi.DG_NODES_GAUSS, mach=MACH, reynolds=RE, riemann=_abi.DG_RIEMANN_LXF)
    return mesh, q0, base


# DRAM bytes per DOF of one k_volume<6, gauss, float> launch, measured with ncu
# (dram__bytes_read.sum + dram__bytes_write.sum = 444.8 MB over 2,985,984 DOF, 24^3 elements, N=5).
VOLUME_DRAM_BYTES_PER_DOF = 149.0
# The unit that binds k_volume<6, gauss, float> in the same ncu capture: the L1/shared-memory pipe
# (l1tex__throughput.avg.pct_of_peak_sustained_elapsed), ahead of DRAM.
VOLUME_L1TEX_FRAC = 0.73
# Executed FP64 floating-point operations per DOF and RK stage of the plain form: ncu SASS counts
# dadd + dmul + 2 dfma of k_volume (1562.0), k_flux (95.5) and k_update_tma (217.0) per DOF, on the
# 8^3-element N=5 case (the same kernels and per-DOF work as the 32^3 workload).
FP64_FLOP_PER_DOF_STAGE = 1874.5


def volume_bytes(P: int, word: int) -> float:
    """Algorithmic bytes per DOF of k_volume (NS): reads Q (5 FP64), Ja (9) and 1/J (1), and per face
    point of its six sides (6 P^2 / P^3 = 6/P per DOF) the neighbour's Q trace (5) and the side
    geometry n, Jf (4), all in the storage word; writes the viscous normal fluxes (5 per face point)
    and QDot (5)."""
    face = 6.0 / P
    return 5 * 8 + word * (9 + 1 + (5 + 4) * face + 5 * face + 5)


def run_gpu_arm(args, rank, world, local, case):
    import ctypes as C

    from horses3d_gb300 import _abi
    from horses3d_gb300.control import Config
    from horses3d_gb300.problems import rel_l2
    from horses3d_gb300.solver import NavierStokesDG

    mesh, q0, base = case
    ndof = mesh.ndof
    dof_stage_per_step = 3.0 * ndof
    L = _abi.lib()

    def timed(precision, dt=None):
        g = NavierStokesDG(mesh, Config(**base, precision=precision))
        g.set_state(q0)
        if dt is None:
            dt = g.max_time_step(CFL, CFL)
        t = g.run_steps(args.warmup, 0.0, dt=dt)
        g.synchronize()
        _barrier(world)
        ms = C.c_double()
        _abi.check(L.dg_time_steps(g._h, args.steps, t, dt, 0.0, 0.0, C.byref(ms)), "dg_time_steps")
        _barrier(world)
        return g, dt, ms.value

    from horses3d_gb300._abi import DG_PRECISION_FP64, DG_PRECISION_MIXED

    gp, dt, ms_plain = timed(DG_PRECISION_FP64)  # dt: the FP64 MaxTimeStep at t=0, shared by both forms
    with ClockSampler(local) as clk:
        gm, _, ms_mixed = timed(DG_PRECISION_MIXED, dt)
    clocks = clk.summary()
    # the mixed form with the gradient contractions on the tensor cores (A/B against gm)
    gt, _, ms_tc = timed(_abi.DG_PRECISION_MIXED_TC, dt)
    ms_tc = _allreduce_max(ms_tc, world)
    q_tc = gt.Q.copy()
    kt_tc = np.zeros(5)
    _abi.check(L.dg_kernel_times(gt._h, 10, 0.0, dt, _abi.f64ptr(kt_tc)), "dg_kernel_times")
    gt.close()
    ms_mixed = _allreduce_max(ms_mixed, world)
    ms_plain = _allreduce_max(ms_plain, world)
    value = world * dof_stage_per_step * args.steps / (ms_mixed * 1e-3)
    plain = world * dof_stage_per_step * args.steps / (ms_plain * 1e-3)
    # accuracy of the mixed form against the FP64 form after the same steps
    q_mixed, q_fp64 = gm.Q.copy(), gp.Q.copy()  # after warm-up + timed steps (the kernel timing below moves Q)
    acc = rel_l2(q_mixed, q_fp64)

    # per-kernel launch times of the mixed form (dominant kernel for the roofline)
    kt = np.zeros(5)
    _abi.check(L.dg_kernel_times(gm._h, 10, 0.0, dt, _abi.f64ptr(kt)), "dg_kernel_times")
    kt_plain = np.zeros(5)
    _abi.check(L.dg_kernel_times(gp._h, 3, 0.0, dt, _abi.f64ptr(kt_plain)), "dg_kernel_times")
    names = ["volume", "flux", "update", "traces", "unused"]
    P = ORDER + 1
    hbm, peak_kind = _peaks()
    alg = volume_bytes(P, 4) * ndof
    achieved = alg / (kt[0] * 1e-3) / 1e9
    traffic = VOLUME_DRAM_BYTES_PER_DOF * ndof if P == 6 else None
    roofline = {"bound": "hbm", "kernel": "k_volume<6,gauss,float>", "achieved": round(achieved, 1),
                "peak": hbm, "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / hbm, 4),
                "traffic": traffic, "alg_bytes_per_launch": alg,
                "traffic_note": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one k_volume launch on the "
                                "24^3-element case (149.0 B/DOF), scaled by the DOF count",
                "limiter": {"unit": "l1tex (shared-memory operand loads)", "throughput_frac": VOLUME_L1TEX_FRAC,
                            "source": "ncu l1tex__throughput.avg.pct_of_peak_sustained_elapsed, same capture"}}
    # the step's other two kernels and the whole step against the same HBM peak (algorithmic bytes:
    # update 224 B/DOF (stage 1, no QDot store), flux 160 B per face point = 480/P B/DOF, step average
    # volume + flux + update with the last stage's QDot store)
    upd_b, flux_b = 224.0, 480.0 / P
    step_b = volume_bytes(P, 4) + flux_b + upd_b + 20.0 / 3.0
    roofline["other_kernels"] = {
        "k_update_tma": {"alg_bytes_per_dof": upd_b, "achieved": round(upd_b * ndof / (kt[2] * 1e-3) / 1e9, 1),
                         "frac": round(upd_b * ndof / (kt[2] * 1e-3) / 1e9 / hbm, 4)},
        "k_flux": {"alg_bytes_per_dof": flux_b, "achieved": round(flux_b * ndof / (kt[1] * 1e-3) / 1e9, 1),
                   "frac": round(flux_b * ndof / (kt[1] * 1e-3) / 1e9 / hbm, 4)}}
    per_gpu = value / world
    roofline["step"] = {"alg_bytes_per_dof_stage": round(step_b, 1), "achieved": round(per_gpu * step_b / 1e9, 1),
                        "frac": round(per_gpu * step_b / 1e9 / hbm, 4)}

    # the plain form's compute roofline: FP64 pipe (measured FMA rate of this GPU)
    fp64_peak = C.c_double()
    _abi.check(L.dg_measure_fp64_peak(C.byref(fp64_peak)), "dg_measure_fp64_peak")
    plain_roof = {"bound": "fp64", "peak_tflops": round(fp64_peak.value, 3), "peak_kind": "measured (FMA chains)",
                  "hbm_frac": round(plain * 1016.0 / 1e9 / hbm, 4), "hbm_bytes_per_dof_stage": 1016.0}
    if FP64_FLOP_PER_DOF_STAGE:
        ach = plain * FP64_FLOP_PER_DOF_STAGE / 1e12
        plain_roof.update({"achieved_tflops": round(ach, 3), "fp64_frac": round(ach / fp64_peak.value, 4),
                           "fp64_flop_per_dof_stage": FP64_FLOP_PER_DOF_STAGE})

    # e2e through the C ABI with host buffers (IntegrateInTime-shaped loop)
    import torch

    pinned = torch.empty(q0.size, dtype=torch.float64).pin_memory()
    pinned.numpy()[:] = q0
    out = torch.empty(q0.size, dtype=torch.float64).pin_memory()
    qp = C.cast(pinned.data_ptr(), C.POINTER(C.c_double))
    op = C.cast(out.data_ptr(), C.POINTER(C.c_double))
    e2e_steps = max(1, args.steps)
    hist = np.zeros((e2e_steps, 5))
    nan = C.c_int()
    t_end = C.c_double()

    def e2e_rate(precision):
        ge = NavierStokesDG(mesh, Config(**base, precision=precision))

        def once():
            # IntegrateInTime through the C ABI: every step MaxTimeStep (CFL) + TakeRK3Step + t += dt +
            # ComputeMaxResiduals / checkForNan on the device (dg_integrate), one host synchronization
            _abi.check(L.dg_upload_state(ge._h, qp), "dg_upload_state")
            _abi.check(L.dg_integrate(ge._h, e2e_steps, 0.0, 0.0, CFL, CFL, C.byref(t_end), _abi.f64ptr(hist),
                                      C.byref(nan)), "dg_integrate")
            _abi.check(L.dg_download(ge._h, _abi.DG_FIELD_Q, op), "dg_download")

        once()  # warm-up
        runs = []
        for _ in range(3):  # the median of three timed runs (one run alone varies by up to 20 %)
            _barrier(world)
            t0 = time.perf_counter()
            once()
            runs.append(_allreduce_max(time.perf_counter() - t0, world))
        ge.close()
        return world * dof_stage_per_step * e2e_steps / statistics.median(runs)

    e2e_value = e2e_rate(DG_PRECISION_MIXED)
    e2e_fp64 = e2e_rate(DG_PRECISION_FP64)
    qbytes = 8 * q0.size
    e2e = {"value": e2e_value, "unit": "DOF*stage/s", "h2d_bytes_per_step": int(qbytes / e2e_steps + 16),
           "d2h_bytes_per_step": int(qbytes / e2e_steps + 48 + 8 / e2e_steps),
           "loop": "upload Q from pinned host memory; dg_integrate (per step: CFL dt, RK3 step, residuals and "
                   "NaN check on the device, one graph per step); download Q and the residual history; "
                   "median of three timed runs after one warm-up run",
           "plain_fp64": {"value": e2e_fp64, "unit": "DOF*stage/s",
                          "note": "the same loop with the plain FP64 form (same precision as the CPU reference)"}}

    return {
        "value": value, "ms_per_step": ms_mixed / args.steps, "plain": plain,
        "plain_ms_per_step": ms_plain / args.steps, "mixed_over_plain": value / plain,
        "plain_roofline": plain_roof, "q_mixed": q_mixed, "q_fp64": q_fp64, "dt_fixed": dt, "q_tc": q_tc,
        "tensor_core_form": {"value": world * dof_stage_per_step * args.steps / (ms_tc * 1e-3),
                             "ms_per_step": ms_tc / args.steps,
                             "kernel_ms": dict(zip(names, [round(float(v), 5) for v in kt_tc])),
                             "rel_l2_vs_fp64": [float(v) for v in rel_l2(q_tc, q_fp64)],
                             "note": "mixed form with the gradient contractions and Q traces of the volume kernel "
                                     "on the tensor cores (tcgen05 TF32 split products in TMEM)"},
        "rel_l2_mixed_vs_fp64": [float(v) for v in acc], "roofline": roofline, "e2e": e2e, "clocks": clocks,
        "kernel_ms_mixed": dict(zip(names, [round(float(v), 5) for v in kt])),
        "kernel_ms_fp64": dict(zip(names, [round(float(v), 5) for v in kt_plain])), "ndof": ndof, "dt": dt,
        "gpu_launches": int(args.steps * (3 * 3 + 1)),
    }


# ------------------------------------------------------------------ secondary workloads ----------
# The other benchmark configurations, measured one at a time with --workload NAME (one JSON line
# each). Every one reports the mixed form against the plain FP64 form on the same GPU, with the
# same fixed dt (MaxTimeStep at t=0 of the FP64 form), and the relative L2 difference of the two.
SECONDARY = {
    "tgv8_n3_gl_roe": "Taylor-Green 8^3 elements, N=3 Gauss-Lobatto, standard form, Roe, BR1, M=0.1, Re=1600, 100 steps",
    "split16_n4_pirozzoli": "Taylor-Green 16^3, N=4 Gauss-Lobatto, split form (Pirozzoli two-point flux), LxF, BR1, "
                            "+-1% seeded velocity perturbation, 200 steps",
    "aniso24_vortex": "p-anisotropic 24^3 box, (Nx,Ny,Nz) i.i.d. uniform {2..7} (seed 4), Euler isentropic vortex "
                      "(strength 5, M=0.5) advected diagonally, Gauss, LxF, 500 steps",
    "batch64": "64 independent NS cases: 8^3..12^3 periodic boxes, uniform N in {2..6}, M ~ U[0.1,0.8], "
               "Re ~ U[100,3000], Taylor-Green or isentropic vortex by seed (seed 5), Gauss, LxF, 200 steps",
}


def build_secondary(name: str):
    """(meshes, FP64 configs, initial states, steps) of a secondary workload."""
    from horses3d_gb300 import _abi, problems
    from horses3d_gb300.control import Config
    from horses3d_gb300.mesh import HexMesh

    two_pi = 2 * np.pi
    if name == "tgv8_n3_gl_roe":
        m = HexMesh.box(8, [0, 0, 0], [two_pi] * 3, 3, node_type=_abi.DG_NODES_GAUSS_LOBATTO)
        c = Config(order=3, nodes=_abi.DG_NODES_GAUSS_LOBATTO, mach=0.1, reynolds=1600.0, riemann=_abi.DG_RIEMANN_ROE)
        return [m], [c], [problems.taylor_green(m.x, 0.1)], 100
    if name == "split16_n4_pirozzoli":
        m = HexMesh.box(16, [0, 0, 0], [two_pi] * 3, 4, node_type=_abi.DG_NODES_GAUSS_LOBATTO)
        c = Config(order=4, nodes=_abi.DG_NODES_GAUSS_LOBATTO, mach=0.1, reynolds=1600.0, riemann=_abi.DG_RIEMANN_LXF,
                   inviscid=_abi.DG_INVISCID_SPLIT, averaging=_abi.DG_AVG_PIROZZOLI)
        return [m], [c], [problems.taylor_green(m.x, 0.1, perturbation=0.01, seed=2)], 200
    if name == "aniso24_vortex":
        n = 24
        orders = np.random.default_rng(4).integers(2, 8, size=(n ** 3, 3)).astype(np.int32)
        m = HexMesh.box(n, [-5.0] * 3, [5.0] * 3, orders, node_type=_abi.DG_NODES_GAUSS)
        c = Config(order=7, nodes=_abi.DG_NODES_GAUSS, flow="euler", mach=0.5, riemann=_abi.DG_RIEMANN_LXF)
        return [m], [c], [problems.isentropic_vortex(m.x, 0.5, strength=5.0, period=10.0)], 500
    if name == "batch64":
        rng = np.random.default_rng(5)
        meshes, cfgs, qs = [], [], []
        for _ in range(64):
            n = int(rng.integers(8, 13))
            N = int(rng.integers(2, 7))
            mach = float(rng.uniform(0.1, 0.8))
            re = float(rng.uniform(100.0, 3000.0))
            vortex = bool(rng.integers(0, 2))
            if vortex:
                m = HexMesh.box(n, [-5.0] * 3, [5.0] * 3, N, node_type=_abi.DG_NODES_GAUSS)
                q = problems.isentropic_vortex(m.x, mach, strength=5.0, period=10.0)
            else:
                m = HexMesh.box(n, [0, 0, 0], [two_pi] * 3, N, node_type=_abi.DG_NODES_GAUSS)
                q = problems.taylor_green(m.x, mach)
            meshes.append(m)
            cfgs.append(Config(order=N, nodes=_abi.DG_NODES_GAUSS, mach=mach, reynolds=re, riemann=_abi.DG_RIEMANN_LXF))
            qs.append(q)
        return meshes, cfgs, qs, 200
    raise ValueError(f"unknown workload {name}")


def run_secondary(name: str, args):
    import dataclasses

    from horses3d_gb300 import _abi
    from horses3d_gb300.batch import CaseBatch
    from horses3d_gb300.problems import rel_l2

    meshes, cfgs, qs, steps = build_secondary(name)
    steps = args.steps if args.steps_given else steps
    ndof = sum(m.ndof for m in meshes)

    def make(precision):
        b = CaseBatch(meshes, [dataclasses.replace(c, precision=precision) for c in cfgs])
        b.set_state(qs)
        return b

    def timed(b, dts):
        b.set_clock(np.zeros(len(meshes)), dts)
        b.run_steps(args.warmup)
        b.set_clock(np.zeros(len(meshes)), dts)
        b.set_state(qs)
        return b.run_steps(steps)

    if len(meshes) == 1 and meshes[0].uniform_order() is not None:
        # one uniform case: the uniform-order kernels (the batch path would also run it)
        from horses3d_gb300.solver import NavierStokesDG

        def make_single(precision):
            g = NavierStokesDG(meshes[0], dataclasses.replace(cfgs[0], precision=precision))
            g.set_state(qs[0])
            return g

        g64 = make_single(_abi.DG_PRECISION_FP64)
        dt = g64.max_time_step(CFL, CFL)
        ms = {}
        outs = {}
        for prec, g in ((_abi.DG_PRECISION_FP64, g64), (_abi.DG_PRECISION_MIXED, make_single(_abi.DG_PRECISION_MIXED))):
            g.run_steps(args.warmup, 0.0, dt=dt)
            g.set_state(qs[0])
            import ctypes as C

            t = C.c_double()
            _abi.check(_abi.lib().dg_time_steps(g._h, steps, 0.0, dt, 0.0, 0.0, C.byref(t)), "dg_time_steps")
            ms[prec] = t.value
            outs[prec] = [g.Q]
        kt = np.zeros(5)
        gm = make_single(_abi.DG_PRECISION_MIXED)
        _abi.check(_abi.lib().dg_kernel_times(gm._h, 10, 0.0, dt, _abi.f64ptr(kt)), "dg_kernel_times")
        kernels = dict(zip(["volume", "flux", "update", "traces"], [round(float(v), 5) for v in kt[:4]]))
        launches = steps * 9
    else:
        b64 = make(_abi.DG_PRECISION_FP64)
        dts = b64.max_time_steps(CFL, CFL)
        bm = make(_abi.DG_PRECISION_MIXED)
        t_tune = time.perf_counter()
        if not args.no_autotune:
            b64.autotune(5)  # elements per CTA of every order triple (cached for the process)
            bm.autotune(5)
        t_tune = time.perf_counter() - t_tune
        ms = {_abi.DG_PRECISION_FP64: timed(b64, dts), _abi.DG_PRECISION_MIXED: timed(bm, dts)}
        outs = {_abi.DG_PRECISION_FP64: b64.get(), _abi.DG_PRECISION_MIXED: bm.get()}
        kt = np.zeros(5)
        _abi.check(_abi.lib().dg_kernel_times(bm._h, 10, 0.0, 0.0, _abi.f64ptr(kt)), "dg_kernel_times")
        kernels = dict(zip(["volume", "face_flux", "update", "traces", "face_jump"], [round(float(v), 5) for v in kt]))
        kernels["autotune_s"] = round(t_tune, 2)
        launches = steps * 3 * (4 if cfgs[0].flow == "ns" else 3)
    errs = np.array([rel_l2(a, b, m.quadrature_weights())
                     for a, b, m in zip(outs[_abi.DG_PRECISION_MIXED], outs[_abi.DG_PRECISION_FP64], meshes)])
    mixed = 3.0 * ndof * steps / (ms[_abi.DG_PRECISION_MIXED] * 1e-3)
    plain = 3.0 * ndof * steps / (ms[_abi.DG_PRECISION_FP64] * 1e-3)
    cpu = None
    if not args.no_cpu_baseline:  # one oracle RK3 step of every case, on all host cores
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle as oracle_mod

        t0 = time.perf_counter()
        for m, c, q in zip(meshes, cfgs, qs):
            o = oracle_mod.Oracle(m, c.physics(), c.options())
            o.set_state(q)
            o.rk3_step(0.0, 1e-4)
        el = time.perf_counter() - t0
        cpu = {"value": 3.0 * ndof / el, "unit": "DOF*stage/s", "cores": os.cpu_count() or 1, "kind": "port",
               "sample": f"one RK3 step of every case ({el:.1f} s)"}
    line = {"workload": name, "metric": "DOF*RK-stage updates/s", "value": mixed, "unit": "DOF*stage/s",
            "n_gpus": 1, "steps": steps, "warmup": args.warmup,
            "ms_per_step": ms[_abi.DG_PRECISION_MIXED] / steps, "higher_is_better": True,
            "dtype": "f32 fluxes / f64 state", "data": "synthetic",
            "config": {"workload": SECONDARY[name], "cases": len(meshes), "ndof": ndof,
                       "elements": sum(m.n_elements for m in meshes), "dt": "CFL 0.4 at t=0 per case, fixed"},
            "plain_fp64": {"value": plain, "ms_per_step": ms[_abi.DG_PRECISION_FP64] / steps},
            "mixed_over_plain": mixed / plain,
            "rel_l2_mixed_vs_fp64_max": [float(v) for v in errs.max(axis=0)],
            "kernel_ms_mixed": kernels, "gpu_launches": launches, "cpu_baseline": cpu}
    print(json.dumps(line))


def oracle_steps(case, steps: int, dt: float):
    """The FP64 oracle on the host cores (OpenMP, all threads): `steps` RK3 steps of size dt from the
    workload's initial state. Returns (DOF*stage/s, seconds, final Q)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle

    mesh, q0, base = case
    from horses3d_gb300.control import Config

    cfg = Config(**base)
    o = oracle.Oracle(mesh, cfg.physics(), cfg.options())
    o.set_state(q0)
    t0 = time.perf_counter()
    for s in range(steps):
        o.rk3_step(s * dt, dt)
    el = time.perf_counter() - t0
    return 3.0 * mesh.ndof * steps / el, el, o.get(0)


def reference_arm(args):
    """The CPU reference timing: the oracle (FP64, OpenMP on all host threads) on its own build of the
    workload's mesh and geometry; W untimed then K timed RK3 steps with the fixed CFL dt at t=0. Only
    oracle/ is loaded (the product modules imported here are ctypes declarations and numpy initial
    conditions)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle

    from horses3d_gb300 import _abi, problems
    from horses3d_gb300.control import Config

    oracle.build()
    mesh = oracle.BoxMesh(args.elements, [0.0] * 3, [2 * np.pi] * 3, ORDER, node_type=_abi.DG_NODES_GAUSS, warp=WARP,
                          patch_order=ORDER)
    cfg = Config(order=ORDER, nodes=_abi.DG_NODES_GAUSS, mach=MACH, reynolds=RE, riemann=_abi.DG_RIEMANN_LXF)
    o = oracle.Oracle(mesh, cfg.physics(), cfg.options())
    o.set_state(problems.taylor_green(mesh.x, MACH))
    dt = o.max_dt(CFL, CFL)
    t = 0.0
    for _ in range(args.warmup):
        o.rk3_step(t, dt)
        t += dt
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.rk3_step(t, dt)
        t += dt
    el = time.perf_counter() - t0
    return 3.0 * mesh.ndof * args.steps / el, el, mesh.ndof


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--elements", type=int, default=N_ELEM, help="elements per direction (profiling runs)")
    ap.add_argument("--profile", choices=["mixed", "fp64", "mixed_tc"], default=None,
                    help="profiling run: only warm-up + timed steps of one form, no extra legs")
    ap.add_argument("--workload", choices=["tgv32_curvilinear", *SECONDARY], default="tgv32_curvilinear",
                    help="the headline workload (default) or one of the other benchmark configurations")
    ap.add_argument("--no-autotune", action="store_true", help="variable-order workloads: default item sizes")
    args = ap.parse_args()
    args.steps_given = "--steps" in sys.argv
    rank, world, local = _dist()
    if world > 1:
        import torch.distributed as dist

        if args.impl == "gb300":
            import torch

            torch.cuda.set_device(local)  # one GPU per rank, before NCCL picks one
        dist.init_process_group("nccl" if args.impl == "gb300" else "gloo")
    threads = os.cpu_count() or 1
    metric = "DOF*RK-stage updates/s"
    config = {"workload": WORKLOAD, "elements": args.elements ** 3, "order": ORDER,
              "ndof": (args.elements * (ORDER + 1)) ** 3,
              "nodes": "gauss", "riemann": "lax-friedrichs", "viscous": "br1", "mach": MACH, "reynolds": RE,
              "warp": WARP, "dt": "CFL 0.4 at t=0, fixed", "l2": "inputs larger than L2 (Q alone 283 MB)",
              "parallelism": f"replicas x{world}"}
    if args.impl == "reference":
        if rank != 0:
            return
        rate, el, ndof = reference_arm(args)
        line = {"impl": "reference", "metric": metric, "value": rate, "unit": "DOF*stage/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": el * 1e3 / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": config,
                "cpu_baseline": {"value": rate, "unit": "DOF*stage/s", "cores": threads, "kind": "port",
                                 "sample": f"{args.steps} timed RK3 steps (after {args.warmup} untimed) of the full "
                                           f"{args.elements}^3 N={ORDER} workload ({ndof} DOF), {el:.1f} s"},
                "e2e": {"value": rate, "unit": "DOF*stage/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "note": "Fortran reference not buildable here (no Fortran compiler); the oracle port of its "
                        "loops runs on all host threads, on the oracle's own mesh and geometry"}
        print(json.dumps(line))
        return
    from horses3d_gb300 import build as product_build

    if rank == 0:
        product_build.build()
    _barrier(world)
    if args.workload != "tgv32_curvilinear":
        if rank == 0:
            run_secondary(args.workload, args)
        return
    case = build_case(args.elements)
    if args.profile:
        from horses3d_gb300.control import Config
        from horses3d_gb300.solver import NavierStokesDG

        mesh, q0, base = case
        prec = {"fp64": 0, "mixed": 1, "mixed_tc": 2}[args.profile]
        g = NavierStokesDG(mesh, Config(**base, precision=prec))
        g.set_state(q0)
        dt = g.max_time_step(CFL, CFL)
        t = g.run_steps(args.warmup, 0.0, dt=dt)
        t = g.run_steps(args.steps, t, dt=dt)
        # then the monitored device loop (CFL dt, residuals, NaN check) for as many steps
        t, _ = g.integrate_on_device(args.steps, t, cfl=CFL, dcfl=CFL)
        print(json.dumps({"profile": args.profile, "elements": args.elements, "ndof": mesh.ndof, "t_end": t}))
        return
    r = run_gpu_arm(args, rank, world, local, case)
    cpu = None
    vs_oracle = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # the oracle over the same W+K fixed-dt steps from the same state: the CPU baseline's timing
        # and the accuracy of both GPU forms against the FP64 oracle
        rate, el, q_ref = oracle_steps(case, args.warmup + args.steps, r["dt_fixed"])
        cpu = {"value": rate, "unit": "DOF*stage/s", "cores": threads, "kind": "port",
               "sample": f"{args.warmup + args.steps} RK3 steps of the full workload ({el:.1f} s)"}
        from horses3d_gb300.problems import rel_l2

        vs_oracle = {"steps": args.warmup + args.steps,
                     "mixed": [float(v) for v in rel_l2(r["q_mixed"], q_ref)],
                     "plain_fp64": [float(v) for v in rel_l2(r["q_fp64"], q_ref)],
                     "tensor_core_form": [float(v) for v in rel_l2(r["q_tc"], q_ref)]}
    if rank != 0:
        return
    line = {"metric": metric, "value": r["value"], "unit": "DOF*stage/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 fluxes / f64 state", "data": "synthetic", "config": config,
            "plain_fp64": {"value": r["plain"], "ms_per_step": r["plain_ms_per_step"], "roofline": r["plain_roofline"]},
            "mixed_over_plain": r["mixed_over_plain"], "rel_l2_mixed_vs_fp64": r["rel_l2_mixed_vs_fp64"],
            "rel_l2_vs_oracle": vs_oracle, "tensor_core_form": r["tensor_core_form"],
            "roofline": r["roofline"], "cpu_baseline": cpu, "e2e": r["e2e"], "clocks": r["clocks"],
            "gpu_launches": r["gpu_launches"], "kernel_ms_mixed": r["kernel_ms_mixed"],
            "kernel_ms_fp64": r["kernel_ms_fp64"]}
    print(json.dumps(line))


if __name__ == "__main__":
    main()
