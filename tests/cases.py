"""Small versions of the benchmark configurations, shared by the parity tests."""
from __future__ import annotations

import numpy as np

from horses3d_gb300 import _abi, problems
from horses3d_gb300.control import Config
from horses3d_gb300.mesh import HexMesh

TWO_PI = 2.0 * np.pi


def tgv_case(n=4, order=3, nodes=_abi.DG_NODES_GAUSS_LOBATTO, riemann=_abi.DG_RIEMANN_ROE,
             inviscid=_abi.DG_INVISCID_STANDARD, averaging=_abi.DG_AVG_STANDARD, mach=0.1, reynolds=1600.0,
             warp=0.0, perturbation=0.0, seed=0, precision=_abi.DG_PRECISION_FP64, flow="ns"):
    mesh = HexMesh.box(n, [0, 0, 0], [TWO_PI] * 3, order, node_type=nodes, warp=warp,
                       patch_order=order if warp else 0)
    cfg = Config(order=order, nodes=nodes, flow=flow, mach=mach, reynolds=reynolds, riemann=riemann,
                 averaging=averaging, inviscid=inviscid, precision=precision)
    q0 = problems.taylor_green(mesh.x, mach, perturbation=perturbation, seed=seed)
    return mesh, cfg, q0


def vortex_case(n=4, order=3, nodes=_abi.DG_NODES_GAUSS, mach=0.5, precision=_abi.DG_PRECISION_FP64):
    L = 10.0
    mesh = HexMesh.box(n, [-L / 2] * 3, [L / 2] * 3, order, node_type=nodes)
    cfg = Config(order=order, nodes=nodes, flow="euler", mach=mach, riemann=_abi.DG_RIEMANN_LXF, precision=precision)
    q0 = problems.isentropic_vortex(mesh.x, mach, strength=5.0, period=L)
    return mesh, cfg, q0


def convergence_case(order=7, precision=_abi.DG_PRECISION_FP64):
    """The reference's NavierStokes/Convergence case: periodic [-1,1]x[0,2]x[-1,1] with 4^3 elements
    (UnitCube4x4.mesh), Gauss nodes, Roe, BR1, M=0.3, Re=10, manufactured source."""
    mesh = HexMesh.box(4, [-1, 0, -1], [1, 2, 1], order, node_type=_abi.DG_NODES_GAUSS)
    cfg = Config(order=order, nodes=_abi.DG_NODES_GAUSS, mach=0.3, reynolds=10.0, riemann=_abi.DG_RIEMANN_ROE,
                 precision=precision, source=_abi.DG_SOURCE_MMS_CONVERGENCE, cfl=0.5, dcfl=1.0e5, t_final=1.0,
                 n_steps=1000000)
    q0, _ = problems.mms_convergence_state(mesh.x, 0.0)
    return mesh, cfg, q0


def convergence_variant_case(variant, precision=_abi.DG_PRECISION_FP64):
    """NavierStokes/Convergence_energy and Convergence_entropy: the Convergence case on Gauss-Lobatto
    nodes in split form at CFL 1, with the energy gradient variables (Roe, Pirozzoli) or the entropy
    gradient variables (matrix dissipation, Chandrasekar) (Convergence_*/Convergence.control)."""
    mesh = HexMesh.box(4, [-1, 0, -1], [1, 2, 1], 7, node_type=_abi.DG_NODES_GAUSS_LOBATTO)
    if variant == "energy":
        riemann, avg, gv = _abi.DG_RIEMANN_ROE, _abi.DG_AVG_PIROZZOLI, _abi.DG_GRADVARS_ENERGY
    else:
        riemann, avg, gv = _abi.DG_RIEMANN_MATRIX_DISS, _abi.DG_AVG_CHANDRASEKAR, _abi.DG_GRADVARS_ENTROPY
    cfg = Config(order=7, nodes=_abi.DG_NODES_GAUSS_LOBATTO, mach=0.3, reynolds=10.0, riemann=riemann,
                 inviscid=_abi.DG_INVISCID_SPLIT, averaging=avg, gradient_variables=gv, precision=precision,
                 source=_abi.DG_SOURCE_MMS_CONVERGENCE, cfl=1.0, dcfl=1.0e5, t_final=1.0, n_steps=1000000)
    q0, _ = problems.mms_convergence_state(mesh.x, 0.0)
    return mesh, cfg, q0


# Goldens of Convergence_energy and Convergence_entropy (SETUP/ProblemFile.f90:618-633, tol 1e-11 on x+1).
CONVERGENCE_VARIANT_GOLDENS = {
    "energy": (np.array([6.2838924111412731E-01, 1.8880402299553984E+00, 2.5257816906017094E+00,
                         4.4137338696617938E+00, 2.5153751482782658E+00]),
               np.array([6.7174769052792914E-06, 7.8936751849804373E-06, 2.8203611177044557E-06,
                         6.6884144365250127E-06, 1.4116624697295942E-05]),
               np.array([1.2370219075207763E-04, 1.1813999720732922E-04, 4.0653170754839378E-05,
                         1.2358578587070169E-04, 2.1723315094097264E-04])),
    "entropy": (np.array([6.2929844029491377E-01, 1.8894710750845625E+00, 2.5264755519384234E+00,
                          4.4146672499485859E+00, 2.5157533917446182E+00]),
                np.array([3.3102799903292017E-05, 3.6405407003671022E-05, 1.5957629488942332E-05,
                          3.4132613560424396E-05, 6.6811198249671421E-05]),
                np.array([9.2273153574772720E-04, 9.6259031804949867E-04, 3.8474183309141608E-04,
                          8.7717012428247660E-04, 1.6750805236722724E-03])),
}


# Goldens of Solver/test/NavierStokes/Convergence/SETUP/ProblemFile.f90:617-635 (tol 1e-11 on x+1).
CONVERGENCE_RESIDUALS = np.array([6.2801762330611588E-01, 1.8889640334957627E+00, 2.5256897695536247E+00,
                                  4.4142472296503827E+00, 2.5163928650671146E+00])
CONVERGENCE_Q_ERRORS = np.array([1.0983475326313417E-06, 1.4788256133056976E-06, 4.5499827613507929E-07,
                                 9.0819927730318800E-07, 2.5402026557722347E-06])
CONVERGENCE_QDOT_ERRORS = np.array([1.1342700947907287E-05, 1.1638989807665964E-05, 3.5549224957856481E-06,
                                    1.0769093706709006E-05, 2.0658954210939997E-05])
# The error norm of that test uses these tabulated Gauss-Lobatto weights (ProblemFile.f90:643-650).
WLGL7 = np.array([0.035714285714286, 0.210704227143506, 0.341122692483504, 0.412458794658704,
                  0.412458794658704, 0.341122692483504, 0.210704227143506, 0.035714285714286])


def convergence_errors(mesh, q, qdot, t):
    qe, qde = problems.mms_convergence_state(mesh.x, t)
    w3 = (WLGL7[None, None, :] * WLGL7[None, :, None] * WLGL7[:, None, None]).reshape(-1)
    J = mesh.jacobian.reshape(mesh.n_elements, -1)
    dq = (q - qe).reshape(mesh.n_elements, -1, 5)
    dqd = (qdot - qde).reshape(mesh.n_elements, -1, 5)
    err = np.sqrt(np.einsum("ep,p,epv->v", J, w3, dq ** 2))
    qerr = np.sqrt(np.einsum("ep,p,epv->v", J, w3, dqd ** 2))
    return err, qerr


def lamb_vector_case(precision=_abi.DG_PRECISION_FP64):
    """The reference's NavierStokes/LambVector case: periodic [0, 2 pi]^3 with 8^3 elements
    (TaylorGreen8.mesh), N=5 Gauss nodes, Roe, BR1, M=0.08, Re=1600, dt=0.005 to t=0.100001,
    manufactured source (LambVector/TaylorGreen.control)."""
    mesh = HexMesh.box(8, [0, 0, 0], [TWO_PI] * 3, 5, node_type=_abi.DG_NODES_GAUSS)
    cfg = Config(order=5, nodes=_abi.DG_NODES_GAUSS, mach=0.08, reynolds=1600.0, riemann=_abi.DG_RIEMANN_ROE,
                 precision=precision, source=_abi.DG_SOURCE_MMS_LAMB_VECTOR, dt=0.005, t_final=0.100001,
                 n_steps=10000)
    return mesh, cfg, problems.mms_lamb_vector_state(mesh.x, 0.0)


# Golden of Solver/test/NavierStokes/LambVector/SETUP/ProblemFile.f90:753-756 (tol 1e-7).
LAMB_VECTOR_L2 = 3.4755642143319206E-05
# Gauss weights N=5 tabulated in that test (ProblemFile.f90:587-594).
WG5 = np.array([0.17132449237917019, 0.36076157304813833, 0.46791393457269093, 0.46791393457269093,
                0.36076157304813833, 0.17132449237917019])


def lamb_vector_l2_error(mesh, q, t):
    """sqrt(sum_e sum_ijk w_i w_j w_k J |Q_exact - Q|^2 / K) (ProblemFile.f90:637-750)."""
    qe = problems.mms_lamb_vector_state(mesh.x, t)
    w3 = (WG5[None, None, :] * WG5[None, :, None] * WG5[:, None, None]).reshape(-1)
    J = mesh.jacobian.reshape(mesh.n_elements, -1)
    d2 = np.sum(((q - qe).reshape(mesh.n_elements, -1, 5)) ** 2, axis=2)
    return float(np.sqrt(np.sum(J * w3[None, :] * d2) / mesh.n_elements))


GOLDEN_DIR = __import__("pathlib").Path(__file__).resolve().parent / "golden"

# Root of a reference source tree, when one is mounted (read only by the fallback below).
REFERENCE_ENV = "HORSES3D_REFERENCE"


def reference_file(rel: str, tmp_dir=None):
    """A file of the reference tree by its path within the project (e.g.
    "Solver/test/TestMeshes/UnitCube4x4.mesh"): the committed gzip fixture of that name
    (tests/golden/make_fixtures.py) decompressed into tmp_dir (a temporary directory when None), else
    the file under the root named by $HORSES3D_REFERENCE, else None (the caller skips)."""
    import gzip
    import os
    import tempfile
    from pathlib import Path

    name = Path(rel).name
    fixture = GOLDEN_DIR / f"{name}.gz"
    if fixture.exists():
        out = Path(tmp_dir if tmp_dir is not None else tempfile.mkdtemp(prefix="h3d_ref_")) / name
        if not out.exists():
            out.write_bytes(gzip.decompress(fixture.read_bytes()))
        return out
    root = os.environ.get(REFERENCE_ENV)
    if root and (Path(root) / rel).exists():
        return Path(root) / rel
    return None

# Solver/test/NavierStokes/{Energy,Entropy}ConservingTest/SETUP/ProblemFile.f90:555-561 (tol 1e-11 on
# x+1, 1e-10 for the y-momentum)
CONSERVING_GOLDENS = {
    "EnergyConservingTest": np.array([8.4536070422136675E+01, 2.1762123673954497E+02, 6.4602872675548434E-11,
                                      4.0133134577655784E+02, 2.3743041720710371E+03]),
    "EntropyConservingTest": np.array([8.2631424496364474E+01, 2.2430272815501075E+02, 6.4161760571618557E-11,
                                       4.1620680221184398E+02, 2.3047571785589912E+03]),
}


def conserving_cylinder_config(test):
    """The configuration of {Energy,Entropy}ConservingTest.control: N=5 on Gauss-Lobatto nodes (split
    form), central fluxes, Pirozzoli + energy / Chandrasekar + entropy gradient variables, M=0.3,
    Re=200, AoA phi 90, CFL 0.3 for 10 steps, no-slip walls on the cylinder and the side walls."""
    energy = test == "EnergyConservingTest"
    cfg = Config(order=5, nodes=_abi.DG_NODES_GAUSS_LOBATTO, mach=0.3, reynolds=200.0, riemann=_abi.DG_RIEMANN_CENTRAL,
                 inviscid=_abi.DG_INVISCID_SPLIT,
                 averaging=_abi.DG_AVG_PIROZZOLI if energy else _abi.DG_AVG_CHANDRASEKAR,
                 gradient_variables=_abi.DG_GRADVARS_ENERGY if energy else _abi.DG_GRADVARS_ENTROPY,
                 cfl=0.3, dcfl=0.3, n_steps=10, aoa_theta=0.0, aoa_phi=90.0)
    cfg.periodic = [("bottom", "top"), ("back", "front")]
    cfg.boundaries = {z: {"type": "noslipwall"} for z in ("innercylinder", "left", "right")}
    return cfg


def cylinder_mesh(cfg, tmp_dir):
    """CylinderNSpol3.mesh from the committed fixture (tests/golden/make_fixtures.py)."""
    import gzip

    path = __import__("pathlib").Path(tmp_dir) / "CylinderNSpol3.mesh"
    path.write_bytes(gzip.decompress((GOLDEN_DIR / "CylinderNSpol3.mesh.gz").read_bytes()))
    return HexMesh.from_specmesh(path, cfg.order, node_type=cfg.nodes, periodic=cfg.periodic_spec())


# The NavierStokes Cylinder family (Solver/test/NavierStokes/<case>/SETUP/ProblemFile.f90): the five
# residuals after 100 CFL steps from the free stream, FTAssertEqual on value + 1 with the case's
# tolerance, and the mesh fixture of the case.
CYLINDER_GOLDENS = {
    # Cylinder/SETUP/ProblemFile.f90:556-560,572-595
    "Cylinder": (np.array([8.8131248889811715e+00, 1.7608838068776613e+01, 1.9037533106262516e-01,
                           2.4301352846288605e+01, 2.4063786464536835e+02]), 1e-11),
    # CylinderDucros/SETUP/ProblemFile.f90:555-559,570-593
    "CylinderDucros": (np.array([9.49419906221126, 24.2427358262976, 0.231929845707823, 27.3961550687737,
                                 259.972329181719]), 1e-11),
    # CylinderChandrasekarRoe/SETUP/ProblemFile.f90:538-542,548-571
    "CylinderChandrasekarRoe": (np.array([9.292005572719354, 24.258016397589838, 0.2388511827572224,
                                          28.435107391243378, 253.03319158649319]), 1e-7),
    # CylinderDifferentOrders/SETUP/ProblemFile.f90:556-560,572-595
    "CylinderDifferentOrders": (np.array([9.5806856005342933e+00, 2.0804408993372231e+01, 3.7668665836122439e-01,
                                          2.8294964263463125e+01, 2.6470704194989690e+02]), 1e-11),
}


def cylinder_case_config(case):
    """<case>.control of the Cylinder family: M=0.3, Re=200, AoA phi 90, CFL = dCFL = 0.3, 100 steps,
    a no-slip wall on the cylinder, free-slip walls at bottom/top, inflow at back/left/front and
    outflow at right. Cylinder: N=3 Gauss, Roe. CylinderDucros: split form (Gauss-Lobatto), standard
    Roe, Ducros average. CylinderChandrasekarRoe: split form, Roe, Chandrasekar average.
    CylinderDifferentOrders: Roe, Re=45, CFL = dCFL = 0.2, per-element (Nx, Ny, Nz) from
    OrdersN2N3N4N5_anisotropy.csv. CylinderDucros sets the Roe dissipation scaling lambda to 0.9."""
    split = case in ("CylinderDucros", "CylinderChandrasekarRoe")
    cfg = Config(order=3, nodes=_abi.DG_NODES_GAUSS_LOBATTO if split else _abi.DG_NODES_GAUSS, mach=0.3,
                 reynolds=200.0, riemann=_abi.DG_RIEMANN_STD_ROE if case == "CylinderDucros" else _abi.DG_RIEMANN_ROE,
                 inviscid=_abi.DG_INVISCID_SPLIT if split else _abi.DG_INVISCID_STANDARD,
                 averaging={"CylinderDucros": _abi.DG_AVG_DUCROS,
                            "CylinderChandrasekarRoe": _abi.DG_AVG_CHANDRASEKAR}.get(case, _abi.DG_AVG_STANDARD),
                 cfl=0.3, dcfl=0.3, n_steps=100, aoa_theta=0.0, aoa_phi=90.0, convergence_tolerance=1e-10)
    if case == "CylinderDucros":
        cfg.lambda_stab = 0.9
    if case == "CylinderDifferentOrders":
        cfg.order_file = "MESH/OrdersN2N3N4N5_anisotropy.csv"
        cfg.reynolds = 45.0
        cfg.cfl = cfg.dcfl = 0.2
    cfg.boundaries = {"innercylinder": {"type": "noslipwall"}, "bottom": {"type": "freeslipwall"},
                      "top": {"type": "freeslipwall"}, "back": {"type": "inflow"}, "left": {"type": "inflow"},
                      "front": {"type": "inflow"}, "right": {"type": "outflow"}}
    return cfg


def cylinder_case_mesh(case, cfg, tmp_dir):
    """The case's mesh (and orders) from the committed fixtures (tests/golden/make_fixtures.py)."""
    import gzip
    from pathlib import Path

    from horses3d_gb300.control import read_order_file

    name = "CylinderNSpol3_1elem_y.mesh" if case == "CylinderDifferentOrders" else "CylinderNSpol3.mesh"
    path = Path(tmp_dir) / name
    path.write_bytes(gzip.decompress((GOLDEN_DIR / f"{name}.gz").read_bytes()))
    orders = cfg.order
    if cfg.order_file is not None:
        op = Path(tmp_dir) / Path(cfg.order_file).name
        op.write_bytes(gzip.decompress((GOLDEN_DIR / f"{op.name}.gz").read_bytes()))
        orders = read_order_file(op)
    return HexMesh.from_specmesh(path, orders, node_type=cfg.nodes, periodic=cfg.periodic_spec())


# Euler BoxAroundCircle and BoxAroundCirclePirozzoli (Solver/test/Euler/<case>/SETUP/ProblemFile.f90):
# the five residuals after 1000 CFL steps from the free stream, FTAssertEqual on value + 1, tol 1e-11.
BOX_AROUND_CIRCLE_GOLDENS = {
    # BoxAroundCircle/SETUP/ProblemFile.f90:349-353,363-391
    "BoxAroundCircle": np.array([3.9167069726447580e-03, 7.0027671589173224e-02, 3.6068228611380296e-13,
                                 8.2231956082004870e-02, 0.10659815868258372]),
    # BoxAroundCirclePirozzoli/SETUP/ProblemFile.f90:323-327,337-365
    "BoxAroundCirclePirozzoli": np.array([3.2245412233756249e-03, 7.2948338786761158e-02, 7.8482433396760149e-12,
                                          6.3956090995916370e-02, 9.8435366345196243e-02]),
}


def box_around_circle_config(case):
    """<case>.control: Euler, N=3, standard Roe, CFL 0.7, M=0.3, AoA 0, 1000 steps; free-slip walls
    on the cylinder, bottom and top, inflow on front, back, left and right. The Pirozzoli case runs
    the split form (Gauss-Lobatto) with the Pirozzoli average."""
    split = case == "BoxAroundCirclePirozzoli"
    cfg = Config(order=3, nodes=_abi.DG_NODES_GAUSS_LOBATTO if split else _abi.DG_NODES_GAUSS, flow="euler",
                 mach=0.3, reynolds=0.0, riemann=_abi.DG_RIEMANN_STD_ROE,
                 inviscid=_abi.DG_INVISCID_SPLIT if split else _abi.DG_INVISCID_STANDARD,
                 averaging=_abi.DG_AVG_PIROZZOLI if split else _abi.DG_AVG_STANDARD, cfl=0.7, dcfl=0.7,
                 n_steps=1000, aoa_theta=0.0, aoa_phi=0.0, convergence_tolerance=1e-10)
    cfg.boundaries = {z: {"type": "freeslipwall"} for z in ("innercylinder", "bottom", "top")}
    cfg.boundaries.update({z: {"type": "inflow"} for z in ("front", "back", "left", "right")})
    return cfg


def box_around_circle_mesh(cfg, tmp_dir):
    """BoxAroundCircle3D_extended_pol3.mesh from the committed fixture (tests/golden/make_fixtures.py)."""
    import gzip

    path = __import__("pathlib").Path(tmp_dir) / "BoxAroundCircle3D_extended_pol3.mesh"
    path.write_bytes(gzip.decompress((GOLDEN_DIR / f"{path.name}.gz").read_bytes()))
    return HexMesh.from_specmesh(path, cfg.order, node_type=cfg.nodes, periodic=cfg.periodic_spec())


# NavierStokes TaylorGreen (Solver/test/NavierStokes/TaylorGreen/SETUP/ProblemFile.f90:317-366): after 5
# CFL steps the five residuals (tol 1e-7 on value + 1) and the volume monitors kinetic energy, its
# rate (on value + 1) and enstrophy (tol 1e-11). Euler TaylorGreenKEPEC
# (Solver/test/Euler/TaylorGreenKEPEC/SETUP/ProblemFile.f90:337-395): after 10 steps the residuals
# (1e-7), kinetic energy (1e-11), its rate and the entropy rate (1e-11 on value + 1).
TAYLOR_GREEN_GOLDENS = {
    "TaylorGreen": {
        "residuals": np.array([1.6417830052388520e-05, 1.2677577061211545e-01, 1.2677577048633804e-01,
                               2.4981129585617484e-01, 6.2174425106488129e-01]),
        "kinetic_energy": 1.2499879367819486e-01,
        "kinetic_energy_rate": -4.2807806718622574e-04,
        "enstrophy": 3.7499683882517909e-01,
    },
    "TaylorGreenKEPEC": {
        "residuals": np.array([1.1131779208842484e-04, 0.12741606758485369, 0.12741606776695064,
                               0.24998271835184718, 0.62461894702221510]),
        "kinetic_energy": 0.12500000000766839,
        "kinetic_energy_rate": 2.3284871259485850e-06,
        "entropy_rate": 2.346803715467861e-08,
    },
}


def taylor_green_reference_case(test="TaylorGreen", n=32):
    """TaylorGreen.control: N=3 Gauss, Roe, BR1, CFL = dCFL = 0.4, M=0.08, Re=1600, 5 steps, periodic.
    TaylorGreenKEPEC.control: Euler, split form with the Chandrasekar average (Gauss-Lobatto), central
    flux, N=3, CFL 0.4, M=0.08, 10 steps. Their mesh, TaylorGreen32.mesh, is not in the reference tree;
    a generated periodic box of n^3 straight elements on [0, 2 pi]^3 (the domain of the
    TaylorGreen8.mesh that is there) stands in for it. The initial condition is the tests' own
    (TaylorGreen ProblemFile.f90:64-148): rho 1, the Taylor-Green velocity, and
    p = 100 + (cos 2x cos 2z + 2 cos 2y + 2 cos 2x + cos 2y cos 2z) / 16."""
    if test == "TaylorGreen":
        cfg = Config(order=3, nodes=_abi.DG_NODES_GAUSS, mach=0.08, reynolds=1600.0, riemann=_abi.DG_RIEMANN_ROE,
                     cfl=0.4, dcfl=0.4, n_steps=5, convergence_tolerance=1e-10)
    else:
        cfg = Config(order=3, nodes=_abi.DG_NODES_GAUSS_LOBATTO, flow="euler", mach=0.08, reynolds=0.0,
                     riemann=_abi.DG_RIEMANN_CENTRAL, inviscid=_abi.DG_INVISCID_SPLIT,
                     averaging=_abi.DG_AVG_CHANDRASEKAR, cfl=0.4, dcfl=0.4, n_steps=10, convergence_tolerance=1e-10)
    cfg.periodic = [("front", "back"), ("bottom", "top"), ("left", "right")]
    mesh = HexMesh.box(n, [0, 0, 0], [TWO_PI] * 3, 3, node_type=cfg.nodes)
    x, y, z = mesh.x[:, 0], mesh.x[:, 1], mesh.x[:, 2]
    u = np.sin(x) * np.cos(y) * np.cos(z)
    v = -np.cos(x) * np.sin(y) * np.cos(z)
    p = 100.0 + (np.cos(2 * x) * np.cos(2 * z) + 2 * np.cos(2 * y) + 2 * np.cos(2 * x) + np.cos(2 * y) * np.cos(2 * z)) / 16.0
    q = np.stack([np.ones_like(u), u, v, np.zeros_like(u), p / 0.4 + 0.5 * (u * u + v * v)], axis=1).ravel()
    return mesh, cfg, q


def entropy_rate(mesh, q, qdot):
    """The entropy-rate volume monitor (VolumeIntegrals.f90:322-331 over the volume): the quadrature of
    QDot . U with U the entropy variables of NSGradientVariables_ENTROPY."""
    Q = q.reshape(-1, 5)
    D = qdot.reshape(-1, 5)
    rho = Q[:, 0]
    rv2 = np.sum(Q[:, 1:4] ** 2, axis=1) / rho
    p = 0.4 * (Q[:, 4] - 0.5 * rv2)
    U = np.stack([(1.4 - (np.log(p) - 1.4 * np.log(rho))) / 0.4 - 0.5 * rv2 / p, Q[:, 1] / p, Q[:, 2] / p,
                  Q[:, 3] / p, -rho / p], axis=1)
    w = mesh.quadrature_weights()
    return np.sum(w * np.sum(D * U, axis=1)) / np.sum(w)


def volume_monitors(mesh, q, qdot, ux=None, uy=None, uz=None):
    """Kinetic energy, its rate and enstrophy per unit volume (VolumeMonitor.f90:298-310 with
    VolumeIntegrals.f90:179-286): quadratures of 1/2 |rho V|^2 / rho, of u . d(rho V)/dt - |u|^2/2
    d(rho)/dt, and of 1/2 |curl u|^2 with the velocity gradients of getVelocityGradients_State."""
    w = mesh.quadrature_weights()
    vol = np.sum(w)
    Q = q.reshape(-1, 5)
    D = qdot.reshape(-1, 5)
    ke = np.sum(w * 0.5 * np.sum(Q[:, 1:4] ** 2, axis=1) / Q[:, 0]) / vol
    vel = Q[:, 1:4] / Q[:, [0]]
    rate = np.sum(w * (np.sum(vel * D[:, 1:4], axis=1) - 0.5 * np.sum(vel ** 2, axis=1) * D[:, 0])) / vol
    if ux is None:
        return ke, rate, None
    inv = 1.0 / Q[:, 0]
    ud = Q[:, 1:4] * (inv * inv)[:, None]
    g = [inv[:, None] * G.reshape(-1, 5)[:, 1:4] - ud * G.reshape(-1, 5)[:, [0]] for G in (ux, uy, uz)]
    om2 = (g[1][:, 2] - g[2][:, 1]) ** 2 + (g[2][:, 0] - g[0][:, 2]) ** 2 + (g[0][:, 1] - g[1][:, 0]) ** 2
    return ke, rate, 0.5 * np.sum(w * om2) / vol


# Euler UniformFlow (Solver/test/Euler/UniformFlow/SETUP/ProblemFile.f90:320-323): per polynomial order,
# the iterations to a maximum residual of 1e-10 (exact) and that final residual (FTAssertEqual, 1e-3).
UNIFORM_FLOW_GOLDENS = {3: (1821, 9.7985624521602423e-11), 4: (3090, 9.7825050715404729e-11),
                        5: (4164, 9.7454147241309180e-11)}


def uniform_flow_config(order=5):
    """UniformFlow.control: Euler, Box27.mesh, Gauss nodes, Rusanov, CFL 0.4, M=0.5, AoA 0, inflow on
    every side (the six zones of one "#define boundary left__right__front__back__bottom__top" block),
    steady state to a maximum residual of 1e-10 (at most 5000 steps)."""
    cfg = Config(order=order, nodes=_abi.DG_NODES_GAUSS, flow="euler", mach=0.5, reynolds=0.0,
                 riemann=_abi.DG_RIEMANN_RUSANOV, cfl=0.4, dcfl=0.4, n_steps=5000, aoa_theta=0.0, aoa_phi=0.0,
                 convergence_tolerance=1e-10)
    cfg.boundaries = {z: {"type": "inflow"} for z in ("left", "right", "front", "back", "bottom", "top")}
    return cfg


def box27_mesh(cfg, tmp_dir):
    """Box27.mesh (27 unit cubes) from the committed fixture (tests/golden/make_fixtures.py)."""
    import gzip

    path = __import__("pathlib").Path(tmp_dir) / "Box27.mesh"
    path.write_bytes(gzip.decompress((GOLDEN_DIR / "Box27.mesh.gz").read_bytes()))
    return HexMesh.from_specmesh(path, cfg.order, node_type=cfg.nodes, periodic=cfg.periodic_spec())


def uniform_flow_state(cfg, mesh):
    """UserDefinedInitialCondition of UniformFlow (ProblemFile.f90:64-144): the free stream, with the
    density of node (3,3,3) of every element raised by 5 % (energy unchanged)."""
    q = free_stream_state(cfg, mesh).reshape(-1, 5)
    P = cfg.order + 1
    q[3 + P * (3 + P * 3)::P ** 3, 0] *= 1.05
    return q.ravel()


def free_stream_state(cfg, mesh):
    rho, u, v, w, p = cfg.free_stream()
    return np.tile([rho, rho * u, rho * v, rho * w, p / 0.4 + 0.5 * rho * (u * u + v * v + w * w)], mesh.ndof)


def ftassert_equal(expected, actual, tol):
    """FTAssertEqual of two reals (ftobject/Comparisons.f90:238-255): relative tolerance, absolute
    below tol."""
    x, y = float(expected), float(actual)
    lim = tol if x <= tol else tol * max(abs(x), abs(y))
    return abs(x - y) <= lim


def ftassert_close(expected, actual, tol=1e-11):
    """FTAssertEqual on (value + 1) as the reference test does (ftobject/Comparisons.f90:238-255)."""
    x, y = np.asarray(expected) + 1.0, np.asarray(actual) + 1.0
    lim = np.where(x <= tol, tol, tol * np.maximum(np.abs(x), np.abs(y)))
    return np.all(np.abs(x - y) <= lim)


def quadrature_weights(mesh):
    """w_i w_j w_k J at every node (for rel-L2 norms)."""
    return mesh.quadrature_weights()


def random_orders(n_elements, lo, hi, seed):
    """(Nx, Ny, Nz) per element drawn i.i.d. uniform from {lo..hi} (numpy PCG64 with the seed)."""
    return np.random.default_rng(seed).integers(lo, hi + 1, size=(n_elements, 3)).astype(np.int32)


def aniso_tgv_case(n=3, lo=1, hi=4, seed=1, nodes=_abi.DG_NODES_GAUSS, riemann=_abi.DG_RIEMANN_ROE, warp=0.0,
                   mach=0.1, reynolds=1600.0, precision=_abi.DG_PRECISION_FP64, perturbation=0.01):
    """Taylor-Green vortex on a p-anisotropic periodic box (faces at the larger order of their sides)."""
    orders = random_orders(n ** 3, lo, hi, seed)
    mesh = HexMesh.box(n, [0, 0, 0], [TWO_PI] * 3, orders, node_type=nodes, warp=warp,
                       patch_order=hi if warp else 0)
    cfg = Config(order=hi, nodes=nodes, flow="ns", mach=mach, reynolds=reynolds, riemann=riemann, precision=precision)
    q0 = problems.taylor_green(mesh.x, mach, perturbation=perturbation, seed=seed)
    return mesh, cfg, q0


def aniso_vortex_case(n=3, lo=2, hi=5, seed=2, nodes=_abi.DG_NODES_GAUSS, riemann=_abi.DG_RIEMANN_LXF,
                      mach=0.5, precision=_abi.DG_PRECISION_FP64, averaging=_abi.DG_AVG_STANDARD):
    """Euler isentropic vortex (strength 5) advected diagonally on a p-anisotropic periodic box."""
    L = 10.0
    orders = random_orders(n ** 3, lo, hi, seed)
    mesh = HexMesh.box(n, [-L / 2] * 3, [L / 2] * 3, orders, node_type=nodes)
    cfg = Config(order=hi, nodes=nodes, flow="euler", mach=mach, riemann=riemann, averaging=averaging,
                 precision=precision)
    q0 = problems.isentropic_vortex(mesh.x, mach, strength=5.0, period=L)
    return mesh, cfg, q0


# Proper rotations of the reference cube (det +1), as matrices acting on local coordinates.
CUBE_ROTATIONS = [
    np.array([[0, -1, 0], [1, 0, 0], [0, 0, 1]]),   # 90 deg about zeta
    np.array([[1, 0, 0], [0, 0, -1], [0, 1, 0]]),   # 90 deg about xi
    np.array([[0, 0, 1], [0, 1, 0], [-1, 0, 0]]),   # 90 deg about eta
    np.array([[0, 0, 1], [1, 0, 0], [0, 1, 0]]),    # cyclic xi -> eta -> zeta
    np.array([[-1, 0, 0], [0, -1, 0], [0, 0, 1]]),  # 180 deg about zeta
    np.array([[0, 1, 0], [1, 0, 0], [0, 0, -1]]),   # 180 deg about the xi=eta diagonal
]
_CORNERS = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]])


def rotated_box_specmesh(path, n=4, length=TWO_PI, seed=0):
    """A periodic n^3 box of straight hexahedra written as a SpecMesh file in which every interior
    element lists its corners in a rotated local frame (a proper rotation of the reference cube, chosen
    by seed), so the faces between elements carry non-zero leftIndexes2Right rotations."""
    rng = np.random.default_rng(seed)
    h = length / n
    m1 = n + 1
    nid = lambda i, j, k: 1 + i + m1 * (j + m1 * k)
    lines = [f"{m1 ** 3} {n ** 3} 1"]
    for k in range(m1):
        for j in range(m1):
            for i in range(m1):
                lines.append(f"{i * h!r} {j * h!r} {k * h!r}")
    for k in range(n):
        for j in range(n):
            for i in range(n):
                ids = [nid(i + a, j + b, k + c) for a, b, c in _CORNERS]
                names = ["front" if j == 0 else "---", "back" if j == n - 1 else "---",
                         "bottom" if k == 0 else "---", "right" if i == n - 1 else "---",
                         "top" if k == n - 1 else "---", "left" if i == 0 else "---"]
                if all(nm == "---" for nm in names):
                    R = CUBE_ROTATIONS[int(rng.integers(len(CUBE_ROTATIONS)))]
                    old = {tuple(c): ids[q] for q, c in enumerate(_CORNERS)}
                    ids = [old[tuple(int(v) for v in (R @ (2 * c - 1) + 1) // 2)] for c in _CORNERS]
                lines.append(" ".join(str(v) for v in ids))
                lines.append("0 0 0 0 0 0")
                lines.append(" ".join(names))
    path.write_text("\n".join(lines) + "\n")
    return path


def rotated_tgv_case(path, order, nodes=_abi.DG_NODES_GAUSS, riemann=_abi.DG_RIEMANN_ROE, n=4, seed=0,
                     flow="ns", inviscid=_abi.DG_INVISCID_STANDARD, averaging=_abi.DG_AVG_STANDARD):
    """Taylor-Green vortex (+1% perturbation) on the rotated-element box; order may be per element."""
    rotated_box_specmesh(path, n=n, seed=seed)
    mesh = HexMesh.from_specmesh(path, order, node_type=nodes)
    cfg = Config(order=int(np.max(order)), nodes=nodes, flow=flow, mach=0.2, reynolds=800.0, riemann=riemann,
                 inviscid=inviscid, averaging=averaging)
    q0 = problems.taylor_green(mesh.x, 0.2, perturbation=0.01, seed=seed + 1)
    return mesh, cfg, q0
