"""Element partitions and their halo exchange, on the CPU.

The partitioner (horses3d_gb300.partition) splits a periodic box into element blocks; every rank
holds one block, runs the oracle on it (OraclePartition) and exchanges, over torch.distributed with
the gloo backend, the face data the reference's MPI faces move between the phases of the
right-hand side (the face Q, then the face gradients; MPI_Face.f90:203-383). The partitioned
right-hand side and RK3 steps (dt reduced with MIN over the ranks) must reproduce the single-domain
oracle on the same mesh to 1e-13. The GPU side of the same partitions is tested in
tests/test_gpu_partition.py."""
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

import cases
import oracle
from horses3d_gb300 import _abi
from horses3d_gb300.partition import partition_mesh

ROOT = Path(__file__).resolve().parents[1]
TOL = 1e-13


def _case(kind):
    if kind == "ns_gl":
        return cases.tgv_case(n=4, order=3, nodes=_abi.DG_NODES_GAUSS_LOBATTO, perturbation=0.02, seed=5)
    if kind == "ns_gauss_warped":
        return cases.tgv_case(n=4, order=3, nodes=_abi.DG_NODES_GAUSS, warp=0.1, perturbation=0.02, seed=6)
    if kind == "euler_vortex":
        return cases.vortex_case(n=4, order=3)
    raise ValueError(kind)


def test_partition_lists_pair_up():
    """Every face lies in the parts of its elements; a cut face is sent by one part and received by
    the other at the same position of their lists; every element side of a part has a face."""
    mesh, _, _ = _case("ns_gl")
    for n_parts in (2, 3, 5):
        parts = partition_mesh(mesh, n_parts)
        assert sum(p.n_elements for p in parts) == mesh.n_elements
        assert sum(p.ndof for p in parts) == mesh.ndof
        for p in parts:
            fe = np.ctypeslib.as_array(p.desc.face_elem, shape=(2 * p.desc.n_faces,)).reshape(-1, 2)
            fs = np.ctypeslib.as_array(p.desc.face_side, shape=(2 * p.desc.n_faces,)).reshape(-1, 2)
            own = [(e, s) for (e, s) in zip(fe.reshape(-1), fs.reshape(-1)) if 0 <= e < p.n_elements]
            assert sorted(own) == sorted((e, s) for e in range(p.n_elements) for s in range(1, 7))
            for n in p.neighbours:
                q = parts[n.rank]
                back = next(m for m in q.neighbours if m.rank == p.rank)
                assert np.array_equal(n.global_faces, back.global_faces)
                assert np.all(n.send_slots < 6 * p.n_elements) and np.all(back.recv_slots >= 6 * q.n_elements)
                assert np.array_equal(n.own_side, 3 - back.own_side)


KINDS = ("ns_gl", "ns_gauss_warped", "euler_vortex")


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), OMP_NUM_THREADS="2")
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "oracle"))
    sys.path.insert(0, str(ROOT / "tests"))
    import torch
    import torch.distributed as dist

    import oracle as orc
    from horses3d_gb300.partition import allreduce, dist_exchange, partition_mesh as pm

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        for kind in KINDS:
            out.put((kind,) + _one_case(rank, world, kind, dist_exchange, allreduce, pm, orc, torch))
    finally:
        dist.destroy_process_group()


def _one_case(rank, world, kind, dist_exchange, allreduce, pm, orc, torch):
    mesh, cfg, q0 = _case(kind)
    part = pm(mesh, world)[rank]

    def exchange(sends, like):
        got = dist_exchange({k: torch.from_numpy(v) for k, v in sends.items()},
                            {k: torch.from_numpy(v) for k, v in like.items()})
        return {k: v.numpy() for k, v in got.items()}

    p = orc.OraclePartition(part, cfg.physics(), cfg.options())
    p.set_state(part.local_state(q0))
    orc.partition_rhs([p], 0.0, exchange)
    full = orc.Oracle(mesh, cfg.physics(), cfg.options())
    full.set_state(q0)
    ref = part.local_state(full.rhs(0.0))
    err_rhs = float(np.max(np.abs(p.get(1) - ref)) / np.max(np.abs(ref)))
    t = 0.0
    for _ in range(3):
        dt = allreduce(p.max_dt(0.4, 0.4), "min")  # MaxTimeStep's MIN over the ranks
        assert dt == full.max_dt(0.4, 0.4)
        orc.partition_rk3_step([p], t, dt, exchange)
        full.rk3_step(t, dt)
        t += dt
    ref = part.local_state(full.get(0))
    err_steps = float(np.max(np.abs(p.get(0) - ref)) / np.max(np.abs(ref)))
    return rank, err_rhs, err_steps, len(part.neighbours)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_reproduce_the_single_domain_oracle():
    """Navier-Stokes on Gauss-Lobatto and on warped Gauss nodes, Euler vortex: right-hand side and
    three CFL steps, two ranks."""
    pytest.importorskip("torch")
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=300) for _ in range(2 * len(KINDS)))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted({r[0] for r in results}) == sorted(KINDS)
    for kind, rank, err_rhs, err_steps, n_nb in results:
        assert n_nb == 1  # two slabs of a periodic box: each part's only neighbour is the other
        assert err_rhs <= TOL and err_steps <= TOL, (kind, rank, err_rhs, err_steps)
