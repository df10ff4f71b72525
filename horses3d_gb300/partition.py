"""Element partitions of a mesh and the halo exchange between them (one partition per GPU).

This is the reference's MPI domain decomposition (HexMesh.f90:1199-1730 UpdateMPIFacesSolution /
UpdateMPIFacesGradients, MPI_Face.f90:203-383, the MIN/MAX reductions of the time step and the
residuals in DGSEMClass.f90:770-868,1019-1021) on the C ABI's partition contexts:

* ``partition_mesh`` splits the elements into contiguous blocks (the element order of the generated
  boxes is a structured sweep, so a block is a slab) and builds, per part, a mesh description of
  its own elements and of every face that touches them. A face to a remote element names it as a
  ghost element ``n_elements + g``; the global face keeps its sides, rotation and geometry, so both
  partitions evaluate a cut face's flux from the same data and get the same bits.
* The exchange lists pair, for every neighbour, this part's own face slots with the neighbour's
  ghost slots, faces in ascending global order on both sides.
* ``PartitionSolver`` drives one partition context; ``rk3_step`` / ``rhs`` advance a list of
  partitions held by this process, with an exchange function that moves the per-neighbour buffers
  (``dist_exchange`` over torch.distributed: NCCL for device tensors, gloo for host tensors; or
  ``local_exchange`` for several partitions in one process).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _abi


@dataclass
class Neighbour:
    rank: int
    faces: np.ndarray       # local face indices of the shared faces, ascending global face id
    global_faces: np.ndarray
    own_side: np.ndarray    # 1 or 2: the side of each face that belongs to this part
    send_slots: np.ndarray  # own element-face slots, 6 * local element + side - 1
    recv_slots: np.ndarray  # ghost slots of the neighbour's elements


@dataclass
class Partition:
    rank: int
    n_parts: int
    elements: np.ndarray    # global ids of the own elements (ascending)
    ghosts: np.ndarray      # global ids of the remote elements across the cut faces (ascending)
    faces: np.ndarray       # global ids of the faces of this part (ascending)
    node_slice: slice       # this part's nodes within the global node order
    neighbours: list[Neighbour]
    desc: _abi.DgMeshDesc = None
    arrays: dict = field(default_factory=dict)  # keeps the description's arrays alive

    @property
    def n_elements(self) -> int:
        return len(self.elements)

    @property
    def n_ghost(self) -> int:
        return len(self.ghosts)

    @property
    def ndof(self) -> int:
        return self.node_slice.stop - self.node_slice.start

    def local_state(self, q_global: np.ndarray) -> np.ndarray:
        """This part's slice of a global state (5 values per node)."""
        return np.ascontiguousarray(q_global[5 * self.node_slice.start:5 * self.node_slice.stop])

    def send_slots(self) -> np.ndarray:
        return np.concatenate([n.send_slots for n in self.neighbours]).astype(np.int32) if self.neighbours else \
            np.zeros(0, np.int32)

    def recv_slots(self) -> np.ndarray:
        return np.concatenate([n.recv_slots for n in self.neighbours]).astype(np.int32) if self.neighbours else \
            np.zeros(0, np.int32)


def _view(ptr, n, dtype=None):
    a = np.ctypeslib.as_array(ptr, shape=(n,))
    return a if dtype is None else a.astype(dtype)


def partition_mesh(mesh, n_parts: int, part_of_element: np.ndarray | None = None) -> list[Partition]:
    """Partitions of a mesh (anything with a ``desc`` DgMeshDesc, ``n_elements`` and ``ndof``):
    contiguous element blocks unless part_of_element is given (it must be non-decreasing, so that
    every part's nodes stay contiguous in the global node order)."""
    d = mesh.desc
    K, F = int(d.n_elements), int(d.n_faces)
    order = _view(d.order, 3 * K).reshape(K, 3)
    npe = np.prod(order + 1, axis=1).astype(np.int64)
    eoff = np.concatenate([[0], np.cumsum(npe)])
    nf = _view(d.face_nf, 2 * F).reshape(F, 2)
    fpts = ((nf[:, 0] + 1) * (nf[:, 1] + 1)).astype(np.int64)
    foff = np.concatenate([[0], np.cumsum(fpts)])
    face_elem = _view(d.face_elem, 2 * F).reshape(F, 2)
    face_side = _view(d.face_side, 2 * F).reshape(F, 2)
    face_rot = _view(d.face_rotation, F)
    face_bnd = _view(d.face_boundary, F) if d.face_boundary else None
    nd = int(eoff[-1])
    node_arrays = {name: (_view(getattr(d, name), w * nd), w) for name, w in (
        ("x", 3), ("ja_xi", 3), ("ja_eta", 3), ("ja_zeta", 3), ("jacobian", 1), ("inv_jacobian", 1))}
    npts = int(foff[-1])
    face_arrays = {name: (_view(getattr(d, name), w * npts), w) for name, w in (
        ("face_normal", 3), ("face_t1", 3), ("face_t2", 3), ("face_jacobian", 1))}
    if part_of_element is None:
        part_of_element = np.concatenate([np.full(len(b), r, np.int32)
                                          for r, b in enumerate(np.array_split(np.arange(K), n_parts))])
    part_of_element = np.asarray(part_of_element, dtype=np.int32)
    if len(part_of_element) != K or np.any(np.diff(part_of_element) < 0) or part_of_element.min() < 0 or \
            part_of_element.max() >= n_parts:
        raise ValueError("part_of_element must assign every element to 0..n_parts-1, non-decreasing")
    pL = part_of_element[face_elem[:, 0]]
    pR = np.where(face_elem[:, 1] >= 0, part_of_element[np.maximum(face_elem[:, 1], 0)], -1)

    parts = []
    for r in range(n_parts):
        own = np.nonzero(part_of_element == r)[0]
        if len(own) == 0:
            raise ValueError(f"part {r} has no elements")
        e0 = int(own[0])
        Kr = len(own)
        fid = np.nonzero((pL == r) | (pR == r))[0]
        other = np.where(pL[fid] == r, face_elem[fid, 1], face_elem[fid, 0])
        other_part = np.where(pL[fid] == r, pR[fid], pL[fid])
        cut = (other >= 0) & (other_part != r)
        ghosts = np.unique(other[cut])
        local = np.full(K, -1, np.int64)
        local[own] = np.arange(Kr)
        local[ghosts] = Kr + np.arange(len(ghosts))
        fe = face_elem[fid].astype(np.int64)
        le = np.where(fe >= 0, local[np.maximum(fe, 0)], -1).astype(np.int32)
        arrays = {
            "order": np.ascontiguousarray(np.concatenate([order[own], order[ghosts]]).reshape(-1), dtype=np.int32),
            "face_elem": np.ascontiguousarray(le.reshape(-1)),
            "face_side": np.ascontiguousarray(face_side[fid].reshape(-1), dtype=np.int32),
            "face_rotation": np.ascontiguousarray(face_rot[fid], dtype=np.int32),
            "face_nf": np.ascontiguousarray(nf[fid].reshape(-1), dtype=np.int32),
        }
        n0, n1 = int(eoff[e0]), int(eoff[e0 + Kr])
        for name, (a, w) in node_arrays.items():
            arrays[name] = np.ascontiguousarray(a[w * n0:w * n1])
        pts = np.concatenate([np.arange(foff[f], foff[f + 1]) for f in fid]) if len(fid) else np.zeros(0, np.int64)
        for name, (a, w) in face_arrays.items():
            arrays[name] = np.ascontiguousarray(a.reshape(-1, w)[pts].reshape(-1))
        if face_bnd is not None:
            arrays["face_boundary"] = np.ascontiguousarray(face_bnd[fid], dtype=np.int32)
        desc = _abi.DgMeshDesc()
        desc.n_elements = Kr
        desc.node_type = d.node_type
        desc.n_faces = len(fid)
        desc.n_boundaries = d.n_boundaries
        desc.boundaries = d.boundaries
        for name, a in arrays.items():
            ctype = C.c_int32 if a.dtype == np.int32 else C.c_double
            setattr(desc, name, a.ctypes.data_as(C.POINTER(ctype)))
        if face_bnd is None:
            desc.face_boundary = None
        neighbours = []
        for q in sorted(set(other_part[cut].tolist())):
            sel = np.nonzero(cut & (other_part == q))[0]  # positions within fid, ascending global id
            own_side = np.where(pL[fid[sel]] == r, 1, 2).astype(np.int32)
            e_own = np.where(own_side == 1, fe[sel, 0], fe[sel, 1])
            e_gh = np.where(own_side == 1, fe[sel, 1], fe[sel, 0])
            s_own = np.where(own_side == 1, face_side[fid[sel], 0], face_side[fid[sel], 1])
            s_gh = np.where(own_side == 1, face_side[fid[sel], 1], face_side[fid[sel], 0])
            neighbours.append(Neighbour(
                rank=q, faces=sel.astype(np.int32), global_faces=fid[sel], own_side=own_side,
                send_slots=(6 * local[e_own] + s_own - 1).astype(np.int32),
                recv_slots=(6 * local[e_gh] + s_gh - 1).astype(np.int32)))
        parts.append(Partition(rank=r, n_parts=n_parts, elements=own, ghosts=ghosts, faces=fid,
                               node_slice=slice(n0, n1), neighbours=neighbours, desc=desc, arrays=arrays))
    return parts


# ------------------------------------------------------------------------------ exchanges ----
def local_exchange(sends: dict) -> dict:
    """Partitions held by one process: sends[(r, q)] is r's buffer for q; returns recvs[(q, r)]
    (q's buffer from r) = the same data."""
    return {(q, r): buf for (r, q), buf in sends.items()}


def dist_exchange(sends: dict, recv_like: dict) -> dict:
    """One partition per process over torch.distributed: sends[(r, q)] for this rank r; recv_like
    [(r, q)] is a buffer of the size q sends to r. Returns recvs[(r, q)]."""
    import torch.distributed as dist

    ops = []
    recvs = {}
    for (r, q), buf in sends.items():
        ops.append(dist.P2POp(dist.isend, buf, q))
    for (r, q), like in recv_like.items():
        recvs[(r, q)] = like
        ops.append(dist.P2POp(dist.irecv, like, q))
    if ops:
        for req in dist.batch_isend_irecv(ops):
            req.wait()
    return recvs


def allreduce(value: float, op: str) -> float:
    """MIN or MAX of a host scalar over the ranks (identity without torch.distributed)."""
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return value
    import torch

    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MIN if op == "min" else dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------------- GPU partitions ----
class PartitionSolver:
    """One partition context (dg_create_partition) with its device exchange buffers (torch)."""

    def __init__(self, part: Partition, config, device: int = 0):
        import torch

        self.part = part
        self.config = config
        self.ns = config.flow == "ns"
        L = _abi.lib()
        h = C.c_void_p()
        _abi.check(L.dg_create_partition(C.byref(part.desc), part.n_ghost, C.byref(config.physics()),
                                         C.byref(config.options()), C.byref(h)), "dg_create_partition")
        self._h = h
        send, recv = part.send_slots(), part.recv_slots()
        _abi.check(L.dg_halo_set_slots(h, len(send), _abi.i32ptr(send), len(recv), _abi.i32ptr(recv)),
                   "dg_halo_set_slots")
        self.slot_bytes = int(L.dg_halo_slot_bytes(h))
        self.dtype = torch.float64 if config.precision == _abi.DG_PRECISION_FP64 else torch.float32
        self.per_slot = self.slot_bytes // (8 if self.dtype == torch.float64 else 4)
        dev = torch.device("cuda", device)
        self.send_buf = torch.empty(max(1, len(send)) * self.per_slot, dtype=self.dtype, device=dev)
        self.recv_buf = torch.empty(max(1, len(recv)) * self.per_slot, dtype=self.dtype, device=dev)
        # per neighbour slices of the buffers (same order on both sides)
        self.slices = {}
        a = 0
        for n in part.neighbours:
            self.slices[n.rank] = slice(a * self.per_slot, (a + len(n.send_slots)) * self.per_slot)
            a += len(n.send_slots)

    def close(self):
        if getattr(self, "_h", None):
            _abi.lib().dg_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def set_state(self, q_local: np.ndarray) -> None:
        q = np.ascontiguousarray(q_local, dtype=np.float64)
        _abi.check(_abi.lib().dg_upload_state(self._h, _abi.f64ptr(q)), "dg_upload_state")

    def set_energy_reference(self, e_ref: float) -> None:
        _abi.check(_abi.lib().dg_set_energy_reference(self._h, e_ref), "dg_set_energy_reference")

    def get(self, field: int = _abi.DG_FIELD_Q) -> np.ndarray:
        out = np.empty(5 * self.part.ndof)
        _abi.check(_abi.lib().dg_download(self._h, field, _abi.f64ptr(out)), "dg_download")
        return out

    def pack(self, field: int) -> dict:
        _abi.check(_abi.lib().dg_halo_pack(self._h, field, C.c_void_p(self.send_buf.data_ptr())), "dg_halo_pack")
        return {(self.part.rank, q): self.send_buf[s] for q, s in self.slices.items()}

    def recv_like(self) -> dict:
        return {(self.part.rank, q): self.recv_buf[s] for q, s in self.slices.items()}

    def unpack(self, field: int, recvs: dict) -> None:
        for q, s in self.slices.items():
            buf = recvs[(self.part.rank, q)]
            if buf.data_ptr() != self.recv_buf[s].data_ptr():
                self.recv_buf[s].copy_(buf)
        import torch

        torch.cuda.synchronize(self.recv_buf.device)
        _abi.check(_abi.lib().dg_halo_unpack(self._h, field, C.c_void_p(self.recv_buf.data_ptr())), "dg_halo_unpack")

    def stage(self, k: int, phase: int, t: float, dt: float) -> None:
        _abi.check(_abi.lib().dg_partition_stage(self._h, k, phase, t, dt), "dg_partition_stage")

    def max_dt_local(self, cfl: float, dcfl: float) -> float:
        dt = C.c_double()
        _abi.check(_abi.lib().dg_max_dt(self._h, cfl, dcfl, C.byref(dt)), "dg_max_dt")
        return dt.value

    def residuals_local(self):
        r = np.zeros(5)
        nan = C.c_int()
        rc = _abi.lib().dg_residuals(self._h, _abi.f64ptr(r), C.byref(nan))
        if rc not in (_abi.DG_OK, _abi.DG_ERR_NAN):
            _abi.check(rc, "dg_residuals")
        return r, bool(nan.value)


def _exchange(solvers, field, exchange):
    sends = {}
    for s in solvers:
        sends.update(s.pack(field))
    if exchange is None:
        recvs = local_exchange(sends)
    else:
        like = {}
        for s in solvers:
            like.update(s.recv_like())
        recvs = exchange(sends, like)
    for s in solvers:
        s.unpack(field, recvs)


def _stage(solvers, k, t, dt, exchange):
    _exchange(solvers, _abi.DG_HALO_Q_TRACES, exchange)
    for s in solvers:
        s.stage(k, 0, t, dt)
    if solvers and solvers[0].ns:
        _exchange(solvers, _abi.DG_HALO_VISCOUS_FLUX, exchange)
    for s in solvers:
        s.stage(k, 1, t, dt)


def rhs(solvers, t: float, exchange=None) -> None:
    """ComputeTimeDerivative on every partition of `solvers` (QDot, then get(DG_FIELD_QDOT)).
    exchange: None for partitions all held here, else dist_exchange."""
    _stage(solvers, -1, t, 0.0, exchange)


def rk3_step(solvers, t: float, dt: float, exchange=None) -> None:
    """TakeRK3Step on every partition: per stage the Q trace exchange, the volume phase, the viscous
    flux exchange and the surface phase with the stage update."""
    for k in range(3):
        _stage(solvers, k, t, dt, exchange)


def max_time_step(solvers, cfl: float, dcfl: float) -> float:
    """MaxTimeStep: the minimum over the partitions here and, under torch.distributed, over the ranks."""
    return allreduce(min(s.max_dt_local(cfl, dcfl) for s in solvers), "min")


def mean_energy(parts_and_states) -> float:
    """The mean energy over all partitions' nodes (the shared energy reference of the mixed form)
    from (Partition, local state) pairs held here, summed over the ranks."""
    tot = sum(float(np.sum(q.reshape(-1, 5)[:, 4])) for _, q in parts_and_states)
    cnt = sum(p.ndof for p, _ in parts_and_states)
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        import torch

        device = "cuda" if dist.get_backend() == "nccl" else "cpu"
        t = torch.tensor([tot, float(cnt)], dtype=torch.float64, device=device)
        dist.all_reduce(t)
        tot, cnt = float(t[0]), float(t[1])
    return tot / cnt
