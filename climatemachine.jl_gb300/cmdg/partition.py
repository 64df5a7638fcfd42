"""Element partition and face-halo exchange for multi-rank runs (host side).

The reference's only parallel strategy is an element partition with one
ghost-face exchange of the state per stage (src/Arrays/MPIStateArrays.jl:
411-575, src/Numerics/DGMethods/DGModel.jl:125-412; stacks are not split,
src/Numerics/Mesh/BrickMesh.jl:531).  This module restates that plan for the
library's brick element order (e = iz + nz (ix + nx iy)):

* ``ColumnPartition`` gives each rank a contiguous range of whole element
  columns, so vertical faces never cross ranks;
* ``halo_plan`` lists, for every pair of ranks, the (element, face) pairs
  whose face nodes one side needs from the other, in an order both sides
  derive without communication;
* ``exchange_faces`` packs the face nodes of a rank's state into one buffer
  per peer and swaps them with ``torch.distributed`` point-to-point calls
  (host-staged: CPU tensors), returning the ghost faces;
* ``local_layout`` appends one ghost slot per received face after the local
  elements and rewrites the 6-neighbour connectivity rows so that a stage
  kernel reading the neighbour's node ``(nb, vP)`` finds the ghost face in
  the slot.

Every GPU of this build runs the hot path alone (replicas, ``bench.py``
under torchrun); the exchange is exercised by CPU ranks in the tests.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch

NSTATE = 5


def face_nodes(N: int, f: int) -> np.ndarray:
    """Volume node indices of face f (0..5 = xi1-, xi1+, xi2-, xi2+, xi3-,
    xi3+) in the in-face order a + (N+1) b (src/Numerics/Mesh/Grids.jl:580-597)."""
    Nq = N + 1
    a, b = np.meshgrid(np.arange(Nq), np.arange(Nq), indexing="xy")
    a, b = a.ravel(), b.ravel()
    side = N if f & 1 else 0
    if f < 2:
        return side + Nq * (a + Nq * b)
    if f < 4:
        return a + Nq * (side + Nq * b)
    return a + Nq * (b + Nq * side)


@dataclass
class ColumnPartition:
    """Whole element columns of an (nx, ny, nz) brick split into ``world``
    contiguous, balanced ranges."""

    ne: tuple
    periodic: tuple
    N: int
    world: int

    def __post_init__(self):
        nx, ny, nz = self.ne
        ncol = nx * ny
        if self.world < 1 or self.world > ncol:
            raise ValueError("need 1 <= world <= number of columns")
        base, extra = divmod(ncol, self.world)
        sizes = [base + (1 if r < extra else 0) for r in range(self.world)]
        self.col_start = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)

    @property
    def nelem(self):
        return self.ne[0] * self.ne[1] * self.ne[2]

    def elements(self, rank: int) -> range:
        nz = self.ne[2]
        return range(int(self.col_start[rank]) * nz, int(self.col_start[rank + 1]) * nz)

    def owner(self, e: int) -> int:
        return int(np.searchsorted(self.col_start, e // self.ne[2], side="right") - 1)

    def neighbor(self, e: int, f: int) -> int:
        """Element across face f of element e, or -1 on a wall."""
        nx, ny, nz = self.ne
        iz, c = e % nz, e // nz
        idx = [c % nx, c // nx, iz]
        d, step = f // 2, (1 if f & 1 else -1)
        idx[d] += step
        if idx[d] < 0 or idx[d] >= self.ne[d]:
            if not self.periodic[d]:
                return -1
            idx[d] %= self.ne[d]
        return int(idx[2] + nz * (idx[0] + nx * idx[1]))


def halo_plan(part: ColumnPartition, rank: int):
    """{peer: [(element, face), ...]} of the faces ``rank`` receives from each
    peer (the peer's element and its face that touches ``rank``), and the
    faces it sends to each peer in the order the peer expects them."""
    recv = {}
    for e in part.elements(rank):
        for f in range(4):  # vertical faces stay inside a column
            e2 = part.neighbor(e, f)
            if e2 < 0:
                continue
            s = part.owner(e2)
            if s != rank:
                recv.setdefault(s, set()).add((e2, f ^ 1))
    recv = {s: sorted(v) for s, v in recv.items()}
    send = {}
    for s in range(part.world):
        if s == rank:
            continue
        for e in part.elements(s):
            for f in range(4):
                e2 = part.neighbor(e, f)
                if e2 >= 0 and part.owner(e2) == rank:
                    send.setdefault(s, set()).add((e2, f ^ 1))
    send = {s: sorted(v) for s, v in send.items()}
    return recv, send


def pack(part: ColumnPartition, rank: int, Q_local: torch.Tensor, faces) -> torch.Tensor:
    """Face nodes of local elements, (len(faces), 5, Nfp)."""
    e0 = part.elements(rank).start
    out = torch.empty((len(faces), NSTATE, (part.N + 1) ** 2), dtype=Q_local.dtype)
    for i, (e, f) in enumerate(faces):
        out[i] = Q_local[e - e0][:, torch.from_numpy(face_nodes(part.N, f))]
    return out


def exchange_faces(part: ColumnPartition, rank: int, Q_local: torch.Tensor, group=None):
    """Swap face halos with every peer (one packed buffer per direction and
    peer, non-blocking point-to-point); returns {(element, face): (5, Nfp)}."""
    import torch.distributed as dist

    recv_plan, send_plan = halo_plan(part, rank)
    Nfp = (part.N + 1) ** 2
    reqs, bufs = [], {}
    for s, faces in sorted(send_plan.items()):
        buf = pack(part, rank, Q_local, faces).contiguous()
        reqs.append(dist.isend(buf, dst=s, group=group, tag=666))
        bufs[("send", s)] = buf
    for s, faces in sorted(recv_plan.items()):
        buf = torch.empty((len(faces), NSTATE, Nfp), dtype=Q_local.dtype)
        reqs.append(dist.irecv(buf, src=s, group=group, tag=666))
        bufs[("recv", s)] = buf
    for r in reqs:
        r.wait()
    ghosts = {}
    for s, faces in recv_plan.items():
        buf = bufs[("recv", s)]
        for i, key in enumerate(faces):
            ghosts[key] = buf[i]
    return ghosts


def local_layout(part: ColumnPartition, rank: int, Q_local: torch.Tensor, ghosts):
    """State with one ghost slot per received face appended after the local
    elements (only that face's nodes are set) and the connectivity rows
    [6 neighbours or -tag, vertical index, 0] of the local elements remapped
    to local and ghost slots."""
    elems = part.elements(rank)
    e0, nloc = elems.start, len(elems)
    keys = sorted(ghosts)
    slot = {k: nloc + i for i, k in enumerate(keys)}
    Np = (part.N + 1) ** 3
    Q = torch.full((nloc + len(keys), NSTATE, Np), float("nan"), dtype=Q_local.dtype)
    Q[:nloc] = Q_local
    for k, i in slot.items():
        Q[i][:, torch.from_numpy(face_nodes(part.N, k[1]))] = ghosts[k]
    nbr = np.zeros((nloc, 8), dtype=np.int32)
    for e in elems:
        row = nbr[e - e0]
        for f in range(6):
            e2 = part.neighbor(e, f)
            if e2 < 0:
                row[f] = -(2 if f & 1 else 1)
            elif part.owner(e2) == rank:
                row[f] = e2 - e0
            else:
                row[f] = slot[(e2, f ^ 1)]
        row[6] = e % part.ne[2]
    return Q, nbr
