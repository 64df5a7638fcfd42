"""Multi-rank host logic on CPU ranks (gloo, world_size 2): the column
partition, the face-halo plan and exchange, and the ghost-slot layout a
partitioned stage kernel would read.  The oracle checks that each rank's
tendency, computed from its own elements plus the exchanged ghost faces
only, equals the single-rank tendency of those elements exactly."""
import os
import socket

import numpy as np
import pytest
import torch

from cmdg import partition as P


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_partition_owns_every_element_once_and_plans_are_symmetric():
    for ne, per, world in [((4, 3, 2), (1, 1, 0), 2), ((5, 4, 3), (1, 0, 0), 3), ((2, 2, 4), (0, 0, 1), 4)]:
        part = P.ColumnPartition(ne, per, 3, world)
        owned = np.concatenate([np.arange(part.elements(r).start, part.elements(r).stop) for r in range(world)])
        assert np.array_equal(np.sort(owned), np.arange(part.nelem))
        plans = [P.halo_plan(part, r) for r in range(world)]
        for r in range(world):
            recv, send = plans[r]
            for s, faces in recv.items():
                assert plans[s][1][r] == faces
                assert all(part.owner(e) == s for e, _ in faces)
            for s, faces in send.items():
                assert all(part.owner(e) == r for e, _ in faces)


def _rank_main(rank, world, port, result_dir):
    import torch.distributed as dist

    import oracle as O

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        ne, N, L = (4, 3, 2), 3, 2500.0
        om = O.OracleModel(N, ne, (0, 0, 0), (L, L, L), periodic=(1, 1, 0), orientation="flat", gravity=True,
                           ref_state=True, profile="dry_adiabatic", T_surface=300.0, T_min=0.0)
        Q0 = om.init_bubble(rc=900.0, xc=1100.0, yc=1300.0, zc=800.0)
        rng = np.random.default_rng(5)
        Q0[:, 1:4] += rng.uniform(-2, 2, size=Q0[:, 1:4].shape)
        ref = om.tendency(Q0)
        part = P.ColumnPartition(ne, (1, 1, 0), N, world)
        elems = part.elements(rank)
        Q_local = torch.from_numpy(Q0[elems.start:elems.stop].copy())
        ghosts = P.exchange_faces(part, rank, Q_local)
        # the full-mesh state a rank can see: its elements and the ghost faces
        Qv = np.full_like(Q0, np.nan)
        Qv[elems.start:elems.stop] = Q0[elems.start:elems.stop]
        for (e2, f2), vals in ghosts.items():
            Qv[e2][:, P.face_nodes(N, f2)] = vals.numpy()
        got = om.tendency(Qv)[elems.start:elems.stop]
        exact = np.array_equal(got, ref[elems.start:elems.stop])
        # ghost-slot layout: the neighbour node each face node reads is the exchanged one
        Ql, nbr = P.local_layout(part, rank, Q_local, ghosts)
        ok_layout = True
        for i, e in enumerate(elems):
            for f in range(6):
                nb = nbr[i, f]
                e2 = part.neighbor(e, f)
                if e2 < 0:
                    ok_layout &= nb < 0
                    continue
                want = Q0[e2][:, P.face_nodes(N, f ^ 1)]
                ok_layout &= np.array_equal(Ql[nb][:, P.face_nodes(N, f ^ 1)].numpy(), want)
        np.save(os.path.join(result_dir, f"rank{rank}.npy"),
                np.array([exact, ok_layout, len(ghosts), sum(len(v) for v in P.halo_plan(part, rank)[0].values())]))
    finally:
        dist.destroy_process_group()


def test_halo_exchange_reproduces_single_rank_tendency(tmp_path):
    import torch.multiprocessing as mp

    world = 2
    mp.spawn(_rank_main, args=(world, free_port(), str(tmp_path)), nprocs=world, join=True)
    for r in range(world):
        exact, ok_layout, nghost, nplanned = np.load(tmp_path / f"rank{r}.npy")
        assert exact and ok_layout
        assert nghost == nplanned > 0
