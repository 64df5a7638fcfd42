"""Checkpoint files (the reference's write_checkpoint / read_checkpoint /
rm_checkpoint, src/Driver/Checkpoint/Checkpoint.jl:21-127): naming per rank
and number, exact round trip of h_Q, h_aux and t, the reference's error on a
missing file, and rejection of a damaged file.  Host-only."""
import json
import os
import struct

import numpy as np
import pytest

from cmdg import checkpoint as ck


def arrays(seed=3, nelem=7, Np=27):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((nelem, 5, Np)), rng.standard_normal((nelem, 3, Np))


def test_file_name_follows_the_reference(tmp_path):
    p = ck.checkpoint_path(str(tmp_path), "rising bubble", 3, 12)
    assert os.path.basename(p) == "rising_bubble_checkpoint_mpirank0003_num0012.cmdg"


@pytest.mark.parametrize("rank", [0, 1])
def test_round_trip_is_exact(tmp_path, rank):
    Q, A = arrays(seed=rank)
    t = 123.456789012345
    path = ck.write_checkpoint_arrays(Q, A, t, str(tmp_path), "bubble", rank=rank, num=5)
    assert os.path.exists(path) and not os.path.exists(path + ".tmp")
    Q2, A2, t2 = ck.read_checkpoint(str(tmp_path), "bubble", rank=rank, num=5)
    assert t2 == t
    assert Q2.shape == Q.shape and A2.shape == A.shape
    assert np.array_equal(Q2, Q) and np.array_equal(A2, A)


def test_layout_is_column_major_julia_order(tmp_path):
    """The h_Q record is the bytes of a Julia (Np, nstate, nelem) array: the
    header names that shape and the data start on a 64-byte boundary."""
    Q, A = arrays()
    path = ck.write_checkpoint_arrays(Q, A, 0.0, str(tmp_path), "x")
    raw = open(path, "rb").read()
    assert raw[:8] == ck.MAGIC
    (hlen,) = struct.unpack("<Q", raw[8:16])
    meta = json.loads(raw[16:16 + hlen])
    d = meta["arrays"]["h_Q"]
    assert d["shape"] == [Q.shape[2], Q.shape[1], Q.shape[0]] and d["offset"] % 64 == 0
    col = np.frombuffer(raw[d["offset"]:d["offset"] + d["nbytes"]], "<f8").reshape(d["shape"], order="F")
    assert np.array_equal(col[:, :, 4], Q[4].T)  # Q[e, s, n] == col[n, s, e]


def test_missing_file_raises_like_the_reference(tmp_path):
    with pytest.raises(FileNotFoundError, match="Cannot restore from checkpoint"):
        ck.read_checkpoint(str(tmp_path), "none", 0, 0)


def test_damaged_files_are_rejected(tmp_path):
    Q, A = arrays()
    path = ck.write_checkpoint_arrays(Q, A, 1.0, str(tmp_path), "d")
    raw = bytearray(open(path, "rb").read())
    open(path, "wb").write(raw[: len(raw) - 100])  # truncated
    with pytest.raises(ValueError, match="truncated"):
        ck.read_checkpoint(str(tmp_path), "d")
    raw[0:8] = b"NOTACKPT"
    open(path, "wb").write(raw)
    with pytest.raises(ValueError, match="not a cmdg checkpoint"):
        ck.read_checkpoint(str(tmp_path), "d")


def test_rm_checkpoint(tmp_path):
    Q, A = arrays()
    path = ck.write_checkpoint_arrays(Q, A, 1.0, str(tmp_path), "r", rank=1, num=2)
    ck.rm_checkpoint(str(tmp_path), "r", rank=1, num=2)
    assert not os.path.exists(path)
    ck.rm_checkpoint(str(tmp_path), "r", rank=1, num=2)  # force = true: no error


def test_fp32_record_round_trip(tmp_path):
    Q, A = arrays()
    Qp = Q.astype(np.float32)
    ck.write_checkpoint_arrays(Q, A, 2.0, str(tmp_path), "p", h_Qp=Qp)
    rec, t = ck.read_checkpoint_records(str(tmp_path), "p")
    assert t == 2.0 and rec["h_Qp"].dtype == np.float32 and np.array_equal(rec["h_Qp"], Qp)
    Q2, A2, _ = ck.read_checkpoint(str(tmp_path), "p")
    assert np.array_equal(Q2, Q) and np.array_equal(A2, A)
