"""Checkpoint / restart of a DG state, mirroring ClimateMachine.jl's
``write_checkpoint`` / ``read_checkpoint`` / ``rm_checkpoint``
(src/Driver/Checkpoint/Checkpoint.jl:21-127).

The reference saves, per MPI rank, ``h_Q`` (the state, ``(Np, nstate,
nelem)``), ``h_aux`` (the auxiliary state) and the solver time ``t`` with
JLD2 into ``"<name>_checkpoint_mpirank%04d_num%04d.jld2"`` (blanks in
``name`` replaced by underscores).  This module keeps the file naming, the
three records and their meaning; the container is a self-describing raw
file instead of HDF5/JLD2 (no HDF5 library is available to this package):

    bytes 0..7     magic ``CMDGCKP1``
    bytes 8..15    header length H (little-endian uint64)
    bytes 16..     H bytes of UTF-8 JSON: {"t", "name", "rank", "num",
                   "arrays": {"h_Q": {"dtype", "shape", "offset", "nbytes"},
                   "h_aux": {...}}, "aux_fields": [...]}
    then           the arrays, each starting on a 64-byte boundary, stored
                   column-major with the Julia shape ``shape`` (``(Np,
                   nstate, nelem)``), i.e. exactly the bytes of
                   ``Q.realdata`` -- a Julia reader ``read!``s them into an
                   ``Array{Float64}(undef, shape...)``.

``h_Q`` is always the full FP64 state (a mixed-precision model's FP32
perturbation is converted back), so a checkpoint restarts either precision.
A mixed-precision model also stores its FP32 perturbation state as ``h_Qp``
(``dtype`` ``<f4``): ``restart_ode_state`` restarts such a model from it bit
for bit (the FP64 sum q_ref + q' rounds perturbations more than 2^29 below
the reference value, so the FP64 record alone does not round-trip them).
``h_aux`` holds this library's auxiliary state, the reference state
``(rho_ref, rhoe_ref, p_ref)`` at the nodes (the rest of the reference's aux
-- coordinates, geopotential, metric-derived fields -- is rebuilt from the
mesh and the parameters when a model is created, as
``restart_auxiliary_state`` would restore it).
"""
from __future__ import annotations

import json
import os
import struct

import numpy as np

MAGIC = b"CMDGCKP1"
ALIGN = 64
AUX_FIELDS = ["rho_ref", "rhoe_ref", "p_ref"]


def checkpoint_path(checkpoint_dir: str, name: str, rank: int, num: int) -> str:
    """``"%s_checkpoint_mpirank%04d_num%04d"`` of the reference with this
    container's extension (Checkpoint.jl:47-53)."""
    nm = name.replace(" ", "_")
    return os.path.join(checkpoint_dir, "%s_checkpoint_mpirank%04d_num%04d.cmdg" % (nm, rank, num))


DTYPES = {"<f8": np.float64, "<f4": np.float32}


def _as_host(a, dtype=np.float64) -> np.ndarray:
    if hasattr(a, "detach"):  # torch tensor on any device
        a = a.detach().to("cpu").numpy()
    a = np.ascontiguousarray(a, dtype=dtype)
    if a.ndim != 3:
        raise ValueError(f"expected a (nelem, nstate, Np) array, got shape {a.shape}")
    return a


def write_checkpoint_arrays(h_Q, h_aux, t: float, checkpoint_dir: str, name: str, rank: int = 0, num: int = 0,
                            aux_fields=None, h_Qp=None) -> str:
    """write_checkpoint(Q, A, odesolver, checkpoint_dir, name, mpicomm, num)
    with the arrays and the time given directly (and optionally the FP32
    perturbation state of a mixed model); returns the file path.  The file
    is written under a temporary name and renamed into place."""
    arrays = {"h_Q": _as_host(h_Q), "h_aux": _as_host(h_aux)}
    if h_Qp is not None:
        arrays["h_Qp"] = _as_host(h_Qp, np.float32)
    meta = {"format": "cmdg-checkpoint", "version": 1, "t": float(t), "name": name, "rank": int(rank),
            "num": int(num), "aux_fields": list(aux_fields or AUX_FIELDS), "arrays": {}}
    # two passes: the header length fixes the array offsets
    header = b""
    for _ in range(3):
        off = (16 + len(header) + ALIGN - 1) // ALIGN * ALIGN
        for k, a in arrays.items():
            meta["arrays"][k] = {"dtype": "<f8" if a.dtype == np.float64 else "<f4",
                                 "shape": [a.shape[2], a.shape[1], a.shape[0]], "offset": off, "nbytes": a.nbytes}
            off = (off + a.nbytes + ALIGN - 1) // ALIGN * ALIGN
        new = json.dumps(meta, sort_keys=True).encode()
        if len(new) == len(header):
            break
        header = new
    os.makedirs(checkpoint_dir, exist_ok=True)
    path = checkpoint_path(checkpoint_dir, name, rank, num)
    tmp = path + ".tmp"
    with open(tmp, "wb") as fh:
        fh.write(MAGIC)
        fh.write(struct.pack("<Q", len(header)))
        fh.write(header)
        for k, a in arrays.items():
            fh.seek(meta["arrays"][k]["offset"])
            fh.write(a.astype(a.dtype.newbyteorder("<"), copy=False).tobytes(order="C"))
    os.replace(tmp, path)
    return path


def read_checkpoint(checkpoint_dir: str, name: str, rank: int = 0, num: int = 0):
    """read_checkpoint(checkpoint_dir, name, array_type, mpicomm, num) ->
    ``(h_Q, h_aux, t)``, host arrays shaped (nelem, nstate, Np) (the memory
    of the reference's (Np, nstate, nelem) arrays).  Raises like the
    reference when the file is missing (Checkpoint.jl:115-121)."""
    rec, t = read_checkpoint_records(checkpoint_dir, name, rank, num)
    return rec["h_Q"], rec["h_aux"], t


def read_checkpoint_records(checkpoint_dir: str, name: str, rank: int = 0, num: int = 0):
    """Every record of a checkpoint file as a dict of host arrays, and t."""
    path = checkpoint_path(checkpoint_dir, name, rank, num)
    if not os.path.isfile(path):
        raise FileNotFoundError(f"Cannot restore from checkpoint in {path}, file not found")
    with open(path, "rb") as fh:
        if fh.read(8) != MAGIC:
            raise ValueError(f"{path} is not a cmdg checkpoint")
        (hlen,) = struct.unpack("<Q", fh.read(8))
        meta = json.loads(fh.read(hlen).decode())
        out = {}
        size = os.fstat(fh.fileno()).st_size
        if "h_Q" not in meta["arrays"] or "h_aux" not in meta["arrays"]:
            raise ValueError(f"{path}: h_Q or h_aux missing")
        for k, d in meta["arrays"].items():
            if d["dtype"] not in DTYPES or d["offset"] + d["nbytes"] > size:
                raise ValueError(f"{path}: record {k} is truncated or of an unknown type")
            dt = DTYPES[d["dtype"]]
            Np, ns, ne = d["shape"]
            if Np * ns * ne * np.dtype(dt).itemsize != d["nbytes"]:
                raise ValueError(f"{path}: record {k} has an inconsistent shape")
            fh.seek(d["offset"])
            out[k] = np.frombuffer(fh.read(d["nbytes"]), dtype=d["dtype"]).reshape(ne, ns, Np).astype(dt)
    return out, float(meta["t"])


def rm_checkpoint(checkpoint_dir: str, name: str, rank: int = 0, num: int = 0) -> None:
    """rm_checkpoint(checkpoint_dir, name, mpicomm, num) (Checkpoint.jl:79-99)."""
    try:
        os.remove(checkpoint_path(checkpoint_dir, name, rank, num))
    except FileNotFoundError:
        pass


def write_checkpoint(dg, Q, odesolver, checkpoint_dir: str, name: str, rank: int = 0, num: int = 0) -> str:
    """write_checkpoint for a DGModel's state ``Q`` (FP64, or the FP32
    perturbation of a mixed model) and its solver's time."""
    h_Q = dg.full_state(Q)
    t = odesolver.gettime() if hasattr(odesolver, "gettime") else float(odesolver)
    return write_checkpoint_arrays(h_Q, dg.reference_state(), t, checkpoint_dir, name, rank, num,
                                   h_Qp=Q if dg.mixed else None)


def restart_ode_state(dg, checkpoint_dir: str, name: str, rank: int = 0, num: int = 0):
    """restart_ode_state (src/Numerics/DGMethods/DGModel.jl:429-443) from a
    checkpoint file: the device state in the model's own representation and
    the checkpoint time.  A mixed model takes the stored FP32 perturbation
    when the file has one (bitwise restart), else converts h_Q."""
    import torch

    rec, t = read_checkpoint_records(checkpoint_dir, name, rank, num)
    if dg.mixed and "h_Qp" in rec:
        return torch.from_numpy(rec["h_Qp"]).to(dg.device), t
    return dg.init_ode_state(rec["h_Q"]), t
