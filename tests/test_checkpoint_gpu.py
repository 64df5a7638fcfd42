"""Restart from a checkpoint (write_checkpoint -> read_checkpoint ->
restart_ode_state, src/Driver/Checkpoint/Checkpoint.jl and
src/Numerics/DGMethods/DGModel.jl:429-443) continues a run bit for bit, in
FP64 and in mixed precision; the FP64 record h_Q restarts a mixed model to
within the rounding of q_ref + q'."""
import pytest
import torch

import cmdg
from cmdg import checkpoint as ck
from cmdg import workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g

    g.build()
    torch.cuda.set_device(0)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_restart_is_bitwise(tmp_path, precision):
    dg = workloads.bubble_model(ne=(4, 4, 4), N=4, precision=precision)
    Q0 = workloads.rising_bubble(dg.grid.coordinates())
    dt = 0.05
    Qa = dg.init_ode_state(Q0)
    la = cmdg.LSRK54CarpenterKennedy(dg, Qa, dt=dt)
    cmdg.solve_(Qa, la, numberofsteps=4)

    Qb = dg.init_ode_state(Q0)
    lb = cmdg.LSRK54CarpenterKennedy(dg, Qb, dt=dt)
    cmdg.solve_(Qb, lb, numberofsteps=2)
    ck.write_checkpoint(dg, Qb, lb, str(tmp_path), "restart test", rank=0, num=1)
    h_Q, h_aux, t = ck.read_checkpoint(str(tmp_path), "restart test", rank=0, num=1)
    assert t == pytest.approx(2 * dt, rel=1e-15)
    assert (h_aux == dg.reference_state()).all()
    Qc, t2 = ck.restart_ode_state(dg, str(tmp_path), "restart test", rank=0, num=1)
    assert t2 == t and Qc.dtype == Qb.dtype
    lc = cmdg.LSRK54CarpenterKennedy(dg, Qc, dt=dt, t0=t)
    cmdg.solve_(Qc, lc, numberofsteps=2)
    assert torch.equal(Qc, Qa)
    assert lc.gettime() == pytest.approx(la.gettime(), rel=1e-15)


def test_mixed_restart_from_the_fp64_record_alone(tmp_path):
    dg = workloads.bubble_model(ne=(4, 4, 4), N=4, precision="mixed")
    Q = dg.init_ode_state(workloads.rising_bubble(dg.grid.coordinates()))
    lsrk = cmdg.LSRK54CarpenterKennedy(dg, Q, dt=0.05)
    cmdg.solve_(Q, lsrk, numberofsteps=2)
    ck.write_checkpoint_arrays(dg.full_state(Q), dg.reference_state(), lsrk.gettime(), str(tmp_path), "f64")
    Qr, _ = ck.restart_ode_state(dg, str(tmp_path), "f64")
    full = dg.full_state(Q)
    assert torch.allclose(dg.full_state(Qr), full, rtol=1e-15, atol=0.0)
