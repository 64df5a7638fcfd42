"""Restart from a checkpoint (write_checkpoint -> read_checkpoint ->
init_ode_state, src/Driver/Checkpoint/Checkpoint.jl and
restart_ode_state, src/Numerics/DGMethods/DGModel.jl:429-443) continues a
run bit for bit, in FP64 and in mixed precision."""
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
    Qc = dg.init_ode_state(h_Q)
    lc = cmdg.LSRK54CarpenterKennedy(dg, Qc, dt=dt, t0=t)
    cmdg.solve_(Qc, lc, numberofsteps=2)
    assert torch.equal(Qc, Qa)
    assert lc.gettime() == pytest.approx(la.gettime(), rel=1e-15)
