"""Failure detection on the GPU without a fault.

The persistent stage kernel stages every element's state and RK register
with bulk copies that complete on shared-memory barriers; each wait on such
a barrier is bounded.  The test hook cmdg_model_set_staging_test arms the
barriers without issuing the copies, so every wait runs out after a few
hundred polls: the kernel must then report bit 1 of the status word and
return, and the context must stay usable (the next launches give the same
result as before the hook was set).  Nothing here faults, traps or hangs.
"""
import numpy as np
import pytest
import torch

import cmdg
import oracle as O
from cmdg import _lib, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g

    g.build()
    torch.cuda.set_device(0)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_bounded_staging_wait_runs_out_and_reports_it(precision):
    L = _lib.load()
    dg = workloads.bubble_model(ne=(2, 2, 3), N=4, precision=precision)
    dg.set_kernel("node", 2)  # two resident CTAs walk the 12 elements with staged copies
    xyz = dg.grid.coordinates()
    Q0 = workloads.rising_bubble(xyz, rc=900.0, center=(1100.0, 1300.0, 900.0))
    Q0[:, 1:4] += np.random.default_rng(3).uniform(-1, 1, size=Q0[:, 1:4].shape)
    Q = dg.init_ode_state(Q0)
    good = dg.new_state(torch.float64)
    dg(good, Q, None, 0.0)
    assert dg.status_word() == 0

    assert L.cmdg_model_set_staging_test(dg.h, 1, 256) == 0
    junk = dg.new_state(torch.float64)
    dg(junk, Q, None, 0.0)
    torch.cuda.synchronize()
    assert dg.status_word() & 2, "the bounded wait did not report that it ran out"

    assert L.cmdg_model_set_staging_test(dg.h, 0, 0) == 0
    again = dg.new_state(torch.float64)
    dg(again, Q, None, 0.0)
    torch.cuda.synchronize()
    assert dg.status_word() == 0
    assert torch.equal(again, good)


def test_fused_steps_refuse_caller_refreshed_terms():
    """A model whose source is refreshed by the caller at every stage time
    cannot be stepped by the fused LSRK54 call (it would use stale terms)."""
    L = 1 / 20
    om = O.OracleModel(2, (2, 2, 2), (-L,) * 3, (L,) * 3, periodic=(1, 1, 1))
    dg = cmdg.DGModel(cmdg.AtmosModel(), cmdg.ArraysGrid(2, om.vgeo, om.vmapP + 1, om.elemtobndy))
    src = dg.new_state(torch.float64)
    dg.set_mms(src, None, zero_enthalpy=False)
    Q = dg.new_state(torch.float64)
    lsrk = cmdg.LSRK54CarpenterKennedy(dg, Q, dt=1e-3)
    with pytest.raises(cmdg.CmdgError, match="CMDG_ERR_STATE"):
        cmdg.dostep_(Q, lsrk, None, 0.0)
