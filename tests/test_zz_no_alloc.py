"""The allocation-free LSRK54 entry point (cmdg_lsrk54_step_noalloc).

Some hosts cannot let the library call cudaMalloc: an arena or pool
allocator that owns all of the device's memory, or a host that forbids
allocation after start-up.  For them the stage buffers live in a fixed
device array inside libcmdg.so, reserved when a model is created.  This file
checks, through the C ABI, that two calls in a row give bit for bit the
states of the allocating entry point (both run the same stage kernels on the
same inputs in the same order), that a call after the first takes no device
memory, and that a state too large for the fixed array is refused.  It is
collected last on purpose.
"""
import ctypes

import numpy as np
import pytest
import torch

import cmdg
from cmdg import _lib, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g

    g.build_library()
    torch.cuda.set_device(0)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_noalloc_matches_allocating_entry_point_on_two_calls(precision):
    L = _lib.load()
    # one model steps through the allocating entry point, the other only
    # through the allocation-free one (so it never owns stage buffers)
    dga = workloads.bubble_model(ne=(6, 5, 7), N=4, precision=precision)
    dgb = workloads.bubble_model(ne=(6, 5, 7), N=4, precision=precision)
    xyz = dga.grid.coordinates()
    Q0 = workloads.rising_bubble(xyz, rc=900.0, center=(1100.0, 1300.0, 900.0))
    Q0[:, 1:4] += np.random.default_rng(5).uniform(-1, 1, size=Q0[:, 1:4].shape)
    Qa = dga.init_ode_state(Q0)
    Qb = Qa.clone()
    dQa = torch.zeros(Qa.shape, dtype=torch.float64, device="cuda")
    dQb = torch.zeros_like(dQa)
    dt = dga.courant_dt(Qa, 0.4)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ref_fn = L.cmdg_lsrk54_step_mixed if precision == "mixed" else L.cmdg_lsrk54_step
    for call in range(2):
        assert ref_fn(dga.h, _ptr(Qa), _ptr(dQa), 0.0, dt, 2, stream) == 0
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc = L.cmdg_lsrk54_step_noalloc(dgb.h, _ptr(Qb), _ptr(dQb), 0.0, dt, 2, stream)
        assert rc == 0, L.cmdg_last_error()
        torch.cuda.synchronize()
        if call == 1:
            # the first call may still load the stage kernels' code; after it
            # a call takes no device memory
            assert torch.cuda.mem_get_info()[0] == free_before
        assert torch.equal(Qa, Qb), call
        assert torch.isfinite(dgb.full_state(Qb)).all()
    assert dga.status_word() == 0
    assert dgb.status_word() == 0


def test_noalloc_rejects_a_state_beyond_its_fixed_buffers():
    L = _lib.load()
    # 22^3 elements at N=4 in FP32: 26.6 MB per state, above the 24 MiB limit
    dg = workloads.bubble_model(ne=(22, 22, 22), N=4, precision="mixed")
    Q = dg.new_state()
    dQ = torch.zeros(Q.shape, dtype=torch.float64, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = L.cmdg_lsrk54_step_noalloc(dg.h, _ptr(Q), _ptr(dQ), 0.0, 0.01, 1, stream)
    assert rc == 1
    assert b"exceeds the allocation-free limit" in L.cmdg_last_error()
