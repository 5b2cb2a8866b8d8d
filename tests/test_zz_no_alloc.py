"""xlbg_step_diag_noalloc gives the same results as xlbg_step_diag.

The allocation-free entry point serves callers that cannot allocate device
memory around a step (hosts whose own pool owns the device heap, loops that must
not call cudaMalloc/cudaFree because those can synchronise the device).  It keeps
its scratch in static device arrays inside libxlbg.so.  This test calls it
through the C ABI twice in a row, next to the caller-scratch entry point, on a
layout that uses both scratch arrays (Regularized inlet -> aux recovery; a
halfway bounce-back sphere -> momentum-exchange force), and compares populations
(exactly, as every parity test here does) and the FP64 mass / force (rtol 1e-12,
the tolerance of the diagnostics tests).

This file is collected last on purpose.
"""

import ctypes

import numpy as np
import pytest

from xlb_gb300 import _lib
from _scenarios import Scenario


@pytest.mark.gpu
def test_noalloc_matches_step_diag_two_calls():
    import torch

    sc = Scenario("D3Q19", (16, 10, 10), "channel_regularized", policy="fp32")
    sc.randomize(seed=21)
    f_0, f_1, bcm, mm = sc.gpu_fields()
    bits, rec, scratch = sc.stepper._aux_state(bcm, mm)
    assert rec is not None and rec.numel() > 0
    sphere = sc.xbcs[3]
    lib = _lib.load()
    desc = sc.stepper.desc
    stream = _lib.stream_handle()
    a0, a1 = f_0.clone(), f_1.clone()
    b0, b1 = f_0.clone(), f_1.clone()
    slots = torch.zeros(_lib.DIAG_SLOTS * 4, dtype=torch.float64, device="cuda")
    out_a = torch.empty(4, dtype=torch.float64, device="cuda")
    out_b = torch.empty(4, dtype=torch.float64, device="cuda")
    P = _lib.ptr
    for call in range(2):
        _lib.check(lib.xlbg_step_diag(desc, P(a0), P(a1), P(bcm), P(bits), P(rec), rec.numel(), P(scratch),
                                      sc.omega, call, sphere.id, P(slots), P(out_a), stream))
        _lib.check(lib.xlbg_step_diag_noalloc(desc, P(b0), P(b1), P(bcm), P(bits), P(rec), rec.numel(),
                                              sc.omega, call, sphere.id, P(out_b), stream))
        torch.cuda.synchronize()
        assert torch.equal(a0, b0) and torch.equal(a1, b1), f"populations differ on call {call}"
        da, db = out_a.cpu().numpy(), out_b.cpu().numpy()
        assert np.all(np.isfinite(db)) and db[0] > 0
        assert np.allclose(db, da, rtol=1e-12, atol=1e-12), (call, da, db)
        a0, a1 = a1, a0
        b0, b1 = b1, b0


@pytest.mark.gpu
def test_noalloc_rejects_oversized_recovery_list():
    import torch

    sc = Scenario("D3Q19", (16, 10, 10), "channel_regularized", policy="fp32")
    f_0, f_1, bcm, mm = sc.gpu_fields()
    bits, rec, _ = sc.stepper._aux_state(bcm, mm)
    out = torch.empty(4, dtype=torch.float64, device="cuda")
    P = _lib.ptr
    too_many = _lib.NOALLOC_REC_SCRATCH_BYTES // (19 * 4) + 1
    st = _lib.load().xlbg_step_diag_noalloc(sc.stepper.desc, P(f_0), P(f_1), P(bcm), P(bits), P(rec), too_many,
                                            sc.omega, 0, -1, P(out), _lib.stream_handle())
    assert st == _lib.ERR_ARG
    assert b"exceeds" in _lib.load().xlbg_last_error()
    # a count whose byte size overflows 64 bits is refused too, not wrapped into range
    st = _lib.load().xlbg_step_diag_noalloc(sc.stepper.desc, P(f_0), P(f_1), P(bcm), P(bits), P(rec), 1 << 60,
                                            sc.omega, 0, -1, P(out), _lib.stream_handle())
    assert st == _lib.ERR_ARG
    assert b"exceeds" in _lib.load().xlbg_last_error()
    assert ctypes.sizeof(ctypes.c_double) == 8
