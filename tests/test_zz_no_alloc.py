"""p3t_soft_force_noalloc: the soft force for callers that cannot allocate
device memory (their device buffers come from another runtime's arena, or
their process may not call cudaMalloc).  The test allocates the device
buffers itself, as such a caller would hand them over, calls the entry point
through the C ABI twice in a row on different inputs, and checks each result
against the allocating entry point p3t_soft_force_host on the same input:
neighbour fields bit-exact, forces within the soft tests' tolerance (the two
run the same kernel, so they agree to the last bit).  Collected last, so a
run that stops at the first failure has run every other test first."""
import ctypes

import numpy as np
import pytest

from gplum_gb300 import _lib, soft
from gplum_gb300.layout import FORCE_DTYPE
from tests.common import lists_for, prepared_state, records, rel_err

pytestmark = pytest.mark.gpu
VP = ctypes.c_void_p


def _device_copy(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1).copy()).cuda()


def _call_noalloc(lib, torch, P, epj, L, expect=0):
    bufs = {k: _device_copy(torch, L[k]) for k in ("i_off", "i_idx", "j_off", "j_idx", "s_off", "s_idx", "spj")}
    d_epj = _device_copy(torch, epj)
    d_force = torch.full((len(epj) * FORCE_DTYPE.itemsize,), 0xAB, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    st = lib.p3t_soft_force_noalloc(len(epj), VP(d_epj.data_ptr()), L["n_group"],
                                    *(VP(bufs[k].data_ptr()) for k in ("i_off", "i_idx", "j_off", "j_idx",
                                                                       "s_off", "s_idx")),
                                    VP(bufs["spj"].data_ptr()), len(L["spj"]), ctypes.c_double(P.eps2), 0,
                                    VP(d_force.data_ptr()), VP(stream.cuda_stream))
    assert st == expect, st
    return d_force.cpu().numpy().view(FORCE_DTYPE)


def test_no_alloc_soft_force_matches_allocating_entry_point(gpu):
    torch = pytest.importorskip("torch")
    lib = _lib.host_lib()
    for seed, n in ((12, 3000), (13, 5000)):
        P, d, s = prepared_state(n=n, seed=seed, ecc_hill=4.0, inc_hill=2.0)
        epi, epj = records(s)
        L = lists_for(s, P)
        want = soft.soft_force_host(P, epj, L, precision=0, trace_mode=0)
        got = _call_noalloc(lib, torch, P, epj, L)
        for k in ("number", "rank", "id_max", "id_min"):
            np.testing.assert_array_equal(got[k], want[k], err_msg=k)
        assert rel_err(got["acc"], want["acc"]).max() <= 1e-6
        assert (np.abs(got["phi"] - want["phi"]) <= 1e-6 * np.abs(want["phi"])).all()


def test_no_alloc_rejects_more_bodies_than_its_scratch(gpu):
    lib = _lib.host_lib()
    st = lib.p3t_soft_force_noalloc(65537, None, 1, None, None, None, None, None, None, None, 0,
                                    ctypes.c_double(0.0), 0, None, None)
    assert st < 0


def test_no_alloc_reports_bad_lists_then_recovers(gpu):
    """A list entry out of range is clamped by the kernel and returned as
    status 2; malformed offsets return 2 before any force kernel runs (the
    output keeps its fill); the next clean call returns 0 with the right
    result -- the status word does not carry over."""
    torch = pytest.importorskip("torch")
    lib = _lib.host_lib()
    P, d, s = prepared_state(n=2000, seed=14, ecc_hill=4.0, inc_hill=2.0)
    epi, epj = records(s)
    L = lists_for(s, P)
    bad = dict(L)
    bad["j_idx"] = L["j_idx"].copy()
    bad["j_idx"][len(bad["j_idx"]) // 2] = len(epj)  # one past the last body
    _call_noalloc(lib, torch, P, epj, bad, expect=2)
    dec = dict(L)
    dec["j_off"] = L["j_off"].copy()
    dec["j_off"][1] = dec["j_off"][2] + 1  # decreasing
    got = _call_noalloc(lib, torch, P, epj, dec, expect=2)
    assert (got.view(np.uint8) == 0xAB).all()
    want = soft.soft_force_host(P, epj, L, precision=0, trace_mode=0)
    got = _call_noalloc(lib, torch, P, epj, L, expect=0)
    for k in ("number", "rank", "id_max", "id_min"):
        np.testing.assert_array_equal(got[k], want[k], err_msg=k)
    assert rel_err(got["acc"], want["acc"]).max() <= 1e-6
