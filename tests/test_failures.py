"""Malformed caller input is rejected on the host before any device work
(GPLUM itself trusts FDPS's lists and stops with PS::Abort on a broken
invariant, src/main_p3t.cpp:160-203; a C caller here gets a status code).
Every case below returns before the library touches a GPU, so it runs on
CPU: status 2 (list index or offset out of range) for bad lists,
-cudaErrorInvalidValue (-1) for the no-allocation entry point's limits."""
import ctypes

import numpy as np

from gplum_gb300 import _lib

VP = ctypes.c_void_p
BAD_INDEX = 2
INVALID_VALUE = -1


def _p(a):
    return a.ctypes.data_as(VP) if a is not None else None


def _lists(n_group=3, per=4):
    off = np.arange(0, (n_group + 1) * per, per, dtype=np.int32)
    idx = np.zeros(n_group * per, np.int32)
    return off, idx


def test_upload_lists_rejects_bad_offsets():
    lib = _lib.host_lib()
    off, idx = _lists()
    spj = np.zeros(80, np.uint8)
    dec = off.copy()
    dec[2] = dec[1] - 1  # decreasing
    start = off + 1      # does not start at 0
    for i_off, j_off, s_off in ((dec, off, off), (off, dec, off), (off, off, dec), (start, off, off)):
        r = lib.p3t_upload_lists(3, _p(i_off), _p(idx), _p(j_off), _p(idx), _p(s_off), _p(idx), _p(spj), 1)
        assert r == BAD_INDEX
    # entries promised by the offsets but no array
    assert lib.p3t_upload_lists(3, _p(off), None, _p(off), _p(idx), _p(off), _p(idx), _p(spj), 1) == BAD_INDEX
    # superparticles promised but absent; negative counts
    assert lib.p3t_upload_lists(3, _p(off), _p(idx), _p(off), _p(idx), _p(off), _p(idx), None, 1) == BAD_INDEX
    assert lib.p3t_upload_lists(-1, _p(off), _p(idx), _p(off), _p(idx), _p(off), _p(idx), _p(spj), 1) == BAD_INDEX


def test_host_call_rejects_bad_offsets_and_buffers():
    lib = _lib.host_lib()
    off, idx = _lists()
    dec = off.copy()
    dec[3] = 0
    epj = np.zeros(112 * 12, np.uint8)
    force = np.zeros(32 * 12, np.uint8)
    spj = np.zeros(80, np.uint8)
    args = lambda i_off: (12, _p(epj), 3, _p(i_off), _p(idx), _p(off), _p(idx), _p(off), _p(idx), _p(spj), 1,
                          _p(force))
    assert lib.p3t_soft_force_host(*args(dec)) == BAD_INDEX
    assert lib.p3t_soft_force_host(12, None, 3, _p(off), _p(idx), _p(off), _p(idx), _p(off), _p(idx), _p(spj), 1,
                                   _p(force)) == BAD_INDEX
    assert lib.p3t_upload_particles(-3, _p(epj)) == BAD_INDEX
    assert lib.p3t_upload_particles(3, None) == BAD_INDEX


def test_multiwalk_dispatch_rejects_bad_counts():
    lib = _lib.host_lib()
    rec = np.zeros(112 * 4, np.uint8)
    ptrs = (VP * 2)(_p(rec), _p(rec))
    good = np.array([2, 2], np.int32)
    neg = np.array([2, -1], np.int32)
    nulls = (VP * 2)(_p(rec), None)
    assert lib.p3t_soft_dispatch(0, 2, ptrs, _p(neg), ptrs, _p(good), ptrs, _p(good)) == BAD_INDEX
    assert lib.p3t_soft_dispatch(0, 2, ptrs, _p(good), nulls, _p(good), ptrs, _p(good)) == BAD_INDEX
    assert lib.p3t_soft_dispatch(0, -1, ptrs, _p(good), ptrs, _p(good), ptrs, _p(good)) == BAD_INDEX
    ids = np.zeros(2, np.int32)
    id_ptrs = (VP * 2)(_p(ids), _p(ids))
    assert lib.p3t_soft_dispatch_index(0, 2, ptrs, _p(good), id_ptrs, _p(neg), id_ptrs, _p(good), _p(rec), 4,
                                       None, 0, 1) == BAD_INDEX
    assert lib.p3t_soft_dispatch_index(0, 2, ptrs, _p(good), id_ptrs, _p(good), id_ptrs, _p(good), None, 4,
                                       None, 0, 1) == BAD_INDEX


def test_no_alloc_rejects_over_size_and_null_buffers():
    lib = _lib.host_lib()
    off, idx = _lists()
    buf = np.zeros(1024, np.uint8)
    spj = np.zeros(80, np.uint8)
    # more superparticles than the static scratch holds
    assert lib.p3t_soft_force_noalloc(12, _p(buf), 3, _p(off), _p(idx), _p(off), _p(idx), _p(off), _p(idx),
                                      _p(spj), 65537, 0.0, 0, _p(buf), None) == INVALID_VALUE
    # null buffers where the call would read or write them
    assert lib.p3t_soft_force_noalloc(12, None, 3, _p(off), _p(idx), _p(off), _p(idx), _p(off), _p(idx),
                                      _p(spj), 1, 0.0, 0, _p(buf), None) == INVALID_VALUE
    assert lib.p3t_soft_force_noalloc(12, _p(buf), 3, _p(off), None, _p(off), _p(idx), _p(off), _p(idx),
                                      _p(spj), 1, 0.0, 0, _p(buf), None) == INVALID_VALUE
    assert lib.p3t_soft_force_noalloc(12, _p(buf), 3, _p(off), _p(idx), _p(off), _p(idx), _p(off), _p(idx),
                                      None, 1, 0.0, 0, _p(buf), None) == INVALID_VALUE
    assert lib.p3t_soft_force_noalloc(12, _p(buf), 3, _p(off), _p(idx), _p(off), _p(idx), _p(off), _p(idx),
                                      _p(spj), 1, 0.0, 0, None, None) == INVALID_VALUE


def test_step_cap_setter_range():
    lib = _lib.host_lib()
    assert lib.p3t_set_hard_step_cap(0) == INVALID_VALUE
    assert lib.p3t_set_hard_step_cap((1 << 20) + 1) == INVALID_VALUE
    assert lib.p3t_set_hard_step_cap(1 << 20) == 0


def test_count_status_coding():
    assert _lib.status_bits(-(65536 + 4)) == 4
    assert _lib.status_bits(-(65536 + 18)) == 18
    assert _lib.status_bits(-700) == 0 and _lib.status_bits(3) == 0


def test_form_setters_reject_out_of_range():
    lib = _lib.host_lib()
    try:
        for bad in (-1, 4):
            assert lib.p3t_set_walk(bad) == INVALID_VALUE
        assert lib.p3t_set_walk(3) == 0 and lib.p3t_set_walk(1) == 0
        for cap, store in ((0, 0), (4097, 0), (8, -1)):
            assert lib.p3t_set_walk_limits(cap, store) == INVALID_VALUE
        assert lib.p3t_set_walk_limits(4096, 0) == 0
        for thr, ctas in ((-1.0, 0), (1.0, -1), (1.0, 4097)):
            assert lib.p3t_set_hard_lone(thr, ctas) == INVALID_VALUE
        assert lib.p3t_hard_phase_cycles(None, 14) == INVALID_VALUE
        buf = np.zeros(4, np.uint64)
        assert lib.p3t_hard_phase_cycles(_p(buf), 4) == INVALID_VALUE  # fewer slots than phases
    finally:
        lib.p3t_set_walk(1)
        lib.p3t_set_hard_lone(0.0, 0)
