"""Soft force on the GPU against the CPU oracle (same lists, same records).

Bit-exact: neighbour count, rank sum, id_min, id_max (the FP32 screen of
src/gravity_kernel.hpp:89-112 reproduced operation for operation).
Tolerance: accelerations and potentials against the FP64 restatement of the
functors, per particle |a_gpu - a_64| / |a_64|:
  mixed form  -- median <= 1e-6; 99th percentile no worse than GPLUM's own
                 FP32 functor on the same input, maximum within twice its
                 maximum + 1e-6;
  FP64 form   -- <= 1e-12.
"""
import ctypes

import numpy as np
import pytest

from gplum_gb300 import soft
from gplum_gb300.disk import P3TParams
from gplum_gb300.layout import FORCE_DTYPE, cleared_forces
from oracle import harness as H
from tests.common import lists_for, prepared_state, records, rel_err

pytestmark = pytest.mark.gpu
VP = ctypes.c_void_p


def oracle_lists(mode, L, epi, epj, trace_mode=0):
    lib = H.load("orc")
    n = len(epj)
    args = [L[k].ctypes.data_as(VP) for k in ("i_off", "i_idx", "j_off", "j_idx", "s_off", "s_idx")]
    if mode == 0:
        f = cleared_forces(n)
        lib.orc_soft_lists(0, trace_mode, L["n_group"], *args, epi.ctypes.data_as(VP), epj.ctypes.data_as(VP),
                           L["spj"].ctypes.data_as(VP), f.ctypes.data_as(VP), None, None, 8)
        return f
    acc4 = np.zeros(4 * n)
    ngb4 = np.zeros(4 * n, np.int32)
    lib.orc_soft_lists(1, trace_mode, L["n_group"], *args, epi.ctypes.data_as(VP), epj.ctypes.data_as(VP),
                       L["spj"].ctypes.data_as(VP), None, acc4.ctypes.data_as(VP), ngb4.ctypes.data_as(VP), 8)
    return acc4.reshape(-1, 4), ngb4.reshape(-1, 4)


def check_neighbours(got, want):
    for k in ("number", "rank", "id_max", "id_min"):
        np.testing.assert_array_equal(got[k], want[k], err_msg=k)


def check_mixed_accuracy(got, ref32, a64):
    """Median <= 1e-6; the tail no worse than GPLUM's FP32 functor beyond
    rounding noise (both are FP32 sums that cancel for a few particles)."""
    e_gpu = rel_err(got["acc"], a64[:, :3])
    e_ref = rel_err(ref32["acc"], a64[:, :3])
    assert np.median(e_gpu) <= 1e-6, np.median(e_gpu)
    assert np.percentile(e_gpu, 99) <= max(np.percentile(e_ref, 99), 1e-6)
    assert e_gpu.max() <= 2.0 * e_ref.max() + 1e-6, (e_gpu.max(), e_ref.max())
    ep = np.abs(got["phi"] - a64[:, 3]) / np.abs(a64[:, 3])
    assert ep.max() <= 1e-6, ep.max()
    return e_gpu, e_ref


@pytest.mark.parametrize("n_group_limit", [64, 256, 33, 1])
def test_resident_mixed_matches_oracle(gpu, n_group_limit):
    P = P3TParams(n_group_limit=n_group_limit)
    P, d, s = prepared_state(n=3000 if n_group_limit > 1 else 400, seed=5, ecc_hill=4.0, inc_hill=2.0,
                             params=P, with_acc_d=True)
    epi, epj = records(s)
    L = lists_for(s, P)
    sf = soft.SoftForce(P, precision=0)
    sf.upload_particles(epj)
    sf.upload_lists(L)
    sf.run()
    got = sf.download()
    ref32 = oracle_lists(0, L, epi, epj)
    a64, _ = oracle_lists(1, L, epi, epj)
    check_neighbours(got, ref32)
    check_mixed_accuracy(got, ref32, a64)


def test_resident_fp64_form(gpu):
    P, d, s = prepared_state(n=3000, seed=6, ecc_hill=4.0, inc_hill=2.0, with_acc_d=True)
    epi, epj = records(s)
    L = lists_for(s, P)
    sf = soft.SoftForce(P, precision=1)
    sf.upload_particles(epj)
    sf.upload_lists(L)
    sf.run()
    got = sf.download()
    a64, n64 = oracle_lists(1, L, epi, epj)
    assert rel_err(got["acc"], a64[:, :3]).max() <= 1e-6  # ForceGrav stores float
    np.testing.assert_array_equal(got["number"], n64[:, 0])
    soft.configure(P, precision=0)


def test_larger_disk_and_both_traces(gpu):
    """n = 60000 with group limit 256: every work split of the kernel and
    lists longer than one shared-memory tile; both quadrupole traces."""
    P = P3TParams(n_group_limit=256)
    P, d, s = prepared_state(n=60000, seed=7, a_in=0.9, a_out=1.1, m=2e-10, params=P)
    epi, epj = records(s)
    L = lists_for(s, P)
    sizes = np.diff(L["i_off"])
    assert sizes.max() > 128 and sizes.min() <= 32 and np.diff(L["j_off"]).max() > 128
    for trace in (0, 1):
        sf = soft.SoftForce(P, precision=0, trace_mode=trace)
        sf.upload_particles(epj)
        sf.upload_lists(L)
        sf.run()
        got = sf.download()
        ref32 = oracle_lists(0, L, epi, epj, trace)
        a64, _ = oracle_lists(1, L, epi, epj, trace)
        check_neighbours(got, ref32)
        check_mixed_accuracy(got, ref32, a64)
    soft.configure(P, trace_mode=0)


def test_functor_calls_accumulate_into_records(gpu):
    P, d, s = prepared_state(n=2000, seed=8, ecc_hill=4.0, inc_hill=2.0)
    soft.configure(P)
    epi, epj = records(s)
    L = lists_for(s, P)
    lib = H.load("orc")
    rng = np.random.default_rng(0)
    for g in range(0, L["n_group"], 4):
        ii = L["i_idx"][L["i_off"][g]:L["i_off"][g + 1]]
        ei = np.ascontiguousarray(epi[ii])
        ej = np.ascontiguousarray(epj[L["j_idx"][L["j_off"][g]:L["j_off"][g + 1]]])
        sj = np.ascontiguousarray(L["spj"][L["s_idx"][L["s_off"][g]:L["s_off"][g + 1]]])
        start = cleared_forces(len(ii))
        start["acc"] = rng.normal(0, 1e-4, (len(ii), 3))
        start["number"] = 1
        start["id_max"] = 5
        a, b = start.copy(), start.copy()
        soft.calc_force_epep(ei, ej, a)
        soft.calc_force_epsp(ei, sj, a)
        lib.orc_epep_f32(ei.ctypes.data_as(VP), len(ei), ej.ctypes.data_as(VP), len(ej), b.ctypes.data_as(VP))
        lib.orc_epsp_f32(ei.ctypes.data_as(VP), len(ei), sj.ctypes.data_as(VP), len(sj), b.ctypes.data_as(VP), 0)
        check_neighbours(a, b)
        np.testing.assert_allclose(a["acc"], b["acc"], rtol=0, atol=1e-5 * np.abs(b["acc"]).max())


def _ragged(L, drop_j, drop_s):
    """L with the EPJ lists of the groups in drop_j and the SPJ lists of those
    in drop_s emptied."""
    out = {"n_group": L["n_group"], "spj": L["spj"], "i_off": L["i_off"], "i_idx": L["i_idx"]}
    for k, idx, drop in (("j", "j_idx", drop_j), ("s", "s_idx", drop_s)):
        off = L[k + "_off"]
        parts = [L[idx][off[g]:off[g + 1]] if g not in drop else L[idx][:0] for g in range(L["n_group"])]
        out[k + "_off"] = np.concatenate([[0], np.cumsum([len(x) for x in parts])]).astype(np.int32)
        out[idx] = np.concatenate(parts).astype(np.int32)
    return out


def test_empty_and_ragged_inputs(gpu):
    """Zero-length inputs through every entry point: functor calls with no
    j-particles or no superparticles leave the records as they were; an empty
    system through the host call; groups whose EPJ or SPJ lists are empty
    (resident run and host call) against the oracle on the same lists."""
    P, d, s = prepared_state(n=2000, seed=13, ecc_hill=4.0, inc_hill=2.0)
    soft.configure(P)
    epi, epj = records(s)
    L = lists_for(s, P)
    ii = L["i_idx"][L["i_off"][0]:L["i_off"][1]]
    ei = np.ascontiguousarray(epi[ii])
    start = cleared_forces(len(ii))
    start["acc"] = np.random.default_rng(1).normal(0, 1e-4, (len(ii), 3))
    start["number"] = 2
    start["id_min"] = 7
    a = start.copy()
    soft.calc_force_epep(ei, epj[:0], a)
    soft.calc_force_epsp(ei, L["spj"][:0], a)
    assert a.tobytes() == start.tobytes()
    empty = {"n_group": 0, "spj": L["spj"][:0]}
    for k in ("i", "j", "s"):
        empty[k + "_off"] = np.zeros(1, np.int32)
        empty[k + "_idx"] = np.zeros(0, np.int32)
    assert len(soft.soft_force_host(P, epj[:0], empty)) == 0
    ng = L["n_group"]
    # disjoint: every group keeps one of its lists (a body with neither has phi = 0)
    R = _ragged(L, {g for g in range(ng) if g % 5 == 1}, {g for g in range(ng) if g % 3 == 0 and g % 5 != 1})
    assert (np.diff(R["j_off"]) == 0).any() and (np.diff(R["s_off"]) == 0).any()
    sf = soft.SoftForce(P, precision=0)
    sf.upload_particles(epj)
    sf.upload_lists(R)
    sf.run()
    got = sf.download()
    assert soft.soft_force_host(P, epj, R).tobytes() == got.tobytes()
    ref32 = oracle_lists(0, R, epi, epj)
    a64, _ = oracle_lists(1, R, epi, epj)
    check_neighbours(got, ref32)
    check_mixed_accuracy(got, ref32, a64)


def test_multiwalk_forms_equal_resident(gpu):
    P, d, s = prepared_state(n=5000, seed=9, ecc_hill=4.0, inc_hill=2.0, params=P3TParams(n_group_limit=128))
    soft.configure(P)
    epi, epj = records(s)
    L = lists_for(s, P)
    sf = soft.SoftForce(P)
    sf.upload_particles(epj)
    sf.upload_lists(L)
    sf.run()
    want = sf.download()
    mw = soft.MultiWalk()
    groups = list(range(L["n_group"]))
    batches = [groups[k:k + 17] for k in range(0, len(groups), 17)]
    got = np.zeros(len(epj), FORCE_DTYPE)
    got_idx = np.zeros(len(epj), FORCE_DTYPE)
    for bi, batch in enumerate(batches):
        epis = [epi[L["i_idx"][L["i_off"][g]:L["i_off"][g + 1]]] for g in batch]
        epjs = [epj[L["j_idx"][L["j_off"][g]:L["j_off"][g + 1]]] for g in batch]
        spjs = [L["spj"][L["s_idx"][L["s_off"][g]:L["s_off"][g + 1]]] for g in batch]
        mw.dispatch(bi % 2, epis, epjs, spjs)
        for g, f in zip(batch, mw.retrieve(bi % 2)):
            got[L["i_idx"][L["i_off"][g]:L["i_off"][g + 1]]] = f
        idj = [L["j_idx"][L["j_off"][g]:L["j_off"][g + 1]] for g in batch]
        ids = [L["s_idx"][L["s_off"][g]:L["s_off"][g + 1]] for g in batch]
        mw.dispatch_index(bi % 2, epis, idj, ids, epj, L["spj"], send_flag=(bi == 0))
        for g, f in zip(batch, mw.retrieve(bi % 2)):
            got_idx[L["i_idx"][L["i_off"][g]:L["i_off"][g + 1]]] = f
    assert got.tobytes() == want.tobytes()
    assert got_idx.tobytes() == want.tobytes()


def test_host_one_call_equals_resident(gpu):
    P, d, s = prepared_state(n=3000, seed=10)
    epi, epj = records(s)
    L = lists_for(s, P)
    a = soft.soft_force_host(P, epj, L)
    sf = soft.SoftForce(P)
    sf.upload_particles(epj)
    sf.upload_lists(L)
    sf.run()
    assert a.tobytes() == sf.download().tobytes()


@pytest.mark.parametrize("tiles", [(0, 0, 0), (64, 32, 16), (128, 64, 0), (256, 64, 32), (128, 64, 32, 4), (128, 48, 16, 6)])
def test_work_splits_agree(gpu, tiles):
    """Every work split the autotuner may choose gives the same neighbour
    fields and forces equal to rounding (sub-block partial sums combine in a
    different grouping)."""
    P, d, s = prepared_state(n=20000, seed=9, ecc_hill=3.0, inc_hill=1.5, params=P3TParams(n_group_limit=256))
    epi, epj = records(s)
    L = lists_for(s, P)
    sf = soft.SoftForce(P, precision=0)
    sf.upload_particles(epj)
    sf.upload_lists(L)
    lib = sf.lib
    try:
        lib.p3t_set_soft_tiles(128, 64, 32)
        sf.run(emit_candidates=False)
        ref = sf.download().copy()
        assert lib.p3t_set_soft_tiles(*tiles[:3]) == 0
        if len(tiles) > 3:
            assert lib.p3t_set_soft_occupancy(tiles[3]) == 0
        sf.run(emit_candidates=False)
        got = sf.download()
    finally:
        lib.p3t_set_soft_tiles(128, 64, 32)
        lib.p3t_set_soft_occupancy(5)
    for k in ("number", "rank", "id_max", "id_min"):
        np.testing.assert_array_equal(got[k], ref[k])
    assert rel_err(got["acc"].astype(np.float64), ref["acc"].astype(np.float64)).max() < 1e-6
    assert lib.p3t_set_soft_tiles(40, 64, 32) != 0  # invalid: t_ipt2 < t_s1
    assert lib.p3t_set_soft_tiles(200, 64, 32) != 0  # invalid: neither <= 128 nor 256
    assert lib.p3t_set_soft_occupancy(3) != 0


@pytest.mark.parametrize("ngl,tiles", [(256, (128, 64, 32)), (64, (128, 64, 32)), (256, (256, 32, 0))])
def test_pipelined_staging_bit_identical(gpu, ngl, tiles):
    """The pipelined staging (records copied two tiles ahead, one barrier per
    tile) against gather-then-compute: the same ForceGrav records bit for
    bit, with and without candidate emission, in every work split."""
    P, d, s = prepared_state(n=20000, seed=9, ecc_hill=3.0, inc_hill=1.5, params=P3TParams(n_group_limit=ngl))
    epi, epj = records(s)
    L = lists_for(s, P)
    sf = soft.SoftForce(P, precision=0)
    sf.upload_particles(epj)
    sf.upload_lists(L)
    lib = sf.lib
    out = {}
    try:
        assert lib.p3t_set_soft_tiles(*tiles) == 0
        for pipe in (0, 1):
            assert lib.p3t_set_soft_pipe(pipe) == 0
            for emit in (False, True):
                sf.run(emit_candidates=emit)
                out[pipe, emit] = sf.download().copy()
    finally:
        lib.p3t_set_soft_pipe(0)
        lib.p3t_set_soft_tiles(128, 64, 32)
    for emit in (False, True):
        assert out[1, emit].tobytes() == out[0, emit].tobytes()
