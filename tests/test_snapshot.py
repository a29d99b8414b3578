"""Snapshot files (GPLUM's snapNNNNNN.dat and snap_tmp.dat): the library's
host writer against GPLUM's own FileHeader / FPGrav writers compiled from the
reference headers (oracle/_ref), byte for byte, on a state after start-up and
two tree steps; the readers on those files; the FPGrav layout of the binary
record against GPLUM's compiled class.  No GPU."""
import ctypes

import numpy as np
import pytest

from gplum_gb300 import snapshot
from gplum_gb300.disk import P3TParams, make_disk
from oracle import harness as H

pytestmark = pytest.mark.skipif(not H.ref_available(), reason="reference build (oracle/_ref) not available")

# GPLUM's FPGrav (individual cutoffs, quadrupole, collisions): sizeof, sizeof(FileHeader), then the
# byte offsets of id_local myrank pos r_out r_search id mass vel acc_d acc acc_s jerk_d jerk_s acc_gd
# phi phi_d phi_s v_disp r_out_inv time dt acc0 r_planet f neighbor id_cluster n_cluster inDomain
# isSent isDead isMerged -- the layout csrc/snapshot_io.cpp writes
LAYOUT = [344, 128, 0, 4, 8, 32, 40, 48, 56, 64, 88, 112, 136, 160, 184, 208, 232, 240, 248, 256, 264, 272,
          280, 288, 296, 304, 312, 328, 336, 340, 341, 342, 343]

VEC = ("pos", "vel", "acc", "acc_d", "jerk_d", "acc_s", "jerk_s")
SCAL = ("mass", "r_planet", "f", "phi", "phi_d", "phi_s", "r_out", "r_search", "r_out_inv", "v_disp", "time", "dt",
        "acc0")
INTS = ("number", "rank", "id_max", "id_min", "n_cluster", "dead", "merged")


@pytest.fixture(scope="module")
def ref_state():
    P = P3TParams()
    d = make_disk(600, 1e-9, 0.99, 1.01, ecc_hill=2.0, inc_hill=1.0, seed=21, f=150.0)
    s = H.CpuSystem("ref", P)
    lf = H.tree_lists_fn(P)
    H.p3t_init(s, d, lf)
    ncol = sum(len(H.p3t_step(s, st, lf)["cols"]) for st in (1, 2))
    s.f("set_id_local")()
    arrays = {k: s.get(k) for k in VEC + SCAL}
    arrays["id"] = s.get("id")
    arrays["id_cluster"] = s.get("id_cluster")
    for k in INTS:
        arrays[k] = s.get(k).astype(np.int32)
    return s, arrays, ncol


def test_fpgrav_layout_matches_gplum():
    s = H.CpuSystem("ref", P3TParams())
    out = (ctypes.c_longlong * 40)()
    s.f("fpgrav_layout")(out)
    assert list(out)[:len(LAYOUT)] == LAYOUT


@pytest.mark.parametrize("binary", [0, 1])
def test_host_writer_matches_gplum_byte_for_byte(ref_state, tmp_path, binary):
    s, arrays, ncol = ref_state
    e_init = np.array([-1.25e-3, 2.5e-4, -1.5e-3, -1.0e-9, -1.2e-9, 2.0e-10, 0.0])
    e_now = np.array([-1.2500001e-3, 2.5e-4, -1.5e-3, -1.1e-9, -1.3e-9, 2.0e-10, 3.0e-15])
    t, id_next = 2 * 2.0**-7, int(arrays["id"].max()) + 1
    want, got = tmp_path / "ref.dat", tmp_path / "ours.dat"
    e0 = e_init.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    e1 = e_now.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    assert s.f("write_snapshot")(str(want).encode(), binary, ctypes.c_double(t), id_next, e0, e1) == 0
    hdr = snapshot.Header(time=t, id_next=id_next, e_init=e_init, e_now=e_now)
    src = arrays if binary else {k: arrays[k] for k in snapshot.ASCII_FIELDS}
    snapshot.write_host(got, binary, hdr, src)
    a, b = want.read_bytes(), got.read_bytes()
    assert len(a) == len(b) and a == b
    assert len(a) == (128 + 344 * len(arrays["id"]) if binary else len(a))


@pytest.mark.parametrize("binary", [0, 1])
def test_reader_recovers_the_written_bodies(ref_state, tmp_path, binary):
    s, arrays, _ = ref_state
    path = tmp_path / "snap.dat"
    e = np.arange(7, dtype=np.float64) * 1e-4
    hdr = snapshot.Header(time=0.5, id_next=777, e_init=e, e_now=-e)
    snapshot.write_host(path, binary, hdr, arrays)
    h, got = snapshot.read_host(path, binary)
    assert h.n_body == len(arrays["id"]) and h.id_next == 777 and h.time == 0.5
    if binary:
        np.testing.assert_array_equal(h.e_init, e)
        for k in VEC + SCAL + INTS + ("id", "id_cluster"):
            np.testing.assert_array_equal(got[k].reshape(arrays[k].shape), arrays[k], err_msg=k)
    else:
        # the ASCII header carries etot ekin ephi_sun ephi_planet edisp at 16 digits
        np.testing.assert_allclose(h.e_init[[0, 1, 2, 3, 6]], e[[0, 1, 2, 3, 6]], rtol=1e-15)
        text = np.loadtxt(path, skiprows=1)
        np.testing.assert_array_equal(got["id"], text[:, 0].astype(np.int64))
        np.testing.assert_array_equal(got["mass"], text[:, 1])
        np.testing.assert_array_equal(got["pos"], text[:, 4:7])
        np.testing.assert_array_equal(got["vel"], text[:, 7:10])
        np.testing.assert_array_equal(got["number"], text[:, 10].astype(np.int32))
        np.testing.assert_allclose(got["pos"], arrays["pos"], rtol=1e-15, atol=0)


def test_ascii_without_header_reads_as_initial_conditions(ref_state, tmp_path):
    s, arrays, _ = ref_state
    path = tmp_path / "INIT.dat"
    snapshot.write_host(path, 0, snapshot.Header(), {k: arrays[k] for k in snapshot.ASCII_FIELDS})
    lines = path.read_text().splitlines()
    headless = tmp_path / "INIT_noheader.dat"
    headless.write_text("\n".join(lines[1:]) + "\n")
    h, got = snapshot.read_host(headless, 0)
    assert h.n_body == len(arrays["id"]) and h.time == 0.0
    np.testing.assert_array_equal(got["id"], arrays["id"])


def test_reader_rejects_a_truncated_file(ref_state, tmp_path):
    s, arrays, _ = ref_state
    path = tmp_path / "snap_tmp.dat"
    snapshot.write_host(path, 1, snapshot.Header(), arrays)
    data = path.read_bytes()
    path.write_bytes(data[:-100])
    with pytest.raises(RuntimeError):
        snapshot.read_host(path, 1)
