"""The FDPS-side binding of the multiwalk pair (tests/cxx/multiwalk_binding.cpp,
the DispatchP3T / RetrieveP3T callbacks INTEGRATION.md gives for
src/main_p3t.cpp:351-355), compiled as C++:

* against GPLUM's own record classes (its particle.h over the PS shim),
  where the reference tree is present: the build succeeds only if EPIGrav,
  EPJGrav, MySPJQuadrupole and ForceGrav have, member by member, the layouts
  the C ABI reads and writes (static_asserts);
* against the library's C structs, linked with the library and run on the
  GPU the way FDPS runs a multiwalk force: every body's ForceGrav record
  equals, bit for bit, the resident path's on the same lists.
"""
import os
import subprocess

import numpy as np
import pytest

from oracle import harness as H

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cxx", "multiwalk_binding.cpp")


def test_gplum_classes_have_the_abi_layouts():
    ref = H.ref_source_dir()
    if ref is None:
        pytest.skip("no reference build (GPLUM's source tree is not present here)")
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-w", "-DGPLUM_TYPES", "-DUSE_INDIVIDUAL_CUTOFF", "-DUSE_QUAD",
           "-DCOLLISION", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "oracle", "ref_shim"),
           "-iquote", ref, SRC]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


@pytest.mark.gpu
def test_compiled_multiwalk_binding_runs_on_the_gpu(gpu, tmp_path):
    from gplum_gb300 import build, soft
    from tests.common import lists_for, prepared_state, records

    exe = tmp_path / "multiwalk_binding"
    libdir = os.path.dirname(build.LIB)
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), SRC, "-L", libdir, "-lgplum_p3t",
           f"-Wl,-rpath,{libdir}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    P, d, s = prepared_state(n=4000, seed=41, ecc_hill=4.0, inc_hill=2.0)
    epi, epj = records(s)
    L = lists_for(s, P)
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        np.array([len(epj), L["n_group"], len(L["spj"])], np.int64).tofile(f)
        P.vector().tofile(f)
        epj.tofile(f)
        L["spj"].tofile(f)
        for k in ("i_off", "i_idx", "j_off", "j_idx", "s_off", "s_idx"):
            np.ascontiguousarray(L[k], np.int32).tofile(f)
    out = tmp_path / "out.bin"
    r = subprocess.run([str(exe), str(inp), str(out), "64"], capture_output=True, text=True)
    assert r.returncode == 0, (r.stdout, r.stderr)
    got = np.fromfile(out, dtype=soft.FORCE_DTYPE)
    want = soft.soft_force_host(P, epj, L)
    assert got.tobytes() == want.tobytes()
