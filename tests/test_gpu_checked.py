"""The bounds-checked build (librc_gb300_checked.so, -DGB_CHECKED): the FP32
tiled kernels test every shared-memory, GCF, record and visibility index
against its array and count violations instead of faulting.  A child
interpreter loads that library (RC_GB300_CHECKED=1), checks that the counter
counts (a self-test that only computes out-of-range indices), runs the
engine, batch and allocation-free parity cases through the checked kernels,
and reports the violations: there must be none."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_CHILD = r"""
import ctypes as C, json, sys
sys.path.insert(0, sys.argv[1])
from rc_gb300 import lib
L = lib.load()
v = C.c_int64()
out = {"library": L._name}
assert L.gb_checked_violations(C.byref(v)) == 0
assert L.gb_checked_selftest() == 0
L.gb_checked_violations(C.byref(v))
out["selftest"] = v.value
import tests.test_gpu_engine as E
import tests.test_gpu_batch as B
import tests.test_zz_no_alloc as N
for args in [(32, 256, 32), (16, 128, 16), (64, 512, 32), (8, 256, 8), (32, 512, 64),
             (25, 256, 32), (9, 128, 16)]:
    E.test_fp32_tiled_grid_matches_fp64_oracle(*args)
for args in [(24, 0, 0), (8, 512, 64), (32, 256, 32)]:
    E.test_largest_supports(*args)
E.test_fp32_adjoint_identity()
E.test_gcf_on_an_8_byte_boundary()
E.test_single_visibility_each_plane()
B.test_batch_matches_oracle_per_member_and_in_a_graph()
N.test_noalloc_matches_planned_entry_point_twice()
L.gb_checked_violations(C.byref(v))
out["violations"] = v.value
print(json.dumps(out))
"""


def test_checked_kernels_see_no_out_of_range_index():
    from rc_gb300 import build as B

    lib_path = B.build(checked=True)
    env = dict(os.environ, RC_GB300_CHECKED="1", RC_GB300_AUTOBUILD="0")
    r = subprocess.run([sys.executable, "-c", _CHILD, ROOT], env=env, capture_output=True,
                       text=True, timeout=1500)
    assert r.returncode == 0, r.stderr[-4000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert os.path.samefile(out["library"], lib_path)
    assert out["selftest"] == 2
    assert out["violations"] == 0


def test_normal_build_reports_no_checking():
    import ctypes as C

    from rc_gb300 import lib

    L = lib.load()
    v = C.c_int64()
    assert L.gb_checked_violations(C.byref(v)) == 0 and v.value == -1
    assert L.gb_checked_selftest() == lib.ERR_ARG
