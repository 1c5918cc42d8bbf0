"""libbsc's BWT-stage names (bsc_bwt_encode / bsc_bwt_decode) through the shim
object, from a C program linked the way libbsc would be: known answers from
the golden vectors, and the inverse back to the input."""
import json
import os
import subprocess

import pytest

from test_native_abi import build_shim_caller

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "bwt_vectors.json")


@pytest.mark.parametrize("name", ["banana", "period3", "bsc_rs_test_0", "headers"])
def test_shim_matches_golden_vectors(tmp_path, name):
    vec = next(v for v in json.load(open(GOLDEN))["vectors"] if v["name"] == name)
    t = bytes.fromhex(vec["input"])
    if not t or b"\0" in t or len(t) > 4096:
        pytest.skip("not passable as a C string argument")
    exe = build_shim_caller(tmp_path)
    r = subprocess.run([str(exe).encode(), t], capture_output=True, timeout=120)
    assert r.returncode == 0, r.stderr
    first, second = r.stdout.split(b"\n")[:2]
    u, idx = first[:len(t)], int(first[len(t) + 1:])
    assert u == bytes.fromhex(vec["bwt"]) and idx == vec["index"]
    assert second == t
