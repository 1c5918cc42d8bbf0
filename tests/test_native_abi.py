"""The C-ABI library builds, loads and exports every entry point the header
declares (no compute calls: this runs without a GPU)."""
import ctypes
import os
import re
import subprocess

import pytest

from qz_gb300 import build, native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "qzgpu.h")


def declared_functions(path=HEADER):
    src = open(path).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(qzgpu_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return native.load()


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("qzgpu_init", "qzgpu_bwt_encode", "qzgpu_bwt_decode", "qzgpu_bwt_encode_batch",
                 "qzgpu_bwt_decode_batch", "qzgpu_bwt_encode_device", "qzgpu_bwt_decode_device"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", native.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\sT\s+(\w+)", out))
    missing = [f for f in declared_functions() if f not in exported]
    assert not missing, missing
    for f in declared_functions():
        assert f in native.SIGNATURES, f"binding lacks {f}"
        getattr(lib, f)


def test_error_strings_and_aux_rate(lib):
    assert native.error_string(-6) == "data corrupt"
    assert native.error_string(0) == "no error"
    # largest power of two <= max(n/8, 1)
    assert lib.qzgpu_aux_rate(0) == 1
    assert lib.qzgpu_aux_rate(7) == 1
    assert lib.qzgpu_aux_rate(16) == 2
    assert lib.qzgpu_aux_rate(26_214_400) == 2_097_152


def test_kernels_built_for_sm103a(lib):
    # one -gencode target, sm_103a, for every translation unit
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    objs = [os.path.join(build.OUT, os.path.basename(s) + ".o") for s in build.sources()]
    assert all(os.path.exists(o) for o in objs)


def test_no_cpu_fallback_without_gpu(lib):
    # With no usable GPU the library reports an error instead of computing.
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from qz_gb300 import bwt

    with pytest.raises(native.QzGpuError) as e:
        bwt.bwt_encode(b"ACGTACGT")
    assert e.value.code in (native.QZGPU_GPU_NOT_SUPPORTED, native.QZGPU_GPU_ERROR)


C_CALLER = r"""
/* A plain C caller of the boundary: the header is valid C and every entry
 * point links from a C program (the binding a Rust, Go or C host would make). */
#include <stdio.h>
#include "qzgpu.h"

int main(int argc, char **argv) {
    if (argc < 2) return 0; /* linked, not run: no GPU needed */
    unsigned char t[8] = "ACGTACGT";
    unsigned char num = 0;
    int idx[4];
    int rc = qzgpu_bwt_encode(t, 8, &num, idx, QZGPU_FEATURE_FASTMODE);
    qzgpu_storage *st = 0;
    qzgpu_storage_create(&st, 1 << 20, 4);
    qzgpu_storage_destroy(st);
    qzgpu_streams_info info;
    qzgpu_fastq_streams(t, 0, 0, 0, 0, 0, 0, 0, &info);
    printf("%d %s\n", rc, qzgpu_error_string(rc));
    return qzgpu_bwt_decode_noalloc(0, 0, 0, 1, 0);
}
"""


def test_c_program_compiles_and_links(lib, tmp_path):
    src = tmp_path / "caller.c"
    src.write_text(C_CALLER)
    exe = tmp_path / "caller"
    libdir = os.path.dirname(native.LIB_PATH)
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-pedantic", "-I", os.path.join(ROOT, "include"),
                        str(src), "-o", str(exe), "-L", libdir, "-lqzgpu", f"-Wl,-rpath,{libdir}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    # the program loads the library (no compute call without an argument)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr



SHIM_CALLER = r"""
/* A libbsc-side caller: it knows only libbsc's BWT-stage names and links
 * against the shim object plus the library, as libbsc would once its own bwt
 * object is left out.  With a block as argument it sorts it and prints the
 * transform and primary index, then inverts it in place. */
#include <stdio.h>
#include <string.h>
#include "qzgpu_bsc_shim.h"

int main(int argc, char **argv) {
    if (argc < 2) return 0; /* linked, not run: no GPU needed */
    unsigned char t[4096];
    int n = (int)strlen(argv[1]);
    if (n > 4096) return 2;
    memcpy(t, argv[1], (size_t)n);
    int idx = bsc_bwt_encode(t, n, NULL, NULL, 1);
    if (idx < 0) return 3;
    printf("%.*s %d\n", n, (const char *)t, idx);
    if (bsc_bwt_decode(t, n, idx, 0, NULL, 1) != 0) return 4;
    printf("%.*s\n", n, (const char *)t);
    return 0;
}
"""


def build_shim_caller(tmp_path):
    build.build()
    src = tmp_path / "bsc_caller.c"
    src.write_text(SHIM_CALLER)
    exe = tmp_path / "bsc_caller"
    libdir = os.path.dirname(native.LIB_PATH)
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-pedantic", "-I", os.path.join(ROOT, "include"),
                        str(src), build.SHIM_OBJ, "-o", str(exe), "-L", libdir, "-lqzgpu", f"-Wl,-rpath,{libdir}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_bsc_shim_exports_libbsc_names_and_links(lib, tmp_path):
    out = subprocess.run(["nm", "--defined-only", build.SHIM_OBJ], capture_output=True, text=True,
                         check=True).stdout
    assert set(re.findall(r"\sT\s+(\w+)", out)) == {"bsc_bwt_encode", "bsc_bwt_decode"}
    exe = build_shim_caller(tmp_path)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
