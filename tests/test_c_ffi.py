"""A plain-C caller of the C ABI (tests/c/ffi_c1.c, the sequence an FFI
binding follows): include/pisco_gb300.h compiles as strict C99 and the
program links against libpisco_gb300.so (CPU); on the GPU it reproduces the
reference Convolver's TOD on the CPU-runnable workload, with sky-order TOD
bit-identical to scan order (checked inside the program), and its map equals
the map-making oracle's on the same TOD."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, rel_max

SRC = os.path.join(ROOT, "tests", "c", "ffi_c1.c")


def compile_ffi(tmp_path):
    from pisco4cmb_gb300 import _lib

    _lib.load()
    exe = str(tmp_path / "ffi_c1")
    libdir = os.path.dirname(_lib.lib_path())
    cmd = ["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-O2",
           "-I", os.path.join(ROOT, "include"), SRC, "-o", exe, "-L", libdir, "-lpisco_gb300",
           "-Wl,-rpath," + libdir, "-lm"]
    subprocess.check_call(cmd)
    return exe


def test_c_header_and_program_compile_and_link(tmp_path):
    assert os.path.exists(compile_ffi(tmp_path))


@pytest.mark.gpu
def test_c_program_matches_reference(gpu, golden_c1, tmp_path):
    import oracle as O

    g = golden_c1
    exe = compile_ffi(tmp_path)
    nside = int(g["nside_sky"])
    n = g["ra"].size
    g["sky"].astype(np.float32).tofile(tmp_path / "sky.f32")
    scan = np.stack([g["ra"], g["dec"], g["pa"]]).astype(np.float32)
    scan.tofile(tmp_path / "scan.f32")
    r = subprocess.run([exe, str(nside), str(n), str(tmp_path / "sky.f32"),
                        str(tmp_path / "scan.f32"), str(tmp_path / "tod.f32"),
                        str(tmp_path / "map.f32")], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    tod = np.fromfile(tmp_path / "tod.f32", np.float32).reshape(2, n)
    assert rel_max(tod[0], g["tod_a"]) < 1e-6
    assert rel_max(tod[1], g["tod_b"]) < 1e-6
    ra, dec, pa = (np.stack([x, x]) for x in scan)
    ata, atd = O.map_accumulate(nside, ra, dec, pa, np.float32([0.0, np.pi / 2]), tod)
    I, Q, U, hits = O.map_solve(ata, atd)
    m = np.fromfile(tmp_path / "map.f32", np.float32).reshape(4, -1)
    A = ata.reshape(-1, 3, 3)
    seen = ata[0::9] >= 3
    cond = np.full(A.shape[0], np.inf)
    cond[seen] = np.linalg.cond(A[seen])
    ok = cond < 1e8
    assert np.array_equal(m[3][ok | ~seen], hits[ok | ~seen].astype(np.float32))
    for k, ref in enumerate((I, Q, U)):
        assert np.allclose(m[k][ok], ref[ok], rtol=1e-5, atol=1e-4)
