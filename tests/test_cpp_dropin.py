"""The C++ drop-in headers: a reference-style caller compiles against
include/pisco unchanged (CPU), and on the GPU reproduces the reference
Convolver's TOD on the CPU-runnable workload."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, rel_max

SRC = os.path.join(ROOT, "tests", "cpp", "dropin_c1.cpp")


def compile_dropin(tmp_path):
    from pisco4cmb_gb300 import _lib

    _lib.load()
    exe = str(tmp_path / "dropin_c1")
    libdir = os.path.dirname(_lib.lib_path())
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include", "pisco"), SRC, "-o", exe,
           "-L", libdir, "-lpisco_gb300", "-Wl,-rpath," + libdir]
    subprocess.check_call(cmd)
    return exe


def test_dropin_headers_compile_and_link(tmp_path):
    assert os.path.exists(compile_dropin(tmp_path))


@pytest.mark.gpu
def test_dropin_program_matches_reference(gpu, golden_c1, tmp_path):
    g = golden_c1
    exe = compile_dropin(tmp_path)
    sky = g["sky"].astype(np.float32)
    scan = np.stack([g["ra"], g["dec"], g["pa"]]).astype(np.float32)
    sky.tofile(tmp_path / "sky.f32")
    scan.tofile(tmp_path / "scan.f32")
    n = g["ra"].size
    r = subprocess.run([exe, str(int(g["nside_sky"])), str(n), str(tmp_path / "sky.f32"),
                        str(tmp_path / "scan.f32"), str(tmp_path / "g.f32"), str(tmp_path / "c.f32"),
                        str(tmp_path / "m.f32")],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    for f in ("g.f32", "c.f32"):
        out = np.fromfile(tmp_path / f, np.float32).reshape(2, n)
        assert rel_max(out[0], g["tod_a"]) < 1e-6
        assert rel_max(out[1], g["tod_b"]) < 1e-6
    # SkyMap on the GPU TOD against the map-making oracle on the same TOD
    import oracle as O

    tod = np.fromfile(tmp_path / "g.f32", np.float32).reshape(2, n)
    nside = int(g["nside_sky"])
    ra, dec, pa = (np.stack([x, x]) for x in scan)
    ata, atd = O.map_accumulate(nside, ra, dec, pa, np.float32([0.0, np.pi / 2]), tod)
    I, Q, U, hits = O.map_solve(ata, atd)
    m = np.fromfile(tmp_path / "m.f32", np.float32).reshape(4, -1)
    A = ata.reshape(-1, 3, 3)
    seen = ata[0::9] >= 3
    cond = np.full(A.shape[0], np.inf)
    cond[seen] = np.linalg.cond(A[seen])
    ok = cond < 1e8
    assert np.array_equal(m[3][ok | ~seen], hits[ok | ~seen].astype(np.float32))
    for k, ref in enumerate((I, Q, U)):
        assert np.allclose(m[k][ok], ref[ok], rtol=1e-5, atol=1e-4)
