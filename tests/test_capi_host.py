"""C-ABI library checks that need no GPU: it loads, exports every entry
point the headers declare, and its host-side HEALPix/PolBeam helpers agree
with the oracle and the reference fixtures."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, has_gpu


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            txt = open(os.path.join(inc, f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(pisco_\w+)\s*\(", txt))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    from pisco4cmb_gb300 import _lib

    L = _lib.load()
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    bound = {s[0] for s in _lib.SIGNATURES}
    assert set(names) <= bound, sorted(set(names) - bound)
    assert L.pisco_abi_version() == 1


def test_host_healpix_matches_oracle(oracle_mod):
    from pisco4cmb_gb300 import ang2pix, pix2ang

    rng = np.random.default_rng(3)
    for nside in (1, 4, 64, 1024, 8192):
        pix = rng.integers(0, 12 * nside * nside, 5000)
        th, ph = pix2ang(nside, pix)
        to, po = oracle_mod.pix2ang(nside, pix)
        assert np.array_equal(th, to) and np.array_equal(ph, po)
        t = np.arccos(rng.uniform(-1, 1, 5000))
        p = rng.uniform(0, 2 * np.pi, 5000)
        assert np.array_equal(ang2pix(nside, t, p), oracle_mod.ang2pix(nside, t, p))


def test_polbeam_matches_reference_bit_exact(golden_c1, golden_ellip):
    from pisco4cmb_gb300 import PolBeam, beam_npix_for_radius

    for g, fw, ep in ((golden_c1, (2.0, 2.0, 0.0), 0.01), (golden_ellip, (1.8, 1.4, 30.0), 0.02)):
        nsb = int(g["nside_beam"])
        npb = int(g["npix_beam"])
        b = PolBeam(nsb, npb, ep, "p")
        assert b.get_rho_max() == float(g["rho_max"])
        b.make_unpol_gaussian_elliptical_beams(*fw)
        b.build(int(g["nside_sky"]))
        pa, pb = b.planes()
        assert np.array_equal(pa, g["beam_a"]) and np.array_equal(pb, g["beam_b"])
    assert beam_npix_for_radius(256, np.deg2rad(5.0)) == int(golden_c1["npix_beam"])


def test_argument_errors_are_reported_not_fatal():
    from pisco4cmb_gb300 import PiscoInvalidArgument, PolBeam, _lib, pix2ang

    with pytest.raises(PiscoInvalidArgument):
        pix2ang(0, [0])
    with pytest.raises(PiscoInvalidArgument):
        pix2ang(4, [192])
    with pytest.raises(PiscoInvalidArgument):
        PolBeam(16, 12 * 16 * 16, 0.0, "p")
    with pytest.raises(PiscoInvalidArgument):
        PolBeam(16, 10, 0.0, "x")
    L = _lib.load()
    h = ctypes.c_void_p()
    bad = _lib.RunConfig(nStreams=0)
    assert L.pisco_create(ctypes.byref(bad), ctypes.byref(h)) == _lib.PISCO_ERR_INVALID_CONFIG
    assert b"invalid configuration" in L.pisco_last_error(None)
    assert L.pisco_destroy(None) == _lib.PISCO_ERR_INVALID_ARGUMENT
    assert L.pisco_set_sky(None, 4, None, None, None, None, 0) == _lib.PISCO_ERR_INVALID_ARGUMENT


@pytest.mark.skipif(has_gpu(), reason="checks the no-device path")
def test_create_without_device_reports_cuda_error():
    from pisco4cmb_gb300 import _lib

    L = _lib.load()
    h = ctypes.c_void_p()
    st = L.pisco_create(None, ctypes.byref(h))
    assert st == _lib.PISCO_ERR_CUDA and not h.value
