"""The oracle's HEALPix restatement, pinned three ways (CPU only):

1. against vectors produced by the reference's own device HEALPix port
   (src/GpuConvolver/cuda/cudaHealpix.cu, compiled for the host by
   oracle/build_ref.sh; fixtures in tests/golden/golden_healpix.npz) with the
   reference test's tolerances (tests/cudaHealpix/test_pix2ang.cu:107-112:
   pix2ang within 1e-10, ang2pix exact);
2. query_disc against its definition (every pixel centre within the radius,
   brute force), which the reference never tested;
3. HEALPix invariants (npix, ring structure, ang2pix(pix2ang(p)) == p).
"""
import numpy as np
import pytest

from conftest import load_golden

NSIDES = (1, 2, 4, 64, 256, 2048, 8192)


@pytest.mark.parametrize("nside", NSIDES)
def test_pix2ang_matches_reference_port(oracle_mod, golden_healpix, nside):
    g = golden_healpix
    th, ph = oracle_mod.pix2ang(nside, g["pix_%d" % nside])
    assert np.max(np.abs(th - g["theta_%d" % nside])) <= 1e-10
    assert np.max(np.abs(ph - g["phi_%d" % nside])) <= 1e-10


@pytest.mark.parametrize("nside", NSIDES)
def test_ang2pix_and_interp_match_reference_port(oracle_mod, golden_healpix, nside):
    g = golden_healpix
    t, p = g["atheta_%d" % nside], g["aphi_%d" % nside]
    assert np.array_equal(oracle_mod.ang2pix(nside, t, p), g["apix_%d" % nside])
    pix, w = oracle_mod.get_interpol(nside, t, p)
    assert np.array_equal(pix, g["ipix_%d" % nside])
    assert np.max(np.abs(w - g["iwgt_%d" % nside])) <= 1e-12


def test_rho_sigma_chi_matches_reference(oracle_mod, golden_healpix):
    rin, rout = golden_healpix["rsc_in"], golden_healpix["rsc_out"]
    rho, sig, chi = oracle_mod.rho_sigma_chi(*rin)
    assert np.array_equal(rho, rout[0]) or np.max(np.abs(rho - rout[0])) <= 1e-12
    assert np.max(np.abs(sig - rout[1])) <= 1e-12
    assert np.max(np.abs(chi - rout[2])) <= 1e-12


@pytest.mark.parametrize("nside", (1, 2, 8, 64, 256, 1024))
def test_roundtrip_exhaustive(oracle_mod, nside):
    pix = np.arange(12 * nside * nside)
    th, ph = oracle_mod.pix2ang(nside, pix)
    assert np.array_equal(oracle_mod.ang2pix(nside, th, ph), pix)
    # HEALPix invariants: equal-area rings, polar-cap centres at z = 1 - i^2/(3 nside^2)
    z = np.cos(th)
    ring1 = pix < 4 if nside > 1 else pix < 4
    np.testing.assert_allclose(z[ring1], 1 - 1.0 / (3 * nside * nside), atol=1e-14)


def _vec(th, ph):
    return np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], -1)


@pytest.mark.parametrize("nside,rdeg", [(16, 40.0), (64, 5.0), (256, 3.0), (1024, 1.0), (8, 120.0)])
def test_query_disc_is_the_brute_force_disc(oracle_mod, nside, rdeg):
    rng = np.random.default_rng(20261203 + nside)
    r = np.deg2rad(rdeg)
    pix = np.arange(12 * nside * nside)
    V = _vec(*oracle_mod.pix2ang(nside, pix))
    ties = 0
    for k in range(60):
        t0 = np.arccos(rng.uniform(-1, 1))
        if k < 6:
            t0 = rng.uniform(0, 1.2 * r)           # pole inside or near the disc
        elif k < 12:
            t0 = np.pi - rng.uniform(0, 1.2 * r)
        p0 = rng.uniform(-np.pi, 3 * np.pi)       # unnormalised phi on purpose
        d = oracle_mod.query_disc(nside, t0, p0, r)
        assert np.all(np.diff(d) > 0)
        dist = np.arccos(np.clip(V @ _vec(t0, p0), -1, 1))
        diff = np.setxor1d(d, pix[dist <= r])
        near = np.abs(dist[diff] - r) < 1e-12
        ties += int(near.sum())
        assert near.all(), "disc differs from the definition away from a tie"
    assert ties <= 2


def test_query_disc_whole_sky(oracle_mod):
    assert np.array_equal(oracle_mod.query_disc(4, 0.3, 0.2, np.pi), np.arange(192))
