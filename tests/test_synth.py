"""Seeded synthetic inputs (CPU): deterministic, finite, the stated shapes."""
import numpy as np

from pisco4cmb_gb300 import synth


def test_grf_sky_seeded_and_normalised():
    a = synth.grf_sky(16, 1, dtype=np.float64)
    b = synth.grf_sky(16, 1, dtype=np.float64)
    assert np.array_equal(a, b)
    assert a.shape == (4, 12 * 16 * 16) and np.all(a[3] == 0)
    np.testing.assert_allclose(a[:3].std(axis=1), [100.0, 10.0, 10.0], rtol=1e-12)
    c = synth.grf_sky(16, 2, dtype=np.float64)
    assert not np.allclose(a, c)


def test_grf_high_m_stays_finite():
    # lambda_mm underflows for m ~ lmax at mid latitudes: scaled recurrence
    m = synth.grf_map(64, 191, [3, 4])
    assert np.isfinite(m).all() and abs(m.std() - 1.0) < 1e-12 and np.abs(m).max() < 10


def test_ring_geometry_matches_healpix(oracle_mod):
    for nside in (1, 4, 32):
        z, n, phi0, start = synth.ring_geometry(nside)
        assert n.sum() == 12 * nside * nside
        th, ph = oracle_mod.pix2ang(nside, start)
        np.testing.assert_allclose(np.cos(th), z, atol=1e-14)
        np.testing.assert_allclose(ph, phi0, atol=1e-14)


def test_scans():
    ra, dec, psi = synth.raster_scan(20000)
    assert ra.size == 20000 and abs(np.rad2deg(dec).min() + 30.0) < 1e-9
    assert np.rad2deg(dec).max() <= 30.0 + 1e-9
    assert set(np.round(np.rad2deg(psi)).astype(int)) == {0, 45, 90, 135}
    ra, dec, psi = synth.sweep_scan(2_000_000, 2)
    assert abs(np.rad2deg(dec).max() - (-80 + 0.05 * 488)) < 1e-9
    assert np.rad2deg(psi).min() >= 0 and np.rad2deg(psi).max() < 180
    ra, dec, psi = synth.pole_heavy_scan(10000, 3)
    near = np.abs(np.abs(dec) - np.pi / 2) <= np.deg2rad(1.0)
    assert abs(near.mean() - 0.1) < 0.01
    fx, fy = synth.elliptical_fwhm(1.5, 0.05)
    assert abs((fx - fy) / (fx + fy) - 0.05) < 1e-12 and abs(np.sqrt(fx * fy) - 1.5) < 1e-12
    dets = synth.c4_detectors()
    assert len(dets) == 48 and all(1.0 <= d["radius_deg"] <= 5.0 for d in dets)
    assert all(1e4 <= d["nsamples"] <= 1e6 for d in dets)
