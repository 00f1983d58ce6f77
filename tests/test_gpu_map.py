"""Binned map-maker (GPU) against the oracle's restatement of SkyMap
(skymap.cpp:68-231), which tests/test_oracle_map.py pins to the reference
SkyMap compiled from its own sources."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _scan(ndet, ns, seed, dtype=np.float32):
    rng = np.random.default_rng(seed)
    ra = rng.uniform(0, 2 * np.pi, (ndet, ns))
    dec = np.arcsin(rng.uniform(-1, 1, (ndet, ns)))
    dec[:, :8] = np.pi / 2 - 1e-3  # near the pole
    pa = rng.uniform(-np.pi, np.pi, (ndet, ns))
    data = rng.normal(size=(ndet, ns))
    pol = np.array([0.0, np.pi / 2, np.pi / 4, 0.3][:ndet], np.float32)
    return [x.astype(dtype) for x in (ra, dec, pa, data)] + [pol]


def _read_normal(m):
    return m.get_normal()


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_map_matches_oracle(gpu, dtype):
    from pisco4cmb_gb300 import SkyMap

    nside = 16
    m = SkyMap(nside)
    ata = atd = None
    for seed in (1, 2):  # two calls: totals carry over
        ra, dec, pa, data, pol = _scan(3, 3000, seed, dtype)
        m.accumulate_data(ra.shape[1], ra, dec, pa, 3, pol, data)
        ata, atd = O.map_accumulate(nside, ra, dec, pa, pol, data, ata, atd)
    m.solve_map()
    g_ata, g_atd = _read_normal(m)
    # CUDA's and the host's cos/sin may differ in the last bit
    assert np.allclose(g_ata, ata, rtol=1e-13, atol=1e-12)
    assert np.allclose(g_atd, atd, rtol=1e-13, atol=1e-11)
    I, Q, U, hits = O.map_solve(ata, atd)
    A = ata.reshape(-1, 3, 3)
    seen = ata[0::9] >= 3
    cond = np.full(A.shape[0], np.inf)
    cond[seen] = np.linalg.cond(A[seen])
    ok = cond < 1e8
    gh = m.get_hitmap()
    assert np.array_equal(gh[ok | ~seen], hits[ok | ~seen])
    for mine, ref in zip((m.get_stokes_I(), m.get_stokes_Q(), m.get_stokes_U()), (I, Q, U)):
        assert np.allclose(mine[ok], ref[ok], rtol=1e-5, atol=1e-5)
    low = (gh > 0) & (gh < 3)
    assert np.any(low) and not np.any(m.get_stokes_I()[low])


def test_map_singular_and_sparse_pixels(gpu):
    """A pixel seen at one angle only (exactly singular: hits 0, AtD kept as
    the values) and a pixel with 2 hits (I = Q = U = 0, hits 2)."""
    from pisco4cmb_gb300 import SkyMap

    nside = 16
    ra = np.array([1.0] * 6 + [4.0] * 2, np.float32)
    dec = np.array([0.2] * 6 + [-0.7] * 2, np.float32)
    pa = np.zeros(8, np.float32)
    data = np.arange(1, 9, dtype=np.float32)
    m = SkyMap(nside)
    m.accumulate_data(8, ra, dec, pa, 1, [0.0], data)
    m.solve_map()
    ata, atd = O.map_accumulate(nside, ra, dec, pa, [0.0], data)
    I, Q, U, hits = O.map_solve(ata, atd)
    th = np.pi / 2 - dec.astype(np.float64)
    p1 = int(O.ang2pix(nside, th[:1], ra[:1].astype(np.float64))[0])
    p2 = int(O.ang2pix(nside, th[6:7], ra[6:7].astype(np.float64))[0])
    gh = m.get_hitmap()
    assert gh[p1] == hits[p1] == 0 and gh[p2] == hits[p2] == 2
    assert m.get_stokes_I()[p1] == I[p1] == np.float32(atd[3 * p1])
    assert m.get_stokes_Q()[p1] == Q[p1] and m.get_stokes_U()[p1] == U[p1]
    assert m.get_stokes_I()[p2] == 0 and m.get_stokes_Q()[p2] == 0
    assert gh.sum() == 2


def test_map_device_entry_equals_host(gpu):
    import torch

    from pisco4cmb_gb300 import SkyMap

    ra, dec, pa, data, pol = _scan(2, 5000, 5)
    a = SkyMap(32)
    a.accumulate_data(5000, ra, dec, pa, 2, pol, data)
    a.solve_map()
    b = SkyMap(32)
    t = [torch.tensor(x, device="cuda") for x in (ra, dec, pa, data)]
    b.accumulate_device(5000, t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr(), 2, pol,
                        t[3].data_ptr())
    b.solve_map()
    for x, y in zip(_read_normal(a), _read_normal(b)):
        assert np.array_equal(x, y)
    assert np.array_equal(a.get_stokes_Q(), b.get_stokes_Q())
    assert np.array_equal(a.get_hitmap(), b.get_hitmap())


def test_map_recovers_a_pixelised_sky(gpu):
    """TOD made from a pixelised sky, d = I + Q cos 2psi + U sin 2psi at the
    sample's pixel, maps back to that sky wherever the angles are spread."""
    from pisco4cmb_gb300 import SkyMap

    nside = 8
    rng = np.random.default_rng(9)
    npix = 12 * nside * nside
    sky = rng.normal(size=(3, npix))
    n = 200_000
    ra = rng.uniform(0, 2 * np.pi, n)
    dec = np.arcsin(rng.uniform(-1, 1, n))
    pa = rng.uniform(-np.pi, np.pi, n)
    pix = O.ang2pix(nside, np.pi / 2 - dec, ra)
    psi = -pa  # detector angle 0
    d = sky[0, pix] + sky[1, pix] * np.cos(2 * psi) + sky[2, pix] * np.sin(2 * psi)
    m = SkyMap(nside)
    m.accumulate_data(n, ra, dec, pa, 1, [0.0], d)
    m.solve_map()
    assert np.all(m.get_hitmap() >= 3)
    for k, got in enumerate((m.get_stokes_I(), m.get_stokes_Q(), m.get_stokes_U())):
        assert np.abs(got - sky[k]).max() < 1e-5


def test_map_rejects_bad_pointing_and_keeps_the_rest(gpu):
    from pisco4cmb_gb300 import PiscoInvalidArgument, SkyMap

    ra, dec, pa, data, pol = _scan(1, 1000, 3)
    dec[0, 10] = np.float32(2.0)  # |dec| > pi/2
    ra[0, 11] = np.float32(np.nan)
    m = SkyMap(16)
    with pytest.raises(PiscoInvalidArgument):
        m.accumulate_data(1000, ra, dec, pa, 1, pol, data)
    keep = np.ones(1000, bool)
    keep[[10, 11]] = False
    ata, atd = O.map_accumulate(16, ra[:, keep], dec[:, keep], pa[:, keep], pol, data[:, keep])
    g_ata, g_atd = _read_normal(m)
    assert np.allclose(g_ata, ata, rtol=1e-13, atol=1e-12)
