"""Pins of the map-making oracle (CPU): the dgesv restatement against LAPACK
(scipy), and accumulate + solve against the reference SkyMap compiled from
its own sources (oracle/_ref)."""
import numpy as np
import pytest

import oracle as O


def _scan(nside, ndet, ns, seed, pole=True):
    rng = np.random.default_rng(seed)
    ra = rng.uniform(0, 2 * np.pi, (ndet, ns)).astype(np.float32)
    dec = np.arcsin(rng.uniform(-1, 1, (ndet, ns))).astype(np.float32)
    if pole:
        dec[:, :10] = np.float32(np.pi / 2 - 1e-3)
    pa = rng.uniform(-np.pi, np.pi, (ndet, ns)).astype(np.float32)
    data = rng.normal(size=(ndet, ns)).astype(np.float32)
    pol = np.array([0.0, np.pi / 2, np.pi / 4, 0.3][:ndet], np.float32)
    return ra, dec, pa, pol, data


def test_dgesv3_matches_lapack():
    lapack = pytest.importorskip("scipy.linalg.lapack")
    rng = np.random.default_rng(0)
    cases = [rng.normal(size=(3, 3)) for _ in range(300)]
    cases += [np.diag([1.0, 1e-9, 1e9]) + 1e-3 * rng.normal(size=(3, 3)) for _ in range(50)]
    # a normal-equations matrix of a few polarisation angles (the map-maker's case)
    for _ in range(100):
        k = int(rng.integers(3, 9))
        ang = rng.uniform(0, np.pi, k)
        v = np.stack([np.ones(k), np.cos(2 * ang), np.sin(2 * ang)])
        cases.append(v @ v.T)
    for a in cases:
        b = rng.normal(size=3)
        info, x, _, _ = O.dgesv3(a, b)
        _, _, xs, infos = lapack.dgesv(a, b)
        assert info == infos
        if info == 0:
            cond = np.linalg.cond(a)
            assert np.allclose(x, xs, rtol=1e-12 * max(cond, 1.0), atol=0), (a, x, xs)
    # exactly singular: info reports the first zero pivot; b is left unchanged
    a = np.array([[2.0, 2.0, 0.0], [2.0, 2.0, 0.0], [0.0, 0.0, 0.0]])
    b = np.array([1.0, 2.0, 3.0])
    info, x, _, _ = O.dgesv3(a, b)
    _, _, xs, infos = lapack.dgesv(a, b)
    assert info == infos == 2 and np.array_equal(x, b)


@pytest.mark.parametrize("exact", [True, False])
def test_map_matches_reference_skymap(exact):
    if not O.refmap_available():
        pytest.skip("oracle/_ref not built (reference tree absent)")
    nside = 16
    ra, dec, pa, pol, data = _scan(nside, 3, 4000, 1)
    # a pixel seen at one angle only (exactly singular), and pixels with < 3 hits
    ra[0, :5] = np.float32(1.0)
    dec[0, :5] = np.float32(0.2)
    pa[0, :5] = np.float32(0.0)
    pol[0] = 0.0
    ref = O.ref_skymap(nside, ra, dec, pa, pol, data, ncalls=2, exact=exact)
    ata, atd = O.map_accumulate(nside, ra, dec, pa, pol, data)
    ata, atd = O.map_accumulate(nside, ra, dec, pa, pol, data, ata, atd)
    mine = (ata, atd) + O.map_solve(ata, atd)
    if exact:
        for r, m in zip(ref, mine):
            assert np.array_equal(r, m)
    else:
        # The reference's flags let the compiler contract a*b+c into an FMA,
        # so sums differ in the last bits; where the normal matrix is
        # (numerically) singular -- the data are accumulated twice, so some
        # pixels hold two distinct angles only -- whether the last pivot is
        # exactly zero is decided by that rounding.  Compare the rest.
        assert np.allclose(ref[0], mine[0], rtol=1e-13, atol=1e-13)
        assert np.allclose(ref[1], mine[1], rtol=1e-13, atol=1e-12)
        A = ref[0].reshape(-1, 3, 3)
        seen = ref[0][0::9] >= 3
        cond = np.full(A.shape[0], np.inf)
        cond[seen] = np.linalg.cond(A[seen])
        ok = cond < 1e8
        assert np.array_equal(ref[5][ok | ~seen], mine[5][ok | ~seen])
        for k in (2, 3, 4):
            assert np.allclose(ref[k][ok], mine[k][ok], rtol=1e-5, atol=1e-5)
    hits = mine[5]
    assert np.any(hits == 0) and np.any((hits > 0) & (hits < 3))
    low = (hits > 0) & (hits < 3)
    assert not np.any(mine[2][low]) and not np.any(mine[3][low])
