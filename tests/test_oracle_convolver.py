"""The oracle's convolution and PolBeam restatements against the reference's
own code (CPU only).

Fixtures (tests/golden/, made by make_golden.py from the reference sources
compiled unmodified against the HEALPix shim): the TOD of the reference
Convolver::exec_convolution and the beams of the reference PolBeam.  When the
reference tree is present (this container), the same checks also run live
against oracle/_ref.
"""
import numpy as np
import pytest

from conftest import rel_max, rel_rms


@pytest.mark.parametrize("case", ["golden_c1", "golden_ellip"])
def test_oracle_f32_matches_reference_convolver(oracle_mod, case, request):
    g = request.getfixturevalue(case)
    sky = g["sky"].astype(np.float32)
    oa, ob = oracle_mod.convolve_f32(g["ra"], g["dec"], g["pa"], int(g["nside_sky"]), sky,
                                     int(g["nside_beam"]), g["beam_a"], g["beam_b"])
    # float per-pair products: only rounding/contraction differences remain
    assert rel_max(oa, g["tod_a"]) < 1e-6
    assert rel_max(ob, g["tod_b"]) < 1e-6


def test_oracle_polbeam_bit_exact(oracle_mod, golden_c1, golden_ellip):
    g = golden_c1
    ba, bb = oracle_mod.gaussian_beams(int(g["nside_beam"]), int(g["npix_beam"]), 2.0, 2.0, 0.0,
                                       0.01, int(g["nside_sky"]))
    assert np.array_equal(ba, g["beam_a"]) and np.array_equal(bb, g["beam_b"])
    assert oracle_mod.beam_rho_max(int(g["nside_beam"]), int(g["npix_beam"])) == float(g["rho_max"])
    g = golden_ellip
    ba, bb = oracle_mod.gaussian_beams(int(g["nside_beam"]), int(g["npix_beam"]), 1.8, 1.4, 30.0,
                                       0.02, int(g["nside_sky"]))
    assert np.array_equal(ba, g["beam_a"]) and np.array_equal(bb, g["beam_b"])


def test_oracle_f64_close_to_reference(oracle_mod, golden_c1):
    g = golden_c1
    da, db = oracle_mod.convolve_f64(g["ra"].astype(np.float64), g["dec"].astype(np.float64),
                                     g["pa"].astype(np.float64), int(g["nside_sky"]),
                                     g["sky"].astype(np.float32).astype(np.float64),
                                     int(g["nside_beam"]), g["beam_a"], g["beam_b"])
    # all-double arithmetic vs the reference's float products: ~1e-7 of rms
    assert rel_rms(da, g["tod_a"]) < 1e-6
    assert rel_rms(db, g["tod_b"]) < 1e-6


def test_oracle_live_against_ref_build(oracle_mod, golden_ellip):
    if not oracle_mod.ref_available():
        pytest.skip("oracle/_ref not built (reference tree absent)")
    g = golden_ellip
    sky = g["sky"].astype(np.float32)
    qa, qb = oracle_mod.ref_convolve(g["ra"], g["dec"], g["pa"], int(g["nside_sky"]), sky,
                                     int(g["nside_beam"]), g["beam_a"], g["beam_b"])
    # (a bad polFlag is not probed here: the reference throws it from inside
    # its OpenMP loop, convolver.cpp:38-70, which terminates the process)
    assert np.array_equal(qa, g["tod_a"]) and np.array_equal(qb, g["tod_b"])


def test_oracle_adjoint_is_transpose(oracle_mod):
    """<A x, y> == <x, A^T y> for the double forward and its adjoint."""
    rng = np.random.default_rng(5)
    ns, nb = 16, 64
    npb = oracle_mod.beam_npix_for_radius(nb, np.deg2rad(8.0))
    ba = rng.normal(size=(4, npb))
    bb = rng.normal(size=(4, npb))
    n = 300
    ra, dec, pa = rng.uniform(0, 6.28, n), np.arcsin(rng.uniform(-1, 1, n)), rng.uniform(0, 3, n)
    x = rng.normal(size=(4, 12 * ns * ns))
    ya, yb = rng.normal(size=n), rng.normal(size=n)
    fa, fb = oracle_mod.convolve_f64(ra, dec, pa, ns, x, nb, ba, bb)
    g = oracle_mod.adjoint_f64(ra, dec, pa, ns, nb, ba, bb, ya, yb)
    lhs = fa @ ya + fb @ yb
    rhs = float(np.sum(x * g))
    assert abs(lhs - rhs) <= 1e-10 * abs(lhs)
