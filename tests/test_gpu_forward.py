"""Parity of the CUDA forward forms, called through the C ABI (GPU).

Tolerances (relative to the TOD rms):
* PLAIN vs the reference Convolver (golden fixtures, float API): max 1e-6 --
  same float per-pair products, only rounding/contraction order differs.
* FP64 vs the oracle's all-double form on the same inputs: max 1e-12.
* TUNED vs FP64 on the same float inputs: rms 1e-6 (the target), and every
  beam-pixel decision identical (tested through the TOD at 1e-6 max).
"""
import numpy as np
import pytest

from conftest import rel_max, rel_rms

pytestmark = pytest.mark.gpu


def make_conv(g, form="plain", sky64=False, beam64=False, ptg64=False, cfg=None):
    from pisco4cmb_gb300 import GPUConvolver, RunConfig, Scan, Sky

    c = GPUConvolver(cfg or RunConfig(), form=form)
    sky = g["sky"] if sky64 else g["sky"].astype(np.float32)
    c.update_sky(Sky(int(g["nside_sky"]), sky[0], sky[1], sky[2], None))
    a = [g["beam_a"][k].astype(np.float64 if beam64 else np.float32) for k in range(4)]
    b = [g["beam_b"][k].astype(np.float64 if beam64 else np.float32) for k in range(4)]
    c.set_beam_planes(int(g["nside_beam"]), int(g["npix_beam"]), a, b)
    dt = np.float64 if ptg64 else np.float32
    n = g["ra"].size
    c.update_scan(Scan(n, g["ra"].astype(dt), g["dec"].astype(dt), g["pa"].astype(dt)))
    return c


def run(c, n, dtype=np.float32, form=None, polflag="p"):
    a = np.full(n, np.nan, dtype)
    b = np.full(n, np.nan, dtype)
    c.exec_convolution(a, b, polFlag=polflag, form=form)
    return a, b


@pytest.mark.parametrize("case", ["golden_c1", "golden_ellip"])
def test_plain_matches_reference_convolver(gpu, case, request):
    g = request.getfixturevalue(case)
    c = make_conv(g)
    a, b = run(c, g["ra"].size)
    assert rel_max(a, g["tod_a"]) < 1e-6
    assert rel_max(b, g["tod_b"]) < 1e-6


@pytest.mark.parametrize("case", ["golden_c1", "golden_ellip"])
def test_fp64_matches_double_oracle(gpu, oracle_mod, case, request):
    g = request.getfixturevalue(case)
    c = make_conv(g, form="fp64", sky64=True, beam64=True, ptg64=True)
    a, b = run(c, g["ra"].size, np.float64)
    oa, ob = oracle_mod.convolve_f64(g["ra"].astype(np.float64), g["dec"].astype(np.float64),
                                     g["pa"].astype(np.float64), int(g["nside_sky"]), g["sky"],
                                     int(g["nside_beam"]), g["beam_a"].astype(np.float64),
                                     g["beam_b"].astype(np.float64))
    assert rel_max(a, oa) < 1e-12
    assert rel_max(b, ob) < 1e-12


@pytest.mark.parametrize("case", ["golden_c1", "golden_ellip"])
def test_tuned_matches_fp64(gpu, case, request):
    g = request.getfixturevalue(case)
    ref = make_conv(g, form="fp64", ptg64=True)
    ra, rb = run(ref, g["ra"].size, np.float64)
    c = make_conv(g, form="tuned", ptg64=True)
    a, b = run(c, g["ra"].size, np.float64)
    assert rel_rms(a, ra) < 1e-6 and rel_rms(b, rb) < 1e-6
    assert rel_max(a, ra) < 1e-6 and rel_max(b, rb) < 1e-6


@pytest.mark.parametrize("case", ["golden_c1", "golden_ellip"])
def test_tuned_decisions_within_margin(gpu, case, request):
    """Worst FP32 decision error of TUNED, as a fraction of its FP64 margin."""
    g = request.getfixturevalue(case)
    c = make_conv(g, form="tuned", ptg64=True)
    worst, tuned_pairs = c.tuned_calibrate(with_pairs=True)
    assert 0.0 <= worst < 0.5, worst
    # the TUNED disc (FP32 edge angle, FP64 re-check) is HEALPix query_disc's exactly
    assert tuned_pairs == c.count_pairs()
    a, b = run(c, g["ra"].size)
    nf = c.last_fallbacks()
    assert 0 <= nf < 0.02 * c.count_pairs()


def test_tuned_disc_exact_on_random_pointings(gpu, oracle_mod):
    """Pair counts of the TUNED disc equal the exact disc on random and
    pole-grazing pointings, for several sky/beam resolutions."""
    from pisco4cmb_gb300 import GPUConvolver, PolBeam, Scan, Sky

    rng = np.random.default_rng(77)
    for nss, nsb, rdeg in ((16, 64, 9.0), (128, 512, 2.5), (512, 1024, 1.3), (2048, 4096, 0.6)):
        npb = oracle_mod.beam_npix_for_radius(nsb, np.deg2rad(rdeg))
        beam = PolBeam(nsb, npb, 0.0, "p")
        beam.make_unpol_gaussian_elliptical_beams(rdeg / 2, rdeg / 2, 0.0)
        beam.build(nss)
        n = 4000
        ra = rng.uniform(-1, 7, n)
        dec = np.arcsin(rng.uniform(-1, 1, n))
        dec[:400] = np.pi / 2 - rng.uniform(0, 1.5 * np.deg2rad(rdeg), 400)
        dec[400:800] = -np.pi / 2 + rng.uniform(0, 1.5 * np.deg2rad(rdeg), 400)
        c = GPUConvolver(form="tuned")
        c.update_sky(Sky(nss, *np.zeros((3, 12 * nss * nss), np.float32), None))
        c.update_beam(beam)
        c.update_scan(Scan(n, ra, dec, rng.uniform(0, 3, n)))
        worst, tp = c.tuned_calibrate(with_pairs=True)
        assert tp == c.count_pairs() and worst < 0.5


def test_tuned_unnormalised_pointing(gpu, oracle_mod):
    """dec beyond +-90 deg and ra outside [0, 2pi): the reference chain takes
    them as given; TUNED must agree with the FP64 form on the same inputs."""
    from pisco4cmb_gb300 import GPUConvolver, PolBeam, Scan, Sky

    rng = np.random.default_rng(13)
    nss, nsb = 64, 256
    npb = oracle_mod.beam_npix_for_radius(nsb, np.deg2rad(5.0))
    beam = PolBeam(nsb, npb, 0.01, "p")
    beam.make_unpol_gaussian_elliptical_beams(2.0, 1.6, 40.0)
    beam.build(nss)
    n = 3000
    ra = rng.uniform(-20, 20, n)
    dec = rng.uniform(-2.5, 2.5, n)
    pa = rng.uniform(-30, 30, n)
    sky = rng.normal(size=(3, 12 * nss * nss)).astype(np.float32)
    outs = {}
    for form in ("tuned", "fp64"):
        c = GPUConvolver(form=form)
        c.update_sky(Sky(nss, *sky, None))
        c.update_beam(beam)
        c.update_scan(Scan(n, ra, dec, pa))
        a = np.zeros(n)
        b = np.zeros(n)
        c.exec_convolution(a, b)
        outs[form] = (a, b)
    assert rel_max(outs["tuned"][0], outs["fp64"][0]) < 1e-6
    assert rel_max(outs["tuned"][1], outs["fp64"][1]) < 1e-6


def test_nonfinite_pointing_gives_nan(gpu, golden_c1):
    from pisco4cmb_gb300 import Scan

    g = golden_c1
    for form in ("plain", "tuned", "fp64"):
        c = make_conv(g, form=form)
        ra = g["ra"][:64].astype(np.float64).copy()
        ra[5] = np.nan
        dec = g["dec"][:64].astype(np.float64).copy()
        dec[9] = np.inf
        c.update_scan(Scan(64, ra, dec, g["pa"][:64].astype(np.float64)))
        a, b = run(c, 64)
        assert np.isnan(a[5]) and np.isnan(a[9]) and np.isnan(b[5])
        assert np.isfinite(np.delete(a, [5, 9])).all()


def test_bilinear_matches_oracle(gpu, oracle_mod, golden_ellip):
    g = golden_ellip
    c = make_conv(g, form="fp64", sky64=True, beam64=True, ptg64=True)
    c.set_interp(True)
    a, b = run(c, g["ra"].size, np.float64)
    oa, ob = oracle_mod.convolve_f64(g["ra"].astype(np.float64), g["dec"].astype(np.float64),
                                     g["pa"].astype(np.float64), int(g["nside_sky"]), g["sky"],
                                     int(g["nside_beam"]), g["beam_a"].astype(np.float64),
                                     g["beam_b"].astype(np.float64), interp=1)
    # bilinear weights use the ring colatitudes (acos/atan2); the CUDA and host
    # libm results differ by an ulp and the ring spacing (~1e-2 rad) scales
    # that to ~1e-14 in the weights, hence 1e-10 rather than 1e-12
    assert rel_max(a, oa) < 1e-10 and rel_max(b, ob) < 1e-10
    c2 = make_conv(g, form="plain")
    c2.set_interp(True)
    pa_, pb_ = run(c2, g["ra"].size)
    fa, fb = oracle_mod.convolve_f32(g["ra"], g["dec"], g["pa"], int(g["nside_sky"]),
                                     g["sky"].astype(np.float32), int(g["nside_beam"]),
                                     g["beam_a"], g["beam_b"], interp=1)
    assert rel_max(pa_, fa) < 1e-6 and rel_max(pb_, fb) < 1e-6


@pytest.mark.parametrize("case", ["golden_c1", "golden_ellip"])
def test_tuned_bilinear_matches_plain(gpu, oracle_mod, case, request):
    """TUNED with the bilinear lookup builds get_interpol's stencil in FP32
    (continuous weights: no FP64 re-evaluation except at the boresight).
    Against PLAIN's FP64 stencil and the FP64 oracle: the FP32 errors of r and
    sigma (~1e-7 relative) move the weights by ~1e-5 at most, times the beam's
    change over one pixel, so 1e-6 (rms) and 1e-5 (max) of the TOD rms."""
    g = request.getfixturevalue(case)
    n = g["ra"].size
    c = make_conv(g, form="tuned", ptg64=True)
    c.set_interp(True)
    a, b = run(c, n, np.float64)
    p = make_conv(g, form="plain", ptg64=True)
    p.set_interp(True)
    pa_, pb_ = run(p, n, np.float64)
    oa, ob = oracle_mod.convolve_f64(g["ra"].astype(np.float64), g["dec"].astype(np.float64),
                                     g["pa"].astype(np.float64), int(g["nside_sky"]),
                                     g["sky"].astype(np.float32).astype(np.float64),
                                     int(g["nside_beam"]), g["beam_a"].astype(np.float64),
                                     g["beam_b"].astype(np.float64), interp=1)
    rms = float(np.sqrt(np.mean(oa ** 2)))
    for mine, ref in ((a, pa_), (b, pb_), (a, oa), (b, ob)):
        d = mine - ref
        assert np.sqrt(np.mean(d ** 2)) <= 1e-6 * rms
        assert np.abs(d).max() <= 1e-5 * rms
    # the nearest lookup is unchanged by switching back
    c.set_interp(False)
    na, _ = run(c, n, np.float64)
    q = make_conv(g, form="tuned", ptg64=True)
    qa, _ = run(q, n, np.float64)
    assert np.array_equal(na, qa)


def test_polflag_tail_and_determinism(gpu, golden_c1):
    from pisco4cmb_gb300 import PiscoInvalidArgument, RunConfig

    g = golden_c1
    n = g["ra"].size
    # ptgPerConv that does not divide n: the reference drops the tail; here
    # every sample is computed
    c = make_conv(g, cfg=RunConfig(ptgPerConv=7777))
    a1, b1 = run(c, n)
    assert np.all(np.isfinite(a1)) and np.all(np.isfinite(b1))
    a2, b2 = run(c, n)
    assert np.array_equal(a1, a2) and np.array_equal(b1, b2)  # deterministic
    a = np.full(n, np.nan, np.float32)
    c.exec_convolution(a, None, polFlag="a")
    assert np.array_equal(a, a1)
    b = np.full(n, np.nan, np.float32)
    c.exec_convolution(None, b, polFlag="b")
    assert np.array_equal(b, b1)
    with pytest.raises(PiscoInvalidArgument):
        c.exec_convolution(a, b, polFlag="x")


def test_convolver_dropin_api(gpu, golden_c1):
    from pisco4cmb_gb300 import Convolver, PolBeam, PiscoInvalidArgument, Scan, Sky

    g = golden_c1
    sky = g["sky"].astype(np.float32)
    beam = PolBeam(int(g["nside_beam"]), int(g["npix_beam"]), 0.01, "p")
    beam.make_unpol_gaussian_elliptical_beams(2.0, 2.0, 0.0)
    beam.build(int(g["nside_sky"]))
    n = g["ra"].size
    conv = Convolver(Scan(n, g["ra"], g["dec"], g["pa"]),
                     Sky(int(g["nside_sky"]), sky[0], sky[1], sky[2], np.zeros_like(sky[0])), beam)
    a = np.zeros(n, np.float32)
    b = np.zeros(n, np.float32)
    conv.exec_convolution("p", a, b)
    assert rel_max(a, g["tod_a"]) < 1e-6 and rel_max(b, g["tod_b"]) < 1e-6
    with pytest.raises(PiscoInvalidArgument):
        conv.exec_convolution("q", a, b)


def test_pair_count_and_empty_scan(gpu, oracle_mod, golden_ellip):
    from pisco4cmb_gb300 import Scan

    g = golden_ellip
    c = make_conv(g)
    want = sum(oracle_mod.query_disc(int(g["nside_sky"]), np.pi / 2 - float(np.float64(d)),
                                     float(np.float64(r)), float(g["rho_max"])).size
               for r, d in zip(g["ra"], g["dec"]))
    assert c.count_pairs() == want
    c.update_scan(Scan(0, np.zeros(0, np.float32), np.zeros(0, np.float32), np.zeros(0, np.float32)))
    a = np.zeros(0, np.float32)
    c.exec_convolution(a, a.copy())
    c.sync()


def test_edge_pointings(gpu, oracle_mod):
    """Poles, ra wrap, negative ra, tiny and whole-ring discs, nside 1 sky."""
    from pisco4cmb_gb300 import GPUConvolver, PolBeam, Scan, Sky

    rng = np.random.default_rng(9)
    for nss, nsb, rdeg in ((1, 64, 10.0), (8, 128, 20.0), (64, 512, 2.0)):
        npix = 12 * nss * nss
        sky = rng.normal(size=(3, npix))
        beam = PolBeam(nsb, oracle_mod.beam_npix_for_radius(nsb, np.deg2rad(rdeg)), 0.0, "p")
        beam.make_unpol_gaussian_elliptical_beams(rdeg / 2, rdeg / 3, 10.0)
        beam.build(nss)
        ra = np.array([0.0, 2 * np.pi - 1e-9, -0.3, 7.0, 1.0, 2.0, 3.0, 0.5])
        dec = np.array([np.pi / 2, -np.pi / 2, 0.1, -0.2, np.pi / 2 - 1e-7, -np.pi / 2 + 1e-4,
                        0.0, 1.0])
        pa = rng.uniform(-3, 3, ra.size)
        c = GPUConvolver(form="fp64")
        c.update_sky(Sky(nss, *sky, None))
        c.update_beam(beam)
        c.update_scan(Scan(ra.size, ra, dec, pa))
        a = np.zeros(ra.size)
        b = np.zeros(ra.size)
        c.exec_convolution(a, b)
        pa_, pb_ = beam.planes()
        oa, ob = oracle_mod.convolve_f64(ra, dec, pa, nss, sky, nsb, pa_.astype(np.float64),
                                         pb_.astype(np.float64))
        np.testing.assert_allclose(a, oa, rtol=0, atol=1e-12 * max(1.0, np.abs(oa).max()))
        np.testing.assert_allclose(b, ob, rtol=0, atol=1e-12 * max(1.0, np.abs(ob).max()))


def test_largest_sky_and_beam(gpu, oracle_mod):
    """nside 8192 sky (805M pixels, the ring table at its largest) and an
    nside 8192 beam: the TUNED disc equals the exact one, TUNED agrees with
    the FP64 form, and per-sample disc sizes match the oracle's query_disc."""
    import torch

    from pisco4cmb_gb300 import GPUConvolver, PolBeam

    nss = nsb = 8192
    npix = 12 * nss * nss
    g = torch.Generator(device="cuda").manual_seed(5)
    sky = torch.randn((npix, 4), generator=g, device="cuda", dtype=torch.float32)
    sky[:, 3] = 0.0
    rdeg = 0.1
    npb = oracle_mod.beam_npix_for_radius(nsb, np.deg2rad(rdeg))
    beam = PolBeam(nsb, npb, 0.01, "p")
    beam.make_unpol_gaussian_elliptical_beams(0.04, 0.035, 30.0)
    beam.build(nss)
    rng = np.random.default_rng(31)
    n = 400
    ra = rng.uniform(0, 2 * np.pi, n)
    dec = np.arcsin(rng.uniform(-1, 1, n))
    dec[:20] = np.pi / 2 - rng.uniform(0, 0.004, 20)
    dec[20:40] = -np.pi / 2 + rng.uniform(0, 0.004, 20)
    pa = rng.uniform(0, np.pi, n)
    t = [torch.tensor(x, device="cuda") for x in (ra, dec, pa)]
    outs = {}
    for form in ("tuned", "fp64"):
        c = GPUConvolver(form=form)
        c.set_sky_device(nss, sky.data_ptr(), False)
        c.update_beam(beam)
        c.set_scan_device(n, *[x.data_ptr() for x in t])
        o = [torch.empty(n, dtype=torch.float64, device="cuda") for _ in range(2)]
        c.forward_device(o[0].data_ptr(), o[1].data_ptr(), out_f64=True)
        c.sync()
        outs[form] = [x.cpu().numpy() for x in o]
        if form == "tuned":
            worst, tp = c.tuned_calibrate(with_pairs=True)
            pairs = c.count_pairs()
            assert tp == pairs and worst < 0.5
        c.close()
    rho = oracle_mod.beam_rho_max(nsb, npb)
    ref_pairs = sum(oracle_mod.query_disc(nss, np.pi / 2 - d, r, rho).size for r, d in zip(ra, dec))
    assert pairs == ref_pairs
    for k in range(2):
        assert rel_max(outs["tuned"][k], outs["fp64"][k]) < 1e-6


def test_random_configuration_sweep(gpu, oracle_mod):
    """Seeded sweep of sky nside, beam nside, radius, ellipticity and
    pointings (a tenth within the beam radius of either pole): TUNED against
    the FP64 form with each lookup (nearest: rms error 1e-6 of the TOD rms and
    max error 1e-6 of the largest TOD value, every decision within its margin
    and the disc exactly HEALPix's; bilinear: 1e-5), PLAIN against FP64 (1e-6).
    Discs hold a few sky pixels at least (radius >= 1.5 sky pixels): with
    mostly empty discs the TOD is mostly zero and an error relative to its
    rms says little."""
    from pisco4cmb_gb300 import GPUConvolver, PolBeam, Scan, Sky, synth

    rng = np.random.default_rng(20261203)
    for _ in range(24):
        nss = int(2 ** rng.integers(4, 11))            # 16 .. 1024
        nsb = int(2 ** rng.integers(7, 12))            # 128 .. 2048
        pix_deg = np.rad2deg(np.sqrt(4 * np.pi / (12 * nss * nss)))
        rdeg = float(rng.uniform(max(0.3, 1.5 * pix_deg), max(6.0, 3.0 * pix_deg)))
        while not (nsb * np.sqrt(3 * (1 - np.cos(np.deg2rad(rdeg)))) + 2 < nsb):
            nsb *= 2
        npb = oracle_mod.beam_npix_for_radius(nsb, np.deg2rad(rdeg))
        beam = PolBeam(nsb, npb, float(rng.uniform(0, 0.05)), "p")
        fx, fy = synth.elliptical_fwhm(rdeg / 2.5, float(rng.uniform(-0.1, 0.1)))
        beam.make_unpol_gaussian_elliptical_beams(fx, fy, float(rng.uniform(0, 180)))
        beam.build(nss)
        n = 1500
        ra = rng.uniform(0, 2 * np.pi, n)
        dec = np.arcsin(rng.uniform(-1, 1, n))
        k = n // 20
        dec[:k] = np.pi / 2 - rng.uniform(0, np.deg2rad(rdeg), k)
        dec[k:2 * k] = -np.pi / 2 + rng.uniform(0, np.deg2rad(rdeg), k)
        pa = rng.uniform(-np.pi, np.pi, n)
        sky = rng.normal(size=(3, 12 * nss * nss)).astype(np.float32)
        out = {}
        for form, interp in (("fp64", False), ("tuned", False), ("plain", False),
                             ("fp64", True), ("tuned", True)):
            c = GPUConvolver(form=form)
            c.update_sky(Sky(nss, *sky, None))
            c.update_beam(beam)
            c.set_interp(interp)
            c.update_scan(Scan(n, ra, dec, pa))
            a = np.zeros(n)
            b = np.zeros(n)
            c.exec_convolution(a, b)
            out[form, interp] = (a, b)
            if form == "tuned" and not interp:
                worst, tp = c.tuned_calibrate(with_pairs=True)
                assert tp == c.count_pairs() and worst < 0.5, (nss, nsb, rdeg, worst)
            c.close()
        case = (nss, nsb, round(rdeg, 3))

        def close(x, ref, tol):
            d = x - ref
            return (np.sqrt(np.mean(d ** 2)) <= tol * np.sqrt(np.mean(ref ** 2))
                    and np.abs(d).max() <= tol * np.abs(ref).max())

        for x in range(2):
            assert close(out["tuned", False][x], out["fp64", False][x], 1e-6), case
            assert close(out["plain", False][x], out["fp64", False][x], 1e-6), case
            assert close(out["tuned", True][x], out["fp64", True][x], 1e-5), case


def test_wide_fine_beam_both_lookups(gpu, oracle_mod):
    """Beam nside 8192 out to 5 deg (1,533,000 pixels; polar-cap rings up to
    ~1,240, where the FP32 stencil's longitude weights carry ~1e-4 absolute
    error): TUNED against the FP64 form with each lookup, nearest at the TUNED
    tolerance (1e-6), bilinear at 1e-5 (rms and max, relative to the TOD)."""
    from pisco4cmb_gb300 import GPUConvolver, PolBeam, Scan, Sky

    nss, nsb, rdeg = 256, 8192, 5.0
    npb = oracle_mod.beam_npix_for_radius(nsb, np.deg2rad(rdeg))
    beam = PolBeam(nsb, npb, 0.01, "p")
    beam.make_unpol_gaussian_elliptical_beams(2.2, 1.8, 35.0)
    beam.build(nss)
    rng = np.random.default_rng(41)
    n = 1000
    ra = rng.uniform(0, 2 * np.pi, n)
    dec = np.arcsin(rng.uniform(-1, 1, n))
    dec[:50] = np.pi / 2 - rng.uniform(0, np.deg2rad(rdeg), 50)
    pa = rng.uniform(0, np.pi, n)
    sky = rng.normal(size=(3, 12 * nss * nss)).astype(np.float32)
    out = {}
    for form in ("tuned", "fp64"):
        for interp in (False, True):
            c = GPUConvolver(form=form)
            c.update_sky(Sky(nss, *sky, None))
            c.update_beam(beam)
            c.set_interp(interp)
            c.update_scan(Scan(n, ra, dec, pa))
            a = np.zeros(n)
            b = np.zeros(n)
            c.exec_convolution(a, b)
            out[form, interp] = (a, b)
            c.close()
    for interp, tol in ((False, 1e-6), (True, 1e-5)):
        for x in range(2):
            ref = out["fp64", interp][x]
            d = out["tuned", interp][x] - ref
            rms = np.sqrt(np.mean(ref ** 2))
            assert np.sqrt(np.mean(d ** 2)) <= tol * rms, (interp, np.sqrt(np.mean(d ** 2)) / rms)
            assert np.abs(d).max() <= tol * np.abs(ref).max(), (interp, np.abs(d).max() / rms)


def test_exact_and_near_pole_pointings(gpu, oracle_mod):
    """Boresights exactly at the poles, one ulp on either side of them (the
    frame flip of the TUNED geometry is decided there), and at dec = +-pi/2
    given in float32: TUNED against the FP64 form with each lookup, and the
    nearest lookup's disc exactly HEALPix's."""
    from pisco4cmb_gb300 import GPUConvolver, PolBeam, Scan, Sky

    nss, nsb = 128, 512
    npb = oracle_mod.beam_npix_for_radius(nsb, np.deg2rad(3.0))
    beam = PolBeam(nsb, npb, 0.01, "p")
    beam.make_unpol_gaussian_elliptical_beams(1.3, 1.1, 15.0)
    beam.build(nss)
    hp = np.pi / 2
    decs = [hp, -hp, np.nextafter(hp, 0), np.nextafter(-hp, 0), np.nextafter(hp, 4),
            np.nextafter(-hp, -4), float(np.float32(hp)), float(np.float32(-hp)),
            hp - 1e-9, -hp + 1e-9]
    ras = [0.0, 1.0, np.pi, 5.5, 2 * np.pi, -0.3]
    ra = np.array([r for r in ras for _ in decs])
    dec = np.array([d for _ in ras for d in decs])
    pa = np.linspace(0, 2 * np.pi, ra.size)
    n = ra.size
    sky = np.random.default_rng(3).normal(size=(3, 12 * nss * nss)).astype(np.float32)
    out = {}
    for form in ("tuned", "fp64"):
        for interp in (False, True):
            c = GPUConvolver(form=form)
            c.update_sky(Sky(nss, *sky, None))
            c.update_beam(beam)
            c.set_interp(interp)
            c.update_scan(Scan(n, ra, dec, pa))
            a = np.zeros(n)
            b = np.zeros(n)
            c.exec_convolution(a, b)
            out[form, interp] = (a, b)
            if form == "tuned" and not interp:
                worst, tp = c.tuned_calibrate(with_pairs=True)
                assert tp == c.count_pairs() and worst < 0.5
            c.close()
    for interp, tol in ((False, 1e-6), (True, 1e-5)):
        for x in range(2):
            assert rel_max(out["tuned", interp][x], out["fp64", interp][x]) < tol, interp
