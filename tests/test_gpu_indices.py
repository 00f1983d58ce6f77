"""Integer decisions made on the device, bit for bit against the oracle (GPU).

The forward kernels never materialise their pair lists, so these tests ask
the library for a record of every (sample, disc pixel) pair the kernels
visit (pisco_debug_pairs: the TUNED record runs the TUNED per-sample body
itself) and compare it with the oracle's CPU restatement:

* the disc: each sample's set of sky pixels equals HEALPix query_disc's
  (oracle.query_disc), exactly -- a swapped edge pixel fails;
* the nearest beam pixel of every pair equals the oracle's
  ang2pix(rho_sigma_chi(...)) chain, in both the PLAIN and the TUNED form;
* chi: PLAIN's FP64 chi within 1e-9 rad of the oracle's; the angle of the
  FP32 phasor (cos 2chi, sin 2chi) each form multiplies by within 1e-6 rad
  of 2 chi / 2 (the reference's own K1 test allows |dchi| <= 1e-6,
  tests/cudaConvolution/test_sky_to_beam_matching_kernel.cu:188-216);
* the bilinear stencil: PLAIN's four pixels equal get_interpol's and its
  weights agree to 1e-8; TUNED's FP32 stencil, as a weight map over beam
  pixels, within 1e-6 (r + 1) of the oracle's renormalised one, r the
  largest ring index of the beam grid the disc reaches (the FP32 error of
  the pair's ring position and longitude, about 2e-7 relative, scaled by the
  ring's size);
* HEALPix RING on the device for every pixel of nside 1 ... 8192: ang2pix
  of pix2ang gives the pixel back, pix2ang agrees with the oracle within
  1e-10 and ang2pix of the oracle's angles is exact (the reference's
  tests/cudaHealpix/test_pix2ang.cu:80-114 asks the same); get_interpol's
  pixels equal the oracle's, its weights to 4e-15 nside.

Workloads: the reference K1 test's shape (sky and beam nside 256, 5 deg,
5,000 pointings uniform in colatitude, tests/cudaConvolution/
test_sky_to_beam_matching_kernel.cu:109-133, seeded here), the CPU-runnable
workload's golden pointings, and the production shapes (sky 1024 / beam
2048 / 3 deg; sky 2048 / beam 4096 / 1 deg) with pointings at and near
both poles.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _beam(nsb, radius_deg, fwhm, e, phi0, nss):
    from pisco4cmb_gb300 import PolBeam, beam_npix_for_radius, synth

    beam = PolBeam(nsb, beam_npix_for_radius(nsb, np.deg2rad(radius_deg)), 0.01, "p")
    fx, fy = synth.elliptical_fwhm(fwhm, e)
    beam.make_unpol_gaussian_elliptical_beams(fx, fy, phi0)
    beam.build(nss)
    return beam


def _conv(nss, beam, ra, dec, pa, form, bilinear=False, seed=3):
    from pisco4cmb_gb300 import GPUConvolver, Scan, Sky

    rng = np.random.default_rng(seed)
    sky = rng.normal(size=(3, 12 * nss * nss)).astype(np.float32)
    c = GPUConvolver(form=form)
    c.update_sky(Sky(nss, sky[0], sky[1], sky[2], None))
    c.update_beam(beam)
    c.update_scan(Scan(ra.size, ra, dec, pa))
    if bilinear:
        c.set_interp(True)
    return c


def _oracle_discs(O, nss, rho, ra, dec):
    lists = [O.query_disc(nss, np.pi / 2 - dec[i], ra[i], rho) for i in range(ra.size)]
    sample = np.repeat(np.arange(ra.size), [x.size for x in lists]).astype(np.int32)
    sky = np.concatenate(lists).astype(np.int32)
    order = np.lexsort((sky, sample))
    return sample[order], sky[order]


def _workload(name):
    from pisco4cmb_gb300 import synth

    rng = np.random.default_rng(20261204)
    if name == "k1":  # the reference K1 test's shape, seeded
        n = 5000
        ra = rng.uniform(0, 2 * np.pi, n)
        dec = np.pi / 2 - rng.uniform(0, np.pi, n)
        pa = rng.uniform(0, np.pi, n)
        return 256, (256, 5.0, 2.0, 0.0, 0.0), ra, dec, pa
    if name == "c1":  # the CPU-runnable workload's raster (first 2,000 samples)
        from conftest import load_golden

        g = load_golden("golden_c1.npz")
        s = slice(0, 2000)
        return 64, (256, 5.0, 2.0, 0.0, 0.0), g["ra"][s].astype(np.float64), \
            g["dec"][s].astype(np.float64), g["pa"][s].astype(np.float64)
    # production shapes: sweep samples plus pointings at and within a beam
    # radius of both poles (exact poles, ring-boundary latitudes)
    nss, nsb, r, fwhm, e = (1024, 2048, 3.0, 1.5, 0.05) if name == "c2" else \
        (2048, 4096, 1.0, 0.5, 0.02)
    # 125 samples spread over the whole 2M-sample sweep (c2) or the 4M-sample
    # pole-heavy scan (c3)
    full = synth.sweep_scan(2_000_000, 2) if name == "c2" else synth.pole_heavy_scan(4_000_000, 3)
    ra_s, dec_s, pa_s = (x[::len(x) // 125] for x in full)
    k = 120
    ra_p = rng.uniform(0, 2 * np.pi, k)
    dec_p = np.where(rng.uniform(size=k) < 0.5, 1, -1) * (np.pi / 2 - np.deg2rad(
        rng.uniform(0, 1.2 * r, k)))
    dec_p[:4] = [np.pi / 2, -np.pi / 2, np.pi / 2 - 1e-9, -np.pi / 2 + 1e-12]
    pa_p = rng.uniform(0, np.pi, k)
    ra = np.concatenate([ra_s, ra_p])
    dec = np.concatenate([dec_s, dec_p])
    pa = np.concatenate([pa_s, pa_p])
    return nss, (nsb, r, fwhm, e, 25.0), ra, dec, pa


@pytest.mark.parametrize("name", ["k1", "c1", "c2", "c3"])
def test_disc_and_beam_pixels_bit_exact(gpu, oracle_mod, name):
    O = oracle_mod
    nss, (nsb, r, fwhm, e, phi0), ra, dec, pa = _workload(name)
    beam = _beam(nsb, r, fwhm, e, phi0, nss)
    rho = O.beam_rho_max(nsb, beam.nPixels)
    o_sample, o_sky = _oracle_discs(O, nss, rho, ra, dec)
    o_bp, o_chi = O.match_pairs(ra[o_sample], dec[o_sample], pa[o_sample], o_sky, nss, nsb)
    for form in ("plain", "tuned"):
        c = _conv(nss, beam, ra, dec, pa, form)
        rec = c.debug_pairs()
        c.close()
        # the disc: same (sample, pixel) set, every pair visited once
        assert np.array_equal(rec["sample"], o_sample), form
        assert np.array_equal(rec["sky_pix"], o_sky), form
        # the nearest beam pixel of every pair, also those beyond the map
        assert np.array_equal(rec["beam_pix"].astype(np.int64), o_bp), form
        inside = o_bp < beam.nPixels
        assert np.array_equal((rec["flags"] & 2) == 0, inside), form
        c2, s2 = np.cos(2 * o_chi), np.sin(2 * o_chi)
        if form == "plain":
            d = np.angle(np.exp(1j * (rec["chi"] - o_chi)))
            assert np.max(np.abs(d)) <= 1e-9
        # chi as the form applies it, exp(2i chi), the phasor of unit length:
        # PLAIN rounds FP64 cos 2chi, sin 2chi to float (the reference K1
        # test's |dchi| <= 1e-6); TUNED forms the phasor from FP32 boresight-
        # frame components, whose rounding grows as 1 / rho for pairs next to
        # the boresight (measured worst 1.2e-6 rad at sky nside 1024, 2.2e-6
        # at 2048): within 1e-5 rad, and 1e-7 rad rms
        m = inside
        z = rec["c2chi"][m].astype(np.float64) + 1j * rec["s2chi"][m].astype(np.float64)
        dchi = 0.5 * np.angle(z * np.exp(-2j * o_chi[m]))
        tol = 1e-6 if form == "plain" else 1e-5
        assert np.max(np.abs(dchi)) <= tol, (form, np.max(np.abs(dchi)))
        assert np.sqrt(np.mean(dchi ** 2)) <= 1e-7, form
        assert np.max(np.abs(np.abs(z) - 1.0)) <= 2e-6, form
        if form == "tuned":
            # most pairs decided in FP32; the near-boundary ones redone in FP64
            redone = np.count_nonzero(rec["flags"] & 1)
            assert redone < 0.01 * rec["sample"].size


def _weight_maps(pix, w, npix_beam):
    """Per pair, the stencil as {beam pixel: weight} over the stored map,
    renormalised; returned as a sparse (pair, pixel) -> weight dict."""
    out = {}
    inside = (pix >= 0) & (pix < npix_beam)
    ws = np.where(inside, w, 0.0).sum(axis=1)
    for i in range(pix.shape[0]):
        if ws[i] <= 0:
            continue
        for k in range(4):
            if inside[i, k] and w[i, k] != 0:
                key = (i, int(pix[i, k]))
                out[key] = out.get(key, 0.0) + w[i, k] / ws[i]
    return out


@pytest.mark.parametrize("name", ["k1", "c2"])
def test_bilinear_stencils(gpu, oracle_mod, name):
    O = oracle_mod
    nss, (nsb, r, fwhm, e, phi0), ra, dec, pa = _workload(name)
    n = 400 if name == "k1" else 60
    sel = np.r_[0:n // 2, ra.size - n // 2:ra.size]
    ra, dec, pa = ra[sel], dec[sel], pa[sel]
    beam = _beam(nsb, r, fwhm, e, phi0, nss)
    rho_max = O.beam_rho_max(nsb, beam.nPixels)
    o_sample, o_sky = _oracle_discs(O, nss, rho_max, ra, dec)
    th, ph = O.pix2ang(nss, o_sky)
    rho, sig, chi = O.rho_sigma_chi(ra[o_sample], dec[o_sample], -pa[o_sample], ph, np.pi / 2 - th)
    o_pix, o_w = O.get_interpol(nsb, rho, sig)
    # PLAIN: get_interpol's stencil itself
    c = _conv(nss, beam, ra, dec, pa, "plain", bilinear=True)
    rec = c.debug_pairs()
    c.close()
    assert np.array_equal(rec["sample"], o_sample) and np.array_equal(rec["sky_pix"], o_sky)
    assert np.array_equal(rec["stencil_pix"].astype(np.int64), o_pix)
    # weights: rho = acos(cos rho) amplifies the last-bit differences of the
    # device's and the host's sin/cos by 1 / rho next to the boresight
    # (measured up to 1.4e-9); the beam value they weight is FP32 (6e-8)
    assert np.max(np.abs(rec["stencil_w"] - o_w)) <= 1e-8
    # TUNED: the FP32 stencil, as a weight map over the stored beam pixels
    c = _conv(nss, beam, ra, dec, pa, "tuned", bilinear=True)
    rec = c.debug_pairs()
    c.close()
    assert np.array_equal(rec["sample"], o_sample) and np.array_equal(rec["sky_pix"], o_sky)
    keep = (rec["flags"] & 2) == 0
    got = _weight_maps(rec["stencil_pix"][keep], rec["stencil_w"][keep], beam.nPixels)
    want = _weight_maps(o_pix[keep], o_w[keep], beam.nPixels)
    worst = max(abs(got.get(k, 0.0) - want.get(k, 0.0)) for k in set(got) | set(want))
    r_max = nsb * np.sqrt(3.0 * (1.0 - np.cos(rho_max)))
    assert worst <= 1e-6 * (r_max + 1.0), (worst, r_max)
    # pairs with no stencil pixel in the map: the same in both
    o_in = ((o_pix >= 0) & (o_pix < beam.nPixels)).any(axis=1)
    assert np.array_equal(keep, o_in)


def _dev_hpx(nside, pix_t):
    import torch

    from pisco4cmb_gb300 import _lib

    L = _lib.load()
    n = pix_t.numel()
    th = torch.empty(n, dtype=torch.float64, device="cuda")
    ph = torch.empty(n, dtype=torch.float64, device="cuda")
    st = L.pisco_hpx_pix2ang_device(nside, n, ctypes.c_void_p(pix_t.data_ptr()),
                                    ctypes.c_void_p(th.data_ptr()), ctypes.c_void_p(ph.data_ptr()),
                                    None)
    assert st == 0, L.pisco_last_error(None)
    return th, ph


def _dev_ang2pix(nside, th, ph):
    import torch

    from pisco4cmb_gb300 import _lib

    L = _lib.load()
    out = torch.empty(th.numel(), dtype=torch.int64, device="cuda")
    st = L.pisco_hpx_ang2pix_device(nside, th.numel(), ctypes.c_void_p(th.data_ptr()),
                                    ctypes.c_void_p(ph.data_ptr()),
                                    ctypes.c_void_p(out.data_ptr()), None)
    assert st == 0, L.pisco_last_error(None)
    return out


def test_device_healpix_every_pixel_nside_1_to_8192(gpu, oracle_mod):
    import torch

    O = oracle_mod
    rng = np.random.default_rng(81)
    nside = 1
    while nside <= 8192:
        npix = 12 * nside * nside
        pix = torch.arange(npix, dtype=torch.int64, device="cuda")
        th, ph = _dev_hpx(nside, pix)
        # every pixel: ang2pix(pix2ang(p)) == p on the device
        back = _dev_ang2pix(nside, th, ph)
        assert torch.equal(back, pix), nside
        del back
        # against the oracle: every pixel up to nside 1024; beyond, both polar
        # caps' first and last 200,000 pixels and 2,000,000 random ones
        if npix <= 12 * 1024 * 1024:
            idx = np.arange(npix)
        else:
            idx = np.unique(np.concatenate([np.arange(200000), np.arange(npix - 200000, npix),
                                            rng.integers(0, npix, 2000000)]))
        it = torch.from_numpy(idx).cuda()
        dth = th[it].cpu().numpy()
        dph = ph[it].cpu().numpy()
        del th, ph, pix
        oth, oph = O.pix2ang(nside, idx)
        assert np.max(np.abs(dth - oth)) <= 1e-10, nside
        assert np.max(np.abs(dph - oph)) <= 1e-10, nside
        # ang2pix of the oracle's angles is exact
        got = _dev_ang2pix(nside, torch.from_numpy(oth).cuda(), torch.from_numpy(oph).cuda())
        assert np.array_equal(got.cpu().numpy(), idx), nside
        # random angles (uniform on the sphere, plus the poles)
        m = 500000
        t = np.arccos(rng.uniform(-1, 1, m))
        t[:2] = [0.0, np.pi]
        f = rng.uniform(-4 * np.pi, 4 * np.pi, m)
        got = _dev_ang2pix(nside, torch.from_numpy(t).cuda(), torch.from_numpy(f).cuda())
        assert np.array_equal(got.cpu().numpy(), O.ang2pix(nside, t, f)), nside
        torch.cuda.empty_cache()
        nside *= 2


def test_device_get_interpol(gpu, oracle_mod):
    import torch

    from pisco4cmb_gb300 import _lib

    O = oracle_mod
    L = _lib.load()
    rng = np.random.default_rng(82)
    for nside in (1, 2, 4, 16, 256, 1024, 4096, 8192):
        m = 300000
        t = np.arccos(rng.uniform(-1, 1, m))
        t[:4] = [0.0, np.pi, 1e-9, np.pi - 1e-9]
        f = rng.uniform(0, 2 * np.pi, m)
        tt, ft = torch.from_numpy(t).cuda(), torch.from_numpy(f).cuda()
        pix = torch.empty((m, 4), dtype=torch.int64, device="cuda")
        w = torch.empty((m, 4), dtype=torch.float64, device="cuda")
        st = L.pisco_hpx_get_interpol_device(nside, m, ctypes.c_void_p(tt.data_ptr()),
                                             ctypes.c_void_p(ft.data_ptr()),
                                             ctypes.c_void_p(pix.data_ptr()),
                                             ctypes.c_void_p(w.data_ptr()), None)
        assert st == 0, L.pisco_last_error(None)
        op, ow = O.get_interpol(nside, t, f)
        assert np.array_equal(pix.cpu().numpy(), op), nside
        # weights (theta - theta_a) / (theta_b - theta_a): one ulp of the
        # ring colatitudes over a ring spacing of about pi / (4 nside)
        assert np.max(np.abs(w.cpu().numpy() - ow)) <= 4e-15 * nside + 1e-15, nside


def test_device_healpix_rejects_bad_input(gpu):
    import torch

    from pisco4cmb_gb300 import _lib

    L = _lib.load()
    pix = torch.tensor([0, 48], dtype=torch.int64, device="cuda")  # 48 = npix at nside 2
    th = torch.empty(2, dtype=torch.float64, device="cuda")
    ph = torch.empty(2, dtype=torch.float64, device="cuda")
    st = L.pisco_hpx_pix2ang_device(2, 2, ctypes.c_void_p(pix.data_ptr()),
                                    ctypes.c_void_p(th.data_ptr()), ctypes.c_void_p(ph.data_ptr()),
                                    None)
    assert st == _lib.PISCO_ERR_INVALID_ARGUMENT
    assert torch.isnan(th[1]) and not torch.isnan(th[0])
    assert L.pisco_hpx_pix2ang_device(0, 2, None, None, None, None) == \
        _lib.PISCO_ERR_INVALID_ARGUMENT
