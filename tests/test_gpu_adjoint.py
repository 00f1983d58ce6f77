"""Adjoint and autograd (GPU).

* transpose: <A x, y> == <x, A^T y> for the sky and for the beam maps
  (relative 1e-6: FP32 per-pair contributions);
* against the oracle's FP64 adjoint (orc_adjoint_f64) on the same inputs;
* DETERMINISTIC mode is bit-reproducible; ATOMIC agrees with it to 1e-6;
* torch.autograd gradients of L = 1/2 |TOD - TOD_target|^2 against central
  finite differences (step 1e-3) of the FP64 forward, for 64 random sky
  pixels and the beam FWHM, ellipticity and pointing offset (dx, dy).
"""
import math

import numpy as np
import pytest

from conftest import rel_max

pytestmark = pytest.mark.gpu


def _case(seed=3, nss=32, nsb=256, rdeg=4.0, n=3000):
    import torch

    import oracle as O
    from pisco4cmb_gb300 import GPUConvolver, PolBeam, Sky, synth

    rng = np.random.default_rng(seed)
    sky = rng.normal(size=(3, 12 * nss * nss))
    npb = O.beam_npix_for_radius(nsb, np.deg2rad(rdeg))
    beam = PolBeam(nsb, npb, 0.01, "p")
    fx, fy = synth.elliptical_fwhm(1.2, 0.05)
    beam.make_unpol_gaussian_elliptical_beams(fx, fy, 20.0)
    beam.build(nss)
    ra = rng.uniform(0, 2 * np.pi, n)
    dec = np.arcsin(rng.uniform(-1, 1, n))
    dec[:30] = np.pi / 2 - rng.uniform(0, 0.06, 30)
    pa = rng.uniform(0, np.pi, n)
    conv = GPUConvolver(form="tuned")
    conv.update_sky(Sky(nss, *sky.astype(np.float32), None))
    conv.update_beam(beam)
    t = [torch.tensor(x, device="cuda") for x in (ra, dec, pa)]
    conv.set_scan_device(n, t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr())
    conv._keep = t
    return conv, sky, beam, ra, dec, pa, nss, nsb, rng


def _fwd(conv, n, form="tuned"):
    import torch

    a = torch.empty(n, dtype=torch.float64, device="cuda")
    b = torch.empty(n, dtype=torch.float64, device="cuda")
    conv.forward_device(a.data_ptr(), b.data_ptr(), out_f64=True, form=form)
    conv.sync()
    return a.cpu().numpy(), b.cpu().numpy()


def _adj(conv, ga, gb, deterministic=True, beam=False, sky_iqu=False):
    import torch

    npix = conv._npix_sky
    g = [torch.tensor(x, device="cuda") for x in (ga, gb)]
    gs = torch.full((npix, 4), float("nan"), dtype=torch.float64, device="cuda")
    gbm = torch.empty((conv._keep_npb, 8), dtype=torch.float64, device="cuda") if beam else None
    conv.adjoint_device(g[0].data_ptr(), g[1].data_ptr(), True, gs.data_ptr(),
                        gbm.data_ptr() if beam else 0, out_f64=True, deterministic=deterministic,
                        sky_iqu=sky_iqu)
    conv.sync()
    return gs.cpu().numpy(), (gbm.cpu().numpy() if beam else None)


def test_adjoint_is_transpose_and_matches_fp64_oracle(gpu, oracle_mod):
    conv, sky, beam, ra, dec, pa, nss, nsb, rng = _case()
    conv._keep_npb = beam.nPixels
    n = ra.size
    ta, tb = _fwd(conv, n)
    ya, yb = rng.normal(size=n), rng.normal(size=n)
    gs, _ = _adj(conv, ya, yb)
    x4 = np.concatenate([sky, np.zeros((1, sky.shape[1]))]).astype(np.float32).astype(np.float64)
    lhs = ta @ ya + tb @ yb
    rhs = float(np.sum(x4.T * gs))
    assert abs(lhs - rhs) <= 1e-6 * abs(lhs)
    ba, bb = beam.planes()
    go = oracle_mod.adjoint_f64(ra, dec, pa, nss, nsb, ba.astype(np.float64), bb.astype(np.float64),
                                ya, yb)
    scale = np.abs(go).max()
    assert np.abs(gs.T - go).max() <= 2e-6 * scale


def test_deterministic_and_atomic_modes(gpu):
    conv, sky, beam, ra, *_ = _case(seed=5)
    conv._keep_npb = beam.nPixels
    rng = np.random.default_rng(1)
    ya, yb = rng.normal(size=ra.size), rng.normal(size=ra.size)
    g1, b1 = _adj(conv, ya, yb, True, beam=True)
    g2, b2 = _adj(conv, ya, yb, True, beam=True)
    assert np.array_equal(g1, g2) and np.array_equal(b1, b2)
    g3, b3 = _adj(conv, ya, yb, False, beam=True)
    assert np.abs(g3 - g1).max() <= 1e-5 * np.abs(g1).max()
    assert np.abs(b3 - b1).max() <= 1e-5 * np.abs(b1).max()


def test_sky_iqu_only(gpu):
    """PISCO_ADJ_SKY_IQU: I, Q, U columns as with V, V column zero."""
    import torch

    conv, sky, beam, ra, *_ = _case(seed=6)
    conv._keep_npb = beam.nPixels
    rng = np.random.default_rng(4)
    # a beam with V components, so that the full V gradient is not zero
    d = torch.tensor(rng.normal(size=(beam.nPixels, 8)).astype(np.float32), device="cuda")
    conv.set_beam_device(beam.nside, beam.nPixels, d.data_ptr())
    ya, yb = rng.normal(size=ra.size), rng.normal(size=ra.size)
    full, bfull = _adj(conv, ya, yb, True, beam=True)
    iqu, biqu = _adj(conv, ya, yb, True, beam=True, sky_iqu=True)
    assert np.array_equal(full[:, :3], iqu[:, :3]) and np.array_equal(bfull, biqu)
    assert not np.any(iqu[:, 3]) and np.any(full[:, 3])
    at, _ = _adj(conv, ya, yb, False, sky_iqu=True)
    assert not np.any(at[:, 3])
    assert np.abs(at[:, :3] - full[:, :3]).max() <= 1e-5 * np.abs(full).max()


def test_beam_adjoint_is_transpose(gpu):
    """TOD is linear in the beam maps: <A(delta), y> == <delta, A_beam^T y>."""
    import torch

    conv, sky, beam, ra, *_ = _case(seed=8)
    npb = beam.nPixels
    conv._keep_npb = npb
    rng = np.random.default_rng(2)
    ya, yb = rng.normal(size=ra.size), rng.normal(size=ra.size)
    _, gbm = _adj(conv, ya, yb, True, beam=True)
    delta = rng.normal(size=(npb, 8)).astype(np.float32)
    d = torch.tensor(delta, device="cuda")
    conv.set_beam_device(beam.nside, npb, d.data_ptr())
    ta, tb = _fwd(conv, ra.size)
    lhs = ta @ ya + tb @ yb
    rhs = float(np.sum(delta.astype(np.float64) * gbm))
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs)


def test_autograd_against_finite_differences(gpu):
    """Loss 1/2 |TOD - target|^2; sky leaf tensor and beam parameters."""
    import torch

    from pisco4cmb_gb300 import GPUConvolver, Sky
    from pisco4cmb_gb300.autograd import beam_pixel_coords, convolve, gaussian_polbeam
    from pisco4cmb_gb300 import synth

    rng = np.random.default_rng(20261203 + 5)
    nss, nsb, rdeg = 32, 256, 4.0
    from pisco4cmb_gb300 import beam_npix_for_radius

    npb = beam_npix_for_radius(nsb, math.radians(rdeg))
    n = 4000
    ra, dec, pa = synth.sweep_scan(n, 5, dec0=-40.0, per_sweep=400, ddec=2.0)
    sky0 = synth.grf_sky(nss, 5, dtype=np.float64)[:3].T.copy()
    target_sky = sky0 + 0.05 * synth.grf_sky(nss, 55, dtype=np.float64)[:3].T
    conv = GPUConvolver(form="tuned")
    conv.update_sky(Sky(nss, *np.zeros((3, 12 * nss * nss), np.float32), None))
    t = [torch.tensor(x, device="cuda") for x in (ra, dec, pa)]
    conv.set_scan_device(n, *[x.data_ptr() for x in t])
    rho, sig = beam_pixel_coords(nsb, npb)
    params = dict(fwhm=1.2, ell=0.05, dx=0.0, dy=0.0)

    def beam_of(p):
        return gaussian_polbeam(rho, sig, p["fwhm"], p["ell"], 0.0, p["dx"], p["dy"], 0.01, nss, nsb)

    def tod64(sky_np, p):
        """FP64 forward (same pixel decisions as TUNED) for the finite differences."""
        s4 = torch.tensor(np.concatenate([sky_np, np.zeros((sky_np.shape[0], 1))], 1), device="cuda")
        bab = beam_of(p).to(torch.float32).contiguous()
        conv.set_sky_device(nss, s4.data_ptr(), True)
        conv.set_beam_device(nsb, npb, bab.data_ptr())
        a = torch.empty(n, dtype=torch.float64, device="cuda")
        b = torch.empty(n, dtype=torch.float64, device="cuda")
        conv.forward_device(a.data_ptr(), b.data_ptr(), out_f64=True, form="fp64")
        conv.sync()
        return a.cpu().numpy(), b.cpu().numpy()

    tgt_a, tgt_b = tod64(target_sky, params)

    def loss64(sky_np, p):
        a, b = tod64(sky_np, p)
        return 0.5 * (np.sum((a - tgt_a) ** 2) + np.sum((b - tgt_b) ** 2))

    # autograd
    sky_t = torch.tensor(sky0, device="cuda", requires_grad=True)
    pt = {k: torch.tensor(v, dtype=torch.float64, device="cuda", requires_grad=True)
          for k, v in params.items()}
    ta, tb = convolve(sky_t, beam_of(pt), conv, nss, nsb)
    ga_t = torch.tensor(tgt_a, device="cuda")
    gb_t = torch.tensor(tgt_b, device="cuda")
    L = 0.5 * (((ta.double() - ga_t) ** 2).sum() + ((tb.double() - gb_t) ** 2).sum())
    L.backward()
    gsky = sky_t.grad.cpu().numpy()
    # sky pixels: central differences, step 1e-3
    h = 1e-3
    pix = rng.choice(np.flatnonzero(np.abs(gsky[:, 0]) > 1e-3 * np.abs(gsky[:, 0]).max()), 64,
                     replace=False)
    for p in pix:
        comp = int(rng.integers(0, 3))
        sp, sm = sky0.copy(), sky0.copy()
        sp[p, comp] += h
        sm[p, comp] -= h
        fd = (loss64(sp, params) - loss64(sm, params)) / (2 * h)
        assert abs(fd - gsky[p, comp]) <= 1e-4 * max(abs(fd), 1e-3 * np.abs(gsky).max()), (p, comp, fd, gsky[p, comp])
    # beam parameters: central differences, step 1e-3 (deg for fwhm, rad*1e-3 for offsets)
    steps = dict(fwhm=1e-3, ell=1e-3, dx=1e-3 * math.radians(1.0), dy=1e-3 * math.radians(1.0))
    for k, hk in steps.items():
        pp = dict(params)
        pm = dict(params)
        pp[k] += hk
        pm[k] -= hk
        fd = (loss64(sky0, pp) - loss64(sky0, pm)) / (2 * hk)
        ag = float(pt[k].grad)
        assert abs(fd - ag) <= 2e-3 * abs(fd) + 1e-9, (k, fd, ag)


@pytest.mark.parametrize("deterministic", [True, False])
def test_bilinear_adjoint_is_transpose(gpu, deterministic):
    """With the bilinear lookup the TOD is linear in the sky and in the beam
    maps (each pair's beam value is sum_i w_i beam[b_i]): <A x, y> ==
    <x, A^T y> for both, with the TUNED forward's FP32 stencil on both sides."""
    import torch

    conv, sky, beam, ra, *_ = _case(seed=9)
    npb = beam.nPixels
    conv._keep_npb = npb
    conv.set_interp(True)
    n = ra.size
    rng = np.random.default_rng(12)
    ya, yb = rng.normal(size=n), rng.normal(size=n)
    gs, gbm = _adj(conv, ya, yb, deterministic, beam=True)
    ta, tb = _fwd(conv, n)
    lhs = ta @ ya + tb @ yb
    x4 = np.concatenate([sky, np.zeros((1, sky.shape[1]))]).astype(np.float32).astype(np.float64)
    assert abs(lhs - float(np.sum(x4.T * gs))) <= 1e-6 * abs(lhs)
    delta = rng.normal(size=(npb, 8)).astype(np.float32)
    d = torch.tensor(delta, device="cuda")
    torch.cuda.synchronize()
    conv.set_beam_device(beam.nside, npb, d.data_ptr())
    ta, tb = _fwd(conv, n)
    lhs = ta @ ya + tb @ yb
    assert abs(lhs - float(np.sum(delta.astype(np.float64) * gbm))) <= 1e-5 * abs(lhs)


def test_adjoint_transpose_sweep(gpu):
    """Seeded sweep of sky/beam resolutions, radii and pole-heavy pointings:
    <A x, y> == <x, A^T y> for the sky (I, Q, U, V) and for the beam maps,
    with each lookup and each accumulation mode."""
    import torch

    import oracle as O
    from pisco4cmb_gb300 import GPUConvolver, PolBeam, Sky, synth

    rng = np.random.default_rng(31)
    for _ in range(6):
        nss = int(2 ** rng.integers(4, 9))   # 16 .. 256
        nsb = int(2 ** rng.integers(7, 11))  # 128 .. 1024
        pix_deg = np.rad2deg(np.sqrt(4 * np.pi / (12 * nss * nss)))
        rdeg = float(rng.uniform(max(0.5, 1.5 * pix_deg), max(5.0, 3.0 * pix_deg)))
        npb = O.beam_npix_for_radius(nsb, np.deg2rad(rdeg))
        beam = PolBeam(nsb, npb, 0.01, "p")
        fx, fy = synth.elliptical_fwhm(rdeg / 2.5, float(rng.uniform(-0.1, 0.1)))
        beam.make_unpol_gaussian_elliptical_beams(fx, fy, float(rng.uniform(0, 180)))
        beam.build(nss)
        n = 1200
        ra = rng.uniform(0, 2 * np.pi, n)
        dec = np.arcsin(rng.uniform(-1, 1, n))
        dec[:60] = np.pi / 2 - rng.uniform(0, np.deg2rad(rdeg), 60)
        pa = rng.uniform(0, np.pi, n)
        sky = rng.normal(size=(4, 12 * nss * nss)).astype(np.float32)
        delta = rng.normal(size=(npb, 8)).astype(np.float32)
        ya, yb = rng.normal(size=n), rng.normal(size=n)
        for interp in (False, True):
            conv = GPUConvolver(form="tuned")
            conv.update_sky(Sky(nss, *sky))
            conv.update_beam(beam)
            conv.set_interp(interp)
            t = [torch.tensor(x, device="cuda") for x in (ra, dec, pa)]
            torch.cuda.synchronize()
            conv.set_scan_device(n, t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr())
            conv._keep_npb = npb
            ta, tb = _fwd(conv, n)
            lhs_sky = ta @ ya + tb @ yb
            for det in (True, False):
                gs, gbm = _adj(conv, ya, yb, det, beam=True)
                assert abs(lhs_sky - float(np.sum(sky.astype(np.float64).T * gs))) <= \
                    1e-5 * abs(lhs_sky), (nss, nsb, rdeg, interp, det)
                d = torch.tensor(delta, device="cuda")
                torch.cuda.synchronize()
                conv.set_beam_device(nsb, npb, d.data_ptr())
                xa, xb = _fwd(conv, n)
                lhs_beam = xa @ ya + xb @ yb
                assert abs(lhs_beam - float(np.sum(delta.astype(np.float64) * gbm))) <= \
                    1e-5 * abs(lhs_beam), (nss, nsb, rdeg, interp, det)
                conv.update_beam(beam)
            conv.close()
