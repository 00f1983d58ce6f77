"""Parity at the workload configurations, against the CPU oracle (GPU).

Each test runs the production shapes of one workload -- sky and beam
resolutions, beam radius, FWHM and ellipticity, scan kind -- on a bounded
prefix of its samples that the oracle finishes in seconds, and compares the
GPU result with the oracle's CPU restatement of the reference Convolver
(convolver.cpp:74-183) on the same inputs:

* TUNED (FP32 per-pair geometry, FP64 pointing) against the oracle's
  all-FP64 form on the same float sky and beams: rms <= 1e-6 and max
  <= 1e-5 of the TOD rms (the stated FP32 tolerance);
* the FP64 form against the oracle's all-FP64 form: max <= 1e-12 of the TOD
  rms;
* PLAIN against the oracle's float form (the reference's own arithmetic):
  max <= 1e-6 of the TOD rms.

Workloads (seeded power-law skies, C_l ~ l^-2; the generator's lmax is
limited to 512 here to keep the sky synthesis short -- the 0.5-3 degree
beams average finer structure away):
* sky nside 1024, beam nside 2048 / 3 deg / FWHM 1.5 deg / e 0.05, the
  constant-elevation sweep: the first 1,000 samples and 1,000 spread over
  all 2,000,000;
* sky nside 2048, beam nside 4096 / 1 deg / FWHM 0.5 deg / e 0.02, the
  pole-heavy scan (10 % within 1 deg of a pole): 2,000 samples spread over
  all 4,000,000;
* sky nside 512, 48 detector pairs with radii 1-5 deg, beam nside 1024,
  per-detector offsets up to 2 deg: the batched persistent launch, each
  pair's first 300 samples;
* sky nside 256 leaf tensor, beam nside 1024 / 4 deg / FWHM 1.2 deg /
  e 0.05, four detector pairs on offset sweeps (5,000 samples each): the
  adjoint against the oracle's FP64 adjoint, and torch.autograd gradients
  against central finite differences (step 1e-3) for 64 sky pixels and every
  beam parameter.
"""
import math

import numpy as np
import pytest

from conftest import rel_max, rel_rms

pytestmark = pytest.mark.gpu

LMAX = 512


def _beam(nsb, radius_deg, fwhm, e, nss, phi0=0.0):
    from pisco4cmb_gb300 import PolBeam, beam_npix_for_radius, synth

    beam = PolBeam(nsb, beam_npix_for_radius(nsb, math.radians(radius_deg)), 0.01, "p")
    fx, fy = synth.elliptical_fwhm(fwhm, e)
    beam.make_unpol_gaussian_elliptical_beams(fx, fy, phi0)
    beam.build(nss)
    return beam


def _gpu(form, nss, sky, beam, ra, dec, pa):
    from pisco4cmb_gb300 import GPUConvolver, Scan, Sky

    c = GPUConvolver(form=form)
    c.update_sky(Sky(nss, sky[0], sky[1], sky[2], None))
    c.update_beam(beam)
    c.update_scan(Scan(ra.size, ra, dec, pa))
    a = np.empty(ra.size)
    b = np.empty(ra.size)
    c.exec_convolution(a, b)
    c.close()
    return a, b


def _check_forms(O, nss, sky, beam, ra, dec, pa):
    ba, bb = beam.planes()
    s64 = sky.astype(np.float32).astype(np.float64)
    oa, ob = O.convolve_f64(ra, dec, pa, nss, s64, beam.nside, ba.astype(np.float64),
                            bb.astype(np.float64))
    for form, rms_tol, max_tol in (("tuned", 1e-6, 1e-5), ("fp64", 1e-12, 1e-12)):
        ga, gb = _gpu(form, nss, sky, beam, ra, dec, pa)
        for g, o in ((ga, oa), (gb, ob)):
            assert rel_rms(g, o) <= rms_tol, (form, rel_rms(g, o))
            assert rel_max(g, o) <= max_tol, (form, rel_max(g, o))
    # PLAIN against the reference's arithmetic (float pointing, sky, beams and
    # per-pair products; double sums)
    r32, d32, p32 = (x.astype(np.float32) for x in (ra, dec, pa))
    fa, fb = O.convolve_f32(r32, d32, p32, nss, sky.astype(np.float32), beam.nside, ba, bb)
    pa_, pb_ = _gpu("plain", nss, sky, beam, *(x.astype(np.float64) for x in (r32, d32, p32)))
    assert rel_max(pa_, fa) <= 1e-6 and rel_max(pb_, fb) <= 1e-6


def test_c2_shape_against_oracle(gpu, oracle_mod):
    from pisco4cmb_gb300 import synth

    nss = 1024
    sky = synth.grf_sky(nss, 2, lmax=LMAX, dtype=np.float32, device="cuda")[:3]
    beam = _beam(2048, 3.0, 1.5, 0.05, nss)
    ra, dec, pa = synth.sweep_scan(2_000_000, 2)
    idx = np.r_[0:1000, np.linspace(1000, 2_000_000 - 1, 1000).astype(np.int64)]
    _check_forms(oracle_mod, nss, sky, beam, ra[idx], dec[idx], pa[idx])


def test_c2_shape_bilinear_against_oracle(gpu, oracle_mod):
    """The bilinear beam lookup at the c2 shape: TUNED (FP32 stencil) and the
    FP64 form against the oracle's FP64 get_interpol lookup.  The FP64 form's
    stencil weights differ from the oracle's by up to ~1e-9 next to the
    boresight (acos of a cosine near 1 amplifies last-bit differences of the
    device and host sin/cos), hence 1e-10 of the TOD rms rather than 1e-12."""
    from pisco4cmb_gb300 import GPUConvolver, Scan, Sky, synth

    O = oracle_mod
    nss = 1024
    sky = synth.grf_sky(nss, 2, lmax=LMAX, dtype=np.float32, device="cuda")[:3]
    beam = _beam(2048, 3.0, 1.5, 0.05, nss)
    ra, dec, pa = synth.sweep_scan(2_000_000, 2)
    idx = np.r_[0:500, np.linspace(500, 2_000_000 - 1, 500).astype(np.int64)]
    ra, dec, pa = ra[idx], dec[idx], pa[idx]
    ba, bb = beam.planes()
    oa, ob = O.convolve_f64(ra, dec, pa, nss, sky.astype(np.float64), beam.nside,
                            ba.astype(np.float64), bb.astype(np.float64), interp=1)
    for form, rms_tol, max_tol in (("tuned", 1e-6, 1e-5), ("fp64", 1e-10, 1e-10)):
        c = GPUConvolver(form=form)
        c.update_sky(Sky(nss, sky[0], sky[1], sky[2], None))
        c.update_beam(beam)
        c.set_interp(True)
        c.update_scan(Scan(ra.size, ra, dec, pa))
        a = np.empty(ra.size)
        b = np.empty(ra.size)
        c.exec_convolution(a, b)
        c.close()
        for g, o in ((a, oa), (b, ob)):
            assert rel_rms(g, o) <= rms_tol, (form, rel_rms(g, o))
            assert rel_max(g, o) <= max_tol, (form, rel_max(g, o))


def test_c3_shape_pole_heavy_against_oracle(gpu, oracle_mod):
    from pisco4cmb_gb300 import synth

    nss = 2048
    sky = synth.grf_sky(nss, 3, lmax=LMAX, dtype=np.float32, device="cuda")[:3]
    beam = _beam(4096, 1.0, 0.5, 0.02, nss)
    ra, dec, pa = synth.pole_heavy_scan(4_000_000, 3)
    idx = np.linspace(0, 4_000_000 - 1, 2000).astype(np.int64)
    idx[::10] = np.arange(0, 2000, 10) * 10  # keep the pole samples (every 10th) in the set
    ra, dec, pa = ra[idx], dec[idx], pa[idx]
    assert np.count_nonzero(np.abs(dec) > np.pi / 2 - math.radians(1.0)) >= 150
    _check_forms(oracle_mod, nss, sky, beam, ra, dec, pa)


def test_c4_shape_batched_against_oracle(gpu, oracle_mod):
    import torch

    from pisco4cmb_gb300 import GPUConvolver, Sky, synth

    O = oracle_mod
    nss = 512
    sky = synth.grf_sky(nss, 4, lmax=LMAX, dtype=np.float32, device="cuda")[:3]
    dets = synth.c4_detectors()
    conv = GPUConvolver(form="tuned")
    conv.update_sky(Sky(nss, sky[0], sky[1], sky[2], None))
    m = 300
    rows, keep, cases = [], [], []
    for d, p in enumerate(dets):
        beam = _beam(1024, p["radius_deg"], p["radius_deg"] / 2.5, p["ellipticity"], nss)
        conv.set_beam_slot(d, beam)
        ra, dec, pa = synth.sweep_scan(p["nsamples"], 4, stream=100 + d)
        ra, dec = synth.offset_pointing(ra, dec, p["dx_deg"], p["dy_deg"])
        ra, dec, pa = ra[:m], dec[:m], pa[:m]
        t = [torch.tensor(x, device="cuda") for x in (ra, dec, pa)]
        o = [torch.empty(m, dtype=torch.float64, device="cuda") for _ in range(2)]
        keep.append((t, o))
        cases.append((beam, ra, dec, pa))
        rows.append((d, m, t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr(), o[0].data_ptr(),
                     o[1].data_ptr()))
    descs = conv.det_descs(rows)
    conv.forward_batched(descs, out_f64=True, chunk=64)
    conv.sync()
    s64 = sky.astype(np.float64)
    worst = 0.0
    for (beam, ra, dec, pa), (_, o) in zip(cases, keep):
        ba, bb = beam.planes()
        oa, ob = O.convolve_f64(ra, dec, pa, nss, s64, beam.nside, ba.astype(np.float64),
                                bb.astype(np.float64))
        for g, r in ((o[0].cpu().numpy(), oa), (o[1].cpu().numpy(), ob)):
            worst = max(worst, rel_rms(g, r))
            assert rel_max(g, r) <= 1e-5
    assert worst <= 1e-6, worst
    conv.close()


def _c5_case(ndet=4, per_det=5000):
    from pisco4cmb_gb300 import synth

    ra, dec, pa = [], [], []
    offs = [(0.0, 0.0), (1.0, 0.0), (0.0, 1.0), (-1.0, -1.0)][:ndet]
    for d, (dx, dy) in enumerate(offs):
        r, de, p = synth.sweep_scan(per_det, 5, dec0=-40.0, per_sweep=500, ddec=1.0, stream=200 + d)
        r, de = synth.offset_pointing(r, de, dx, dy)
        ra.append(r)
        dec.append(de)
        pa.append(p)
    return np.concatenate(ra), np.concatenate(dec), np.concatenate(pa)


def test_c5_shape_adjoint_against_fp64_oracle(gpu, oracle_mod):
    import torch

    from pisco4cmb_gb300 import GPUConvolver, Sky, synth

    O = oracle_mod
    nss, nsb = 256, 1024
    sky = synth.grf_sky(nss, 5, lmax=LMAX, dtype=np.float32, device="cuda")[:3]
    beam = _beam(nsb, 4.0, 1.2, 0.05, nss)
    ra, dec, pa = _c5_case(ndet=2)
    n = ra.size
    conv = GPUConvolver(form="tuned")
    conv.update_sky(Sky(nss, sky[0], sky[1], sky[2], None))
    conv.update_beam(beam)
    t = [torch.tensor(x, device="cuda") for x in (ra, dec, pa)]
    conv.set_scan_device(n, *[x.data_ptr() for x in t])
    rng = np.random.default_rng(55)
    ya, yb = rng.normal(size=n), rng.normal(size=n)
    g = [torch.tensor(x, device="cuda") for x in (ya, yb)]
    gs = torch.empty((12 * nss * nss, 4), dtype=torch.float64, device="cuda")
    conv.adjoint_device(g[0].data_ptr(), g[1].data_ptr(), True, gs.data_ptr(), 0, out_f64=True,
                        deterministic=True)
    conv.sync()
    conv.close()
    ba, bb = beam.planes()
    go = O.adjoint_f64(ra, dec, pa, nss, nsb, ba.astype(np.float64), bb.astype(np.float64), ya, yb)
    got = gs.cpu().numpy().T
    scale = np.abs(go).max()
    assert np.abs(got - go).max() <= 2e-6 * scale


def test_c5_shape_gradients_against_finite_differences(gpu):
    """Loss 1/2 |TOD - TOD_target|^2, target from the sky perturbed by a
    seeded 5 % field; sky leaf tensor and beam FWHM, ellipticity and offset."""
    import torch

    from pisco4cmb_gb300 import GPUConvolver, Sky, beam_npix_for_radius, synth
    from pisco4cmb_gb300.autograd import beam_pixel_coords, convolve, gaussian_polbeam

    nss, nsb, rdeg = 256, 1024, 4.0
    npb = beam_npix_for_radius(nsb, math.radians(rdeg))
    ra, dec, pa = _c5_case()
    n = ra.size
    rng = np.random.default_rng(20261203 + 5)
    sky0 = synth.grf_sky(nss, 5, lmax=LMAX, dtype=np.float64, device="cuda")[:3].T.copy()
    target_sky = sky0 + 0.05 * synth.grf_sky(nss, 55, lmax=LMAX, dtype=np.float64,
                                             device="cuda")[:3].T
    conv = GPUConvolver(form="tuned")
    conv.update_sky(Sky(nss, *np.zeros((3, 12 * nss * nss), np.float32), None))
    t = [torch.tensor(x, device="cuda") for x in (ra, dec, pa)]
    conv.set_scan_device(n, *[x.data_ptr() for x in t])
    rho, sig = beam_pixel_coords(nsb, npb)
    params = dict(fwhm=1.2, ell=0.05, dx=0.0, dy=0.0)

    def beam_of(p):
        return gaussian_polbeam(rho, sig, p["fwhm"], p["ell"], 0.0, p["dx"], p["dy"], 0.01, nss, nsb)

    def tod64(sky_np, p):
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

    sky_t = torch.tensor(sky0, device="cuda", requires_grad=True)
    pt = {k: torch.tensor(v, dtype=torch.float64, device="cuda", requires_grad=True)
          for k, v in params.items()}
    ta, tb = convolve(sky_t, beam_of(pt), conv, nss, nsb)
    L = 0.5 * (((ta.double() - torch.tensor(tgt_a, device="cuda")) ** 2).sum() +
               ((tb.double() - torch.tensor(tgt_b, device="cuda")) ** 2).sum())
    L.backward()
    gsky = sky_t.grad.cpu().numpy()
    h = 1e-3
    pix = rng.choice(np.flatnonzero(np.abs(gsky[:, 0]) > 1e-3 * np.abs(gsky[:, 0]).max()), 64,
                     replace=False)
    for p in pix:
        comp = int(rng.integers(0, 3))
        sp, sm = sky0.copy(), sky0.copy()
        sp[p, comp] += h
        sm[p, comp] -= h
        fd = (loss64(sp, params) - loss64(sm, params)) / (2 * h)
        # autograd runs the TUNED operator on the FP32-rounded sky: the
        # residual TOD - target (5 % of the TOD) carries the sky's 6e-8
        # rounding, about 1.2e-6 of the gradient's scale
        assert abs(fd - gsky[p, comp]) <= 1e-4 * abs(fd) + 2e-6 * np.abs(gsky).max(), \
            (p, comp, fd, gsky[p, comp])
    steps = dict(fwhm=1e-3, ell=1e-3, dx=1e-3 * math.radians(1.0), dy=1e-3 * math.radians(1.0))
    for k, hk in steps.items():
        pp, pm = dict(params), dict(params)
        pp[k] += hk
        pm[k] -= hk
        fd = (loss64(sky0, pp) - loss64(sky0, pm)) / (2 * hk)
        ag = float(pt[k].grad)
        assert abs(fd - ag) <= 2e-3 * abs(fd) + 1e-9, (k, fd, ag)
    conv.close()
