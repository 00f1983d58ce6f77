"""Detector pointing from the array centre, on the GPU (BPoint's
focal_plane_to_sky, src/Bpoint/bpoint.cpp:553-674).

* pisco_focal_plane_to_sky (host arrays) and pisco_focal_plane_to_sky_device
  agree with the oracle's restatement within 1e-12 rad for the three output
  frames, at offsets up to 5 deg and array centres up to the poles.
* The beam model's centre offset (dx, dy) (beam plane: x = rho cos sigma,
  y = rho sin sigma, sphtrigo.cpp:27-54) is a focal-plane offset in BPoint's
  convention: moving the Gaussian's centre to (dx, dy) shifts the response
  like moving the detector to receiver offsets (right, up) = (-dy, -dx) with
  the array centre's rotation equal to the scan's position angle.  Checked by
  finite differences of the TOD (bilinear beam lookup, so the TOD is smooth
  in the pointing) along the equator, where the detector's position angle
  does not change to first order: d TOD / d(right) = -d TOD / d(dy) and
  d TOD / d(up) = -d TOD / d(dx) to within the beam grid's sampling.
"""
import ctypes
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_focal_plane_to_sky_matches_oracle(gpu, oracle_mod):
    import torch

    from pisco4cmb_gb300 import _lib, focal_plane_to_sky

    rng = np.random.default_rng(5)
    ns = 20000
    x_ac = rng.uniform(0, 2 * np.pi, ns)
    y_ac = np.arcsin(rng.uniform(-1, 1, ns))
    y_ac[:4] = [np.pi / 2, -np.pi / 2, np.pi / 2 - 1e-9, 0.0]
    rot = rng.uniform(-np.pi, np.pi, ns)
    dx = np.deg2rad(rng.uniform(-5, 5, 24))
    dy = np.deg2rad(rng.uniform(-5, 5, 24))
    pol = np.deg2rad(rng.uniform(0, 180, 24))
    dx[0] = dy[0] = 0.0
    L = _lib.load()
    for flag in (0, 1, 2):
        want = oracle_mod.focal_plane_to_sky(dx, dy, pol, x_ac, y_ac, rot, flag)
        got = focal_plane_to_sky(dx, dy, pol, x_ac, y_ac, rot, flag)
        for g, w in zip(got, want):
            assert np.max(np.abs(np.angle(np.exp(1j * (g - w))))) <= 1e-12, flag
        # device arrays, on a stream
        t = [torch.tensor(v, device="cuda") for v in (dx, dy, pol, x_ac, y_ac, rot)]
        o = [torch.empty((dx.size, ns), dtype=torch.float64, device="cuda") for _ in range(3)]
        st = torch.cuda.Stream()
        torch.cuda.synchronize()
        rc = L.pisco_focal_plane_to_sky_device(
            dx.size, *[ctypes.c_void_p(v.data_ptr()) for v in t[:3]], ns,
            *[ctypes.c_void_p(v.data_ptr()) for v in t[3:]], flag,
            *[ctypes.c_void_p(v.data_ptr()) for v in o], ctypes.c_void_p(st.cuda_stream))
        assert rc == 0, L.pisco_last_error(None)
        st.synchronize()
        for g, h in zip(o, got):
            assert np.array_equal(g.cpu().numpy(), h)
    assert L.pisco_focal_plane_to_sky(1, None, None, None, 1, None, None, None, 3, None, None,
                                      None) == _lib.PISCO_ERR_INVALID_ARGUMENT


def test_beam_centre_offset_is_a_focal_plane_offset(gpu):
    import torch

    from pisco4cmb_gb300 import GPUConvolver, Sky, beam_npix_for_radius, focal_plane_to_sky, synth

    nss, nsb, rdeg, fwhm = 256, 4096, 3.0, 1.2
    npb = beam_npix_for_radius(nsb, math.radians(rdeg))
    n = 3000
    ra = np.linspace(0.2, 2 * np.pi - 0.2, n)
    dec = np.deg2rad(np.linspace(-0.5, 0.5, n))
    pa = np.random.default_rng(3).uniform(0, np.pi, n)
    sky = synth.grf_sky(nss, 5, lmax=512, dtype=np.float32, device="cuda")
    conv = GPUConvolver(form="tuned")
    conv.update_sky(Sky(nss, sky[0], sky[1], sky[2], None))
    conv.set_interp(True)
    ab = torch.empty((npb, 8), dtype=torch.float32, device="cuda")

    def tod(ra_, dec_, pa_, dxb=0.0, dyb=0.0):
        conv.gaussian_beam_device(nsb, npb, 0.01, nss, fwhm, 0.05, 30.0, dxb, dyb, ab.data_ptr(),
                                  set_beam=True)
        t = [torch.tensor(np.ascontiguousarray(v), device="cuda") for v in (ra_, dec_, pa_)]
        conv.set_scan_device(n, *[v.data_ptr() for v in t])
        a = torch.empty(n, dtype=torch.float64, device="cuda")
        b = torch.empty(n, dtype=torch.float64, device="cuda")
        conv.forward_device(a.data_ptr(), b.data_ptr(), out_f64=True)
        conv.sync()
        return np.concatenate([a.cpu().numpy(), b.cpu().numpy()])

    h = math.radians(0.05)

    def fp(right, up):
        x, y, r = focal_plane_to_sky([right], [up], [0.0], ra, dec, pa, 1)
        return tod(x[0], y[0], r[0])

    d_right = (fp(h, 0.0) - fp(-h, 0.0)) / (2 * h)
    d_up = (fp(0.0, h) - fp(0.0, -h)) / (2 * h)
    d_dx = (tod(ra, dec, pa, dxb=h) - tod(ra, dec, pa, dxb=-h)) / (2 * h)
    d_dy = (tod(ra, dec, pa, dyb=h) - tod(ra, dec, pa, dyb=-h)) / (2 * h)
    conv.close()

    def rel(a, b):
        return np.linalg.norm(a - b) / np.linalg.norm(b)

    assert rel(d_right, -d_dy) <= 0.03, rel(d_right, -d_dy)
    assert rel(d_up, -d_dx) <= 0.03, rel(d_up, -d_dx)
    # the other pairings are not the same derivative
    assert rel(d_right, d_dy) > 1.0 and rel(d_right, -d_dx) > 0.5
