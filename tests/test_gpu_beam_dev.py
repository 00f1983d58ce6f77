"""Beams built on the GPU (csrc/beam_dev.cu) against the host builders.

* pisco_beam_build_device (PolBeam::beam_from_fields + build) against the
  host steps (bit-identical to the reference PolBeam): every float within one
  ulp, for Gaussian fields and for GRASP-ingested fields with phases and a
  cross-polar part, each detector selection;
* pisco_beam_gaussian_device against the torch FP64 model (relative 1e-6);
* pisco_beam_gaussian_param_grad_device against the host analytic gradient
  (relative 1e-10) for float32 and float64 gbeam;
* the GaussianBeamFn autograd chain (beam -> TUNED forward -> adjoint ->
  parameter gradient) against the same chain through the host gradient;
* determinism and argument errors.
"""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _ulps(a, b):
    a = np.ascontiguousarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.ascontiguousarray(b, np.float32).view(np.int32).astype(np.int64)
    # map sign-magnitude to a monotone integer line
    a = np.where(a < 0, -(a & 0x7FFFFFFF), a)
    b = np.where(b < 0, -(b & 0x7FFFFFFF), b)
    return np.abs(a - b)


def _conv():
    from pisco4cmb_gb300 import GPUConvolver

    c = GPUConvolver(form="tuned")
    c.configure_execution()
    return c


def _host_beam(nsb, npix, eps, dets, nss, fa, fb):
    from pisco4cmb_gb300 import PolBeam

    b = PolBeam(nsb, npix, eps, dets)
    if fa is not None:
        b.beam_from_fields("a", *fa)
    if fb is not None:
        b.beam_from_fields("b", *fb)
    b.build(nss)
    a, bb = b.planes()
    return np.concatenate([a.T, bb.T], axis=1)  # npix x 8


def _device_beam(conv, nsb, npix, eps, dets, nss, fa, fb, set_beam=False):
    import torch

    ta = torch.tensor(np.stack(fa), dtype=torch.float64, device="cuda") if fa is not None else None
    tb = torch.tensor(np.stack(fb), dtype=torch.float64, device="cuda") if fb is not None else None
    out = torch.empty((npix, 8), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()  # inputs were written on torch's stream
    conv.build_beam_device(nsb, npix, eps, dets, nss, ta.data_ptr() if ta is not None else 0,
                           tb.data_ptr() if tb is not None else 0, out.data_ptr(),
                           set_beam=set_beam)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _gauss_fields(nsb, npix, fx, fy, phi0):
    import ctypes

    from pisco4cmb_gb300._lib import check, load

    f = [np.empty(npix, np.float64) for _ in range(4)]
    check(load().pisco_beam_gaussian_fields(nsb, npix, fx, fy, phi0,
                                            *[x.ctypes.data_as(ctypes.c_void_p) for x in f]))
    return f


@pytest.mark.parametrize("dets", ["p", "a", "b"])
def test_build_device_gaussian_fields(dets):
    from pisco4cmb_gb300 import beam_npix_for_radius

    nsb, nss, eps = 512, 128, 0.02
    npix = beam_npix_for_radius(nsb, np.deg2rad(4.0))
    fa = _gauss_fields(nsb, npix, 1.7, 1.3, 25.0) if dets != "b" else None
    fb = _gauss_fields(nsb, npix, 1.6, 1.4, 115.0) if dets != "a" else None
    host = _host_beam(nsb, npix, eps, dets, nss, fa, fb)
    dev = _device_beam(_conv(), nsb, npix, eps, dets, nss, fa, fb)
    u = _ulps(dev, host)
    assert u.max() <= 1, (u.max(), np.count_nonzero(u))
    assert np.count_nonzero(u) <= 1e-3 * u.size


def test_build_device_grasp_fields():
    """Fields with phases and a cross-polar part (GRASP ingest of the golden
    grid): tilde U and V are non-zero."""
    from pisco4cmb_gb300 import io as pio

    g = load_golden("golden_grasp.npz")
    nsb = int(g["nside"])
    grid = pio.GraspGrid(u=g["sq_u"], v=g["sq_v"], co=g["sq_co"], cx=g["sq_cx"])
    f = [np.ascontiguousarray(x) for x in pio.fields_from_grasp(grid, nsb)]
    npix = f[0].size
    fb = [f[2], f[3], f[0], f[1]]  # the orthogonal detector sees co and cx swapped
    host = _host_beam(nsb, npix, 0.01, "p", 64, f, fb)
    assert np.abs(host[:, 2]).max() > 0 and np.abs(host[:, 3]).max() > 0
    dev = _device_beam(_conv(), nsb, npix, 0.01, "p", 64, f, fb)
    u = _ulps(dev, host)
    assert u.max() <= 1, (u.max(), np.count_nonzero(u))


def test_build_device_sets_beam_and_is_deterministic():
    import torch

    from pisco4cmb_gb300 import Sky, beam_npix_for_radius

    nsb, nss, eps = 256, 32, 0.01
    npix = beam_npix_for_radius(nsb, np.deg2rad(4.0))
    fa = _gauss_fields(nsb, npix, 1.5, 1.2, 10.0)
    conv = _conv()
    d1 = _device_beam(conv, nsb, npix, eps, "p", nss, fa, fa, set_beam=True)
    d2 = _device_beam(conv, nsb, npix, eps, "p", nss, fa, fa, set_beam=True)
    assert np.array_equal(d1, d2)
    rng = np.random.default_rng(4)
    conv.update_sky(Sky(nss, *rng.normal(size=(3, 12 * nss * nss)).astype(np.float32), None))
    n = 2000
    t = [torch.tensor(x, device="cuda") for x in (rng.uniform(0, 6.28, n),
                                                   np.arcsin(rng.uniform(-1, 1, n)),
                                                   rng.uniform(0, 3.14, n))]
    torch.cuda.synchronize()
    conv.set_scan_device(n, t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr())
    out = [torch.empty(n, dtype=torch.float64, device="cuda") for _ in range(4)]
    conv.forward_device(out[0].data_ptr(), out[1].data_ptr(), out_f64=True, form="tuned")
    dab = torch.tensor(d1, device="cuda")
    torch.cuda.synchronize()
    conv.set_beam_device(nsb, npix, dab.data_ptr())
    conv.forward_device(out[2].data_ptr(), out[3].data_ptr(), out_f64=True, form="tuned")
    torch.cuda.synchronize()
    assert torch.equal(out[0], out[2]) and torch.equal(out[1], out[3])


@pytest.mark.parametrize("params", [(1.5, 0.05, 20.0, 0.0, 0.0), (2.0, -0.1, 130.0, 0.003, -0.002)])
def test_gaussian_device_matches_torch_model(params):
    import torch

    from pisco4cmb_gb300 import beam_npix_for_radius
    from pisco4cmb_gb300.autograd import beam_pixel_coords, gaussian_polbeam

    nsb, nss, eps = 512, 64, 0.01
    npix = beam_npix_for_radius(nsb, np.deg2rad(5.0))
    rho, sig = beam_pixel_coords(nsb, npix, device="cpu")
    ref = gaussian_polbeam(rho, sig, *params, epsilon=eps, nside_sky=nss, nside_beam=nsb).numpy()
    conv = _conv()
    out = torch.empty((npix, 8), dtype=torch.float32, device="cuda")
    conv.gaussian_beam_device(nsb, npix, eps, nss, *params, out.data_ptr(), set_beam=False)
    torch.cuda.synchronize()
    dev = out.cpu().numpy()
    scale = np.abs(ref).max()
    assert np.abs(dev - ref).max() <= 1e-6 * scale


@pytest.mark.parametrize("f64", [False, True])
@pytest.mark.parametrize("params", [(1.5, 0.05, 20.0, 0.0, 0.0), (2.0, -0.1, 130.0, 0.003, -0.002)])
def test_param_grad_device_matches_host(params, f64):
    import torch

    from pisco4cmb_gb300 import beam_npix_for_radius, gaussian_beam_param_grad

    nsb, nss, eps = 256, 64, 0.01
    npix = beam_npix_for_radius(nsb, np.deg2rad(5.0))
    gbeam = np.random.default_rng(3).normal(size=(npix, 8))
    if not f64:
        gbeam = gbeam.astype(np.float32)
    host = gaussian_beam_param_grad(nsb, npix, eps, nss, *params, gbeam.astype(np.float64))
    conv = _conv()
    g = torch.tensor(gbeam, device="cuda")
    out = torch.empty(5, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    conv.gaussian_beam_param_grad_device(nsb, npix, eps, nss, *params, g.data_ptr(), f64,
                                         out.data_ptr())
    torch.cuda.synchronize()  # the call ran on the convolver's own stream
    dev = out.cpu().numpy()
    assert np.allclose(dev, host, rtol=1e-10, atol=1e-12 * np.abs(host).max()), (dev, host)
    out2 = torch.empty(5, dtype=torch.float64, device="cuda")
    conv.gaussian_beam_param_grad_device(nsb, npix, eps, nss, *params, g.data_ptr(), f64,
                                         out2.data_ptr())
    torch.cuda.synchronize()
    assert torch.equal(out, out2)


def test_gaussian_beam_autograd_chain():
    """dL/dparams through GaussianBeamFn equals the host gradient applied to
    the adjoint's beam gradient."""
    import torch

    from pisco4cmb_gb300 import beam_npix_for_radius, gaussian_beam_param_grad
    from pisco4cmb_gb300.autograd import convolve, gaussian_beam

    nsb, nss, eps = 256, 32, 0.01
    npix = beam_npix_for_radius(nsb, np.deg2rad(4.0))
    rng = np.random.default_rng(11)
    conv = _conv()
    n = 3000
    t = [torch.tensor(x, device="cuda") for x in (rng.uniform(0, 6.28, n),
                                                   np.arcsin(rng.uniform(-1, 1, n)),
                                                   rng.uniform(0, 3.14, n))]
    torch.cuda.synchronize()
    conv.set_scan_device(n, t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr())
    sky = torch.tensor(rng.normal(size=(12 * nss * nss, 3)), dtype=torch.float32, device="cuda")
    p0 = (1.3, 0.04, 15.0, 0.001, -0.002)
    params = torch.tensor(p0, dtype=torch.float64, device="cuda", requires_grad=True)
    beam = gaussian_beam(params, conv, nsb, npix, eps, nss)
    beam.retain_grad()
    ta, tb = convolve(sky, beam, conv, nss, nsb)
    loss = 0.5 * ((ta ** 2).sum() + (tb ** 2).sum())
    loss.backward()
    host = gaussian_beam_param_grad(nsb, npix, eps, nss, *p0, beam.grad.double().cpu().numpy())
    dev = params.grad.cpu().numpy()
    assert np.allclose(dev, host, rtol=1e-9, atol=1e-12 * np.abs(host).max()), (dev, host)


def test_argument_errors():
    import torch

    from pisco4cmb_gb300 import PiscoInvalidArgument

    conv = _conv()
    out = torch.empty((100, 8), dtype=torch.float32, device="cuda")
    f = torch.zeros((4, 100), dtype=torch.float64, device="cuda")
    with pytest.raises(PiscoInvalidArgument):  # fields of an enabled detector missing
        conv.build_beam_device(64, 100, 0.01, "p", 16, f.data_ptr(), 0, out.data_ptr())
    with pytest.raises(PiscoInvalidArgument):  # misaligned output
        conv.build_beam_device(64, 100, 0.01, "a", 16, f.data_ptr(), 0, out.data_ptr() + 4)
    with pytest.raises(PiscoInvalidArgument):
        conv.gaussian_beam_device(64, 100, 0.01, 16, -1.0, 0.0, 0.0, 0.0, 0.0, out.data_ptr())
    with pytest.raises(PiscoInvalidArgument):
        conv.gaussian_beam_device(64, 100, 0.01, 16, 1.0, 1.0, 0.0, 0.0, 0.0, out.data_ptr())
    with pytest.raises(PiscoInvalidArgument):  # npix beyond the grid
        conv.gaussian_beam_device(4, 1000, 0.01, 16, 1.0, 0.0, 0.0, 0.0, 0.0, out.data_ptr())
