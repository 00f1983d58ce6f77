"""The fused beam-parameter gradient (pisco_adjoint_gaussian_device) (GPU).

The adjoint forms dL/d(fwhm, ellipticity, phi0, dx, dy) of the elliptical
Gaussian pair beam directly, from each pair's share of the model's weight
and derivatives recomputed at its beam pixel, instead of accumulating the
beam-map gradient (eight atomics per pair) and contracting it afterwards.

* It equals the two-step path (pisco_adjoint_device's beam-map gradient,
  DETERMINISTIC, then pisco_beam_gaussian_param_grad_device) to 1e-4 of each
  component: both weight FP32 per-pair products, rounded differently (the
  two-step path rounds the eight beam-gradient values of a pair, the fused
  one their contraction and the model table), and the sums cancel for the
  offsets of a centred beam.
* The parameter gradient is the same on every run and in both modes (the
  mode only selects the sky gradient's accumulation), and the sky gradient
  it returns equals pisco_adjoint_device's bit for bit.
* Through ``autograd.convolve_gaussian`` the gradients match central finite
  differences of the FP64 forward (step 1e-3; 0.5 deg for phi0), for both
  beam lookups.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PARAMS = (1.2, 0.05, 20.0, math.radians(0.1), -math.radians(0.05))


def _case(seed=21, nss=64, nsb=512, rdeg=4.0, n=4000, interp=False):
    import torch

    from pisco4cmb_gb300 import GPUConvolver, Sky, beam_npix_for_radius

    rng = np.random.default_rng(seed)
    npb = beam_npix_for_radius(nsb, math.radians(rdeg))
    conv = GPUConvolver(form="tuned")
    sky = rng.normal(size=(3, 12 * nss * nss)).astype(np.float32)
    conv.update_sky(Sky(nss, sky[0], sky[1], sky[2], None))
    ab = torch.empty((npb, 8), dtype=torch.float32, device="cuda")
    conv.gaussian_beam_device(nsb, npb, 0.01, nss, *PARAMS, ab.data_ptr(), set_beam=True)
    ra = rng.uniform(0, 2 * np.pi, n)
    dec = np.arcsin(rng.uniform(-1, 1, n))
    dec[:40] = np.pi / 2 - rng.uniform(0, math.radians(rdeg), 40)
    pa = rng.uniform(0, np.pi, n)
    t = [torch.tensor(x, device="cuda") for x in (ra, dec, pa)]
    conv.set_scan_device(n, *[x.data_ptr() for x in t])
    conv.set_interp(interp)
    g = [torch.tensor(rng.normal(size=n), device="cuda") for _ in range(2)]
    torch.cuda.synchronize()
    return conv, dict(nss=nss, nsb=nsb, npb=npb, n=n, keep=(t, g, ab), g=g)


def _two_step(conv, c):
    import torch

    npix = 12 * c["nss"] ** 2
    gs = torch.empty((npix, 4), dtype=torch.float64, device="cuda")
    gbm = torch.empty((c["npb"], 8), dtype=torch.float64, device="cuda")
    conv.adjoint_device(c["g"][0].data_ptr(), c["g"][1].data_ptr(), True, gs.data_ptr(),
                        gbm.data_ptr(), out_f64=True, deterministic=True)
    grad = torch.empty(5, dtype=torch.float64, device="cuda")
    conv.gaussian_beam_param_grad_device(c["nsb"], c["npb"], 0.01, c["nss"], *PARAMS,
                                         gbm.data_ptr(), True, grad.data_ptr())
    conv.sync()
    return gs.cpu().numpy(), grad.cpu().numpy()


def _fused(conv, c, deterministic=True, sky=True):
    import torch

    npix = 12 * c["nss"] ** 2
    gs = torch.empty((npix, 4), dtype=torch.float64, device="cuda") if sky else None
    grad = torch.empty(5, dtype=torch.float64, device="cuda")
    conv.adjoint_gaussian_device(c["g"][0].data_ptr(), c["g"][1].data_ptr(), True,
                                 gs.data_ptr() if sky else 0, grad.data_ptr(), PARAMS, 0.01,
                                 c["nss"], out_f64=True, deterministic=deterministic)
    conv.sync()
    return (gs.cpu().numpy() if sky else None), grad.cpu().numpy()


@pytest.mark.parametrize("interp", [False, True])
def test_fused_equals_two_step_path(gpu, interp):
    conv, c = _case(interp=interp)
    gs2, grad2 = _two_step(conv, c)
    gs1, grad1 = _fused(conv, c)
    assert np.array_equal(gs1, gs2)
    assert np.all(np.isfinite(grad1))
    assert np.all(np.abs(grad1 - grad2) <= 1e-4 * np.abs(grad2) + 1e-12), (grad1, grad2)
    # the same on every run, in either mode, with or without the sky gradient
    _, again = _fused(conv, c)
    _, atomic = _fused(conv, c, deterministic=False)
    _, alone = _fused(conv, c, sky=False)
    assert np.array_equal(grad1, again) and np.array_equal(grad1, atomic)
    assert np.array_equal(grad1, alone)
    conv.close()


@pytest.mark.parametrize("interp", [False, True])
def test_convolve_gaussian_against_finite_differences(gpu, interp):
    """Loss 1/2 |TOD - target|^2 through autograd.convolve_gaussian; the
    finite differences run the FP64 form on the library's model beam."""
    import torch

    from pisco4cmb_gb300 import GPUConvolver, Sky, beam_npix_for_radius, synth
    from pisco4cmb_gb300.autograd import convolve_gaussian

    nss, nsb, rdeg = 64, 512, 4.0
    npb = beam_npix_for_radius(nsb, math.radians(rdeg))
    n = 6000
    ra, dec, pa = synth.sweep_scan(n, 5, dec0=-40.0, per_sweep=600, ddec=1.0)
    sky0 = synth.grf_sky(nss, 5, dtype=np.float64)[:3].T.copy()
    conv = GPUConvolver(form="tuned")
    conv.update_sky(Sky(nss, *np.zeros((3, 12 * nss * nss), np.float32), None))
    t = [torch.tensor(x, device="cuda") for x in (ra, dec, pa)]
    conv.set_scan_device(n, *[x.data_ptr() for x in t])
    conv.set_interp(interp)
    ab = torch.empty((npb, 8), dtype=torch.float32, device="cuda")

    def tod64(p):
        s4 = torch.tensor(np.concatenate([sky0, np.zeros((sky0.shape[0], 1))], 1), device="cuda")
        conv.set_sky_device(nss, s4.data_ptr(), True)
        conv.gaussian_beam_device(nsb, npb, 0.01, nss, *p, ab.data_ptr(), set_beam=True)
        a = torch.empty(n, dtype=torch.float64, device="cuda")
        b = torch.empty(n, dtype=torch.float64, device="cuda")
        conv.forward_device(a.data_ptr(), b.data_ptr(), out_f64=True, form="fp64")
        conv.sync()
        return a.cpu().numpy(), b.cpu().numpy()

    target = list(PARAMS)
    target[0] *= 1.05
    target[3] += math.radians(0.05)
    tgt_a, tgt_b = tod64(target)

    def loss64(p):
        a, b = tod64(p)
        return 0.5 * (np.sum((a - tgt_a) ** 2) + np.sum((b - tgt_b) ** 2))

    sky_t = torch.tensor(sky0, device="cuda")
    pt = torch.tensor(PARAMS, dtype=torch.float64, device="cuda", requires_grad=True)
    ta, tb = convolve_gaussian(sky_t, pt, conv, nss, nsb, npb, 0.01)
    L = 0.5 * (((ta.double() - torch.tensor(tgt_a, device="cuda")) ** 2).sum() +
               ((tb.double() - torch.tensor(tgt_b, device="cuda")) ** 2).sum())
    L.backward()
    g = pt.grad.cpu().numpy()
    # phi0 moves a nearly circular beam (e = 0.05) only slightly: a step of
    # 1e-3 deg changes the FP32 beam map by about 15 of its rounding units, so
    # it takes 0.5 deg (central-difference truncation ~1e-4 relative)
    steps = (1e-3, 1e-3, 0.5, 1e-3 * math.radians(1.0), 1e-3 * math.radians(1.0))
    # autograd differentiates the TUNED operator, the differences the FP64 one;
    # with the bilinear lookup the small phi0 component also carries the FP32
    # stencil weights' error (measured 1.4 %), hence its wider bound
    rtol = [2e-3, 2e-3, 2e-2 if interp else 2e-3, 2e-3, 2e-3]
    for k, h in enumerate(steps):
        pp, pm = list(PARAMS), list(PARAMS)
        pp[k] += h
        pm[k] -= h
        fd = (loss64(pp) - loss64(pm)) / (2 * h)
        assert abs(fd - g[k]) <= rtol[k] * abs(fd) + 1e-9, (k, fd, g[k])
    conv.close()
