"""Analytic beam-parameter gradient of the C ABI (pisco_beam_gaussian_param_grad)
against torch autograd of the differentiable Gaussian PolBeam (CPU)."""
import numpy as np
import pytest


@pytest.mark.parametrize("params", [(1.5, 0.05, 20.0, 0.0, 0.0), (2.0, -0.1, 130.0, 0.003, -0.002)])
def test_param_grad_matches_autograd(params):
    torch = pytest.importorskip("torch")
    from pisco4cmb_gb300 import beam_npix_for_radius, gaussian_beam_param_grad
    from pisco4cmb_gb300.autograd import beam_pixel_coords, gaussian_polbeam

    nsb, nss, eps = 256, 64, 0.01
    npix = beam_npix_for_radius(nsb, np.deg2rad(5.0))
    rho, sig = beam_pixel_coords(nsb, npix, device="cpu")
    th = [torch.tensor(v, dtype=torch.float64, requires_grad=True) for v in params]
    beam = gaussian_polbeam(rho, sig, th[0], th[1], th[2], th[3], th[4], epsilon=eps,
                            nside_sky=nss, nside_beam=nsb)
    gbeam = np.random.default_rng(3).normal(size=(npix, 8))
    (beam * torch.tensor(gbeam)).sum().backward()
    ref = np.array([t.grad.item() for t in th])
    mine = gaussian_beam_param_grad(nsb, npix, eps, nss, *params, gbeam)
    assert np.allclose(mine, ref, rtol=1e-9, atol=1e-12 * np.abs(ref).max()), (mine, ref)
