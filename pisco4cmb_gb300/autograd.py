"""PyTorch autograd binding (the pypisco path of the benchmark spec).

``convolve(sky, beam_ab, conv)`` is a ``torch.autograd.Function``: forward =
the TUNED GPU forward through the C ABI, backward = its exact transpose
(``pisco_adjoint_device``), giving dL/dsky (I, Q, U, V) and dL/dbeam (the
eight beam maps).  ``gaussian_polbeam`` builds the PolBeam maps of an
elliptical Gaussian beam with torch operations (the arithmetic of
``make_unpol_gaussian_elliptical_beams`` + ``build``, src/Polbeam/polbeam.cpp:
186-288, 290-372), with a pointing offset (dx, dy) of the beam centre, so
that gradients with respect to FWHM, ellipticity and pointing offset follow
by recomputing the beam weights: dL/dparam = sum_b dL/dbeam_b dbeam_b/dparam.
No per-pair weights are stored.  ``gaussian_beam`` is the same model as a
``torch.autograd.Function`` on the library's kernels (beam built on the GPU
by ``pisco_beam_gaussian_device``, gradient reduced by
``pisco_beam_gaussian_param_grad_device``), for fitting loops that should not
run the beam through torch operations.  ``convolve_gaussian(sky, params,
conv, ...)`` goes one step further: its backward forms dL/dparams inside the
adjoint (``pisco_adjoint_gaussian_device``), weighting each pair by the
model's weight and derivatives recomputed at its beam pixel, so no beam-map
gradient is accumulated at all.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from .api import GPUConvolver, pix2ang

__all__ = ["convolve", "convolve_gaussian", "gaussian_polbeam", "gaussian_beam",
           "beam_pixel_coords", "ConvolveFn", "ConvolveGaussianFn", "GaussianBeamFn"]


def _torch_stream(device=None) -> int:
    """Handle of torch's current stream for the C ABI.  torch reports its
    default (legacy) stream as 0, which the C ABI would take as "the
    context's own stream" (non-blocking, unordered with torch's work), so it
    is passed as cudaStreamLegacy (1) instead."""
    return torch.cuda.current_stream(device).cuda_stream or 1


class ConvolveFn(torch.autograd.Function):
    """TOD (a, b) = A(sky, beam) with the pointing fixed on ``conv``."""

    @staticmethod
    def forward(ctx, sky, beam_ab, conv: GPUConvolver, nside_sky: int, nside_beam: int,
                deterministic: bool):
        if not (sky.is_cuda and beam_ab.is_cuda):
            raise ValueError("sky and beam must be CUDA tensors")
        sky4 = _as_iquv(sky)
        bab = beam_ab.detach().to(torch.float32).contiguous()
        stream = _torch_stream()
        conv.set_sky_device(nside_sky, sky4.data_ptr(), False, stream=stream)
        conv.set_beam_device(nside_beam, bab.shape[0], bab.data_ptr(), False, stream=stream)
        n = conv._n
        out_dt = torch.float64 if sky.dtype == torch.float64 else torch.float32
        ta = torch.empty(n, dtype=out_dt, device=sky.device)
        tb = torch.empty(n, dtype=out_dt, device=sky.device)
        conv.forward_device(ta.data_ptr(), tb.data_ptr(), out_f64=out_dt == torch.float64,
                            stream=stream, form="tuned")
        ctx.save_for_backward(sky4, bab)
        ctx.conv = conv
        ctx.meta = (nside_sky, nside_beam, deterministic, sky.shape, sky.dtype, beam_ab.dtype)
        return ta, tb

    @staticmethod
    def backward(ctx, ga, gb):
        sky4, bab = ctx.saved_tensors
        conv = ctx.conv
        nside_sky, nside_beam, det, sky_shape, sky_dtype, beam_dtype = ctx.meta
        stream = _torch_stream()
        # the context may have been reused since the forward: restore its inputs
        conv.set_sky_device(nside_sky, sky4.data_ptr(), False, stream=stream)
        conv.set_beam_device(nside_beam, bab.shape[0], bab.data_ptr(), False, stream=stream)
        n = conv._n
        ga = (ga if ga is not None else torch.zeros(n, device=sky4.device)).contiguous()
        gb = (gb if gb is not None else torch.zeros(n, device=sky4.device)).contiguous()
        g64 = ga.dtype == torch.float64
        gb = gb.to(ga.dtype)
        want_sky = ctx.needs_input_grad[0]
        want_beam = ctx.needs_input_grad[1]
        gsky = torch.empty((sky4.shape[0], 4), dtype=torch.float64, device=sky4.device) if want_sky else None
        gbeam = torch.empty((bab.shape[0], 8), dtype=torch.float64, device=sky4.device) if want_beam else None
        if want_sky or want_beam:
            # an I, Q, U sky has no V gradient to accumulate
            iqu = len(sky_shape) == 2 and 3 in tuple(sky_shape)
            conv.adjoint_device(ga.data_ptr(), gb.data_ptr(), g64,
                                gsky.data_ptr() if gsky is not None else 0,
                                gbeam.data_ptr() if gbeam is not None else 0, out_f64=True,
                                deterministic=det, stream=stream, sky_iqu=iqu)
        if gsky is not None:
            gsky = _like_sky(gsky, sky_shape).to(sky_dtype)
        if gbeam is not None:
            gbeam = gbeam.to(beam_dtype)
        return gsky, gbeam, None, None, None, None


def _as_iquv(sky: torch.Tensor) -> torch.Tensor:
    """(npix, 4) float32 contiguous from (npix, 3|4) or (3|4, npix)."""
    s = sky.detach()
    if s.dim() != 2:
        raise ValueError("sky must be 2-D")
    if s.shape[0] in (3, 4) and s.shape[1] > 4:
        s = s.t()
    if s.shape[1] == 3:
        s = torch.cat([s, torch.zeros_like(s[:, :1])], dim=1)
    return s.to(torch.float32).contiguous()


def _like_sky(g4: torch.Tensor, shape) -> torch.Tensor:
    if shape[0] in (3, 4) and shape[1] > 4:
        return g4[:, : shape[0]].t().contiguous()
    return g4[:, : shape[1]].contiguous()


def convolve(sky: torch.Tensor, beam_ab: torch.Tensor, conv: GPUConvolver, nside_sky: int,
             nside_beam: int, deterministic: bool = True):
    """Differentiable TUNED forward: returns (tod_a, tod_b)."""
    return ConvolveFn.apply(sky, beam_ab, conv, nside_sky, nside_beam, deterministic)


def beam_pixel_coords(nside_beam: int, npix: int, device="cuda"):
    """(rho, sigma) of the beam grid's pixel centres, as float64 tensors."""
    th, ph = pix2ang(nside_beam, np.arange(npix))
    return (torch.tensor(th, dtype=torch.float64, device=device),
            torch.tensor(ph, dtype=torch.float64, device=device))


def gaussian_polbeam(rho, sigma, fwhm_deg, ellipticity, phi0_deg=0.0, dx=0.0, dy=0.0,
                     epsilon=0.01, nside_sky=1, nside_beam=1):
    """npixB x 8 (a.IQUV, b.IQUV) beam maps of an elliptical Gaussian pair.

    Same arithmetic as PolBeam::make_unpol_gaussian_elliptical_beams +
    build(nsideSky) for a co-polar pair (tilde I = tilde Q = gaussian, tilde
    U = tilde V = 0; a = ((1+eps) G, (1-eps) G, 0, 0) / Na with
    Na = sum(G) (nsideSky/nsideBeam)^2, and b likewise), with the beam centre
    offset by (dx, dy) radians in the beam plane (x = rho cos sigma,
    y = rho sin sigma) and fwhm_x = F sqrt((1+e)/(1-e)),
    fwhm_y = F sqrt((1-e)/(1+e)).  Every parameter may be a tensor that
    requires grad.
    """
    t = lambda v: v if torch.is_tensor(v) else torch.tensor(float(v), dtype=torch.float64,  # noqa: E731
                                                            device=rho.device)
    F, e, p0, dx, dy = t(fwhm_deg), t(ellipticity), t(phi0_deg), t(dx), t(dy)
    d2r = math.pi / 180.0
    fx = F * torch.sqrt((1 + e) / (1 - e))
    fy = F * torch.sqrt((1 - e) / (1 + e))
    sx = d2r * fx / 2.35482
    sy = d2r * fy / 2.35482
    ph = d2r * p0
    ca = torch.cos(ph) ** 2 / (2 * sx * sx) + torch.sin(ph) ** 2 / (2 * sy * sy)
    cb = -torch.sin(2 * ph) / (4 * sx * sx) + torch.sin(2 * ph) / (4 * sy * sy)
    cc = torch.sin(ph) ** 2 / (2 * sx * sx) + torch.cos(ph) ** 2 / (2 * sy * sy)
    x = rho * torch.cos(sigma) - dx
    y = rho * torch.sin(sigma) - dy
    g = torch.exp(-(ca * x * x + 2.0 * cb * x * y + cc * y * y))
    ocmp = (nside_sky / float(nside_beam)) ** 2
    norm = g.sum() * ocmp
    z = torch.zeros_like(g)
    a = torch.stack([(1 + epsilon) * g, (1 - epsilon) * g, z, z], dim=1) / norm
    return torch.cat([a, a], dim=1)


class GaussianBeamFn(torch.autograd.Function):
    """beam_ab (npixB x 8 float32, a.IQUV b.IQUV) of the elliptical Gaussian
    pair model from params = (fwhm_deg, ellipticity, phi0_deg, dx, dy)."""

    @staticmethod
    def forward(ctx, params, conv: GPUConvolver, nside_beam: int, npix: int, epsilon: float,
                nside_sky: int):
        if params.numel() != 5:
            raise ValueError("params must hold (fwhm_deg, ellipticity, phi0_deg, dx, dy)")
        p = [float(v) for v in params.detach().double().cpu().tolist()]
        dev = torch.device("cuda", conv.cfg.deviceId)
        out = torch.empty((int(npix), 8), dtype=torch.float32, device=dev)
        stream = _torch_stream(dev)
        conv.gaussian_beam_device(nside_beam, npix, epsilon, nside_sky, *p, out.data_ptr(),
                                  set_beam=False, stream=stream)
        ctx.conv = conv
        ctx.meta = (nside_beam, npix, epsilon, nside_sky, p, params.dtype, params.device, dev)
        return out

    @staticmethod
    def backward(ctx, gbeam):
        nside_beam, npix, epsilon, nside_sky, p, dtype, pdev, dev = ctx.meta
        g = gbeam.to(dev)
        if g.dtype not in (torch.float32, torch.float64):
            g = g.to(torch.float64)
        g = g.contiguous()
        out = torch.empty(5, dtype=torch.float64, device=dev)
        stream = _torch_stream(dev)
        ctx.conv.gaussian_beam_param_grad_device(nside_beam, npix, epsilon, nside_sky, *p,
                                                 g.data_ptr(), g.dtype == torch.float64,
                                                 out.data_ptr(), stream=stream)
        return out.to(device=pdev, dtype=dtype), None, None, None, None, None


class ConvolveGaussianFn(torch.autograd.Function):
    """TOD (a, b) of a sky and the elliptical Gaussian pair beam of params =
    (fwhm_deg, ellipticity, phi0_deg, dx, dy), the beam built on the GPU.
    The backward forms dL/dparams in the adjoint itself
    (pisco_adjoint_gaussian_device): the model's weights and derivatives are
    recomputed from the parameters at the beam pixels, and no beam-map
    gradient is formed."""

    @staticmethod
    def forward(ctx, sky, params, conv: GPUConvolver, nside_sky: int, nside_beam: int, npix: int,
                epsilon: float, deterministic: bool):
        if not sky.is_cuda:
            raise ValueError("sky must be a CUDA tensor")
        if params.numel() != 5:
            raise ValueError("params must hold (fwhm_deg, ellipticity, phi0_deg, dx, dy)")
        p = [float(v) for v in params.detach().double().cpu().tolist()]
        sky4 = _as_iquv(sky)
        stream = _torch_stream(sky.device)
        bab = torch.empty((int(npix), 8), dtype=torch.float32, device=sky.device)
        conv.set_sky_device(nside_sky, sky4.data_ptr(), False, stream=stream)
        conv.gaussian_beam_device(nside_beam, npix, epsilon, nside_sky, *p, bab.data_ptr(),
                                  set_beam=True, stream=stream)
        n = conv._n
        out_dt = torch.float64 if sky.dtype == torch.float64 else torch.float32
        ta = torch.empty(n, dtype=out_dt, device=sky.device)
        tb = torch.empty(n, dtype=out_dt, device=sky.device)
        conv.forward_device(ta.data_ptr(), tb.data_ptr(), out_f64=out_dt == torch.float64,
                            stream=stream, form="tuned")
        ctx.save_for_backward(sky4, bab)
        ctx.conv = conv
        ctx.meta = (nside_sky, nside_beam, int(npix), float(epsilon), deterministic, p,
                    sky.shape, sky.dtype, params.dtype, params.device)
        return ta, tb

    @staticmethod
    def backward(ctx, ga, gb):
        sky4, bab = ctx.saved_tensors
        conv = ctx.conv
        nside_sky, nside_beam, npix, eps, det, p, sky_shape, sky_dtype, pdt, pdev = ctx.meta
        stream = _torch_stream(sky4.device)
        conv.set_sky_device(nside_sky, sky4.data_ptr(), False, stream=stream)
        conv.set_beam_device(nside_beam, npix, bab.data_ptr(), False, stream=stream)
        n = conv._n
        ga = (ga if ga is not None else torch.zeros(n, device=sky4.device)).contiguous()
        gb = (gb if gb is not None else torch.zeros(n, device=sky4.device)).contiguous()
        g64 = ga.dtype == torch.float64
        gb = gb.to(ga.dtype)
        want_sky = ctx.needs_input_grad[0]
        gsky = torch.empty((sky4.shape[0], 4), dtype=torch.float64, device=sky4.device) if want_sky else None
        grad = torch.empty(5, dtype=torch.float64, device=sky4.device)
        iqu = len(sky_shape) == 2 and 3 in tuple(sky_shape)
        conv.adjoint_gaussian_device(ga.data_ptr(), gb.data_ptr(), g64,
                                     gsky.data_ptr() if gsky is not None else 0, grad.data_ptr(),
                                     p, eps, nside_sky, out_f64=True, deterministic=det,
                                     stream=stream, sky_iqu=iqu)
        if gsky is not None:
            gsky = _like_sky(gsky, sky_shape).to(sky_dtype)
        gp = grad.to(device=pdev, dtype=pdt) if ctx.needs_input_grad[1] else None
        return gsky, gp, None, None, None, None, None, None


def convolve_gaussian(sky: torch.Tensor, params: torch.Tensor, conv: GPUConvolver, nside_sky: int,
                      nside_beam: int, npix: int, epsilon: float = 0.01,
                      deterministic: bool = True):
    """Differentiable TUNED forward with the Gaussian pair beam of ``params``
    (fwhm_deg, ellipticity, phi0_deg, dx, dy): returns (tod_a, tod_b); the
    parameter gradient comes from the fused adjoint."""
    return ConvolveGaussianFn.apply(sky, params, conv, nside_sky, nside_beam, npix, epsilon,
                                    deterministic)


def gaussian_beam(params: torch.Tensor, conv: GPUConvolver, nside_beam: int, npix: int,
                  epsilon: float = 0.01, nside_sky: int = 1) -> torch.Tensor:
    """Differentiable Gaussian pair beam built by the library's kernels."""
    return GaussianBeamFn.apply(params, conv, nside_beam, npix, epsilon, nside_sky)
