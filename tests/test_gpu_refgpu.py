"""The reference's own GPU kernels (K1 fill_pixel_matching_matrix + K2
partial_polarized_convolution, cudaConv2.cu, compiled unmodified for sm_103a
into oracle/_ref/refconv.cubin) with GPUConvolver's host pipeline
(oracle/ref_gpu_harness.cpp), against this library on the same inputs.

The reference computes chi in FP64 but stores it as float, takes cosf/sinf of
it, multiplies in float, adds 16 per-thread double partials per sample with
float atomics (order not fixed): its TOD carries ~1e-7 relative float noise,
so the tolerances are 1e-5 (rms) and 1e-4 (max) of the TOD rms.  Skipped when
the cubin was not built (it needs the reference tree at build time).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _needs_refgpu():
    import oracle

    if not oracle.refgpu_available():
        pytest.skip("reference GPU kernels not built (oracle/_ref/refconv.cubin)")
    return oracle


def _case(n, seed=7, nss=64, nsb=256, rdeg=5.0):
    import oracle as O
    from pisco4cmb_gb300 import PolBeam, synth

    rng = np.random.default_rng(seed)
    sky = rng.normal(size=(3, 12 * nss * nss)).astype(np.float32)
    npb = O.beam_npix_for_radius(nsb, np.deg2rad(rdeg))
    beam = PolBeam(nsb, npb, 0.01, "p")
    fx, fy = synth.elliptical_fwhm(2.0, 0.05)
    beam.make_unpol_gaussian_elliptical_beams(fx, fy, 30.0)
    beam.build(nss)
    ra = rng.uniform(0, 2 * np.pi, n).astype(np.float32)
    dec = np.arcsin(rng.uniform(-1, 1, n)).astype(np.float32)
    dec[:40] = np.float32(np.pi / 2 - 0.01)  # near the pole
    pa = rng.uniform(0, np.pi, n).astype(np.float32)
    return sky, beam, ra, dec, pa, nss, nsb


def _ours(sky, beam, ra, dec, pa, nss, form):
    from pisco4cmb_gb300 import GPUConvolver, Scan, Sky

    c = GPUConvolver(form=form)
    c.update_sky(Sky(nss, sky[0], sky[1], sky[2], None))
    c.update_beam(beam)
    c.update_scan(Scan(ra.size, ra, dec, pa))
    a = np.zeros(ra.size, np.float64)
    b = np.zeros(ra.size, np.float64)
    c.exec_convolution(a, b)
    c.close()
    return a, b


@pytest.mark.parametrize("form", ["plain", "tuned"])
def test_reference_kernels_match(form):
    O = _needs_refgpu()
    sky, beam, ra, dec, pa, nss, nsb = _case(4096 + 300)
    ba, bb = beam.planes()
    ra_, rb_, _ = O.refgpu_convolve(ra, dec, pa, nss, sky, nsb, ba, bb)
    assert ra_.size == 4096  # the reference drops the n % ptgPerConv tail
    a, b = _ours(sky, beam, ra[:4096], dec[:4096], pa[:4096], nss, form)
    rms = float(np.sqrt(np.mean(a ** 2)))
    for mine, ref in ((a, ra_), (b, rb_)):
        d = mine - ref.astype(np.float64)
        assert np.sqrt(np.mean(d ** 2)) <= 1e-5 * rms
        assert np.abs(d).max() <= 1e-4 * rms


def test_reference_pipeline_rejects_nonuniform_chunks():
    """ptgPerConv not a multiple of 2048 would make K2's barriers divergent:
    the harness refuses before any launch."""
    O = _needs_refgpu()
    sky, beam, ra, dec, pa, nss, nsb = _case(3000)
    ba, bb = beam.planes()
    with pytest.raises(RuntimeError):
        O.refgpu_convolve(ra, dec, pa, nss, sky, nsb, ba, bb, ptg_per_conv=1000)
