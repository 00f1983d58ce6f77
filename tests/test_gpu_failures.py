"""Host-side failure paths of the context (GPU, no fault of any kind).

The reference sizes its device buffers from RunConfig.maxMemUsage and
refuses a configuration that does not fit (gpuconvolver.cu:58-70, 74-78);
CUDA errors there end the process (gpuconvolver.cu:8-32).  Here a request
beyond maxMemUsage returns PISCO_ERR_OUT_OF_MEMORY with a message, before
any device memory is touched, and the context stays usable: its previous
sky is still in place and later, smaller inputs work as in a fresh context.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(nss, seed=7, n=1500):
    from pisco4cmb_gb300 import PolBeam, Scan, Sky, beam_npix_for_radius

    rng = np.random.default_rng(seed)
    sky = rng.normal(size=(3, 12 * nss * nss)).astype(np.float32)
    nsb = 128
    beam = PolBeam(nsb, beam_npix_for_radius(nsb, np.deg2rad(4.0)), 0.01, "p")
    beam.make_unpol_gaussian_elliptical_beams(1.6, 1.5, 10.0)
    beam.build(nss)
    ra = rng.uniform(0, 2 * np.pi, n)
    dec = np.arcsin(rng.uniform(-1, 1, n))
    pa = rng.uniform(0, np.pi, n)
    return Sky(nss, sky[0], sky[1], sky[2], None), beam, Scan(n, ra, dec, pa)


def _run(conv, n):
    a = np.zeros(n)
    b = np.zeros(n)
    conv.exec_convolution(a, b)
    return a, b


def test_max_mem_usage_refusal_leaves_context_usable(gpu):
    from pisco4cmb_gb300 import GPUConvolver, PiscoError, RunConfig
    from pisco4cmb_gb300 import _lib

    sky64, beam, scan = _inputs(64)
    n = scan.get_nsamples()
    # 8 MB: the ring table (2.1 MB), an nside-64 sky (0.8 MB), beam, scan and
    # TOD fit; an nside-512 sky (50 MB) does not
    conv = GPUConvolver(RunConfig(maxMemUsage=8 << 20, ptgPerConv=4096), form="tuned")
    conv.update_beam(beam)
    conv.update_sky(sky64)
    conv.update_scan(scan)
    a0, b0 = _run(conv, n)
    assert np.all(np.isfinite(a0)) and np.all(np.isfinite(b0))

    big, _, _ = _inputs(512)
    with pytest.raises(PiscoError) as ei:
        conv.update_sky(big)
    assert ei.value.status == _lib.PISCO_ERR_OUT_OF_MEMORY
    assert "maxMemUsage" in str(ei.value)

    # the refused call touched nothing: the same TOD, bit for bit
    a1, b1 = _run(conv, n)
    assert np.array_equal(a0, a1) and np.array_equal(b0, b1)

    # a smaller sky still fits and gives what a context without a limit gives
    sky32, _, _ = _inputs(32)
    conv.update_sky(sky32)
    a2, b2 = _run(conv, n)
    conv.close()
    ref = GPUConvolver(form="tuned")
    ref.update_beam(beam)
    ref.update_sky(sky32)
    ref.update_scan(scan)
    a3, b3 = _run(ref, n)
    ref.close()
    assert np.array_equal(a2, a3) and np.array_equal(b2, b3)


def test_config_below_one_chunk_is_refused(gpu):
    from pisco4cmb_gb300 import GPUConvolver, PiscoInvalidArgument, RunConfig
    from pisco4cmb_gb300 import _lib

    conv = GPUConvolver(RunConfig(maxMemUsage=1024, ptgPerConv=4096))
    with pytest.raises(PiscoInvalidArgument) as ei:
        conv.configure_execution()
    assert ei.value.status == _lib.PISCO_ERR_INVALID_CONFIG
