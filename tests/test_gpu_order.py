"""Sky-ordered processing (GPU): sorting a launch's samples by sky cell must
leave every TOD value, and the deterministic adjoint, bit for bit unchanged
(every form, host and device entry points, sample sub-ranges, chunked host
calls, a re-set scan, batched descriptors)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NSS, NSB = 64, 256


def _inputs(n, seed):
    import oracle as O
    from pisco4cmb_gb300 import PolBeam, synth

    rng = np.random.default_rng(seed)
    sky = rng.normal(size=(3, 12 * NSS * NSS)).astype(np.float32)
    npb = O.beam_npix_for_radius(NSB, np.deg2rad(4.0))
    beam = PolBeam(NSB, npb, 0.01, "p")
    fx, fy = synth.elliptical_fwhm(1.6, 0.05)
    beam.make_unpol_gaussian_elliptical_beams(fx, fy, 20.0)
    beam.build(NSS)
    # random pointings in time order: neighbouring samples far apart on the sky
    ra = rng.uniform(0, 2 * np.pi, n)
    dec = np.arcsin(rng.uniform(-1, 1, n))
    dec[:16] = np.pi / 2 - rng.uniform(0, 0.03, 16)
    pa = rng.uniform(-np.pi, np.pi, n)
    return sky, beam, ra, dec, pa


def _conv(form, sky, beam, ra, dec, pa, order, ptg=1 << 20):
    from pisco4cmb_gb300 import GPUConvolver, RunConfig, Scan, Sky

    c = GPUConvolver(RunConfig(ptgPerConv=ptg), form=form)
    c.update_sky(Sky(NSS, sky[0], sky[1], sky[2], None))
    c.update_beam(beam)
    c.update_scan(Scan(len(ra), ra, dec, pa))
    c.set_sample_order(order)
    return c


@pytest.mark.parametrize("bilinear", [False, True])
@pytest.mark.parametrize("form", ["tuned", "plain", "fp64"])
def test_sky_order_host_forward_bit_identical(gpu, form, bilinear):
    sky, beam, ra, dec, pa = _inputs(3000, 11)
    out = {}
    for order in ("scan", "sky"):
        for ptg in (1 << 20, 700):  # one chunk, and chunks each sorted on their own
            c = _conv(form, sky, beam, ra, dec, pa, order, ptg)
            c.set_interp(bilinear)
            a = np.zeros(len(ra), np.float64)
            b = np.zeros(len(ra), np.float64)
            c.exec_convolution(a, b)
            out[(order, ptg)] = (a, b)
    ref = out[("scan", 1 << 20)]
    for key, (a, b) in out.items():
        assert np.array_equal(a, ref[0]) and np.array_equal(b, ref[1]), key


def test_sky_order_device_ranges_and_rescan(gpu):
    import torch

    sky, beam, ra, dec, pa = _inputs(5000, 12)
    scan_c = _conv("tuned", sky, beam, ra, dec, pa, "scan")
    sky_c = _conv("tuned", sky, beam, ra, dec, pa, "sky")

    def run(c, begin, n):
        o = [torch.full((n,), float("nan"), dtype=torch.float32, device="cuda") for _ in range(2)]
        c.forward_device(o[0].data_ptr(), o[1].data_ptr(), begin=begin, n=n)
        c.sync()
        return [x.cpu().numpy() for x in o]

    for begin, n in ((0, 5000), (123, 1000), (4000, 1000), (123, 1000), (0, 1)):
        x, y = run(scan_c, begin, n), run(sky_c, begin, n)
        assert np.array_equal(x[0], y[0]) and np.array_equal(x[1], y[1]), (begin, n)
    # a new scan of the same length must not reuse the old order's result
    from pisco4cmb_gb300 import Scan

    _, _, ra2, dec2, pa2 = _inputs(5000, 13)
    for c in (scan_c, sky_c):
        c.update_scan(Scan(5000, ra2, dec2, pa2))
    x, y = run(scan_c, 0, 5000), run(sky_c, 0, 5000)
    assert np.array_equal(x[0], y[0]) and np.array_equal(x[1], y[1])


def test_sky_order_adjoint(gpu):
    import torch

    sky, beam, ra, dec, pa = _inputs(4000, 14)
    rng = np.random.default_rng(3)
    ga = torch.tensor(rng.normal(size=len(ra)), dtype=torch.float32, device="cuda")
    gb = torch.tensor(rng.normal(size=len(ra)), dtype=torch.float32, device="cuda")
    res = {}
    for order in ("scan", "sky"):
        c = _conv("tuned", sky, beam, ra, dec, pa, order)
        for det in (True, False):
            g = torch.zeros((12 * NSS * NSS, 4), dtype=torch.float64, device="cuda")
            c.adjoint_device(ga.data_ptr(), gb.data_ptr(), False, g.data_ptr(), 0, out_f64=True,
                             deterministic=det)
            c.sync()
            res[(order, det)] = g.cpu().numpy()
    assert np.array_equal(res[("scan", True)], res[("sky", True)])
    scale = np.abs(res[("scan", True)]).max()
    assert np.abs(res[("sky", False)] - res[("scan", True)]).max() <= 1e-5 * scale


def test_sky_order_batched_bit_identical(gpu):
    import torch

    from pisco4cmb_gb300 import GPUConvolver, Sky

    conv = GPUConvolver(form="tuned")
    rows, outs = [], {}
    keep = []
    for d, seed in enumerate((21, 22, 23)):
        sky, beam, ra, dec, pa = _inputs(1500 + 700 * d, seed)
        if d == 0:
            conv.update_sky(Sky(NSS, sky[0], sky[1], sky[2], None))
        conv.set_beam_slot(d, beam)
        t = [torch.tensor(x, device="cuda") for x in (ra, dec, pa)]
        o = [torch.full((len(ra),), float("nan"), device="cuda") for _ in range(2)]
        keep.append((t, o))
        rows.append((d, len(ra), t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr(),
                     o[0].data_ptr(), o[1].data_ptr()))
    for sky_order in (False, True):
        descs = conv.det_descs(rows, sky_order=sky_order)
        for _ in range(2):  # capture, then graph replay
            conv.forward_batched(descs, chunk=64)
        conv.sync()
        outs[sky_order] = [[x.cpu().numpy().copy() for x in k[1]] for k in keep]
    for d in range(3):
        for k in range(2):
            assert np.array_equal(outs[False][d][k], outs[True][d][k]), (d, k)
