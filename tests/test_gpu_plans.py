"""Sample plans of the TUNED forward (GPU).

The TUNED forward builds each sample's FP64 geometry (its disc's rings and
edge constants, the boresight frame, the psi phasors) either in a separate
kernel with one thread per sample, into scratch the context keeps, or in
the pair kernel's own warp.  The scratch counts against
RunConfig.maxMemUsage (gpuconvolver.cu:58-70 is the reference's check of
its buffers against it): with room for fewer plans than samples the
forward runs in chunks, with room for fewer than 1024 plans the warps plan
their own samples.  All three give the same TOD bit for bit, for both beam
lookups, with non-finite pointings and pole pointings in the scan, and the
scratch never takes the context beyond maxMemUsage.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PLAN_BYTES = 96


def _setup(conv, nss=128, n=20000, seed=11):
    import torch

    from pisco4cmb_gb300 import PolBeam, Sky, beam_npix_for_radius

    rng = np.random.default_rng(seed)
    sky = rng.normal(size=(3, 12 * nss * nss)).astype(np.float32)
    nsb = 512
    beam = PolBeam(nsb, beam_npix_for_radius(nsb, np.deg2rad(2.5)), 0.01, "p")
    beam.make_unpol_gaussian_elliptical_beams(1.1, 0.9, 20.0)
    beam.build(nss)
    ra = rng.uniform(0, 2 * np.pi, n)
    dec = np.arcsin(rng.uniform(-1, 1, n))
    pa = rng.uniform(0, np.pi, n)
    dec[:6] = [np.pi / 2, -np.pi / 2, np.pi / 2 - 1e-9, -np.pi / 2 + 3e-4, 0.0, 1.2]
    dec[7], ra[8], pa[9] = np.nan, np.inf, np.nan
    conv.update_sky(Sky(nss, sky[0], sky[1], sky[2], None))
    conv.update_beam(beam)
    t = [torch.tensor(v, device="cuda") for v in (ra, dec, pa)]
    conv.set_scan_device(n, *[v.data_ptr() for v in t])
    conv._test_scan = t
    return n


def _tod(conv, n, interp):
    import torch

    conv.set_interp(interp)
    a = torch.empty(n, dtype=torch.float64, device="cuda")
    b = torch.empty(n, dtype=torch.float64, device="cuda")
    conv.forward_device(a.data_ptr(), b.data_ptr(), out_f64=True)
    conv.sync()
    return a.cpu().numpy(), b.cpu().numpy()


@pytest.mark.parametrize("interp", [False, True])
def test_planned_chunked_and_unplanned_forward_agree(gpu, interp):
    from pisco4cmb_gb300 import GPUConvolver, RunConfig

    free = GPUConvolver(form="tuned")
    n = _setup(free)
    before = free.memory_used()
    ra_, rb_ = _tod(free, n, interp)
    # one chunk: the whole scan's plans were allocated
    assert free.memory_used() - before == PLAN_BYTES * n
    free.close()
    assert np.isnan(ra_[7]) and np.isnan(ra_[8]) and np.isnan(rb_[9])
    assert np.isfinite(np.delete(ra_, [7, 8, 9])).all()

    for room, chunks in ((6000, 4), (20000, 1), (1000, 0)):
        conv = GPUConvolver(RunConfig(maxMemUsage=before + PLAN_BYTES * room, ptgPerConv=4096),
                            form="tuned")
        _setup(conv)
        assert conv.memory_used() == before
        a, b = _tod(conv, n, interp)
        used = conv.memory_used()
        conv.close()
        # scratch for min(room, n) plans, none below 1024 plans of room
        assert used - before == (PLAN_BYTES * min(room, n) if chunks else 0), (room, used - before)
        assert np.array_equal(a, ra_, equal_nan=True), (room, np.nanmax(np.abs(a - ra_)))
        assert np.array_equal(b, rb_, equal_nan=True), room


def test_short_scans_and_sub_ranges_use_the_same_plans(gpu):
    """Fewer samples than the minimum plan count, and sub-ranges of the scan
    (begin > 0), give the full forward's TOD."""
    import torch

    from pisco4cmb_gb300 import GPUConvolver

    conv = GPUConvolver(form="tuned")
    n = _setup(conv, n=3000, seed=5)
    ra_, rb_ = _tod(conv, n, False)
    for begin, m in ((0, 500), (1234, 77), (2999, 1)):
        a = torch.empty(m, dtype=torch.float64, device="cuda")
        b = torch.empty(m, dtype=torch.float64, device="cuda")
        conv.forward_device(a.data_ptr(), b.data_ptr(), out_f64=True, begin=begin, n=m)
        conv.sync()
        assert np.array_equal(a.cpu().numpy(), ra_[begin:begin + m], equal_nan=True)
        assert np.array_equal(b.cpu().numpy(), rb_[begin:begin + m], equal_nan=True)
    conv.close()


def test_forwards_on_two_streams_share_the_plan_scratch(gpu):
    """Two forwards of one context on different streams, back to back with
    no host synchronisation: the second waits for the first's use of the
    plan scratch, and both give the single-stream TOD."""
    import torch

    from pisco4cmb_gb300 import GPUConvolver

    conv = GPUConvolver(form="tuned")
    n = _setup(conv, n=40000, seed=9)
    ref = _tod(conv, n, False)
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    outs = []
    for st, (b0, m) in ((s1, (0, n)), (s2, (n // 3, n - n // 3)), (s1, (5, 1000))):
        a = torch.empty(m, dtype=torch.float64, device="cuda")
        b = torch.empty(m, dtype=torch.float64, device="cuda")
        conv.forward_device(a.data_ptr(), b.data_ptr(), out_f64=True, begin=b0, n=m,
                            stream=st.cuda_stream)
        outs.append((b0, m, a, b))
    torch.cuda.synchronize()
    conv.sync()
    for b0, m, a, b in outs:
        assert np.array_equal(a.cpu().numpy(), ref[0][b0:b0 + m], equal_nan=True)
        assert np.array_equal(b.cpu().numpy(), ref[1][b0:b0 + m], equal_nan=True)
    conv.close()


def test_plan_scratch_yields_to_inputs_under_max_mem_usage(gpu):
    """Under a maxMemUsage limit the plan scratch gives way to a larger input:
    the input is accepted, the next forward plans within what is left (here
    in chunks), and its TOD equals that of a context without a limit."""
    import torch

    from pisco4cmb_gb300 import GPUConvolver, RunConfig, Sky

    free = GPUConvolver(form="tuned")
    n = _setup(free)
    before = free.memory_used()
    free.close()
    conv = GPUConvolver(RunConfig(maxMemUsage=before + PLAN_BYTES * n, ptgPerConv=4096),
                        form="tuned")
    _setup(conv)
    _tod(conv, n, False)
    assert conv.memory_used() == before + PLAN_BYTES * n  # the scratch filled the room
    # a larger sky: 12 * 160^2 * 16 B, 1.8 MB more than nside 128, fits only without the scratch
    rng = np.random.default_rng(21)
    nss = 160
    sky = rng.normal(size=(3, 12 * nss * nss)).astype(np.float32)
    conv.update_sky(Sky(nss, sky[0], sky[1], sky[2], None))
    assert conv.memory_used() <= before + PLAN_BYTES * n
    a, b = _tod(conv, n, False)
    assert conv.memory_used() <= before + PLAN_BYTES * n
    conv.close()
    ref = GPUConvolver(form="tuned")
    _setup(ref)
    ref.update_sky(Sky(nss, sky[0], sky[1], sky[2], None))
    ra_, rb_ = _tod(ref, n, False)
    ref.close()
    assert np.array_equal(a, ra_, equal_nan=True) and np.array_equal(b, rb_, equal_nan=True)


def test_adjoint_takes_its_plans_after_its_other_buffers(gpu):
    """The DETERMINISTIC adjoint allocates its fixed-point sky accumulator in
    the call; under a maxMemUsage limit that the forward's plan scratch has
    filled, that allocation frees the scratch, and the adjoint must take its
    plans only afterwards (here: no room for them, so its warps plan).  The
    gradient equals that of a context without a limit, bit for bit."""
    import torch

    from pisco4cmb_gb300 import GPUConvolver, RunConfig

    nss = 128
    npix = 12 * nss * nss
    free = GPUConvolver(form="tuned")
    n = _setup(free, nss=nss)
    before = free.memory_used()
    rng = np.random.default_rng(4)
    g = [torch.tensor(rng.normal(size=n), device="cuda") for _ in range(2)]

    def adjoint(conv):
        out = torch.zeros((npix, 4), dtype=torch.float64, device="cuda")
        conv.adjoint_device(g[0].data_ptr(), g[1].data_ptr(), True, out.data_ptr(), 0, out_f64=True,
                            deterministic=True, sky_iqu=True)
        conv.sync()
        return out.cpu().numpy()

    want = adjoint(free)
    free.close()
    fx = 8 * 4 * npix  # the fixed-point sky accumulator
    cap = before + fx + 3 * 256 * 8 + PLAN_BYTES * n - (1 << 20)
    conv = GPUConvolver(RunConfig(maxMemUsage=cap, ptgPerConv=4096), form="tuned")
    _setup(conv, nss=nss)
    _tod(conv, n, False)
    assert conv.memory_used() == before + PLAN_BYTES * n  # the forward's scratch is in place
    got = adjoint(conv)
    assert conv.memory_used() <= cap
    conv.close()
    assert np.array_equal(got, want)
