"""The allocation-free batched forward, pisco_forward_batched_noalloc (GPU).

Some callers cannot call cudaMalloc: a real-time loop that must not block
on the allocator, a host callback, or a framework whose memory pool owns the
whole GPU and forbids side allocations.  For them the batched forward takes
every input and output as device pointers and keeps its work queue in a
fixed array compiled into the library.

This test calls that entry point through the C ABI twice in a row, with
two different detector sets (different beams, sizes and chunking), and
compares each result with the context-based batched forward
(pisco_forward_batched) on the same inputs.  The two run the same kernel on
the same inputs and each sample's TOD does not depend on how the samples
are cut into work items, so the results must be identical bit for bit.  A
third call runs on a caller-owned stream with one detector's b output left
NULL.  It also checks that sizes beyond the fixed array are refused with a
clear message and no GPU work.

The file is named to be collected last, so a run that stops at the first
failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _detector_set(seed, ndet, nss=64, nsb=256):
    import torch

    from pisco4cmb_gb300 import PolBeam, beam_npix_for_radius, synth

    rng = np.random.default_rng(seed)
    sky = torch.tensor(rng.normal(size=(12 * nss * nss, 4)).astype(np.float32), device="cuda")
    sky[:, 3] = 0
    dets = []
    for _ in range(ndet):
        r = float(rng.uniform(2.0, 6.0))
        npb = beam_npix_for_radius(nsb, np.deg2rad(r))
        beam = PolBeam(nsb, npb, 0.01, "p")
        fx, fy = synth.elliptical_fwhm(r / 2.5, float(rng.uniform(0, 0.1)))
        beam.make_unpol_gaussian_elliptical_beams(fx, fy, float(rng.uniform(0, 180)))
        beam.build(nss)
        a, b = beam.planes()
        ab = torch.tensor(np.concatenate([a.T, b.T], axis=1).copy(), device="cuda")
        n = int(rng.integers(100, 2500))
        ra = torch.tensor(rng.uniform(0, 2 * np.pi, n), device="cuda")
        dec = torch.tensor(np.arcsin(rng.uniform(-1, 1, n)), device="cuda")
        pa = torch.tensor(rng.uniform(0, np.pi, n), device="cuda")
        dets.append(dict(beam=beam, ab=ab, n=n, ra=ra, dec=dec, pa=pa))
    return sky, nss, dets


def _noalloc(sky, nss, dets, chunk, stream=None, no_b=()):
    import torch

    from pisco4cmb_gb300 import _lib

    L = _lib.load()
    arr = (_lib.NoallocDet * len(dets))()
    outs = []
    for i, d in enumerate(dets):
        ta = torch.full((d["n"],), float("nan"), device="cuda")
        tb = torch.full((d["n"],), float("nan"), device="cuda")
        outs.append((ta, tb))
        arr[i] = _lib.NoallocDet(d["beam"].nside, d["beam"].nPixels, d["ab"].data_ptr(), d["n"],
                                 d["ra"].data_ptr(), d["dec"].data_ptr(), d["pa"].data_ptr(),
                                 ta.data_ptr(), None if i in no_b else tb.data_ptr())
    torch.cuda.synchronize()
    handle = None if stream is None else ctypes.c_void_p(stream.cuda_stream)
    st = L.pisco_forward_batched_noalloc(0, nss, ctypes.c_void_p(sky.data_ptr()), arr, len(dets),
                                         chunk, handle)
    assert st == 0, L.pisco_last_error(None)
    torch.cuda.synchronize()
    return [(a.cpu().numpy(), b.cpu().numpy()) for a, b in outs]


def _existing(sky, nss, dets):
    import torch

    from pisco4cmb_gb300 import GPUConvolver, Sky

    conv = GPUConvolver(form="tuned")
    s = sky.cpu().numpy()
    conv.update_sky(Sky(nss, s[:, 0], s[:, 1], s[:, 2], s[:, 3]))
    rows, outs = [], []
    for i, d in enumerate(dets):
        conv.set_beam_slot(i, d["beam"])
        ta = torch.empty(d["n"], device="cuda")
        tb = torch.empty(d["n"], device="cuda")
        outs.append((ta, tb))
        rows.append((i, d["n"], d["ra"].data_ptr(), d["dec"].data_ptr(), d["pa"].data_ptr(),
                     ta.data_ptr(), tb.data_ptr()))
    conv.forward_batched(conv.det_descs(rows))
    conv.sync()
    res = [(a.cpu().numpy(), b.cpu().numpy()) for a, b in outs]
    conv.close()
    return res


def test_noalloc_matches_batched_forward_twice(gpu):
    for seed, ndet, chunk in ((41, 5, 64), (42, 9, 0)):
        sky, nss, dets = _detector_set(seed, ndet)
        got = _noalloc(sky, nss, dets, chunk)
        want = _existing(sky, nss, dets)
        for (ga, gb), (wa, wb) in zip(got, want):
            assert np.all(np.isfinite(ga)) and np.all(np.isfinite(gb))
            assert np.array_equal(ga, wa) and np.array_equal(gb, wb)


def test_noalloc_on_caller_stream_with_a_null_output(gpu):
    import torch

    sky, nss, dets = _detector_set(44, 4)
    want = _existing(sky, nss, dets)
    stream = torch.cuda.Stream()
    got = _noalloc(sky, nss, dets, 128, stream=stream, no_b=(2,))
    for i, ((ga, gb), (wa, wb)) in enumerate(zip(got, want)):
        assert np.array_equal(ga, wa)
        if i == 2:
            assert np.all(np.isnan(gb))  # NULL output: the buffer is never written
        else:
            assert np.array_equal(gb, wb)


def test_noalloc_rejects_sizes_beyond_its_array(gpu):
    import torch

    from pisco4cmb_gb300 import _lib

    L = _lib.load()
    sky, nss, dets = _detector_set(43, 1)
    d = dets[0]
    out = torch.empty(d["n"], device="cuda")
    row = _lib.NoallocDet(d["beam"].nside, d["beam"].nPixels, d["ab"].data_ptr(), d["n"],
                          d["ra"].data_ptr(), d["dec"].data_ptr(), d["pa"].data_ptr(),
                          out.data_ptr(), None)
    many = (_lib.NoallocDet * (_lib.NOALLOC_MAX_DETS + 1))(*([row] * (_lib.NOALLOC_MAX_DETS + 1)))
    st = L.pisco_forward_batched_noalloc(0, nss, ctypes.c_void_p(sky.data_ptr()), many,
                                         _lib.NOALLOC_MAX_DETS + 1, 0, None)
    assert st == _lib.PISCO_ERR_INVALID_ARGUMENT
    assert b"PISCO_NOALLOC_MAX_DETS" in L.pisco_last_error(None)
    long_row = _lib.NoallocDet(d["beam"].nside, d["beam"].nPixels, d["ab"].data_ptr(),
                               _lib.NOALLOC_MAX_ITEMS + 1, d["ra"].data_ptr(), d["dec"].data_ptr(),
                               d["pa"].data_ptr(), None, None)
    one = (_lib.NoallocDet * 1)(long_row)
    st = L.pisco_forward_batched_noalloc(0, nss, ctypes.c_void_p(sky.data_ptr()), one, 1, 1, None)
    assert st == _lib.PISCO_ERR_INVALID_ARGUMENT
    assert b"PISCO_NOALLOC_MAX_ITEMS" in L.pisco_last_error(None)
    huge_row = _lib.NoallocDet(d["beam"].nside, d["beam"].nPixels, d["ab"].data_ptr(),
                               (1 << 62), d["ra"].data_ptr(), d["dec"].data_ptr(),
                               d["pa"].data_ptr(), None, None)
    one = (_lib.NoallocDet * 1)(huge_row)
    st = L.pisco_forward_batched_noalloc(0, nss, ctypes.c_void_p(sky.data_ptr()), one, 1, 1 << 30,
                                         None)
    assert st == _lib.PISCO_ERR_INVALID_ARGUMENT
    assert b"2^40" in L.pisco_last_error(None)
