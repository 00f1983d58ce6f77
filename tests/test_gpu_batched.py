"""Batched multi-detector forward (GPU): uneven beams and sample counts in one
persistent launch must give, per detector, the single-detector TUNED TOD
bit for bit, and agree with the oracle within the TUNED tolerance."""
import json
import os

import numpy as np
import pytest

from conftest import rel_max

pytestmark = pytest.mark.gpu


def _setup(ndet=6, nss=64, nsb=256, seed=4):
    import torch

    import oracle as O
    from pisco4cmb_gb300 import GPUConvolver, PolBeam, Sky, synth

    rng = np.random.default_rng(seed)
    sky = rng.normal(size=(3, 12 * nss * nss)).astype(np.float32)
    conv = GPUConvolver(form="tuned")
    conv.update_sky(Sky(nss, sky[0], sky[1], sky[2], None))
    dets, beams, host = [], [], []
    for d in range(ndet):
        r = float(rng.uniform(2.0, 6.0))
        npb = O.beam_npix_for_radius(nsb, np.deg2rad(r))
        beam = PolBeam(nsb, npb, 0.01, "p")
        fx, fy = synth.elliptical_fwhm(r / 2.5, float(rng.uniform(0, 0.1)))
        beam.make_unpol_gaussian_elliptical_beams(fx, fy, float(rng.uniform(0, 180)))
        beam.build(nss)
        conv.set_beam_slot(d, beam)
        beams.append(beam)
        n = int(np.exp(rng.uniform(np.log(50), np.log(3000))))
        ra = rng.uniform(0, 2 * np.pi, n)
        dec = np.arcsin(rng.uniform(-1, 1, n))
        if d == 0:
            dec[:20] = np.pi / 2 - rng.uniform(0, 0.05, 20)
        pa = rng.uniform(0, np.pi, n)
        t = [torch.tensor(x, device="cuda") for x in (ra, dec, pa)]
        outs = [torch.full((n,), float("nan"), dtype=torch.float32, device="cuda") for _ in range(2)]
        dets.append((d, n, t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr(),
                     outs[0].data_ptr(), outs[1].data_ptr()))
        host.append(dict(ra=ra, dec=dec, pa=pa, t=t, outs=outs, n=n))
    return conv, dets, beams, host, sky, nss, nsb


def test_batched_equals_single_detector_tuned(gpu, oracle_mod):
    from pisco4cmb_gb300 import GPUConvolver, Scan, Sky

    conv, dets, beams, host, sky, nss, nsb = _setup()
    descs = conv.det_descs(dets)
    conv.forward_batched(descs, chunk=64)
    conv.sync()
    first = [[o.cpu().numpy().copy() for o in h["outs"]] for h in host]
    conv.forward_batched(descs, chunk=64)  # graph replay
    conv.sync()
    for d, h in enumerate(host):
        a, b = (o.cpu().numpy() for o in h["outs"])
        assert np.array_equal(a, first[d][0]) and np.array_equal(b, first[d][1])
        single = GPUConvolver(form="tuned")
        single.update_sky(Sky(nss, sky[0], sky[1], sky[2], None))
        single.update_beam(beams[d])
        single.update_scan(Scan(h["n"], h["ra"], h["dec"], h["pa"]))
        sa = np.zeros(h["n"], np.float32)
        sb = np.zeros(h["n"], np.float32)
        single.exec_convolution(sa, sb)
        assert np.array_equal(a, sa) and np.array_equal(b, sb)
        ba, bb = beams[d].planes()
        oa, ob = oracle_mod.convolve_f64(h["ra"], h["dec"], h["pa"], nss, sky.astype(np.float64),
                                         nsb, ba.astype(np.float64), bb.astype(np.float64))
        assert rel_max(a, oa) < 1e-6 and rel_max(b, ob) < 1e-6


def test_batched_bilinear_equals_single_detector(gpu):
    """With the bilinear lookup the batched launch gives each detector the
    single-detector TUNED bilinear TOD bit for bit; switching the lookup
    replaces the captured graph (the launch key holds the lookup)."""
    from pisco4cmb_gb300 import GPUConvolver, Scan, Sky

    conv, dets, beams, host, sky, nss, nsb = _setup(ndet=4, seed=11)
    descs = conv.det_descs(dets)
    conv.forward_batched(descs, chunk=64)
    conv.sync()
    near = [[o.cpu().numpy().copy() for o in h["outs"]] for h in host]
    conv.set_interp(True)
    conv.forward_batched(descs, chunk=64)
    conv.sync()
    for d, h in enumerate(host):
        a, b = (o.cpu().numpy() for o in h["outs"])
        assert not np.array_equal(a, near[d][0])
        single = GPUConvolver(form="tuned")
        single.update_sky(Sky(nss, sky[0], sky[1], sky[2], None))
        single.update_beam(beams[d])
        single.set_interp(True)
        single.update_scan(Scan(h["n"], h["ra"], h["dec"], h["pa"]))
        sa = np.zeros(h["n"], np.float32)
        sb = np.zeros(h["n"], np.float32)
        single.exec_convolution(sa, sb)
        assert np.array_equal(a, sa) and np.array_equal(b, sb)


def test_batched_chunk_sizes_agree(gpu):
    conv, dets, beams, host, *_ = _setup(ndet=4, seed=7)
    descs = conv.det_descs(dets)
    res = []
    for chunk in (1, 37, 4096):
        conv.forward_batched(descs, chunk=chunk)
        conv.sync()
        res.append([o.cpu().numpy().copy() for h in host for o in h["outs"]])
    for r in res[1:]:
        for x, y in zip(res[0], r):
            assert np.array_equal(x, y)


def test_batched_tiles_agree(gpu):
    """Every block shape (4, 8, 16 warps per block) gives the same TOD bit for
    bit: each sample's result does not depend on which warp runs it."""
    from pisco4cmb_gb300 import PiscoInvalidArgument

    conv, dets, beams, host, *_ = _setup(ndet=4, seed=13)
    descs = conv.det_descs(dets)
    res = []
    for warps in (8, 4, 16):
        conv.set_batched_config(128, warps)
        assert conv.batched_config() == (128, warps)
        conv.forward_batched(descs)
        conv.sync()
        res.append([o.cpu().numpy().copy() for h in host for o in h["outs"]])
    for r in res[1:]:
        for x, y in zip(res[0], r):
            assert np.array_equal(x, y)
    with pytest.raises(PiscoInvalidArgument):
        conv.set_batched_config(0, 12)


def test_autotune_and_cache(gpu, tmp_path):
    conv, dets, *_ = _setup(ndet=5, seed=9)
    descs = conv.det_descs(dets)
    path = str(tmp_path / "tune.json")
    chunk, ms = conv.autotune_batched(descs, cache_path=path)
    assert chunk in (32, 64, 128, 256, 512, 1024, 2048, 4096, 8192) and ms > 0
    _, warps = conv.batched_config()
    assert warps in (4, 8, 16)
    data = json.load(open(path))
    assert len(data) == 1 and list(data.values())[0][0] == chunk
    assert list(data.values())[0][2] == warps
    conv.set_batched_config(64, 8 if warps != 8 else 4)
    chunk2, ms2 = conv.autotune_batched(descs, cache_path=path)  # served from the cache
    assert (chunk2, ms2) == (chunk, list(data.values())[0][1])
    assert conv.batched_config() == (chunk, warps)
    conv.forward_batched(descs)  # chunk 0 = the tuned value
    conv.sync()


def test_batched_validation(gpu):
    from pisco4cmb_gb300 import PiscoError, PiscoInvalidArgument, PolBeam

    conv, dets, *_ = _setup(ndet=2, seed=11)
    bad = list(dets)
    bad[1] = (7,) + tuple(bad[1][1:])  # slot never set
    with pytest.raises(PiscoError) as e:
        conv.forward_batched(conv.det_descs(bad))
    assert e.value.status == 3
    bad = list(dets)
    bad[0] = (0, 10, None, None, None, None, None)
    with pytest.raises(PiscoInvalidArgument):
        conv.forward_batched(conv.det_descs(bad))
    wide = PolBeam(16, 12 * 16 * 16 - 40, 0.0, "p")  # far beyond the polar cap
    conv.set_beam_slot(3, wide)
    bad = list(dets)
    bad[0] = (3,) + tuple(bad[0][1:])
    with pytest.raises(PiscoError) as e:
        conv.forward_batched(conv.det_descs(bad))
    assert e.value.status == 6
