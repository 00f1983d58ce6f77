"""On-disk formats (CPU): the reference's sky/tilde-beam/field text files and
its GRASP ingest scripts, pinned against golden_grasp.npz (outputs of the
reference scripts themselves; tests/golden/make_grasp_golden.py)."""
import os

import numpy as np
import pytest

from conftest import load_golden
from pisco4cmb_gb300 import PolBeam, beam_npix_for_radius
from pisco4cmb_gb300 import io as pio

pytest.importorskip("scipy")


@pytest.fixture(scope="module")
def golden():
    return load_golden("golden_grasp.npz")


def _grid(g, key):
    return pio.GraspGrid(u=g[key + "_u"], v=g[key + "_v"], co=g[key + "_co"], cx=g[key + "_cx"])


def _close(mine, ref):
    """Relative to each plane's peak, 1e-10: the fixtures were made with the
    reference's HEALPix port standing in for healpy, whose polar-cap theta
    (acos z) differs from this library's by up to ~1e-14 rad; 1e-10 is the
    reference's own pix2ang tolerance (tests/cudaHealpix/test_pix2ang.cu:107-112).
    Parsing, the tilde combinations and the splines are the same arithmetic."""
    scale = np.abs(ref).max(axis=-1, keepdims=True)
    err = np.abs(mine - ref).max(axis=-1, keepdims=True)
    assert np.all(err <= 1e-10 * scale + 1e-300), (err / scale).ravel()


@pytest.mark.parametrize("key", ["sq", "rect"])
def test_grasp_file_round_trip(tmp_path, golden, key):
    g = _grid(golden, key)
    path = str(tmp_path / ("%s.grd" % key))
    pio.write_grasp_grid(path, g)
    r = pio.read_grasp_grid(path)
    for a in ("u", "v", "co", "cx"):
        assert np.array_equal(getattr(r, a), getattr(g, a)), a


@pytest.mark.parametrize("key", ["sq", "rect"])
@pytest.mark.parametrize("swap", [False, True])
def test_tilde_beams_match_reference_script(tmp_path, golden, key, swap):
    """fields2beams.py (swap=False) and fields2beams_cxisco.py (swap=True)."""
    nside = int(golden["nside"])
    path = str(tmp_path / ("%s.grd" % key))
    pio.write_grasp_grid(path, _grid(golden, key))
    ref = golden[key + ("_tilde_cxisco" if swap else "_tilde")]
    mine = pio.tilde_beams_from_grasp(path, nside, swap_co_cx=swap)
    assert mine.shape == ref.shape
    _close(mine, ref)


def test_fields_match_reference_script(golden):
    """graspbeam_to_healpix.py: magnitudes exactly, phases modulo 2 pi."""
    nside = int(golden["nside"])
    ref = golden["sq_fields"]
    mine = np.stack(pio.fields_from_grasp(_grid(golden, "sq"), nside))
    _close(mine[[0, 2]], ref[[0, 2]])
    dphi = np.angle(np.exp(1j * (mine[[1, 3]] - ref[[1, 3]])))
    assert np.abs(dphi).max() < 1e-10


def test_grasp_to_tilde_file(tmp_path, golden):
    path = str(tmp_path / "beam.grd")
    pio.write_grasp_grid(path, _grid(golden, "sq"))
    out = pio.grasp_to_tilde_file(path, int(golden["nside"]))
    assert os.path.basename(out) == "hpx_tilde_beams_beam.grd"
    _close(pio.read_tilde_beam_txt(out), golden["sq_tilde"])


@pytest.mark.parametrize("nside", [64, 128, 256, 512, 1024])
def test_cap_pixels_match_beam_grid(nside):
    assert pio.beam_cap_pixels(nside) == beam_npix_for_radius(nside, np.deg2rad(5.0))


def test_sky_txt_round_trip(tmp_path):
    rng = np.random.default_rng(5)
    nside = 16
    maps = [rng.standard_normal(12 * nside * nside).astype(np.float32) for _ in range(4)]
    path = str(tmp_path / "cmb.txt")
    pio.write_sky_txt(path, *maps)
    sky = pio.read_sky_txt(path)
    assert sky.nside == nside
    for a, b in zip((sky.sI, sky.sQ, sky.sU, sky.sV), maps):
        assert np.array_equal(a, b)
    pio.write_sky_txt(path, *maps[:3])
    assert np.all(pio.read_sky_txt(path).sV == 0)


def test_sky_txt_rejects_bad_shapes(tmp_path):
    path = str(tmp_path / "bad.txt")
    np.savetxt(path, np.zeros((100, 4)))
    with pytest.raises(ValueError):
        pio.read_sky_txt(path)
    np.savetxt(path, np.zeros((192, 3)))
    with pytest.raises(ValueError):
        pio.read_sky_txt(path)


def test_tilde_files_build_same_beams_as_fields(tmp_path):
    """Beams built from tilde files equal PolBeam's own construction from
    Gaussian fields (the tilde planes are float32 either way)."""
    nsb, nss, eps = 256, 64, 0.01
    npix = beam_npix_for_radius(nsb, np.deg2rad(5.0))
    ref = PolBeam(nsb, npix, eps, "p")
    ref.make_unpol_gaussian_elliptical_beams(1.6, 1.2, 25.0)
    ref.build(nss)
    pa, pb = str(tmp_path / "ta.txt"), str(tmp_path / "tb.txt")
    pio.write_tilde_beam_txt(pa, np.stack([ref.Ia, ref.Qa, ref.Ua, ref.Va]))
    pio.write_tilde_beam_txt(pb, np.stack([ref.Ib, ref.Qb, ref.Ub, ref.Vb]))
    b = pio.polbeam_from_tilde_files(nsb, pa, pb, eps, nss)
    for x, y in zip(b.planes(), ref.planes()):
        assert np.array_equal(x, y)


def test_single_detector_tilde(tmp_path):
    nsb, nss = 128, 32
    npix = beam_npix_for_radius(nsb, np.deg2rad(5.0))
    ref = PolBeam(nsb, npix, 0.0, "a")
    ref.make_unpol_gaussian_elliptical_beams(2.0, 2.0, 0.0)
    ref.build(nss)
    pa = str(tmp_path / "ta.txt")
    pio.write_tilde_beam_txt(pa, np.stack([ref.Ia, ref.Qa, ref.Ua, ref.Va]))
    b = pio.polbeam_from_tilde_files(nsb, pa, None, 0.0, nss, enabledDets="a")
    assert np.array_equal(b.planes()[0], ref.planes()[0])


def test_fields_txt_round_trip(tmp_path, golden):
    f = pio.fields_from_grasp(_grid(golden, "sq"), int(golden["nside"]))
    path = str(tmp_path / "healpix_beam.grd")
    pio.write_fields_txt(path, *f)
    for a, b in zip(pio.read_fields_txt(path), f):
        assert np.array_equal(a, b)


def test_grasp_reader_rejects_truncated(tmp_path, golden):
    path = str(tmp_path / "t.grd")
    pio.write_grasp_grid(path, _grid(golden, "sq"))
    lines = open(path).read().splitlines()
    open(path, "w").write("\n".join(lines[:-5]) + "\n")
    with pytest.raises(ValueError):
        pio.read_grasp_grid(path)
    open(path, "w").write("no header terminator\n1 2 3 4\n")
    with pytest.raises(ValueError):
        pio.read_grasp_grid(path)
