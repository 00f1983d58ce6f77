"""Generate tests/golden/golden_grasp.npz by running the reference's own GRASP
ingest scripts on seeded synthetic GRASP uv-grids.

The scripts (scripts/fields2beams.py, scripts/fields2beams_cxisco.py and
scripts/graspbeam_to_healpix.py of the reference tree, PISCO_REFERENCE,
default: the directory "reference" beside this repository) are executed unmodified with runpy.  Two modules they
import are absent here and are stood in for:

* healpy: ``ang2pix``/``pix2ang`` come from the reference's own HEALPix port
  (src/GpuConvolver/cuda/cudaHealpix.cu, compiled into oracle/_ref by
  oracle/build_ref.sh); ``gnomview``/``orthview`` (plots) return zeros;
* matplotlib.pyplot: a do-nothing mock (plots only).

Grids: "sq" is 61 x 61 over u, v in [-0.1, 0.1] (all three scripts; the
magnitude/phase script needs nx == ny); "rect" is 71 x 51 over
u in [-0.12, 0.12], v in [-0.1, 0.1] (the two tilde-beam scripts).
Beam grid nside 256 (1,512 pixels inside 5 degrees).

Run:  python tests/golden/make_grasp_golden.py
"""
from __future__ import annotations

import os
import runpy
import sys
import tempfile
import types
from unittest import mock

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from pisco4cmb_gb300 import io as pio  # noqa: E402

REF = os.environ.get("PISCO_REFERENCE", os.path.join(os.path.dirname(ROOT), "reference"))
NSIDE = 256


def synthetic_grid(nx, ny, umax, vmax, seed):
    """Elliptical Gaussian co-polar field with a phase ramp, a weaker
    cross-polar lobe pair, plus small seeded noise."""
    rng = np.random.default_rng(seed)
    u = np.linspace(-umax, umax, nx)
    v = np.linspace(-vmax, vmax, ny)
    U, V = np.meshgrid(u, v)  # ny x nx, u fastest
    s1, s2 = 0.012, 0.009
    amp = np.exp(-0.5 * ((U / s1) ** 2 + (V / s2) ** 2))
    co = amp * np.exp(1j * (40.0 * U - 25.0 * V + 0.3))
    cx = 0.15 * (U / s1) * (V / s2) * amp * np.exp(1j * (15.0 * U + 1.1))
    co = co + 1e-4 * (rng.standard_normal(co.shape) + 1j * rng.standard_normal(co.shape))
    cx = cx + 1e-4 * (rng.standard_normal(cx.shape) + 1j * rng.standard_normal(cx.shape))
    return pio.GraspGrid(u=u, v=v, co=co, cx=cx)


def fake_modules():
    hp = types.ModuleType("healpy")

    def ang2pix(nside, theta, phi):
        th = np.atleast_1d(np.asarray(theta, np.float64))
        ph = np.broadcast_to(np.atleast_1d(np.asarray(phi, np.float64)), th.shape)
        p = O.refdev_ang2pix(nside, th, ph)
        return int(p[0]) if np.ndim(theta) == 0 else p

    def pix2ang(nside, pix):
        return O.refdev_pix2ang(nside, np.asarray(pix, np.int64))

    hp.ang2pix = ang2pix
    hp.pix2ang = pix2ang
    hp.gnomview = lambda m, **kw: np.zeros((kw.get("ysize", 1), kw.get("xsize", 1)))
    hp.orthview = lambda *a, **kw: None
    plt = mock.MagicMock()
    plt.subplots.return_value = (mock.MagicMock(), [mock.MagicMock() for _ in range(3)])
    mpl = types.ModuleType("matplotlib")
    mpl.pyplot = plt
    return {"healpy": hp, "matplotlib": mpl, "matplotlib.pyplot": plt}


def run_script(name, grasp_path, out_prefix):
    import scipy.interpolate  # noqa: F401  (imported before the stand-ins go in)
    argv = sys.argv
    sys.argv = [name, grasp_path, str(NSIDE)]
    fakes = fake_modules()
    saved = {k: sys.modules.get(k) for k in fakes}
    sys.modules.update(fakes)
    try:
        with mock.patch("builtins.print", lambda *a, **k: None):
            runpy.run_path(os.path.join(REF, "scripts", name), run_name="__main__")
    finally:
        sys.argv = argv
        for k, m in saved.items():
            if m is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = m
    d = os.path.dirname(grasp_path)
    return np.loadtxt(os.path.join(d, out_prefix + os.path.basename(grasp_path)))


def main():
    out = {"nside": np.int64(NSIDE)}
    grids = {"sq": synthetic_grid(61, 61, 0.1, 0.1, 1), "rect": synthetic_grid(71, 51, 0.12, 0.1, 2)}
    with tempfile.TemporaryDirectory() as tmp:
        for key, g in grids.items():
            path = os.path.join(tmp, "grid_%s.grd" % key)
            pio.write_grasp_grid(path, g)
            out[key + "_u"], out[key + "_v"] = g.u, g.v
            out[key + "_co"], out[key + "_cx"] = g.co, g.cx
            out[key + "_tilde"] = run_script("fields2beams.py", path, "hpx_tilde_beams_").T
            out[key + "_tilde_cxisco"] = run_script("fields2beams_cxisco.py", path,
                                                    "hpx_tilde_beams_").T
            if key == "sq":
                out[key + "_fields"] = run_script("graspbeam_to_healpix.py", path, "healpix_").T
    np.savez_compressed(os.path.join(HERE, "golden_grasp.npz"), **out)
    print("wrote golden_grasp.npz:", {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
