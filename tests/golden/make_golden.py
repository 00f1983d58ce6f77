"""Generate the golden fixtures in tests/golden/ from the reference's own code.

Needs the reference tree (PISCO_REFERENCE, default: the directory "reference" beside this repository) to build
oracle/_ref (see oracle/build_ref.sh).  Outputs, all small .npz files:

* golden_c1.npz      -- the CPU-runnable workload (sky nside 64 float64 I,Q,U;
                        beam nside 256, 5 deg, FWHM 2 deg, epsilon 0.01;
                        20,000 raster samples) with the TOD a/b computed by the
                        reference Convolver (src/Convolver/convolver.cpp) and
                        the beams built by the reference PolBeam
                        (src/Polbeam/polbeam.cpp), both compiled unmodified.
* golden_ellip.npz   -- a second case: elliptical beam (nside 128, 4 deg,
                        FWHM 1.8/1.4 deg, phi0 30 deg), sky nside 32, 3,000
                        seeded random pointings including both poles.
* golden_healpix.npz -- pix2ang / ang2pix / get_interpol vectors from the
                        reference's device HEALPix port
                        (src/GpuConvolver/cuda/cudaHealpix.cu), and
                        rho/sigma/chi from src/Sphtrigo/sphtrigo.cpp.

Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from pisco4cmb_gb300 import synth  # noqa: E402


def c1_case():
    w = synth.WORKLOADS[1]
    sky = synth.grf_sky(w["nside_sky"], 1, dtype=np.float64)
    ra, dec, psi = synth.raster_scan(w["nsamples"])
    ra, dec, psi = (x.astype(np.float32) for x in (ra, dec, psi))
    nsb = w["nside_beam"]
    npb = O.beam_npix_for_radius(nsb, np.deg2rad(w["radius_deg"]))
    ba, bb, rho_max = O.ref_gaussian_beams(nsb, npb, w["fwhm_deg"], w["fwhm_deg"], 0.0,
                                           w["epsilon"], w["nside_sky"])
    ta, tb = O.ref_convolve(ra, dec, psi, w["nside_sky"], sky.astype(np.float32), nsb, ba, bb)
    return dict(sky=sky[:3], ra=ra, dec=dec, pa=psi, nside_sky=w["nside_sky"], nside_beam=nsb,
                npix_beam=npb, beam_a=ba, beam_b=bb, rho_max=rho_max, tod_a=ta, tod_b=tb)


def ellip_case():
    rng = np.random.default_rng(20261203 + 11)
    nss, nsb = 32, 128
    sky = synth.grf_sky(nss, 11, dtype=np.float64)
    n = 3000
    ra = rng.uniform(0, 2 * np.pi, n)
    dec = np.arcsin(rng.uniform(-1, 1, n))
    dec[:100] = np.pi / 2 - np.abs(rng.normal(0, 0.03, 100))   # near north pole
    dec[100:200] = -np.pi / 2 + np.abs(rng.normal(0, 0.03, 100))
    pa = rng.uniform(-np.pi, np.pi, n)
    ra, dec, pa = (x.astype(np.float32) for x in (ra, dec, pa))
    npb = O.beam_npix_for_radius(nsb, np.deg2rad(4.0))
    ba, bb, rho_max = O.ref_gaussian_beams(nsb, npb, 1.8, 1.4, 30.0, 0.02, nss)
    ta, tb = O.ref_convolve(ra, dec, pa, nss, sky.astype(np.float32), nsb, ba, bb)
    return dict(sky=sky[:3], ra=ra, dec=dec, pa=pa, nside_sky=nss, nside_beam=nsb, npix_beam=npb,
                beam_a=ba, beam_b=bb, rho_max=rho_max, tod_a=ta, tod_b=tb)


def healpix_case():
    rng = np.random.default_rng(20261203 + 21)
    out = {}
    for nside in (1, 2, 4, 64, 256, 2048, 8192):
        npix = 12 * nside * nside
        pix = np.unique(np.concatenate([np.arange(min(npix, 600)),
                                        np.arange(max(0, npix - 600), npix),
                                        rng.integers(0, npix, 3000)]))
        th, ph = O.refdev_pix2ang(nside, pix)
        t2 = np.arccos(rng.uniform(-1, 1, 4000))
        t2[:400] = rng.uniform(0, 0.02, 400)
        t2[400:800] = np.pi - rng.uniform(0, 0.02, 400)
        p2 = rng.uniform(0, 2 * np.pi, 4000)
        a2p = O.refdev_ang2pix(nside, t2, p2)
        ipix, iw = O.refdev_get_interpol(nside, t2, p2)
        out.update({"pix_%d" % nside: pix, "theta_%d" % nside: th, "phi_%d" % nside: ph,
                    "atheta_%d" % nside: t2, "aphi_%d" % nside: p2, "apix_%d" % nside: a2p,
                    "ipix_%d" % nside: ipix, "iwgt_%d" % nside: iw})
    n = 8000
    rab = rng.uniform(0, 2 * np.pi, n)
    decb = np.arcsin(rng.uniform(-1, 1, n))
    psib = rng.uniform(-np.pi, np.pi, n)
    off = rng.uniform(0, np.deg2rad(6), n)
    ang = rng.uniform(0, 2 * np.pi, n)
    rap = rab + off * np.cos(ang) / np.maximum(np.cos(decb), 0.05)
    decp = np.clip(decb + off * np.sin(ang), -np.pi / 2, np.pi / 2)
    rho, sig, chi = O.ref_rho_sigma_chi(rab, decb, psib, rap, decp)
    out.update(dict(rsc_in=np.stack([rab, decb, psib, rap, decp]),
                    rsc_out=np.stack([rho, sig, chi])))
    return out


def main():
    O.build_oracle()
    if not O.ref_available():
        O.build_ref()
    if not O.ref_available():
        raise SystemExit("reference tree not available: cannot build oracle/_ref")
    np.savez_compressed(os.path.join(HERE, "golden_c1.npz"), **c1_case())
    np.savez_compressed(os.path.join(HERE, "golden_ellip.npz"), **ellip_case())
    np.savez_compressed(os.path.join(HERE, "golden_healpix.npz"), **healpix_case())
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
