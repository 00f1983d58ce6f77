"""Readers and writers of the reference's on-disk products (host side).

* Sky maps: ``scripts/create_cmb.py:96-97`` writes
  ``numpy.savetxt('cmb.txt', numpy.vstack([I, Q, U, V]).T)``: one row per RING
  pixel, columns I Q U V; the simulation reads it back (``run_wholesky.sh:47-52``).
* Tilde beams: ``scripts/fields2beams.py:172-176`` writes
  ``numpy.savetxt(path, numpy.vstack([tI, tQ, tU, tV]).swapaxes(0, 1))``: one
  row per pixel of the beam grid's polar cap (``ang2pix(nside, 5 deg, 0)``
  rows, ``fields2beams.py:101-103``), columns tilde I Q U V of one detector;
  PolBeam's build step (``polbeam.cpp:204-268``) turns the pair's tilde beams
  into the a/b Stokes beams.
* GRASP fields: ``fields2beams.py:39-56`` reads a GRASP uv-grid file (header
  up to a ``++++`` line, three more lines, the grid ranges and sizes, then one
  row per grid point of complex co- and cross-polar fields), forms the tilde
  Stokes beams of Rosset et al. 2010 (``fields2beams.py:63-66``) and
  interpolates them onto the beam grid with bicubic splines
  (``fields2beams.py:102-122``); ``fields2beams_cxisco.py`` is the same with
  the two field columns swapped (the b detector of a pair).
  ``tilde_beams_from_grasp`` restates both.
* ``scripts/graspbeam_to_healpix.py:47-131`` instead interpolates the field
  magnitudes and phases onto the beam grid and writes them as
  ``healpix_<file>`` (magEco phsEco magEcx phsEcx), the input of
  ``PolBeam.beam_from_fields``; ``fields_from_grasp`` restates it.

The interpolation is scipy's ``RectBivariateSpline`` (cubic, no smoothing),
the routine the reference scripts call; the beam-grid coordinates come from
this library's HEALPix (``pix2ang``/``ang2pix``) in place of healpy.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass

import numpy as np

from .api import PolBeam, Sky, ang2pix, pix2ang


def _nside_of(npix: int) -> int:
    nside = int(round(math.sqrt(npix / 12.0)))
    if nside < 1 or 12 * nside * nside != npix:
        raise ValueError("%d rows is not a HEALPix map (12 nside^2)" % npix)
    return nside


def read_sky_txt(path) -> Sky:
    """A ``cmb.txt`` map (npix rows of I Q U V) as a Sky (float32 planes)."""
    d = np.loadtxt(path, ndmin=2)
    if d.shape[1] != 4:
        raise ValueError("%s: expected 4 columns (I Q U V), got %d" % (path, d.shape[1]))
    nside = _nside_of(d.shape[0])
    p = [np.ascontiguousarray(d[:, k], dtype=np.float32) for k in range(4)]
    return Sky(nside, p[0], p[1], p[2], p[3])


def write_sky_txt(path, I, Q, U, V=None) -> None:
    """Write I, Q, U, V (V = 0 when None) as ``create_cmb.py`` does."""
    I = np.asarray(I, dtype=np.float64)
    V = np.zeros_like(I) if V is None else np.asarray(V, dtype=np.float64)
    _nside_of(I.size)
    np.savetxt(path, np.vstack([I, np.asarray(Q, np.float64), np.asarray(U, np.float64), V]).T)


def read_tilde_beam_txt(path) -> np.ndarray:
    """A ``hpx_tilde_beams_*`` file as a 4 x npix float64 array (tI tQ tU tV)."""
    d = np.loadtxt(path, ndmin=2)
    if d.shape[1] != 4:
        raise ValueError("%s: expected 4 columns (tilde I Q U V), got %d" % (path, d.shape[1]))
    return np.ascontiguousarray(d.T)


def write_tilde_beam_txt(path, tilde) -> None:
    """Write a 4 x npix tilde beam as ``fields2beams.py`` does."""
    t = np.asarray(tilde, dtype=np.float64)
    if t.ndim != 2 or t.shape[0] != 4:
        raise ValueError("tilde beam must be 4 x npix")
    np.savetxt(path, t.swapaxes(0, 1))


def polbeam_from_tilde(nside_beam: int, tilde_a, tilde_b, epsilon: float, nside_sky: int,
                       enabledDets: str = "p") -> PolBeam:
    """PolBeam whose tilde beams are given (4 x npix each; either may be None
    when its detector is disabled), built for a sky of nside_sky."""
    ref = tilde_a if tilde_a is not None else tilde_b
    npix = np.asarray(ref).shape[1]
    beam = PolBeam(nside_beam, npix, epsilon, enabledDets)
    for det, t in (("a", tilde_a), ("b", tilde_b)):
        if t is None:
            continue
        t = np.asarray(t, dtype=np.float32)
        if t.shape != (4, npix):
            raise ValueError("tilde beams of both detectors must be 4 x %d" % npix)
        dst = (beam.Ia, beam.Qa, beam.Ua, beam.Va) if det == "a" else \
            (beam.Ib, beam.Qb, beam.Ub, beam.Vb)
        for k in range(4):
            dst[k][:] = t[k]
    beam.build(nside_sky)
    return beam


def polbeam_from_tilde_files(nside_beam: int, path_a, path_b, epsilon: float, nside_sky: int,
                             enabledDets: str = "p") -> PolBeam:
    """PolBeam from the two ``hpx_tilde_beams_*`` files of a detector pair."""
    ta = read_tilde_beam_txt(path_a) if path_a else None
    tb = read_tilde_beam_txt(path_b) if path_b else None
    return polbeam_from_tilde(nside_beam, ta, tb, epsilon, nside_sky, enabledDets)


# ------------------------------------------------------------------ GRASP grids
@dataclass
class GraspGrid:
    """A GRASP uv-grid: axes u (nx) and v (ny), fields co/cx as ny x nx complex
    arrays (u varies fastest in the file, ``fields2beams.py:57-61``)."""
    u: np.ndarray
    v: np.ndarray
    co: np.ndarray
    cx: np.ndarray


def read_grasp_grid(path) -> GraspGrid:
    """Parse a GRASP uv-grid file as ``fields2beams.py:39-61`` does."""
    with open(path, "r") as f:
        for raw in f:
            if raw.strip() == "++++":
                break
        else:
            raise ValueError("%s: no '++++' line ends the header" % path)
        for _ in range(3):
            f.readline()
        ranges = [float(x) for x in f.readline().split()]
        sizes = [int(x) for x in f.readline().split()]
        rows = np.loadtxt(f, ndmin=2)
    if len(ranges) != 4 or len(sizes) < 2:
        raise ValueError("%s: bad grid ranges or sizes line" % path)
    nx, ny = sizes[0], sizes[1]
    if rows.shape != (nx * ny, 4):
        raise ValueError("%s: expected %d rows of 4 values, got %s" % (path, nx * ny, rows.shape))
    umin, vmin, umax, vmax = ranges
    fld = np.ascontiguousarray(rows).view(complex)
    return GraspGrid(u=np.linspace(umin, umax, nx, endpoint=True),
                     v=np.linspace(vmin, vmax, ny, endpoint=True),
                     co=fld[:, 0].reshape(ny, nx).copy(), cx=fld[:, 1].reshape(ny, nx).copy())


def write_grasp_grid(path, grid: GraspGrid, title: str = "synthetic field") -> None:
    """Write a GRASP uv-grid file that ``read_grasp_grid`` (and the reference
    scripts) read back: free text, ``++++``, KTYPE, NSET ICOMP NCOMP IGRID,
    IX IY, XS YS XE YE, NX NY KLIMIT, then Re/Im of co and cx per point."""
    ny, nx = grid.co.shape
    if grid.cx.shape != (ny, nx) or grid.u.size != nx or grid.v.size != ny:
        raise ValueError("grid axes and fields do not agree")
    rows = np.empty((nx * ny, 4), np.float64)
    rows[:, 0], rows[:, 1] = grid.co.real.ravel(), grid.co.imag.ravel()
    rows[:, 2], rows[:, 3] = grid.cx.real.ravel(), grid.cx.imag.ravel()
    with open(path, "w") as f:
        f.write("%s\n++++\n1\n1 3 2 7\n0 0\n" % title)
        f.write("%.17g %.17g %.17g %.17g\n" % (grid.u[0], grid.v[0], grid.u[-1], grid.v[-1]))
        f.write("%d %d 0\n" % (nx, ny))
        np.savetxt(f, rows, fmt="%.17g")


def _grid_of(src) -> GraspGrid:
    return src if isinstance(src, GraspGrid) else read_grasp_grid(src)


def beam_cap_pixels(nside: int, radius_deg: float = 5.0) -> int:
    """Number of beam-grid pixels the scripts keep: ``ang2pix(nside, r, 0)``
    (``fields2beams.py:102``), i.e. every pixel before the one holding
    (theta = r, phi = 0)."""
    return int(ang2pix(nside, np.array([np.deg2rad(radius_deg)]), np.array([0.0]))[0])


def tilde_from_fields(co, cx):
    """Tilde Stokes beams (Rosset et al. 2010) of complex co/cross-polar fields,
    ``fields2beams.py:63-66``."""
    co = np.asarray(co, complex)
    cx = np.asarray(cx, complex)
    x = co * np.conj(cx)
    return (np.abs(co) ** 2 + np.abs(cx) ** 2, np.abs(co) ** 2 - np.abs(cx) ** 2,
            2.0 * np.real(x), -2.0 * np.imag(x))


def tilde_beams_from_grasp(src, nside: int, swap_co_cx: bool = False,
                           radius_deg: float = 5.0) -> np.ndarray:
    """4 x npix tilde beams (tI tQ tU tV) on the beam grid of ``nside`` from a
    GRASP grid (a path or a GraspGrid): ``fields2beams.py`` (or, with
    ``swap_co_cx``, ``fields2beams_cxisco.py``). The grid's v axis is flipped
    (vh = -sin(rho) cos(sigma)) because GRASP's v points North while the beam
    grid's theta-hat points South at psi = 0 (``fields2beams.py:106-112``)."""
    from scipy.interpolate import RectBivariateSpline
    g = _grid_of(src)
    co, cx = (g.cx, g.co) if swap_co_cx else (g.co, g.cx)
    npix = beam_cap_pixels(nside, radius_deg)
    rho, sigma = pix2ang(nside, np.arange(npix))
    uh = np.sin(rho) * np.sin(sigma)
    vh = -np.sin(rho) * np.cos(sigma)
    out = np.empty((4, npix), np.float64)
    for k, t in enumerate(tilde_from_fields(co, cx)):
        out[k] = RectBivariateSpline(g.v, g.u, t)(vh, uh, grid=False)
    return out


def fields_from_grasp(src, nside: int, radius_deg: float = 5.0):
    """(magEco, phsEco, magEcx, phsEcx) on the beam grid of ``nside`` from a
    GRASP grid, ``graspbeam_to_healpix.py:47-120``: magnitudes and the cosine
    and sine of the phases (taken in [0, 2 pi)) are interpolated separately
    and the phases rebuilt with atan2. That script passes the axes as (u, v)
    with an ny x nx table, so it needs a square grid; so does this."""
    from scipy.interpolate import RectBivariateSpline
    g = _grid_of(src)
    if g.u.size != g.v.size:
        raise ValueError("fields_from_grasp needs a square grid (nx == ny)")
    npix = beam_cap_pixels(nside, radius_deg)
    theta, phi = pix2ang(nside, np.arange(npix))
    uh = np.sin(theta) * np.cos(phi)
    vh = np.sin(theta) * np.sin(phi)
    out = []
    for fld in (g.co, g.cx):
        phs = np.angle(fld)
        phs[phs < 0] += 2.0 * np.pi
        mag = RectBivariateSpline(g.u, g.v, np.abs(fld))(uh, vh, grid=False)
        c = RectBivariateSpline(g.u, g.v, np.cos(phs))(uh, vh, grid=False)
        s = RectBivariateSpline(g.u, g.v, np.sin(phs))(uh, vh, grid=False)
        out += [mag, np.arctan2(s, c)]
    return tuple(out)


def read_fields_txt(path):
    """A ``healpix_*`` file (magEco phsEco magEcx phsEcx per row) as 4 arrays."""
    d = np.loadtxt(path, ndmin=2)
    if d.shape[1] != 4:
        raise ValueError("%s: expected 4 columns, got %d" % (path, d.shape[1]))
    return tuple(np.ascontiguousarray(d[:, k]) for k in range(4))


def write_fields_txt(path, magEco, phsEco, magEcx, phsEcx) -> None:
    """Write beam fields as ``graspbeam_to_healpix.py:129-131`` does."""
    np.savetxt(path, np.vstack([magEco, phsEco, magEcx, phsEcx]).swapaxes(0, 1))


def grasp_to_tilde_file(grasp_path, nside: int, swap_co_cx: bool = False) -> str:
    """``fields2beams.py <grasp_path> <nside>`` without the plots: writes
    ``hpx_tilde_beams_<name>`` beside the input and returns its path."""
    t = tilde_beams_from_grasp(grasp_path, nside, swap_co_cx)
    out = os.path.join(os.path.dirname(grasp_path), "hpx_tilde_beams_" + os.path.basename(grasp_path))
    write_tilde_beam_txt(out, t)
    return out
