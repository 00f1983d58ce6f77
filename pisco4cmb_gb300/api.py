"""Python mirror of the reference API for the convolution path.

Same class names, argument meaning and error behaviour as the reference C++
classes, so a caller of ``Scan``/``Sky``/``PolBeam``/``Convolver``/
``GPUConvolver`` finds the same interface:

* ``Scan(nsamples, ra, dec, pa)``        -- src/Scan/scan.hpp:13-26
* ``Sky(nside, I, Q, U, V)``             -- src/Sky/sky.hpp:15-32
* ``PolBeam(nside, nPixels, epsilon, enabledDets)`` with ``beam_from_fields``,
  ``build``, ``make_unpol_gaussian_elliptical_beams`` -- src/Polbeam/polbeam.hpp:26-84
* ``Convolver(scan, sky, beam).exec_convolution(polFlag, data_a, data_b)``
  -- src/Convolver/convolver.hpp:18-20 (runs on the GPU here)
* ``GPUConvolver(RunConfig)`` with ``configure_execution``, ``update_sky``,
  ``update_beam``, ``update_scan``, ``exec_convolution`` -- src/GpuConvolver/gpuconvolver.hpp:21-34

Every computation goes through libpisco_gb300.so; there is no CPU path.
Differences from the reference, on purpose: every sample is computed (the
reference drops ``nsamples % ptgPerConv`` tail samples,
gpuconvolver.cu:386); errors raise exceptions instead of ``exit(-1)``.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import (FLOAT32, FLOAT64, FORMS, PiscoError, PiscoInvalidArgument, RunConfig,
                   check, load, ptr_array)

__all__ = ["Scan", "Sky", "PolBeam", "Convolver", "GPUConvolver", "SkyMap", "RunConfig",
           "PiscoError", "PiscoInvalidArgument", "beam_npix_for_radius", "pix2ang", "ang2pix",
           "gaussian_beam_param_grad", "focal_plane_to_sky"]


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _dtype_code(a: np.ndarray) -> int:
    if a.dtype == np.float32:
        return FLOAT32
    if a.dtype == np.float64:
        return FLOAT64
    raise PiscoInvalidArgument(1, "arrays must be float32 or float64, got %s" % a.dtype)


# ------------------------------------------------------------------ HEALPix
def pix2ang(nside: int, pix):
    L = load()
    p = np.ascontiguousarray(pix, dtype=np.int64)
    th = np.empty(p.shape, np.float64)
    ph = np.empty(p.shape, np.float64)
    check(L.pisco_hpx_pix2ang(nside, p.size, _ptr(p), _ptr(th), _ptr(ph)), None, "pix2ang")
    return th, ph


def ang2pix(nside: int, theta, phi):
    L = load()
    th = np.ascontiguousarray(theta, dtype=np.float64)
    ph = np.ascontiguousarray(phi, dtype=np.float64)
    out = np.empty(th.shape, np.int64)
    check(L.pisco_hpx_ang2pix(nside, th.size, _ptr(th), _ptr(ph), _ptr(out)), None, "ang2pix")
    return out


def focal_plane_to_sky(det_dx, det_dy, det_pol_angle, x_ac, y_ac, rot_ac, flag: int = 1):
    """BPoint::focal_plane_to_sky (src/Bpoint/bpoint.cpp:553-674) on the GPU:
    detector pointing from the array centre's.  det_*: per detector (receiver
    offsets right / up and polarization angle, radians); x_ac, y_ac, rot_ac:
    per sample; flag 0 Az/El, 1 Ra/Dec, 2 source-relative.  Returns
    (x_det, y_det, rot_det), each ndets x nsamples."""
    L = load()
    dx, dy, dp = (np.ascontiguousarray(np.atleast_1d(v), dtype=np.float64)
                  for v in (det_dx, det_dy, det_pol_angle))
    xa, ya, ra = (np.ascontiguousarray(v, dtype=np.float64) for v in (x_ac, y_ac, rot_ac))
    if not (dx.size == dy.size == dp.size and xa.size == ya.size == ra.size):
        raise PiscoInvalidArgument(1, "detector arrays and sample arrays must match in length")
    out = [np.empty((dx.size, xa.size), np.float64) for _ in range(3)]
    check(L.pisco_focal_plane_to_sky(dx.size, _ptr(dx), _ptr(dy), _ptr(dp), xa.size, _ptr(xa),
                                     _ptr(ya), _ptr(ra), int(flag), *[_ptr(o) for o in out]),
          None, "focal_plane_to_sky")
    return tuple(out)


def beam_npix_for_radius(nside: int, radius_rad: float) -> int:
    n = load().pisco_beam_npix_for_radius(nside, float(radius_rad))
    if n < 0:
        raise PiscoInvalidArgument(1, "bad nside or radius")
    return int(n)


# ------------------------------------------------------------------ API objects
def gaussian_beam_param_grad(nside_beam: int, npix: int, epsilon: float, nside_sky: int,
                             fwhm_deg: float, ellipticity: float, phi0_deg: float, dx: float,
                             dy: float, gbeam) -> np.ndarray:
    """dL/d(fwhm_deg, ellipticity, phi0_deg, dx, dy) of an elliptical Gaussian
    pair beam from dL/dbeam (npix x 8), by pisco_beam_gaussian_param_grad."""
    g = np.ascontiguousarray(gbeam, dtype=np.float64).reshape(-1)
    if g.size != 8 * int(npix):
        raise PiscoInvalidArgument(1, "gbeam must hold npix x 8 values")
    out = np.zeros(5, np.float64)
    check(load().pisco_beam_gaussian_param_grad(int(nside_beam), int(npix), float(epsilon),
                                                int(nside_sky), float(fwhm_deg),
                                                float(ellipticity), float(phi0_deg), float(dx),
                                                float(dy), _ptr(g), _ptr(out)),
          None, "gaussian_beam_param_grad")
    return out


class Scan:
    """Non-owning pointing view: ra, dec, pa arrays of length nsamples (radians)."""

    def __init__(self, nsamples: int, ra, dec, pa):
        self.nsamp = int(nsamples)
        dt = np.float64 if np.asarray(ra).dtype == np.float64 else np.float32
        self.ra = np.ascontiguousarray(ra, dtype=dt)
        self.dec = np.ascontiguousarray(dec, dtype=dt)
        self.pa = np.ascontiguousarray(pa, dtype=dt)
        if min(self.ra.size, self.dec.size, self.pa.size) < self.nsamp:
            raise PiscoInvalidArgument(1, "pointing arrays shorter than nsamples")

    def get_nsamples(self) -> int:
        return self.nsamp

    def get_ra_ptr(self):
        return self.ra

    def get_dec_ptr(self):
        return self.dec

    def get_pa_ptr(self):
        return self.pa


class Sky:
    """Non-owning view of I, Q, U, V HEALPix RING maps."""

    def __init__(self, nside: int, I, Q, U, V=None):
        self.nside = int(nside)
        self.nPixels = 12 * self.nside * self.nside
        dt = np.float64 if np.asarray(I).dtype == np.float64 else np.float32
        self.sI = np.ascontiguousarray(I, dtype=dt)
        self.sQ = np.ascontiguousarray(Q, dtype=dt)
        self.sU = np.ascontiguousarray(U, dtype=dt)
        self.sV = None if V is None else np.ascontiguousarray(V, dtype=dt)
        for m in (self.sI, self.sQ, self.sU) + ((self.sV,) if self.sV is not None else ()):
            if m.size != self.nPixels:
                raise PiscoInvalidArgument(1, "map size does not match 12 nside^2")

    def get_nside(self) -> int:
        return self.nside

    def size(self) -> int:
        return self.nPixels


class PolBeam:
    """Polarized beam of a detector pair as partial RING maps around the pole.

    nPixels pixels per map; rhoMax = pix2ang(nPixels).theta.  Construction
    steps run in libpisco_gb300 (host code) with the reference's arithmetic.
    """

    def __init__(self, nside: int, nPixels: int, epsilon: float, enabledDets: str):
        L = load()
        if enabledDets not in ("a", "b", "p"):
            raise PiscoInvalidArgument(1, "enabledDets must be 'a', 'b' or 'p'")
        self.nside = int(nside)
        self.nPixels = int(nPixels)
        self.epsilon = float(epsilon)
        self.enabledDets = enabledDets
        self.rhoMax = L.pisco_beam_rho_max(self.nside, self.nPixels)
        if self.rhoMax < 0:
            raise PiscoInvalidArgument(1, "nPixels outside the beam grid")
        z = lambda: np.zeros(self.nPixels, np.float32)  # noqa: E731
        self.Ia, self.Qa, self.Ua, self.Va = z(), z(), z(), z()
        self.Ib, self.Qb, self.Ub, self.Vb = z(), z(), z(), z()
        self.aBeams = [z() for _ in range(4)]
        self.bBeams = [z() for _ in range(4)]

    def get_nside(self) -> int:
        return self.nside

    def size(self) -> int:
        return self.nPixels

    def get_rho_max(self) -> float:
        return self.rhoMax

    def beam_from_fields(self, polFlag: str, magEco, phsEco, magEcx, phsEcx) -> None:
        L = load()
        f = [np.ascontiguousarray(x, dtype=np.float64) for x in (magEco, phsEco, magEcx, phsEcx)]
        if polFlag == "a":
            out = (self.Ia, self.Qa, self.Ua, self.Va)
        elif polFlag == "b":
            out = (self.Ib, self.Qb, self.Ub, self.Vb)
        else:
            raise PiscoInvalidArgument(1, "polFlag must be 'a' or 'b'")
        check(L.pisco_beam_from_fields(self.nPixels, *[_ptr(x) for x in f],
                                       *[_ptr(x) for x in out]), None, "beam_from_fields")

    def build(self, nsideSky: int) -> None:
        L = load()
        ta = ptr_array([x.ctypes.data for x in (self.Ia, self.Qa, self.Ua, self.Va)])
        tb = ptr_array([x.ctypes.data for x in (self.Ib, self.Qb, self.Ub, self.Vb)])
        oa = ptr_array([x.ctypes.data for x in self.aBeams])
        ob = ptr_array([x.ctypes.data for x in self.bBeams])
        check(L.pisco_beam_build(self.nside, self.nPixels, self.epsilon,
                                 self.enabledDets.encode(), int(nsideSky), ta, tb, oa, ob),
              None, "build")

    def make_unpol_gaussian_elliptical_beams(self, fwhmx: float, fwhmy: float, phi0: float) -> None:
        L = load()
        f = [np.empty(self.nPixels, np.float64) for _ in range(4)]
        check(L.pisco_beam_gaussian_fields(self.nside, self.nPixels, float(fwhmx), float(fwhmy),
                                           float(phi0), *[_ptr(x) for x in f]), None,
              "make_unpol_gaussian_elliptical_beams")
        if self.enabledDets in ("a", "p"):
            self.beam_from_fields("a", *f)
        if self.enabledDets in ("b", "p"):
            self.beam_from_fields("b", *f)

    def planes(self):
        """(a, b) as 4 x nPixels float32 arrays."""
        return np.stack(self.aBeams), np.stack(self.bBeams)


# ------------------------------------------------------------------ convolvers
class GPUConvolver:
    """Drop-in for the reference GPUConvolver on one GB300.

    ``form``: "tuned" (the default: FP32 per-pair geometry with FP64
    pointing and FP64 re-evaluation near pixel edges; a beam outside its
    domain is convolved by the PLAIN chain automatically), "plain" (the
    reference chain) or "fp64".
    """

    def __init__(self, cfg: RunConfig | None = None, form: str = "tuned"):
        self.cfg = cfg if cfg is not None else RunConfig()
        self.form = form
        if form not in FORMS:
            raise PiscoInvalidArgument(1, "form must be one of %s" % sorted(FORMS))
        self._ctx = None
        self._n = 0

    # the reference allocates in configure_execution (gpuconvolver.cu:72-87)
    def configure_execution(self) -> None:
        L = load()
        h = ctypes.c_void_p()
        st = L.pisco_create(ctypes.byref(self.cfg), ctypes.byref(h))
        if st != 0:
            msg = L.pisco_last_error(None).decode()
            if st in (_lib.PISCO_ERR_INVALID_CONFIG, _lib.PISCO_ERR_INVALID_ARGUMENT):
                raise PiscoInvalidArgument(st, msg)
            raise PiscoError(st, msg)
        self._ctx = h

    @property
    def ctx(self):
        if self._ctx is None:
            self.configure_execution()
        return self._ctx

    def __del__(self):
        if getattr(self, "_ctx", None) is not None:
            try:
                load().pisco_destroy(self._ctx)
            except Exception:  # noqa: BLE001 -- interpreter shutdown
                pass
            self._ctx = None

    def close(self) -> None:
        self.__del__()

    def update_sky(self, sky: Sky) -> None:
        self._npix_sky = sky.nPixels
        V = sky.sV
        check(load().pisco_set_sky(self.ctx, sky.nside, _ptr(sky.sI), _ptr(sky.sQ), _ptr(sky.sU),
                                   _ptr(V), _dtype_code(sky.sI)), self.ctx, "update_sky")

    def update_beam(self, beam: PolBeam) -> None:
        self.set_beam_planes(beam.nside, beam.nPixels, beam.aBeams, beam.bBeams)

    def set_beam_planes(self, nside: int, npix: int, a, b) -> None:
        a = [np.ascontiguousarray(x) for x in a]
        b = [np.ascontiguousarray(x) for x in b]
        dt = _dtype_code(a[0])
        a = [np.ascontiguousarray(x, dtype=a[0].dtype) for x in a]
        b = [np.ascontiguousarray(x, dtype=a[0].dtype) for x in b]
        self._keep = (a, b)
        check(load().pisco_set_beam(self.ctx, int(nside), int(npix),
                                    ptr_array([x.ctypes.data for x in a]),
                                    ptr_array([x.ctypes.data for x in b]), dt),
              self.ctx, "update_beam")

    def update_scan(self, scan: Scan) -> None:
        self._n = scan.nsamp
        check(load().pisco_set_scan(self.ctx, scan.nsamp, _ptr(scan.ra), _ptr(scan.dec),
                                    _ptr(scan.pa), _dtype_code(scan.ra)), self.ctx, "update_scan")

    def set_interp(self, bilinear: bool) -> None:
        check(load().pisco_set_interp(self.ctx, 1 if bilinear else 0), self.ctx, "set_interp")

    def set_sample_order(self, order: str) -> None:
        """"scan" (default) or "sky": process each launch's samples sorted by
        sky cell (TOD identical, written in scan order)."""
        if order not in ("scan", "sky"):
            raise PiscoInvalidArgument(1, "order must be 'scan' or 'sky'")
        check(load().pisco_set_sample_order(self.ctx, 1 if order == "sky" else 0), self.ctx,
              "set_sample_order")

    def exec_convolution(self, data_a: np.ndarray, data_b: np.ndarray, polFlag: str = "p",
                         form: str | None = None) -> None:
        """Fill data_a/data_b (float32 or float64 arrays of nsamples) in place."""
        f = FORMS[form or self.form]
        ref = data_a if data_a is not None else data_b
        dt = _dtype_code(ref)
        for d in (data_a, data_b):
            if d is not None and (not d.flags["C_CONTIGUOUS"] or d.size < self._n or
                                  _dtype_code(d) != dt):
                raise PiscoInvalidArgument(1, "output arrays must be contiguous, of one dtype "
                                              "and hold nsamples values")
        check(load().pisco_forward(self.ctx, polFlag.encode(), _ptr(data_a), _ptr(data_b), dt, f),
              self.ctx, "exec_convolution")

    # ---- resident-input entry points (torch / benchmarks)
    def forward_device(self, d_a: int, d_b: int, out_f64: bool = False, begin: int = 0,
                       n: int | None = None, stream: int = 0, form: str | None = None) -> None:
        n = self._n - begin if n is None else n
        check(load().pisco_forward_device(self.ctx, FORMS[form or self.form], begin, n, d_a or None,
                                          d_b or None, FLOAT64 if out_f64 else FLOAT32,
                                          stream or None), self.ctx, "forward_device")

    def sync(self) -> None:
        check(load().pisco_sync(self.ctx), self.ctx, "sync")

    def memory_used(self) -> int:
        """Device bytes the context holds (what RunConfig.maxMemUsage bounds)."""
        v = ctypes.c_size_t()
        check(load().pisco_memory_used(self.ctx, ctypes.byref(v)), self.ctx, "memory_used")
        return int(v.value)

    def set_scan_device(self, n: int, d_ra: int, d_dec: int, d_pa: int, stream: int = 0) -> None:
        self._n = int(n)
        check(load().pisco_set_scan_device(self.ctx, int(n), d_ra, d_dec, d_pa, stream or None),
              self.ctx, "set_scan_device")

    def set_sky_device(self, nside: int, d_iquv: int, f64: bool, stream: int = 0) -> None:
        self._npix_sky = 12 * int(nside) * int(nside)
        check(load().pisco_set_sky_device(self.ctx, int(nside), d_iquv, FLOAT64 if f64 else FLOAT32,
                                          stream or None), self.ctx, "set_sky_device")

    def count_pairs(self) -> int:
        v = ctypes.c_longlong()
        check(load().pisco_count_pairs(self.ctx, ctypes.byref(v)), self.ctx, "count_pairs")
        return int(v.value)

    # ---- adjoint
    def set_beam_device(self, nside: int, npix: int, d_ab: int, f64: bool = False,
                        stream: int = 0) -> None:
        check(load().pisco_set_beam_device(self.ctx, int(nside), int(npix), d_ab,
                                           FLOAT64 if f64 else FLOAT32, stream or None),
              self.ctx, "set_beam_device")

    def build_beam_device(self, nside: int, npix: int, epsilon: float, enabledDets: str,
                          nside_sky: int, d_fields_a: int, d_fields_b: int, d_ab: int,
                          set_beam: bool = True, stream: int = 0) -> None:
        """PolBeam::beam_from_fields + build on the GPU: d_fields_* = 4 x npix
        device doubles (magEco, phsEco, magEcx, phsEcx), d_ab = npix x 8
        device floats out (a.IQUV, b.IQUV); set_beam makes it this
        convolver's beam."""
        check(load().pisco_beam_build_device(self.ctx, int(nside), int(npix), float(epsilon),
                                             enabledDets.encode(), int(nside_sky),
                                             d_fields_a or None, d_fields_b or None, d_ab,
                                             1 if set_beam else 0, stream or None),
              self.ctx, "build_beam_device")

    def gaussian_beam_device(self, nside: int, npix: int, epsilon: float, nside_sky: int,
                             fwhm_deg: float, ellipticity: float, phi0_deg: float, dx: float,
                             dy: float, d_ab: int, set_beam: bool = True, stream: int = 0) -> None:
        """The elliptical Gaussian pair beam of gaussian_beam_param_grad's
        model, built on the GPU into d_ab (npix x 8 device floats)."""
        check(load().pisco_beam_gaussian_device(self.ctx, int(nside), int(npix), float(epsilon),
                                                int(nside_sky), float(fwhm_deg),
                                                float(ellipticity), float(phi0_deg), float(dx),
                                                float(dy), d_ab, 1 if set_beam else 0,
                                                stream or None),
              self.ctx, "gaussian_beam_device")

    def gaussian_beam_param_grad_device(self, nside: int, npix: int, epsilon: float,
                                        nside_sky: int, fwhm_deg: float, ellipticity: float,
                                        phi0_deg: float, dx: float, dy: float, d_gbeam: int,
                                        g_f64: bool, d_grad: int, stream: int = 0) -> None:
        """dL/d(fwhm_deg, ellipticity, phi0_deg, dx, dy) into d_grad (5 device
        doubles) from d_gbeam = dL/dbeam (npix x 8 device values)."""
        check(load().pisco_beam_gaussian_param_grad_device(
            self.ctx, int(nside), int(npix), float(epsilon), int(nside_sky), float(fwhm_deg),
            float(ellipticity), float(phi0_deg), float(dx), float(dy), d_gbeam,
            FLOAT64 if g_f64 else FLOAT32, d_grad, stream or None),
            self.ctx, "gaussian_beam_param_grad_device")

    def adjoint_device(self, d_ga: int, d_gb: int, g_f64: bool, d_gsky: int, d_gbeam: int,
                       out_f64: bool = False, deterministic: bool = True, begin: int = 0,
                       n: int | None = None, stream: int = 0, sky_iqu: bool = False) -> None:
        """sky_iqu: accumulate I, Q, U only (the V column of the sky gradient
        is written as zero)."""
        n = self._n - begin if n is None else n
        mode = (1 if deterministic else 0) | (2 if sky_iqu else 0)
        check(load().pisco_adjoint_device(self.ctx, begin, n, d_ga, d_gb,
                                          FLOAT64 if g_f64 else FLOAT32, d_gsky or None,
                                          d_gbeam or None, FLOAT64 if out_f64 else FLOAT32,
                                          mode, stream or None),
              self.ctx, "adjoint_device")

    def adjoint_gaussian_device(self, d_ga: int, d_gb: int, g_f64: bool, d_gsky: int,
                                d_grad: int, params, epsilon: float, nside_sky: int,
                                out_f64: bool = False, deterministic: bool = True, begin: int = 0,
                                n: int | None = None, stream: int = 0,
                                sky_iqu: bool = False) -> None:
        """Adjoint with the Gaussian beam-parameter gradient formed directly:
        d_grad (5 device doubles) = dL/d(fwhm_deg, ellipticity, phi0_deg, dx,
        dy) for a context whose beam is that model (gaussian_beam_device with
        ``params``); d_gsky (may be 0) as adjoint_device."""
        n = self._n - begin if n is None else n
        mode = (1 if deterministic else 0) | (2 if sky_iqu else 0)
        f, e, p0, dx, dy = (float(v) for v in params)
        check(load().pisco_adjoint_gaussian_device(
            self.ctx, begin, n, d_ga, d_gb, FLOAT64 if g_f64 else FLOAT32, d_gsky or None,
            FLOAT64 if out_f64 else FLOAT32, mode, float(epsilon), int(nside_sky), f, e, p0, dx,
            dy, d_grad, stream or None), self.ctx, "adjoint_gaussian_device")

    def adjoint(self, g_a: np.ndarray, g_b: np.ndarray, deterministic: bool = True,
                out_f64: bool = True):
        """Host-array adjoint: returns dL/d(I, Q, U, V) as a 4 x npix array."""
        dt = _dtype_code(g_a)
        g_a = np.ascontiguousarray(g_a)
        g_b = np.ascontiguousarray(g_b, dtype=g_a.dtype)
        npix = self._npix_sky
        out = np.zeros((4, npix), np.float64 if out_f64 else np.float32)
        check(load().pisco_adjoint(self.ctx, _ptr(g_a), _ptr(g_b), dt, *[_ptr(out[k]) for k in range(4)],
                                   FLOAT64 if out_f64 else FLOAT32, 1 if deterministic else 0),
              self.ctx, "adjoint")
        return out

    # ---- batched multi-detector forward
    def set_beam_slot(self, slot: int, beam: "PolBeam") -> None:
        a = [np.ascontiguousarray(x, dtype=np.float32) for x in beam.aBeams]
        b = [np.ascontiguousarray(x, dtype=np.float32) for x in beam.bBeams]
        check(load().pisco_set_beam_slot(self.ctx, int(slot), beam.nside, beam.nPixels,
                                         ptr_array([x.ctypes.data for x in a]),
                                         ptr_array([x.ctypes.data for x in b]), FLOAT32),
              self.ctx, "set_beam_slot")

    @staticmethod
    def det_descs(dets, sky_order: bool = False) -> ctypes.Array:
        """dets: iterable of (slot, n, d_ra, d_dec, d_pa, d_tod_a, d_tod_b);
        sky_order: process every pair's samples in sky order."""
        dets = list(dets)
        arr = (_lib.DetDesc * len(dets))()
        flags = _lib.PISCO_DET_SKY_ORDER if sky_order else 0
        for i, (slot, n, ra, dec, pa, ta, tb) in enumerate(dets):
            arr[i] = _lib.DetDesc(int(slot), flags, int(n), ra, dec, pa, ta or None, tb or None)
        return arr

    def forward_batched(self, descs, out_f64: bool = False, chunk: int = 0, stream: int = 0) -> None:
        check(load().pisco_forward_batched(self.ctx, descs, len(descs),
                                           FLOAT64 if out_f64 else FLOAT32, int(chunk),
                                           stream or None), self.ctx, "forward_batched")

    def autotune_batched(self, descs, out_f64: bool = False, cache_path: str | None = None):
        ch = ctypes.c_int()
        ms = ctypes.c_double()
        check(load().pisco_autotune_batched(self.ctx, descs, len(descs),
                                            FLOAT64 if out_f64 else FLOAT32,
                                            cache_path.encode() if cache_path else None,
                                            ctypes.byref(ch), ctypes.byref(ms)),
              self.ctx, "autotune_batched")
        return int(ch.value), float(ms.value)

    def batched_config(self):
        """(chunk, warps per block) the batched launch uses now."""
        ch = ctypes.c_int()
        w = ctypes.c_int()
        check(load().pisco_batched_config(self.ctx, ctypes.byref(ch), ctypes.byref(w)), self.ctx,
              "batched_config")
        return int(ch.value), int(w.value)

    def set_batched_config(self, chunk: int = 0, warps_per_block: int = 8) -> None:
        check(load().pisco_set_batched_config(self.ctx, int(chunk), int(warps_per_block)),
              self.ctx, "set_batched_config")

    def tuned_calibrate(self, begin: int = 0, n: int | None = None, with_pairs: bool = False):
        """Worst FP32 decision error of the TUNED form as a fraction of its
        margin (and, with_pairs, the TUNED disc's pair count)."""
        n = self._n - begin if n is None else n
        v = ctypes.c_double()
        p = ctypes.c_longlong()
        check(load().pisco_tuned_calibrate(self.ctx, begin, n, ctypes.byref(v), ctypes.byref(p)),
              self.ctx, "tuned_calibrate")
        return (float(v.value), int(p.value)) if with_pairs else float(v.value)

    def debug_pairs(self, form: str | None = None, begin: int = 0, n: int | None = None) -> dict:
        """Every (sample, disc pixel) pair the kernels of ``form`` visit over
        samples [begin, begin+n), with their decisions (pisco_debug_pairs):
        a dict of numpy arrays, sorted by (sample, sky pixel)."""
        n = self._n - begin if n is None else n
        L = load()
        f = FORMS[form or self.form]
        tot = ctypes.c_longlong()
        check(L.pisco_debug_pairs(self.ctx, f, begin, n, None, ctypes.byref(tot)), self.ctx,
              "debug_pairs")
        m = int(tot.value)
        out = dict(sample=np.empty(m, np.int32), sky_pix=np.empty(m, np.int32),
                   beam_pix=np.empty(m, np.int32), c2chi=np.empty(m, np.float32),
                   s2chi=np.empty(m, np.float32), chi=np.empty(m, np.float64),
                   flags=np.empty(m, np.int32), stencil_pix=np.empty((m, 4), np.int32),
                   stencil_w=np.empty((m, 4), np.float64))
        rec = _lib.PairDump(m, *[_ptr(out[k]) for k in ("sample", "sky_pix", "beam_pix", "c2chi",
                                                       "s2chi", "chi", "flags", "stencil_pix",
                                                       "stencil_w")])
        check(L.pisco_debug_pairs(self.ctx, f, begin, n, ctypes.byref(rec), ctypes.byref(tot)),
              self.ctx, "debug_pairs")
        order = np.lexsort((out["sky_pix"], out["sample"]))
        return {k: v[order] for k, v in out.items()}

    def last_fallbacks(self) -> int:
        v = ctypes.c_longlong()
        check(load().pisco_last_fallbacks(self.ctx, ctypes.byref(v)), self.ctx, "last_fallbacks")
        return int(v.value)


class Convolver:
    """``Convolver(scan, sky, beam).exec_convolution(polFlag, data_a, data_b)``.

    Same call as the reference CPU Convolver (convolver.cpp:22-72); the work
    runs on the GPU through a private GPUConvolver.  ``polFlag`` other than
    'a', 'b', 'p' raises ``PiscoInvalidArgument`` (std::invalid_argument in
    the reference).
    """

    def __init__(self, scan: Scan, sky: Sky, beam: PolBeam, form: str = "plain"):
        self.scan, self.sky, self.beam = scan, sky, beam
        self.form = form

    def exec_convolution(self, polFlag: str, data_a: np.ndarray, data_b: np.ndarray) -> None:
        if polFlag not in ("a", "b", "p"):
            raise PiscoInvalidArgument(1, "valid polFlags are 'a', 'b' and 'p'")
        g = GPUConvolver(RunConfig(), form=self.form)
        try:
            g.update_sky(self.sky)
            g.update_beam(self.beam)
            g.update_scan(self.scan)
            g.exec_convolution(data_a if polFlag in "ap" else None,
                               data_b if polFlag in "bp" else None, polFlag=polFlag)
        finally:
            g.close()


class SkyMap:
    """Binned map-maker, SkyMap (src/SkyMap/skymap.hpp:13-56), on the GPU.

    ``accumulate_data`` adds TOD into per-pixel normal equations (FP64,
    device-resident, each pixel's totals in the reference's order);
    ``solve_map`` solves them for I, Q, U (``get_stokes_I`` ...,
    ``get_hitmap``).  The accumulators start at zero."""

    INSUFFCOV = 0

    def __init__(self, nside: int, device: int = 0):
        L = load()
        h = ctypes.c_void_p()
        st = L.pisco_map_create(int(nside), int(device), ctypes.byref(h))
        if st != _lib.PISCO_OK:
            text = "SkyMap(%d): %s" % (nside, L.pisco_status_string(st).decode())
            if st == _lib.PISCO_ERR_INVALID_ARGUMENT:
                raise PiscoInvalidArgument(st, text)
            raise PiscoError(st, text)
        self._h = h
        self.nside = int(nside)
        self.nPixels = 12 * self.nside * self.nside
        self._out = None

    def _check(self, st: int, what: str) -> None:
        if st == _lib.PISCO_OK:
            return
        L = load()
        text = "%s: %s (%s)" % (what, L.pisco_map_last_error(self._h).decode(),
                                L.pisco_status_string(st).decode())
        if st == _lib.PISCO_ERR_INVALID_ARGUMENT:
            raise PiscoInvalidArgument(st, text)
        raise PiscoError(st, text)

    def get_nside(self) -> int:
        return self.nside

    def size(self) -> int:
        return self.nPixels

    def reset(self) -> None:
        self._check(load().pisco_map_reset(self._h), "reset")
        self._out = None

    def accumulate_data(self, nsamples: int, ra, dec, pa, ndetectors: int, detPolAngles, data):
        """Host arrays of ndetectors x nsamples values ([det * nsamples + s],
        or shape (ndetectors, nsamples)), float32 as in the reference or
        float64; detPolAngles: ndetectors angles (radians)."""
        f64 = np.asarray(ra).dtype == np.float64
        dt = np.float64 if f64 else np.float32
        arrs = [np.ascontiguousarray(np.asarray(x).reshape(-1), dtype=dt) for x in (ra, dec, pa, data)]
        n = int(nsamples) * int(ndetectors)
        if any(a.size != n for a in arrs):
            raise PiscoInvalidArgument(1, "accumulate_data: arrays must hold ndetectors x nsamples values")
        pol = np.ascontiguousarray(detPolAngles, dtype=np.float32).reshape(-1)
        if pol.size != int(ndetectors):
            raise PiscoInvalidArgument(1, "accumulate_data: one polarisation angle per detector")
        self._check(load().pisco_map_accumulate(self._h, int(nsamples), *[_ptr(a) for a in arrs[:3]],
                                                int(ndetectors), _ptr(pol), _ptr(arrs[3]),
                                                FLOAT64 if f64 else FLOAT32), "accumulate_data")
        self._out = None

    def accumulate_device(self, nsamples: int, d_ra: int, d_dec: int, d_pa: int, ndetectors: int,
                          detPolAngles, d_data: int, f64: bool = False, stream: int = 0) -> None:
        """Device arrays (pointers) of ndetectors x nsamples values."""
        pol = np.ascontiguousarray(detPolAngles, dtype=np.float32).reshape(-1)
        self._check(load().pisco_map_accumulate_device(self._h, int(nsamples), d_ra, d_dec, d_pa,
                                                       int(ndetectors), _ptr(pol), d_data,
                                                       FLOAT64 if f64 else FLOAT32, stream or None),
                    "accumulate_device")
        self._out = None

    def solve_map(self) -> None:
        self._check(load().pisco_map_solve(self._h), "solve_map")
        self._out = None

    def _fetch(self):
        if self._out is None:
            I, Q, U = (np.empty(self.nPixels, np.float32) for _ in range(3))
            hits = np.empty(self.nPixels, np.int32)
            self._check(load().pisco_map_get(self._h, _ptr(I), _ptr(Q), _ptr(U), _ptr(hits)),
                        "get maps")
            self._out = (I, Q, U, hits)
        return self._out

    def get_stokes_I(self) -> np.ndarray:
        return self._fetch()[0]

    def get_stokes_Q(self) -> np.ndarray:
        return self._fetch()[1]

    def get_stokes_U(self) -> np.ndarray:
        return self._fetch()[2]

    def get_hitmap(self) -> np.ndarray:
        return self._fetch()[3]

    def get_normal(self):
        """(AtA 9 x npix, AtD 3 x npix) host copies in the reference's layout."""
        ata = np.empty(9 * self.nPixels, np.float64)
        atd = np.empty(3 * self.nPixels, np.float64)
        self._check(load().pisco_map_get_normal(self._h, _ptr(ata), _ptr(atd)), "get_normal")
        return ata, atd

    def device_arrays(self):
        """(d_iqu, d_hits, d_normal) device pointers (see pisco_map_device_arrays)."""
        a, b, c = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        self._check(load().pisco_map_device_arrays(self._h, ctypes.byref(a), ctypes.byref(b),
                                                   ctypes.byref(c)), "device_arrays")
        return a.value, b.value, c.value

    def close(self) -> None:
        if getattr(self, "_h", None):
            try:
                load().pisco_map_destroy(self._h)
            except Exception:  # noqa: BLE001 -- interpreter shutdown
                pass
            self._h = None

    def __del__(self):
        self.close()
