"""CPU oracle for the polarized-beam convolution -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline / reference
arm of ``bench.py`` may import this package, and only as the checker.  The
product (``pisco4cmb_gb300``) never imports it.

``liboracle.so`` is the plain-C restatement in ``oracle.c`` (see ``oracle.h``
for the reference file:line each function follows).  ``_ref/`` holds, when the
reference tree was available at build time, the reference's own CPU sources
compiled against the HEALPix shim (``build_ref.sh``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libpisco_ref.so")
REFDEV_LIB = os.path.join(HERE, "_ref", "libpisco_refdev.so")
REFGPU_CUBIN = os.path.join(HERE, "_ref", "refconv.cubin")
REFGPU_LIB = os.path.join(HERE, "librefgpu.so")

_i64 = ctypes.c_int64
_dbl = ctypes.c_double
_p = ctypes.c_void_p


def build_oracle(force: bool = False) -> str:
    """Compile oracle.c into liboracle.so (no FMA contraction, OpenMP)."""
    src = os.path.join(HERE, "oracle.c")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(os.path.join(HERE, "oracle.h"))):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
                           "-std=c99", src, "-o", tmp, "-lm"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def build_refgpu(force: bool = False):
    """Compile the harness that runs the reference's GPU kernels
    (ref_gpu_harness.cpp + oracle.c, CUDA driver API) into librefgpu.so;
    None when the CUDA headers are missing."""
    srcs = [os.path.join(HERE, f) for f in ("ref_gpu_harness.cpp", "oracle.c", "oracle.h")]
    if (not force and os.path.exists(REFGPU_LIB)
            and all(os.path.getmtime(REFGPU_LIB) >= os.path.getmtime(f) for f in srcs)):
        return REFGPU_LIB
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    if not os.path.exists(os.path.join(cuda, "include", "cuda.h")):
        return None
    obj = REFGPU_LIB + ".oracle%d.o" % os.getpid()
    tmp = REFGPU_LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-std=c99",
                           "-c", srcs[1], "-o", obj])
    subprocess.check_call(["g++", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
                           "-I", os.path.join(cuda, "include"), "-I", HERE, srcs[0], obj,
                           "-L", os.path.join(cuda, "lib64", "stubs"), "-lcuda", "-o", tmp])
    os.remove(obj)
    os.replace(tmp, REFGPU_LIB)
    return REFGPU_LIB


def refgpu_available() -> bool:
    """The reference-kernel cubin and the harness are both built."""
    return os.path.exists(REFGPU_CUBIN) and os.path.exists(REFGPU_LIB)


def refgpu_convolve(ra, dec, pa, nside_sky, sky, nside_beam, beam_a, beam_b,
                    ptg_per_conv=2048, pix_per_disc=None, nthreads=0):
    """The reference's GPU pipeline (its kernels K1 + K2 with GPUConvolver's
    chunking) on float inputs; sky 3|4 x npix, beams 4 x npixB.  Returns
    (tod_a, tod_b, times) for the first n - n % ptg_per_conv samples; times =
    (total, kernels, query_disc, copies) in seconds."""
    L = ctypes.CDLL(REFGPU_LIB)
    L.refgpu_convolve.restype = ctypes.c_long
    L.refgpu_last_error.restype = ctypes.c_char_p
    ra, dec, pa = (_c(x, np.float32) for x in (ra, dec, pa))
    sky = _c(sky, np.float32)
    if sky.shape[0] == 3:
        sky = np.concatenate([sky, np.zeros((1, sky.shape[1]), np.float32)])
    sky4 = np.ascontiguousarray(sky.T)
    ba = np.ascontiguousarray(_c(beam_a, np.float32).T)
    bb = np.ascontiguousarray(_c(beam_b, np.float32).T)
    n = ra.size
    if pix_per_disc is None:
        # the largest disc (over at most 50,000 evenly spaced samples, plus a
        # 2 % margin beyond that many); the harness reports an overflow
        rho = beam_rho_max(nside_beam, ba.shape[0])
        idx = np.arange(n) if n <= 50_000 else np.linspace(0, n - 1, 50_000).astype(np.int64)
        big = max(int(lib().orc_query_disc_count(nside_sky, float(np.pi / 2 - float(dec[i])),
                                                 float(ra[i]), rho)) for i in idx)
        pix_per_disc = big if n <= 50_000 else int(big * 1.02) + 64
    oa = np.zeros(n, np.float32)
    ob = np.zeros(n, np.float32)
    t = np.zeros(4, np.float64)
    done = L.refgpu_convolve(REFGPU_CUBIN.encode(), ctypes.c_int(nside_sky), _ptr(sky4),
                             ctypes.c_int(nside_beam), ctypes.c_long(ba.shape[0]), _ptr(ba),
                             _ptr(bb), ctypes.c_long(n), _ptr(ra), _ptr(dec), _ptr(pa),
                             ctypes.c_int(ptg_per_conv), ctypes.c_int(int(pix_per_disc)),
                             ctypes.c_int(nthreads), _ptr(oa), _ptr(ob), _ptr(t))
    if done < 0:
        raise RuntimeError("reference GPU pipeline: " + L.refgpu_last_error().decode())
    return oa[:done], ob[:done], tuple(t)


def build_ref() -> bool:
    """Build oracle/_ref from the reference tree when it is present."""
    script = os.path.join(HERE, "build_ref.sh")
    subprocess.check_call(["sh", script])
    return os.path.exists(REF_LIB)


_lib = None


def lib():
    global _lib
    if _lib is None:
        build_oracle()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_query_disc_count.restype = _i64
        L.orc_query_disc_count.argtypes = [_i64, _dbl, _dbl, _dbl]
        L.orc_query_disc_pixels.restype = _i64
        L.orc_query_disc_pixels.argtypes = [_i64, _dbl, _dbl, _dbl, _p, _i64]
        L.orc_beam_npix_for_radius.restype = _i64
        L.orc_beam_npix_for_radius.argtypes = [_i64, _dbl]
        L.orc_beam_rho_max.restype = _dbl
        L.orc_beam_rho_max.argtypes = [_i64, _i64]
        for name in ("orc_pix2ang_many", "orc_ang2pix_many", "orc_get_interpol_many",
                     "orc_gaussian_fields", "orc_beam_from_fields", "orc_beam_build",
                     "orc_convolve_f32", "orc_convolve_f64", "orc_match_pairs",
                     "orc_adjoint_f64"):
            getattr(L, name).restype = None
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_p)


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


# ---------------------------------------------------------------- HEALPix
def pix2ang(nside: int, pix):
    pix = _c(pix, np.int64)
    th = np.empty(pix.shape, np.float64)
    ph = np.empty(pix.shape, np.float64)
    lib().orc_pix2ang_many(_i64(nside), _i64(pix.size), _ptr(pix), _ptr(th), _ptr(ph))
    return th, ph


def ang2pix(nside: int, theta, phi):
    th = _c(theta, np.float64)
    ph = _c(phi, np.float64)
    out = np.empty(th.shape, np.int64)
    lib().orc_ang2pix_many(_i64(nside), _i64(th.size), _ptr(th), _ptr(ph), _ptr(out))
    return out


def get_interpol(nside: int, theta, phi):
    th = _c(theta, np.float64)
    ph = _c(phi, np.float64)
    pix = np.empty((th.size, 4), np.int64)
    w = np.empty((th.size, 4), np.float64)
    lib().orc_get_interpol_many(_i64(nside), _i64(th.size), _ptr(th), _ptr(ph), _ptr(pix), _ptr(w))
    return pix, w


def query_disc(nside: int, theta: float, phi: float, radius: float) -> np.ndarray:
    n = lib().orc_query_disc_count(_i64(nside), _dbl(theta), _dbl(phi), _dbl(radius))
    out = np.empty(max(n, 0), np.int64)
    m = lib().orc_query_disc_pixels(_i64(nside), _dbl(theta), _dbl(phi), _dbl(radius),
                                    _ptr(out), _i64(out.size))
    assert m == n
    return out


def focal_plane_to_sky(det_dx, det_dy, det_pol, x_ac, y_ac, rot_ac, flag: int = 1):
    """BPoint::focal_plane_to_sky restated (bpoint.cpp:553-674): outputs
    (x_det, y_det, rot_det), each ndets x nsamples."""
    dx, dy, dp = (_c(np.atleast_1d(x), np.float64) for x in (det_dx, det_dy, det_pol))
    xa, ya, ra_ = (_c(x, np.float64) for x in (x_ac, y_ac, rot_ac))
    nd, ns = dx.size, xa.size
    out = [np.empty((nd, ns), np.float64) for _ in range(3)]
    lib().orc_focal_plane_to_sky(ctypes.c_int(nd), _ptr(dx), _ptr(dy), _ptr(dp), _i64(ns),
                                 _ptr(xa), _ptr(ya), _ptr(ra_), ctypes.c_int(flag),
                                 *[_ptr(o) for o in out])
    return tuple(out)


def match_pairs(ra, dec, pa, skypix, nside_sky: int, nside_beam: int):
    ra, dec, pa = (_c(x, np.float64) for x in (ra, dec, pa))
    sp = _c(skypix, np.int64)
    bp = np.empty(sp.shape, np.int64)
    chi = np.empty(sp.shape, np.float64)
    lib().orc_match_pairs(_i64(sp.size), _ptr(ra), _ptr(dec), _ptr(pa), _ptr(sp),
                          _i64(nside_sky), _i64(nside_beam), _ptr(bp), _ptr(chi))
    return bp, chi


# ---------------------------------------------------------------- PolBeam
def beam_npix_for_radius(nside: int, radius_rad: float) -> int:
    return int(lib().orc_beam_npix_for_radius(_i64(nside), _dbl(radius_rad)))


def beam_rho_max(nside: int, npix: int) -> float:
    return float(lib().orc_beam_rho_max(_i64(nside), _i64(npix)))


def gaussian_beams(nside: int, npix: int, fwhmx: float, fwhmy: float, phi0: float,
                   epsilon: float, nside_sky: int, dets: str = "p"):
    """PolBeam(nside, npix, eps, dets).make_unpol_gaussian_elliptical_beams + build."""
    L = lib()
    f = [np.empty(npix, np.float64) for _ in range(4)]
    L.orc_gaussian_fields(_i64(nside), _i64(npix), _dbl(fwhmx), _dbl(fwhmy), _dbl(phi0),
                          *[_ptr(x) for x in f])
    tilde = np.zeros((4, npix), np.float32)
    L.orc_beam_from_fields(_i64(npix), *[_ptr(x) for x in f],
                           *[_ptr(tilde[k]) for k in range(4)])
    ta = tilde if dets in "ap" else np.zeros_like(tilde)
    tb = tilde.copy() if dets in "bp" else np.zeros_like(tilde)
    oa = np.empty((4, npix), np.float32)
    ob = np.empty((4, npix), np.float32)
    L.orc_beam_build(_i64(nside), _i64(npix), _dbl(epsilon), ctypes.c_char(dets.encode()),
                     _i64(nside_sky), _ptr(ta), _ptr(tb), _ptr(oa), _ptr(ob))
    return oa, ob


# ---------------------------------------------------------------- convolution
def convolve_f32(ra, dec, pa, nside_sky, sky, nside_beam, beam_a, beam_b, interp=0,
                 polflag="p", nthreads=0):
    """Reference-semantics forward: float inputs/products, double accumulation."""
    ra, dec, pa = (_c(x, np.float32) for x in (ra, dec, pa))
    sky = _c(sky, np.float32)
    beam_a = _c(beam_a, np.float32)
    beam_b = _c(beam_b, np.float32)
    if sky.shape[0] == 3:
        sky = np.concatenate([sky, np.zeros((1, sky.shape[1]), np.float32)])
    npb = beam_a.shape[1]
    oa = np.zeros(ra.size, np.float32)
    ob = np.zeros(ra.size, np.float32)
    lib().orc_convolve_f32(_i64(ra.size), _ptr(ra), _ptr(dec), _ptr(pa), _i64(nside_sky),
                           _ptr(sky), _i64(nside_beam), _i64(npb), _ptr(beam_a), _ptr(beam_b),
                           ctypes.c_int(interp), ctypes.c_char(polflag.encode()),
                           _ptr(oa), _ptr(ob), ctypes.c_int(nthreads))
    return oa, ob


def convolve_f64(ra, dec, pa, nside_sky, sky, nside_beam, beam_a, beam_b, interp=0,
                 polflag="p", nthreads=0):
    """All-double forward (sky, beams, products, accumulation, output)."""
    ra, dec, pa = (_c(x, np.float64) for x in (ra, dec, pa))
    sky = _c(sky, np.float64)
    if sky.shape[0] == 3:
        sky = np.concatenate([sky, np.zeros((1, sky.shape[1]), np.float64)])
    beam_a = _c(beam_a, np.float64)
    beam_b = _c(beam_b, np.float64)
    npb = beam_a.shape[1]
    oa = np.zeros(ra.size, np.float64)
    ob = np.zeros(ra.size, np.float64)
    lib().orc_convolve_f64(_i64(ra.size), _ptr(ra), _ptr(dec), _ptr(pa), _i64(nside_sky),
                           _ptr(sky), _i64(nside_beam), _i64(npb), _ptr(beam_a), _ptr(beam_b),
                           ctypes.c_int(interp), ctypes.c_char(polflag.encode()),
                           _ptr(oa), _ptr(ob), ctypes.c_int(nthreads))
    return oa, ob


def adjoint_f64(ra, dec, pa, nside_sky, nside_beam, beam_a, beam_b, g_a, g_b):
    """Transpose of convolve_f64 (nearest beam pixel): returns 4 x npix."""
    ra, dec, pa, g_a, g_b = (_c(x, np.float64) for x in (ra, dec, pa, g_a, g_b))
    beam_a = _c(beam_a, np.float64)
    beam_b = _c(beam_b, np.float64)
    g = np.zeros((4, 12 * nside_sky * nside_sky), np.float64)
    lib().orc_adjoint_f64(_i64(ra.size), _ptr(ra), _ptr(dec), _ptr(pa), _i64(nside_sky),
                          _i64(nside_beam), _i64(beam_a.shape[1]), _ptr(beam_a), _ptr(beam_b),
                          _ptr(g_a), _ptr(g_b), _ptr(g))
    return g


# ---------------------------------------------------------------- reference (_ref)
_ref = None
_refdev = None


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


def ref_lib():
    global _ref
    if _ref is None:
        L = ctypes.CDLL(REF_LIB)
        L.ref_polbeam_gaussian.restype = ctypes.c_int
        L.ref_convolve.restype = ctypes.c_int
        L.ref_rho_sigma_chi.restype = None
        _ref = L
    return _ref


def refdev_lib():
    global _refdev
    if _refdev is None:
        _refdev = ctypes.CDLL(REFDEV_LIB)
    return _refdev


def ref_gaussian_beams(nside, npix, fwhmx, fwhmy, phi0, epsilon, nside_sky, dets="p"):
    oa = np.empty((4, npix), np.float32)
    ob = np.empty((4, npix), np.float32)
    rm = ctypes.c_double()
    ref_lib().ref_polbeam_gaussian(ctypes.c_int(nside), ctypes.c_long(npix), _dbl(epsilon),
                                   ctypes.c_char(dets.encode()), _dbl(fwhmx), _dbl(fwhmy),
                                   _dbl(phi0), ctypes.c_int(nside_sky), _ptr(oa), _ptr(ob),
                                   ctypes.byref(rm))
    return oa, ob, rm.value


def ref_convolve(ra, dec, pa, nside_sky, sky, nside_beam, beam_a, beam_b, polflag="p",
                 nthreads=0):
    """The reference's own Convolver::exec_convolution (float API)."""
    ra, dec, pa = (_c(x, np.float32) for x in (ra, dec, pa))
    sky = _c(sky, np.float32)
    if sky.shape[0] == 3:
        sky = np.concatenate([sky, np.zeros((1, sky.shape[1]), np.float32)])
    beam_a = _c(beam_a, np.float32)
    beam_b = _c(beam_b, np.float32)
    npb = beam_a.shape[1]
    oa = np.zeros(ra.size, np.float32)
    ob = np.zeros(ra.size, np.float32)
    rc = ref_lib().ref_convolve(ctypes.c_long(ra.size), _ptr(ra), _ptr(dec), _ptr(pa),
                                ctypes.c_int(nside_sky), _ptr(sky[0]), _ptr(sky[1]),
                                _ptr(sky[2]), _ptr(sky[3]), ctypes.c_int(nside_beam),
                                ctypes.c_long(npb), _ptr(beam_a), _ptr(beam_b),
                                ctypes.c_char(polflag.encode()), _ptr(oa), _ptr(ob),
                                ctypes.c_int(nthreads))
    if rc != 0:
        raise ValueError("valid polFlags are 'a', 'b' and 'p'")
    return oa, ob


def refdev_pix2ang(nside, pix):
    pix = _c(pix, np.int64)
    th = np.empty(pix.shape, np.float64)
    ph = np.empty(pix.shape, np.float64)
    refdev_lib().refdev_pix2ang(ctypes.c_int(nside), ctypes.c_long(pix.size), _ptr(pix),
                                _ptr(th), _ptr(ph))
    return th, ph


def refdev_ang2pix(nside, theta, phi):
    th = _c(theta, np.float64)
    ph = _c(phi, np.float64)
    out = np.empty(th.shape, np.int64)
    refdev_lib().refdev_ang2pix(ctypes.c_int(nside), ctypes.c_long(th.size), _ptr(th),
                                _ptr(ph), _ptr(out))
    return out


def refdev_get_interpol(nside, theta, phi):
    th = _c(theta, np.float64)
    ph = _c(phi, np.float64)
    pix = np.empty((th.size, 4), np.int64)
    w = np.empty((th.size, 4), np.float64)
    refdev_lib().refdev_get_interpol(ctypes.c_int(nside), ctypes.c_long(th.size), _ptr(th),
                                     _ptr(ph), _ptr(pix), _ptr(w))
    return pix, w


def _rsc(L, fn, ra_bc, dec_bc, psi_bc, ra_pix, dec_pix):
    arrs = [_c(x, np.float64) for x in (ra_bc, dec_bc, psi_bc, ra_pix, dec_pix)]
    n = arrs[0].size
    out = [np.empty(n, np.float64) for _ in range(3)]
    getattr(L, fn)(ctypes.c_long(n), *[_ptr(a) for a in arrs], *[_ptr(o) for o in out])
    return out


def rho_sigma_chi(*args):
    return _rsc(lib(), "orc_rho_sigma_chi_many", *args)


def ref_rho_sigma_chi(*args):
    return _rsc(ref_lib(), "ref_rho_sigma_chi", *args)


def refdev_rho_sigma_chi(*args):
    return _rsc(refdev_lib(), "refdev_rho_sigma_chi", *args)


# ---------------------------------------------------------------- binned map-making
def map_accumulate(nside, ra, dec, pa, pol, data, ata=None, atd=None):
    """SkyMap::accumulate_data restated (skymap.cpp:68-132).  ra, dec, pa,
    data: (ndet, nsamples) float32 (the reference's types) or float64; pol:
    ndet floats.  Accumulates into and returns (ata 9 x npix, atd 3 x npix),
    interleaved per pixel like the reference's AtA / AtD."""
    npix = 12 * nside * nside
    f64 = np.asarray(ra).dtype == np.float64
    dt = np.float64 if f64 else np.float32
    ra, dec, pa, data = (np.ascontiguousarray(np.atleast_2d(x), dtype=dt) for x in (ra, dec, pa, data))
    ndet, ns = ra.shape
    pol = np.ascontiguousarray(pol, dtype=np.float32).reshape(ndet)
    if ata is None:
        ata = np.zeros(9 * npix, np.float64)
    if atd is None:
        atd = np.zeros(3 * npix, np.float64)
    fn = lib().orc_map_accumulate_f64 if f64 else lib().orc_map_accumulate_f32
    fn(_i64(nside), _i64(ns), _ptr(ra), _ptr(dec), _ptr(pa), ctypes.c_int(ndet), _ptr(pol),
       _ptr(data), _ptr(ata), _ptr(atd))
    return ata, atd


def map_solve(ata, atd):
    """SkyMap::solve_map restated (skymap.cpp:134-231): (I, Q, U, hits)."""
    ata = np.ascontiguousarray(ata, np.float64)
    atd = np.ascontiguousarray(atd, np.float64)
    npix = atd.size // 3
    out = [np.empty(npix, np.float32) for _ in range(3)]
    hits = np.empty(npix, np.int32)
    lib().orc_map_solve(_i64(npix), _ptr(ata), _ptr(atd), *[_ptr(o) for o in out], _ptr(hits))
    return out[0], out[1], out[2], hits


def dgesv3(a, b):
    """LAPACK dgesv restated for one 3 x 3 system: (info, x, lu, ipiv); a is
    the matrix (row-major input, passed column-major as Fortran expects)."""
    A = np.asfortranarray(np.array(a, np.float64)).ravel(order="F").copy()
    B = np.array(b, np.float64).copy()
    ip = np.zeros(3, np.int32)
    info = lib().orc_dgesv3(_ptr(A), _ptr(ip), _ptr(B))
    return info, B, A.reshape(3, 3, order="F"), ip


REFMAP_LIB = os.path.join(HERE, "_ref", "libpisco_refmap.so")
REFMAP_EXACT_LIB = os.path.join(HERE, "_ref", "libpisco_refmap_exact.so")
_refmap = {}


def refmap_available() -> bool:
    return os.path.exists(REFMAP_LIB) and os.path.exists(REFMAP_EXACT_LIB)


def ref_skymap(nside, ra, dec, pa, pol, data, ncalls=1, exact=False):
    """The reference SkyMap (skymap.cpp, compiled unmodified; exact=True: the
    build without floating-point contraction): ncalls x accumulate_data on
    the same float32 (ndet, nsamples) arrays, then solve_map.  Returns
    (ata, atd, I, Q, U, hits)."""
    path = REFMAP_EXACT_LIB if exact else REFMAP_LIB
    if path not in _refmap:
        L = ctypes.CDLL(path)
        L.ref_skymap_run.restype = ctypes.c_int
        _refmap[path] = L
    ra, dec, pa, data = (np.ascontiguousarray(np.atleast_2d(x), dtype=np.float32)
                         for x in (ra, dec, pa, data))
    ndet, ns = ra.shape
    pol = np.ascontiguousarray(pol, dtype=np.float32).reshape(ndet)
    npix = 12 * nside * nside
    ata = np.empty(9 * npix, np.float64)
    atd = np.empty(3 * npix, np.float64)
    I, Q, U = (np.empty(npix, np.float32) for _ in range(3))
    hits = np.empty(npix, np.int32)
    _refmap[path].ref_skymap_run(ctypes.c_int(nside), ctypes.c_int(ns), _ptr(ra), _ptr(dec),
                                 _ptr(pa), ctypes.c_int(ndet), _ptr(pol), _ptr(data),
                                 ctypes.c_int(ncalls), _ptr(ata), _ptr(atd), _ptr(I), _ptr(Q),
                                 _ptr(U), _ptr(hits))
    return ata, atd, I, Q, U, hits
