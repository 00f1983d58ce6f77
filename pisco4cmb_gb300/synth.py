"""Seeded synthetic inputs with the shapes of the five benchmark workloads.

No public data set is used; these generators stand in for CAMB/healpy CMB
maps (reference ``scripts/create_cmb.py``), GRASP beams
(``scripts/fields2beams.py``) and telescope pointing (``src/Bpoint``).

* Sky: independent scalar Gaussian random fields for I, Q, U (V = 0) with
  C_ell ~ ell^-2 for 2 <= ell <= lmax (default 3*nside - 1), synthesised on
  the HEALPix RING grid ring by ring: normalised associated-Legendre
  recurrence in ell (vectorised over m and rings) followed by one inverse FFT
  per ring.  Rescaled to the requested rms.  Runs on torch (CPU or CUDA).
* Beams: elliptical Gaussians through the PolBeam construction
  (``pisco4cmb_gb300.api.PolBeam``), nPixels = ang2pix(nside_beam, radius, 0)
  as in ``scripts/fields2beams.py:102``.  Ellipticity e maps to
  fwhm_x = F*sqrt((1+e)/(1-e)), fwhm_y = F*sqrt((1-e)/(1+e)), i.e.
  e = (fwhm_x - fwhm_y)/(fwhm_x + fwhm_y) at geometric-mean FWHM F.
* Scans: the raster, sweep, pole-heavy and offset-detector scans of the
  workloads (angles in radians; ``pa`` is the position angle the Scan API
  takes, negated internally as in the reference).
"""
from __future__ import annotations

import math
import os

import numpy as np

SEED_BASE = 20261203


def rng_for(config_id: int, stream: int = 0) -> np.random.Generator:
    return np.random.default_rng([SEED_BASE + config_id, stream])


# ------------------------------------------------------------------ rings
def ring_geometry(nside: int):
    """z, number of pixels and first-pixel phi of every RING-scheme ring."""
    nr = 4 * nside - 1
    ring = np.arange(1, nr + 1, dtype=np.int64)
    npix = 12 * nside * nside
    fact2 = 4.0 / npix
    fact1 = 2 * nside * fact2
    north = np.where(ring > 2 * nside, 4 * nside - ring, ring)
    z = np.where(north < nside, 1.0 - north.astype(np.float64) ** 2 * fact2,
                 (2 * nside - north) * fact1)
    z = np.where(ring > 2 * nside, -z, z)
    n_in = np.where(north < nside, 4 * north, 4 * nside)
    shifted = np.where(north < nside, True, ((north - nside) & 1) == 0)
    phi0 = np.where(shifted, np.pi / n_in, 0.0)
    start = np.concatenate([[0], np.cumsum(n_in)[:-1]])
    return z, n_in, phi0, start


def grf_map(nside: int, lmax: int | None, seed, device: str = "cpu",
            lmin: int = 2) -> np.ndarray:
    """One scalar GRF (float64, unit-normalised rms) with C_ell ~ ell^-2."""
    import torch

    if lmax is None:
        lmax = 3 * nside - 1
    rng = np.random.default_rng(seed)
    z, n_in, phi0, start = ring_geometry(nside)
    R = z.size
    dev = torch.device(device)
    zt = torch.tensor(z, dtype=torch.float64, device=dev)
    st = torch.sqrt(torch.clamp(1.0 - zt * zt, min=0.0))
    M = lmax + 1
    # a_lm draws (m >= 0), complex, variance C_ell (real part only at m = 0)
    ell = np.arange(M, dtype=np.float64)
    cl = np.zeros(M)
    cl[lmin:] = ell[lmin:] ** -2.0
    F = torch.zeros((M, R), dtype=torch.complex128, device=dev)
    # Values are carried as v * BIG**E with a per-(m, ring) integer exponent
    # E: lambda_mm ~ sin(theta)^m leaves the double range for large m, and
    # the recurrence started from an underflowed value diverges.  Only rows
    # back at scale E == 0 contribute (E < 0 rows are below 1e-100).
    BIG = 1e100
    lam_mm = torch.full((R,), math.sqrt(1.0 / (4 * math.pi)), dtype=torch.float64, device=dev)
    e_mm = torch.zeros(R, dtype=torch.int32, device=dev)
    # three rotating (m, ring) buffers: lambda_{l, m}, lambda_{l-1, m},
    # lambda_{l-2, m}; step l reads and writes rows m <= l only
    bufs = [torch.zeros((M, R), dtype=torch.float64, device=dev) for _ in range(3)]
    E = torch.zeros((M, R), dtype=torch.int32, device=dev)
    for l in range(0, M):
        cur, lm1, lm2 = bufs[l % 3], bufs[(l - 1) % 3], bufs[(l - 2) % 3]
        if l >= 1:
            m = torch.arange(0, l - 1, dtype=torch.float64, device=dev)
            if m.numel():
                a = torch.sqrt((4.0 * l * l - 1.0) / (l * l - m * m))
                b = torch.sqrt(((l - 1.0) ** 2 - m * m) / (4.0 * (l - 1.0) ** 2 - 1.0))
                cur[: l - 1] = a[:, None] * (zt[None, :] * lm1[: l - 1] - b[:, None] * lm2[: l - 1])
            cur[l - 1] = math.sqrt(2.0 * l + 1.0) * zt * lm1[l - 1]
            lam_mm = -math.sqrt((2.0 * l + 1.0) / (2.0 * l)) * st * lam_mm
            small = (lam_mm.abs() < 1.0 / BIG) & (lam_mm != 0)
            lam_mm = torch.where(small, lam_mm * BIG, lam_mm)
            e_mm = e_mm - small.to(torch.int32)
        cur[l] = lam_mm
        E[l] = e_mm
        # rescale rows that grew past BIG (both retained terms share E)
        big = cur[: l + 1].abs() > BIG
        if bool(big.any()):
            cur[: l + 1] = torch.where(big, cur[: l + 1] / BIG, cur[: l + 1])
            lm1[: l + 1] = torch.where(big, lm1[: l + 1] / BIG, lm1[: l + 1])
            E[: l + 1] += big.to(torch.int32)
        if cl[l] > 0:
            sd = math.sqrt(cl[l])
            re = rng.standard_normal(l + 1) * sd
            im = rng.standard_normal(l + 1) * sd
            re[1:] *= math.sqrt(0.5)
            im[1:] *= math.sqrt(0.5)
            im[0] = 0.0
            alm = torch.tensor(re + 1j * im, dtype=torch.complex128, device=dev)
            live = torch.where(E[: l + 1] == 0, cur[: l + 1], torch.zeros_like(cur[: l + 1]))
            F[: l + 1] += alm[:, None] * live
    # per ring: T(phi_j) = F_0 + 2 Re sum_{m>0} F_m e^{i m phi_j}
    out = np.empty(int(start[-1] + n_in[-1]), np.float64)
    mvec = torch.arange(M, dtype=torch.float64, device=dev)
    Fh = F.clone()
    Fh[1:] *= 2.0
    for r in range(R):
        n = int(n_in[r])
        ph = torch.exp(1j * mvec * float(phi0[r]))
        g = Fh[:, r] * ph
        G = torch.zeros(n, dtype=torch.complex128, device=dev)
        G.index_add_(0, torch.remainder(torch.arange(M, device=dev), n), g)
        vals = torch.fft.ifft(G) * n
        out[int(start[r]):int(start[r]) + n] = vals.real.cpu().numpy()
    out /= out.std()
    return out


def grf_sky(nside: int, config_id: int, rms_i: float = 100.0, rms_qu: float = 10.0,
            lmax: int | None = None, dtype=np.float32, device: str = "cpu") -> np.ndarray:
    """4 x npix I, Q, U, V (V = 0) sky in microkelvin.

    Large skies are cached as .npy under $PISCO_SYNTH_CACHE (default
    /tmp/pisco4cmb_gb300_synth) so repeated runs on one machine reuse them.
    """
    npix = 12 * nside * nside
    cache = None
    if nside >= 256:
        d = os.environ.get("PISCO_SYNTH_CACHE", "/tmp/pisco4cmb_gb300_synth")
        cache = os.path.join(d, "sky_n%d_c%d_l%s_%g_%g.npy" % (nside, config_id, lmax, rms_i, rms_qu))
        if os.path.exists(cache):
            return np.load(cache).astype(dtype)
    sky = np.zeros((4, npix), np.float64)
    for k, rms in enumerate((rms_i, rms_qu, rms_qu)):
        sky[k] = rms * grf_map(nside, lmax, [SEED_BASE + config_id, 100 + k], device=device)
    if cache:
        os.makedirs(os.path.dirname(cache), exist_ok=True)
        tmp = cache + ".tmp%d" % os.getpid()
        np.save(tmp, sky)
        os.replace(tmp + ".npy" if not tmp.endswith(".npy") else tmp, cache)
    return sky.astype(dtype)


# ------------------------------------------------------------------ scans
def raster_scan(n: int = 20000):
    """121 Dec rows (-30..+30 deg, 0.5 deg steps) x 166 RA steps over 0-60 deg,
    truncated at n; psi cycles {0, 45, 90, 135} deg."""
    rows, cols = 121, int(math.ceil(n / 121))
    i = np.arange(n)
    dec = -30.0 + 0.5 * (i // cols)
    ra = 60.0 * (i % cols) / (cols - 1)
    psi = np.array([0.0, 45.0, 90.0, 135.0])[i % 4]
    assert (i // cols).max() < rows
    return np.deg2rad(ra), np.deg2rad(dec), np.deg2rad(psi)


def sweep_scan(n: int, config_id: int, dec0: float = -80.0, ddec: float = 0.05,
               per_sweep: int = 4096, stream: int = 1, shard: int = 0, nshards: int = 1):
    """Constant-elevation sweep: RA advances 360 deg per `per_sweep` samples,
    Dec steps `ddec` deg per sweep from `dec0`; psi uniform in [0, 180) deg.

    shard / nshards: one of nshards interleaved parts of a sweep nshards times
    as dense (shard k is offset by k / nshards of a sample in RA and draws its
    own psi); shard 0 of 1 is the plain sweep."""
    i = np.arange(n, dtype=np.int64)
    ra = 360.0 * ((i % per_sweep) + shard / nshards) / per_sweep
    dec = dec0 + ddec * (i // per_sweep)
    psi = rng_for(config_id, stream + 1000 * shard).uniform(0.0, 180.0, n)
    return np.deg2rad(ra), np.deg2rad(dec), np.deg2rad(psi)


def pole_heavy_scan(n: int, config_id: int, frac: float = 0.1, within_deg: float = 1.0):
    """Sweep scan with every 10th sample replaced by a pointing within
    `within_deg` of the north or south celestial pole."""
    ra, dec, psi = sweep_scan(n, config_id)
    rng = rng_for(config_id, 2)
    sel = np.arange(n) % int(round(1 / frac)) == 0
    k = int(sel.sum())
    colat = np.deg2rad(within_deg) * np.sqrt(rng.uniform(0, 1, k))
    north = rng.uniform(0, 1, k) < 0.5
    dec[sel] = np.where(north, np.pi / 2 - colat, -np.pi / 2 + colat)
    ra[sel] = rng.uniform(0, 2 * np.pi, k)
    return ra, dec, psi


def offset_pointing(ra, dec, dx_deg: float, dy_deg: float):
    """Boresight offset (dx east, dy north) applied in the local tangent frame."""
    dx, dy = np.deg2rad(dx_deg), np.deg2rad(dy_deg)
    dec2 = np.clip(dec + dy, -np.pi / 2, np.pi / 2)
    ra2 = np.mod(ra + dx / np.maximum(np.cos(dec2), 1e-6), 2 * np.pi)
    return ra2, dec2


def elliptical_fwhm(fwhm_deg: float, e: float):
    """(fwhm_x, fwhm_y) in degrees for geometric-mean FWHM and ellipticity e."""
    return fwhm_deg * math.sqrt((1 + e) / (1 - e)), fwhm_deg * math.sqrt((1 - e) / (1 + e))


# ------------------------------------------------------------------ workloads
WORKLOADS = {
    1: dict(name="c1_plain_cpu_runnable", nside_sky=64, nside_beam=256, radius_deg=5.0,
            fwhm_deg=2.0, ellipticity=0.0, epsilon=0.01, nsamples=20000, sky_dtype="float64"),
    2: dict(name="c2_nside1024_beam3deg_2M", nside_sky=1024, nside_beam=2048, radius_deg=3.0,
            fwhm_deg=1.5, ellipticity=0.05, epsilon=0.01, nsamples=2_000_000, sky_dtype="float32"),
    3: dict(name="c3_precision_nside2048_beam1deg_4M", nside_sky=2048, nside_beam=4096,
            radius_deg=1.0, fwhm_deg=0.5, ellipticity=0.02, epsilon=0.01, nsamples=4_000_000,
            sky_dtype="float32", lmax=2048),
    4: dict(name="c4_batched_48pairs_nside512", nside_sky=512, nside_beam=1024, ndet=48,
            epsilon=0.01, sky_dtype="float32"),
    5: dict(name="c5_adjoint_nside256", nside_sky=256, nside_beam=1024, radius_deg=4.0,
            fwhm_deg=1.2, ellipticity=0.05, epsilon=0.01, ndet=4, nsamples=500_000,
            sky_dtype="float32"),
}


def c4_detectors(config_id: int = 4, ndet: int = 48):
    """Per-detector beam radius, FWHM, ellipticity, sample count and offset."""
    rng = rng_for(config_id, 7)
    radius = rng.uniform(1.0, 5.0, ndet)
    fwhm = radius / 2.5
    ell = rng.uniform(0.0, 0.1, ndet)
    ns = np.exp(rng.uniform(math.log(1e4), math.log(1e6), ndet)).astype(np.int64)
    off_r = 2.0 * np.sqrt(rng.uniform(0, 1, ndet))
    off_t = rng.uniform(0, 2 * np.pi, ndet)
    return [dict(radius_deg=float(radius[d]), fwhm_deg=float(fwhm[d]), ellipticity=float(ell[d]),
                 nsamples=int(ns[d]), dx_deg=float(off_r[d] * math.cos(off_t[d])),
                 dy_deg=float(off_r[d] * math.sin(off_t[d]))) for d in range(ndet)]
