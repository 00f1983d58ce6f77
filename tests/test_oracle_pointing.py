"""The oracle's restatement of BPoint::focal_plane_to_sky (CPU).

BPoint (src/Bpoint/bpoint.cpp) cannot be compiled here: it needs SOFA and
the JPL ephemerides, which are not in the reference tree, and it has no
tests or golden vectors of its own.  Its focal_plane_to_sky
(bpoint.cpp:553-674) is spherical trigonometry only; the restatement is
pinned here against an independent construction with rotation vectors:

* the detector's direction in the receiver frame (x right, y up, z along the
  boresight) is (sin dx cos dy, sin dy, cos dx cos dy) -- the polar
  coordinates r = acos(cos dx cos dy), a = atan2(sin dy, sin dx cos dy) of
  the reference;
* on the sky the receiver's up axis has position angle rot (north through
  east) at the array centre and its right axis points to rot - 90 deg;
* the detector's position angle is the direction, north through east, of
  the receiver-frame pole (receiver y axis) seen from the detector.

Checked for the Ra/Dec output (flag 1), and the relations of the Az/El
(flag 0: the longitude step reversed) and source-relative (flag 2: x = -pa)
outputs to it; plus the invariants of zero offset and of the distance.
"""
import numpy as np

import oracle as O


def _unit(lon, lat):
    return np.stack([np.cos(lat) * np.cos(lon), np.cos(lat) * np.sin(lon), np.sin(lat)], -1)


def _vectors(dx, dy, x_ac, y_ac, rot):
    c = _unit(x_ac, y_ac)
    n = np.stack([-np.sin(y_ac) * np.cos(x_ac), -np.sin(y_ac) * np.sin(x_ac), np.cos(y_ac)], -1)
    e = np.stack([-np.sin(x_ac), np.cos(x_ac), np.zeros_like(x_ac)], -1)
    up = np.cos(rot)[:, None] * n + np.sin(rot)[:, None] * e
    right = np.sin(rot)[:, None] * n - np.cos(rot)[:, None] * e
    rx, ry, rz = np.sin(dx) * np.cos(dy), np.sin(dy), np.cos(dx) * np.cos(dy)
    v = rz[:, None] * c + rx[:, None] * right + ry[:, None] * up
    pole = up  # the receiver-frame pole: 90 deg from the boresight along up
    return v, pole


def _pa_at(v, target):
    lon = np.arctan2(v[:, 1], v[:, 0])
    lat = np.arcsin(np.clip(v[:, 2], -1, 1))
    n = np.stack([-np.sin(lat) * np.cos(lon), -np.sin(lat) * np.sin(lon), np.cos(lat)], -1)
    e = np.stack([-np.sin(lon), np.cos(lon), np.zeros_like(lon)], -1)
    t = target - np.sum(target * v, -1)[:, None] * v
    return lon, lat, np.arctan2(np.sum(t * e, -1), np.sum(t * n, -1))


def _wrap(a):
    return np.angle(np.exp(1j * a))


def test_focal_plane_to_sky_against_rotation_vectors(oracle_mod):
    rng = np.random.default_rng(11)
    ns = 4000
    x_ac = rng.uniform(0, 2 * np.pi, ns)
    y_ac = np.arcsin(rng.uniform(-0.98, 0.98, ns))
    rot = rng.uniform(-np.pi, np.pi, ns)
    dxs = np.deg2rad([0.0, 1.0, -2.0, 0.5, 5.0])
    dys = np.deg2rad([0.0, 0.5, 1.5, -3.0, -4.0])
    pol = np.deg2rad([0.0, 90.0, 45.0, -30.0, 10.0])
    x1, y1, r1 = O.focal_plane_to_sky(dxs, dys, pol, x_ac, y_ac, rot, 1)
    x0, _, r0 = O.focal_plane_to_sky(dxs, dys, pol, x_ac, y_ac, rot, 0)
    x2, y2, r2 = O.focal_plane_to_sky(dxs, dys, pol, x_ac, y_ac, rot, 2)
    for d in range(dxs.size):
        v, pole = _vectors(np.full(ns, dxs[d]), np.full(ns, dys[d]), x_ac, y_ac, rot)
        lon, lat, pa = _pa_at(v, pole)
        assert np.max(np.abs(_wrap(x1[d] - lon))) < 1e-12
        assert np.max(np.abs(y1[d] - lat)) < 1e-12
        assert np.max(np.abs(_wrap(r1[d] - pol[d] - pa))) < 1e-11
        # distance from the array centre: acos(cos dx cos dy)
        dist = np.arccos(np.clip(np.sum(v * _unit(x_ac, y_ac), -1), -1, 1))
        assert np.max(np.abs(dist - np.arccos(np.cos(dxs[d]) * np.cos(dys[d])))) < 1e-7
        # Az/El: the longitude step has the other sign; source-relative: x = -pa
        assert np.max(np.abs(_wrap((x0[d] - x_ac) + (x1[d] - x_ac)))) < 1e-12
        assert np.max(np.abs(_wrap(x2[d] + (r2[d] - pol[d])))) < 1e-12
        assert np.array_equal(y2[d], y1[d]) and np.array_equal(r0[d], r1[d])
    # zero offset: the array centre itself, the polarization angle added to rot
    assert np.array_equal(x1[0], x_ac) and np.max(np.abs(y1[0] - y_ac)) < 1e-15
    assert np.max(np.abs(r1[0] - rot)) < 1e-15
