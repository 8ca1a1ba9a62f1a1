"""The packet walk's node test (visit_node_frustum in sparkle_gb300/csrc/traverse.cuh), restated in numpy
float32 (no GPU): for a packet of rays in one octant, the bounds it forms from the extremes of the lanes'
origins and slab reciprocals -- a = s * inv, o = (p - org) * inv, t = fma(q, a, o), the same float32
operations each lane's own test (visit_node) applies to its ray -- contain every lane's near-plane and
far-plane distances, so a child box that passes any lane's own test passes the packet's. (fma is emulated
exactly: q is an integer below 256, so q * a is exact in float64, and the float64 sum rounds to the float32
fma except in double-rounding ties, which random data does not hit.)"""
import numpy as np

F32 = np.float32


def fma32(q, a, o):
    return (np.float64(q) * np.float64(a) + np.float64(o)).astype(F32)


def lane_terms(s, p, org, inv):
    a = (s * inv).astype(F32)
    o = ((p - org).astype(F32) * inv).astype(F32)
    return a, o


def packet_terms(s, p, omin, omax, imin, imax):
    alo, ahi = (s * imin).astype(F32), (s * imax).astype(F32)
    nlo, nhi = (p - omax).astype(F32), (p - omin).astype(F32)
    c = np.stack([(nlo * imin).astype(F32), (nlo * imax).astype(F32), (nhi * imin).astype(F32),
                  (nhi * imax).astype(F32)])
    return alo, ahi, c.min(0), c.max(0)


def slab_inverse(d):
    return np.where(np.abs(d) <= F32(1.1920928955078125e-07), np.copysign(F32(2.0 ** 100), d),
                    (F32(1) / d).astype(F32)).astype(F32)


def test_packet_bounds_contain_every_lane():
    rng = np.random.default_rng(3)
    checked = 0
    for _ in range(3000):
        scale = F32(10.0 ** rng.uniform(-2, 2))
        org0 = (rng.uniform(-100, 100, 3)).astype(F32)
        d0 = rng.normal(size=3)
        d0 /= np.linalg.norm(d0)
        spread = 10.0 ** rng.uniform(-5, -1)
        org = (org0 + rng.normal(scale=spread * scale, size=(32, 3))).astype(F32)
        d = d0 + rng.normal(scale=spread, size=(32, 3))
        d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(F32)
        if not (np.all(np.sign(d) == np.sign(d[0])) and np.all(np.abs(d) > 1.2e-7)):
            continue  # the walk tests such packets lane by lane
        inv = slab_inverse(d)
        e = rng.integers(-10, 6, 3)
        s = (2.0 ** e).astype(F32)  # the node's per-axis plane scale
        p = (org0 + rng.uniform(-200, 200, 3)).astype(F32)  # the node's origin
        q = rng.integers(0, 256, size=(3, 2)).astype(F32)  # two plane bytes per axis
        omin, omax, imin, imax = org.min(0), org.max(0), inv.min(0), inv.max(0)
        alo, ahi, olo, ohi = packet_terms(s, p, omin, omax, imin, imax)
        a, o = lane_terms(s, p, org, inv)
        for k in range(2):
            t_lane = fma32(q[:, k], a, o)  # 32 x 3: each lane's distance to plane byte k on each axis
            lo = fma32(q[:, k], alo, olo)
            hi = fma32(q[:, k], ahi, ohi)
            assert np.all(lo <= t_lane) and np.all(t_lane <= hi), (s, p, q, org, d)
        checked += 1
    assert checked > 1000
