"""CPU tests of the oracle (no GPU): each restated piece is checked against an independent pure-Python /
numpy-float32 restatement of the same reference lines on small cases, and the BVH walks against each
other and against brute force."""
import struct

import numpy as np
import pytest

import oracle
from sparkle_gb300 import abi, scenes

F = np.float32
MASK32 = 0xFFFFFFFF
MASK64 = 0xFFFFFFFFFFFFFFFF


# ---------------------------------------------------------------------------------------------
# Independent restatements (pure Python integers / numpy float32 scalars)
# ---------------------------------------------------------------------------------------------
def splitmix64(state):
    state = (state + 0x9E3779B97F4A7C15) & MASK64
    z = state
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
    return state, z ^ (z >> 31)


def xoshiro128p(seed, n):
    """Sampler.h:16-41: Xoshiro128+ with each state word the low 32 bits of a SplitMix64 output."""
    st, s = seed, []
    for _ in range(4):
        st, z = splitmix64(st)
        s.append(z & MASK32)
    out = []
    for _ in range(n):
        res = (s[0] + s[3]) & MASK32
        t = (s[1] << 9) & MASK32
        s[2] ^= s[0]
        s[3] ^= s[1]
        s[1] ^= s[2]
        s[0] ^= s[3]
        s[2] ^= t
        s[3] = ((s[3] << 11) | (s[3] >> 21)) & MASK32
        out.append(res)
    return out


def xoshiro256ss(seed, n):
    st, s = seed, []
    for _ in range(4):
        st, z = splitmix64(st)
        s.append(z)
    rotl = lambda x, k: ((x << k) | (x >> (64 - k))) & MASK64
    out = []
    for _ in range(n):
        res = (rotl((s[1] * 5) & MASK64, 7) * 9) & MASK64
        t = (s[1] << 17) & MASK64
        s[2] ^= s[0]
        s[3] ^= s[1]
        s[1] ^= s[2]
        s[0] ^= s[3]
        s[2] ^= t
        s[3] = rotl(s[3], 45)
        out.append(res >> 32)
    return out


def dot3(a, b):  # Eigen fixed-size redux order: x0 + (x1 + x2)
    return F(a[0] * b[0]) + F(F(a[1] * b[1]) + F(a[2] * b[2]))


def cross(a, b):
    return [F(a[1] * b[2]) - F(a[2] * b[1]), F(a[2] * b[0]) - F(a[0] * b[2]), F(a[0] * b[1]) - F(a[1] * b[0])]


def mt_reference(o, d, v0, v1, v2):
    """MeshRenderProxy.cpp:128-194 + Ray::InverseAt (identity transform): returns (t, u, v) or None."""
    o, d, v0, v1, v2 = ([F(x) for x in y] for y in (o, d, v0, v1, v2))
    e1 = [F(v1[k] - v0[k]) for k in range(3)]
    e2 = [F(v2[k] - v0[k]) for k in range(3)]
    h = cross(d, e2)
    a = dot3(e1, h)
    if abs(a) < F(1e-6):
        return None
    s = [F(o[k] - v0[k]) for k in range(3)]
    f = F(F(1.0) / a)
    u = F(f * dot3(s, h))
    if u < 0 or u > 1:
        return None
    q = cross(s, e1)
    v = F(f * dot3(d, q))
    if v < 0 or F(u + v) > 1:
        return None
    t = F(f * dot3(e2, q))
    if not t > F(1e-6):
        return None
    lp = [F(o[k] + F(d[k] * t)) for k in range(3)]
    wp_x = F(F(0.0) + (F(F(1.0) * lp[0]) + F(F(F(0.0) * lp[1]) + F(F(0.0) * lp[2]))))
    with np.errstate(divide="ignore", invalid="ignore"):
        wt = F(F(wp_x - o[0]) / d[0])
    if not wt > 0:
        return None
    return wt, u, v


def single_triangle_scene(v0, v1, v2):
    pos = np.array([v0, v1, v2], np.float32)
    n = np.tile(np.array([0, 0, 1], np.float32), (3, 1))
    mesh = abi.Mesh(pos, n, np.array([[0, 1, 2]]))
    return abi.Scene([mesh], [abi.Instance(0, 0)], [abi.Material()])


# ---------------------------------------------------------------------------------------------
# Tests
# ---------------------------------------------------------------------------------------------
@pytest.mark.parametrize("seed", [0, 1, 123456789, 2**32 - 1, 2**40 + 5])
def test_xoshiro128p_matches_restatement(seed):
    u, f = oracle.rng_fill(abi.SPK_RNG_XOSHIRO128P, seed, 64)
    exp = xoshiro128p(seed, 64)
    assert u.tolist() == exp
    # RandomUnit = float(u32) / float(UINT32_MAX) with float(UINT32_MAX) == 2^32
    assert np.array_equal(f, (np.array(exp, np.uint32).astype(np.float32) / F(4294967296.0)).astype(np.float32))


@pytest.mark.parametrize("seed", [0, 7, (3 << 40) ^ 99])
def test_xoshiro256ss_matches_restatement(seed):
    u, _ = oracle.rng_fill(abi.SPK_RNG_XOSHIRO256SS, seed, 64)
    assert u.tolist() == xoshiro256ss(seed, 64)


def test_random_unit_can_reach_one():
    """float(0xFFFFFFFF) rounds to 2^32, so RandomUnit() can return exactly 1.0 (Sampler.h:32-40)."""
    assert F(np.uint32(0xFFFFFFFF)) / F(4294967296.0) == F(1.0)


def test_half_conversion_round_to_nearest_even():
    rng = np.random.default_rng(0)
    vals = np.concatenate([rng.uniform(0, 1, 3000), rng.uniform(0, 70000, 500), 10.0 ** rng.uniform(-9, -4, 500),
                           [0.0, 1.0, 0.5, 65504.0, 65519.0, 65520.0, 2 ** -24, 2 ** -25, 3 * 2 ** -26, 2 ** -14,
                            np.inf]]).astype(np.float32)
    got = np.array([oracle.float_to_half(float(v)) for v in vals], np.uint16)
    exp = vals.astype(np.float16).view(np.uint16)
    assert np.array_equal(got, exp)


def test_moller_trumbore_matches_restatement():
    rng = np.random.default_rng(1)
    tri = ([0.1, 0.2, 0.3], [1.3, 0.1, 0.4], [0.2, 1.1, 0.8])
    sc = oracle.OracleScene(single_triangle_scene(*tri))
    n = 3000
    o = rng.uniform(-1, 2, (n, 3)).astype(np.float32)
    target = rng.uniform(0, 1.2, (n, 3)).astype(np.float32)
    d = target - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = abi.rays_to_array(o, d.astype(np.float32))
    hits, _ = sc.trace(rays)
    n_hit = 0
    for k in range(n):
        exp = mt_reference(rays[k, :3], rays[k, 3:], *tri)
        if exp is None:
            assert hits["prim"][k] == 0xFFFFFFFF, k
        else:
            n_hit += 1
            assert hits["prim"][k] == 0 and hits["face"][k] == 0
            assert (hits["t"][k], hits["u"][k], hits["v"][k]) == exp, k
    assert n_hit > 300


def test_zero_dx_never_hits_a_triangle():
    """world t = (p - o).x / d.x is NaN when d.x == 0 (Ray.h:43-47), so such rays miss every triangle."""
    sc = oracle.OracleScene(single_triangle_scene([-1, -1, 0], [1, -1, 0], [0, 1, 0]))
    rays = np.array([[0, 0, 1, 0, 0, -1], [0.1, 0, 1, 0, 0.6, -0.8], [0, 0, 1, 1e-3, 0, -1]], np.float32)
    rays[2, 3:] /= np.linalg.norm(rays[2, 3:])
    hits, _ = sc.trace(rays)
    assert hits["prim"].tolist()[:2] == [0xFFFFFFFF, 0xFFFFFFFF]
    assert hits["prim"][2] == 0


def test_parallel_and_behind_rays_miss():
    sc = oracle.OracleScene(single_triangle_scene([-1, -1, 0], [1, -1, 0], [0, 1, 0]))
    rays = np.array([[0.3, 0, 1, 1, 0, 0],       # parallel to the plane: |det| < Eps
                     [0.3, 0.01, -1, 0.6, 0, -0.8],  # pointing away: t <= Eps
                     [0.3, 0.01, 1, -0.6, 0, -0.8]], np.float32)  # lands at (-0.45, 0.01, 0): inside
    hits, _ = sc.trace(rays)
    assert hits["prim"].tolist() == [0xFFFFFFFF, 0xFFFFFFFF, 0]


@pytest.mark.parametrize("which", ["cornell", "terrain"])
def test_faithful_and_pruned_walks_agree(which, cornell, small_terrain):
    scene = (cornell if which == "cornell" else small_terrain)[0]
    sc = oracle.OracleScene(scene)
    rays = scenes.random_rays(*scene.world_bounds(), 40_000, seed=2)
    a, oa = sc.trace(rays, traversal=oracle.FAITHFUL)
    b, ob = sc.trace(rays, traversal=oracle.PRUNED)
    assert oa == 0 and ob == 0
    assert np.array_equal(a.view(np.uint8), b.view(np.uint8))


def test_bvh_walk_matches_brute_force_up_to_ties(small_terrain):
    scene = small_terrain[0]
    sc = oracle.OracleScene(scene)
    rays = scenes.random_rays(*scene.world_bounds(), 20_000, seed=3)
    a, _ = sc.trace(rays)
    b = sc.trace_brute(rays)
    assert np.array_equal(a["t"].view(np.uint32), b["t"].view(np.uint32))
    same = (a["prim"] == b["prim"]) & (a["face"] == b["face"])
    assert same.mean() > 0.999


def test_any_hit_implies_closest_hit_exists(cornell):
    scene = cornell[0]
    sc = oracle.OracleScene(scene)
    rays = scenes.random_rays(*scene.world_bounds(), 20_000, seed=4)
    c, _ = sc.trace(rays)
    a, _ = sc.trace(rays, any_hit=True)
    # any-hit reports local t > Eps without the world-t check, so it can only report more hits
    assert np.all((c["prim"] == 0xFFFFFFFF) | (a["prim"] != 0xFFFFFFFF))


def sample_surface_py(mat, ray_dir, normal, tangent, seed):
    """PbrMaterialRenderProxy / DieletricMaterialRenderProxy::SampleSurface restated with numpy float32;
    returns (throughput, w_i, draws, branch)."""
    draws = xoshiro128p(seed, 16)
    pos = [0]

    def unit():
        x = F(np.uint32(draws[pos[0]])) / F(4294967296.0)
        pos[0] += 1
        return F(x)

    def normalize(v):
        z = dot3(v, v)
        if z > 0:
            s = F(np.sqrt(z))
            return [F(x / s) for x in v]
        return v

    n = [F(x) for x in normal]
    tg = [F(x) for x in tangent]
    u_ax = normalize(cross(n, tg))
    v_ax = cross(n, u_ax)
    w_o = [F(-x) for x in ray_dir]
    lo = [dot3(w_o, u_ax), dot3(w_o, v_ax), dot3(w_o, n)]
    base = [F(x) for x in mat.base_color]
    if mat.type == abi.SPK_MAT_DIELECTRIC:
        cos_i, eta_i, eta_t = lo[2], F(1.0), F(mat.eta)
        if not cos_i > 0:
            eta_i, eta_t, cos_i = eta_t, eta_i, F(-cos_i)
        sin_i = F(np.sqrt(F(1 - F(cos_i * cos_i))))
        ref = F(eta_i / eta_t)
        if F(ref * sin_i) >= 1:
            fres = F(1.0)
        else:
            r0 = F(F(1 - ref) / F(1 + ref))
            r0 = F(r0 * r0)
            fres = F(r0 + F(F(1 - r0) * F(np.power(F(1 - cos_i), F(5.0)))))
        if unit() < fres:
            li, branch = [F(-lo[0]), F(-lo[1]), lo[2]], "reflect"
        else:
            ratio = F(F(1.0) / F(mat.eta)) if lo[2] > 0 else F(F(mat.eta) / F(1.0))
            sin2 = F(1 - F(lo[2] * lo[2]))
            st2 = F(F(ratio * ratio) * sin2)
            ct = F(F(np.sqrt(F(1 - st2))) * (F(-1.0) if lo[2] > 0 else F(1.0)))
            li, branch = normalize([F(F(-ratio) * lo[0]), F(F(-ratio) * lo[1]), ct]), "refract"
        thr = base
    else:
        a = F(F(mat.roughness) * F(mat.roughness))
        u1, u2 = unit(), unit()
        v = normalize([F(lo[0] * a), F(lo[1] * a), lo[2]])
        t1 = normalize(cross(v, [F(0), F(0), F(1)])) if v[2] < F(0.999) else [F(1), F(0), F(0)]
        t2 = cross(v, t1)
        r = F(np.sqrt(u1))
        phi = F(F(F(2.0) * F(np.pi)) * u2)
        p1 = F(r * F(np.cos(phi)))
        p2 = F(r * F(np.sin(phi)))
        s = F(F(0.5) * F(1 + v[2]))
        p2 = F(F(F(1 - s) * F(np.sqrt(F(1 - F(p1 * p1))))) + F(s * p2))
        sq = F(np.sqrt(max(F(0), F(F(1 - F(p1 * p1)) - F(p2 * p2)))))
        nn = [F(F(F(p1 * t1[k]) + F(p2 * t2[k])) + F(sq * v[k])) for k in range(3)]
        wm = normalize([F(a * nn[0]), F(a * nn[1]), max(F(0), nn[2])])
        dd = F(dot3(lo, wm) * F(2.0))
        ci = [F(F(wm[k] * dd) - lo[k]) for k in range(3)]
        cos_o, cos_i, cos_m = abs(lo[2]), abs(ci[2]), abs(wm[2])
        lci = dot3(ci, wm)
        valid, fc = False, None
        branch = "diffuse"
        if cos_o > F(1e-6) and cos_i > F(1e-6) and cos_m > F(1e-6):
            p = F(np.power(F(1 - lci), F(5.0)))
            if unit() < F(mat.metallic):
                fc, valid, branch = [F(b + F(F(1 - b) * p)) for b in base], True, "metal"
            elif unit() < F(F(0.04) + F(F(1 - F(0.04)) * p)):
                fc, valid, branch = [F(1)] * 3, True, "specular"
        if valid:
            a2 = F(a * a)
            ggx_i = F(cos_o * F(np.sqrt(F(F(F(F(-cos_i) * a2) + cos_i) * cos_i) + a2)))
            ggx_o = F(cos_i * F(np.sqrt(F(F(F(F(-cos_o) * a2) + cos_o) * cos_o) + a2)))
            occ = F(F(F(F(2.0) * cos_o) * cos_i) / F(ggx_o + ggx_i))
            tan2 = F(F(1 - F(cos_o * cos_o)) / F(cos_o * cos_o))
            norm = F(F(F(2.0) / F(1 + F(np.sqrt(F(1 + F(a2 * tan2)))))) + F(1e-6))
            thr = [F(F(c * occ) / norm) for c in fc]
            li = ci
        else:
            rand = unit()
            theta = F(F(unit() * F(2.0)) * F(np.pi))
            rr = F(np.sqrt(rand))
            dx, dy = F(rr * F(np.cos(theta))), F(rr * F(np.sin(theta)))
            li = [dx, dy, F(np.sqrt(max(F(0), F(F(1.0) - F(F(dx * dx) + F(dy * dy))))))]
            thr = base
    wi = normalize([F(F(F(u_ax[k] * li[0]) + F(v_ax[k] * li[1])) + F(n[k] * li[2])) for k in range(3)])
    return np.array(thr, np.float32), np.array(wi, np.float32), pos[0], branch


@pytest.mark.parametrize("kind", ["lambert", "metal", "glass"])
def test_sample_surface_matches_restatement(kind):
    rng = np.random.default_rng({"lambert": 1, "metal": 2, "glass": 3}[kind])
    mat = abi.spk_material()
    mat.type = abi.SPK_MAT_DIELECTRIC if kind == "glass" else abi.SPK_MAT_PBR
    mat.base_color[:] = [0.7, 0.5, 0.3]
    mat.metallic = {"lambert": 0.0, "metal": 1.0, "glass": 0.0}[kind]
    mat.roughness = {"lambert": 1.0, "metal": 0.3, "glass": 0.0}[kind]
    mat.eta = 1.5
    branches = set()
    for trial in range(300):
        n = rng.standard_normal(3)
        n /= np.linalg.norm(n)
        t = np.cross(n, rng.standard_normal(3))
        t /= np.linalg.norm(t)
        d = rng.standard_normal(3)
        d /= np.linalg.norm(d)
        if kind != "glass" and np.dot(d, n) > 0:
            d = -d
        n, t, d = (x.astype(np.float32) for x in (n, t, d))
        got = oracle.sample_surface(mat, d, n, t, seed=trial)
        thr, wi, draws, branch = sample_surface_py(mat, d, n, t, trial)
        branches.add(branch)
        assert int(got[6]) == draws
        # exact up to the last bits of cos/sin/pow (numpy's float32 vs the C library's)
        np.testing.assert_allclose(got[:3], thr, rtol=2e-5, atol=1e-6)
        np.testing.assert_allclose(got[3:6], wi, rtol=2e-4, atol=2e-5)
    expected = {"lambert": {"diffuse", "specular"}, "metal": {"metal"}, "glass": {"reflect", "refract"}}[kind]
    assert expected <= branches


def test_accumulation_bookkeeping_and_tonemap(cornell):
    scene, cam_args = cornell
    W, H = 12, 10
    cam = scenes.make_camera(cam_args, W, H)
    cfg = abi.make_config(W, H, spp=1, max_spp=3, bounce=3)
    r = oracle.OracleRenderer(oracle.OracleScene(scene), cfg, cam)
    prev = None
    for k in range(5):
        r.render(1)
        c, d = r.sample_counts()
        assert (c, d) == (min(3, k), k + 1)  # cumulated before the frame, dispatched after it
        col, _ = r.gbuffer()
        hdr, out = r.framebuffer()
        w = F(min(3, k)) / F(min(3, k) + 1)
        exp = col if prev is None else (col + (prev - col) * w).astype(np.float32)
        assert np.array_equal(hdr, exp)
        x = (hdr[..., :3] * F(cam.exposure)).astype(np.float32)
        y = (x * (x * F(2.51) + F(0.03))) / (x * (x * F(2.43) + F(0.59)) + F(0.14))
        y = np.clip(y, 0, 1).astype(np.float32)
        assert np.array_equal(out[::-1, :, :3], y.astype(np.float16).view(np.uint16))
        assert np.all(out[..., 3] == 0x3C00)
        prev = hdr


def test_spp_reweights_like_the_reference(cornell):
    """spp only changes the accumulation weight: actual spp = lround(sqrt(spp))^2 (CPURenderer.cpp:102-104)."""
    scene, cam_args = cornell
    cam = scenes.make_camera(cam_args, 8, 8)
    r = oracle.OracleRenderer(oracle.OracleScene(scene), abi.make_config(8, 8, spp=5, bounce=2), cam)
    r.render(3)
    assert r.sample_counts() == (8, 12)  # spp 5 -> 2x2 = 4 per frame


def test_oracle_nee_converges_to_plain(cornell):
    """NEE + MIS (power heuristic) estimates the same image as plain path tracing once the bounce limit no
    longer cuts paths and no sample reaches the 6.0 clamp."""
    scene, cam_args = cornell
    scene = abi.Scene(scene.meshes, scene.instances, list(scene.materials), scene.sky)
    scene.materials[7] = abi.Material.light((2.0, 2.0, 2.0))
    sc = oracle.OracleScene(scene)
    cam = scenes.make_camera(cam_args, 12, 12)
    means = {}
    for nee in (False, True):
        acc = 0.0
        for seed in (1, 2, 3):
            cfg = abi.make_config(12, 12, spp=1, max_spp=1 << 20, bounce=24, enable_nee=nee,
                                  rng=abi.SPK_RNG_XOSHIRO256SS, seed=seed)
            r = oracle.OracleRenderer(sc, cfg, cam)
            r.render(4096, traversal=oracle.PRUNED)
            acc += r.framebuffer()[0][..., :3].astype(np.float64).mean()
        means[nee] = acc / 3
    assert abs(means[True] / means[False] - 1.0) < 1e-2
