"""CPU-only checks: the oracle against the reference's own tables, the oracle's
BVH and intersection against brute force, scene generation, and the C ABI
library's exported symbols (loaded, never called, so no GPU is needed)."""
import ctypes
import hashlib
import json
import os
import re

import numpy as np
import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INF = np.float32(np.inf)


def test_sampler_tables_match_reference_golden():
    """Halton permutations and Sobol matrices regenerated from Faure /
    Joe-Kuo constructions equal the reference's math/halton.inl and
    math/sobol.inl tables (digests in tests/golden/sampler_tables.json)."""
    golden = json.load(open(os.path.join(ROOT, "tests", "golden", "sampler_tables.json")))
    t = oracle.tables()
    for name, g in golden.items():
        a = t[name]
        assert a.size == g["count"]
        assert [int(x) for x in a[:16]] == g["head"], name
        assert hashlib.sha256(a.astype("<u4").tobytes()).hexdigest() == g["sha256"], name


def _rand_tris(rng, n):
    c = rng.uniform(0, 1, (n, 1, 3))
    v = (c + rng.uniform(-0.08, 0.08, (n, 3, 3))).astype(np.float32)
    return v.reshape(-1, 3), np.arange(3 * n, dtype=np.uint32).reshape(-1, 3)


def _brute(rays, tris, spheres):
    """float64 closest hit: (t, kind, index); kind 0 triangle, 1 sphere."""
    o, d = rays[:, None, 0:3].astype(np.float64), rays[:, None, 4:7].astype(np.float64)
    tn, tf = rays[:, 3:4].astype(np.float64), rays[:, 7:8].astype(np.float64)
    v0, v1, v2 = (tris[None, :, k].astype(np.float64) for k in range(3))
    e1, e2 = v1 - v0, v2 - v0
    p = np.cross(d, e2)
    det = np.sum(e1 * p, -1)
    s = o - v0
    with np.errstate(divide="ignore", invalid="ignore"):
        u = np.sum(s * p, -1) / det
        q = np.cross(s, e1)
        v = np.sum(d * q, -1) / det
        t = np.sum(e2 * q, -1) / det
    ok = (u >= 0) & (v >= 0) & (u + v <= 1) & (t >= tn) & (t <= tf) & np.isfinite(t)
    tt = np.where(ok, t, np.inf)
    c, r = spheres[None, :, :3].astype(np.float64), spheres[None, :, 3].astype(np.float64)
    oc = c - o
    a = np.sum(d * d, -1)
    b = np.sum(oc * d, -1) / a
    perp = oc - b[..., None] * d
    l2 = np.sum(perp * perp, -1)
    with np.errstate(invalid="ignore"):
        td = np.sqrt((r * r - l2) / a)
    t0, t1 = b - td, b + td
    ts = np.where((t0 >= tn) & (t0 <= tf), t0, np.where((t1 >= tn) & (t1 <= tf), t1, np.inf))
    ts = np.where(l2 <= r * r, ts, np.inf)
    allt = np.concatenate([tt, ts], 1)
    idx = np.argmin(allt, 1)
    best = allt[np.arange(len(rays)), idx]
    kind = (idx >= tris.shape[1]).astype(int)
    return best, kind, np.where(kind == 0, idx, idx - tris.shape[1])


def test_oracle_bvh_matches_brute_force():
    rng = np.random.default_rng(1)
    v, i = _rand_tris(rng, 300)
    sph = np.concatenate([rng.uniform(0, 1, (60, 3)), rng.uniform(0.01, 0.05, (60, 1))], 1).astype(np.float32)
    sc = oracle.Scene()
    gm, gs = sc.add_mesh(v, i), sc.add_spheres(sph)
    sc.add_instance(gm, 0, 0)
    sc.add_instance(gs, 0, 1)
    sc.commit()
    n = 4000
    org = rng.uniform(-0.5, 1.5, (n, 3))
    tgt = rng.uniform(0, 1, (n, 3))
    d = tgt - org
    rays = np.concatenate([org, np.zeros((n, 1)), d, np.full((n, 1), np.inf)], 1).astype(np.float32)
    f, ids = sc.trace(rays)
    bt, kind, idx = _brute(rays, v.reshape(-1, 3, 3), sph)
    hit = np.isfinite(bt)
    assert np.array_equal(hit, np.isfinite(f[:, 0]) | False) or np.mean(hit != np.isfinite(f[:, 0])) < 1e-3
    both = hit & np.isfinite(f[:, 0])
    rel = np.abs(f[both, 0] - bt[both]) / np.maximum(bt[both], 1e-6)
    assert rel.max() < 1e-4
    agree = (ids[both, 1] == kind[both]) & (ids[both, 0] == idx[both])
    # disagreements only at near-ties
    assert np.all(agree | (rel < 1e-5)), np.flatnonzero(~agree)[:10]
    # occlusion agrees with closest-hit existence
    occ, _ = sc.trace(rays, occlusion=True)
    assert np.array_equal(occ[:, 0] > 0, np.isfinite(f[:, 0]))


def test_oracle_watertight_on_shared_edges_and_vertices():
    """Rays aimed exactly at the vertices and edge midpoints of a flat grid
    all hit: the watertight test leaves no cracks between triangles."""
    n = 17
    xs = np.linspace(0, 1, n, dtype=np.float32)
    X, Z = np.meshgrid(xs, xs)
    v = np.stack([X.ravel(), np.zeros(n * n, np.float32), Z.ravel()], 1)
    idx = []
    for j in range(n - 1):
        for i in range(n - 1):
            a = j * n + i
            idx += [[a, a + n, a + 1], [a + 1, a + n, a + n + 1]]
    sc = oracle.Scene()
    g = sc.add_mesh(v, np.array(idx, np.uint32))
    sc.add_instance(g, 0, 0)
    sc.commit()
    inner = v[(v[:, 0] > 0) & (v[:, 0] < 1) & (v[:, 2] > 0) & (v[:, 2] < 1)]
    mids = 0.5 * (inner[:-1] + inner[1:])
    pts = np.concatenate([inner, mids], 0)
    rays = np.zeros((len(pts), 8), np.float32)
    rays[:, 0], rays[:, 1], rays[:, 2] = pts[:, 0], 1.0, pts[:, 2]
    rays[:, 5], rays[:, 7] = -1.0, np.inf
    f, ids = sc.trace(rays)
    assert np.all(np.isfinite(f[:, 0])) and np.allclose(f[:, 0], 1.0)


def test_scene_generators_deterministic():
    from ospray_gb300 import scenes
    a = scenes.ao_heightfield_scene()
    b = scenes.ao_heightfield_scene()
    assert a["index"].shape == (130050, 3) and a["vertex"].shape == (65536, 3)
    assert a["spheres"].shape == (1000, 4)
    assert np.array_equal(a["vertex"], b["vertex"]) and np.array_equal(a["spheres"], b["spheres"])
    s = a["spheres"]
    assert s[:, 1].max() <= 0.3 and s[:, 3].min() >= 0.005 and s[:, 3].max() <= 0.02
    v, i = scenes.displaced_sphere(6)
    assert i.shape == (32768, 3) and v.shape[0] == 16386


def _header_symbols(path):
    text = open(path).read()
    return sorted(set(re.findall(r"^\s*(?:[\w\s\*]+?)\b(b200_\w+)\s*\(", text, re.M)))


def test_c_abi_library_exports_header_symbols():
    """Every function include/b200.h declares is exported by libb200.so."""
    import ospray_gb300 as og
    syms = _header_symbols(os.path.join(ROOT, "include", "b200.h"))
    assert "b200_trace" in syms and "b200_render_ao" in syms
    lib = ctypes.CDLL(og.lib_path())
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_oracle_volume_gradient_shading_invariants():
    """The SciVis integrator with gradient shading: scale 0 reproduces the
    volume-only renderer exactly; scale 1 keeps every pixel's alpha (the
    shaded opacity 1 - luminance(1 - a) equals a up to rounding) and only
    recolours the volume (lit by a quad and a dim ambient light: darker)."""
    from ospray_gb300 import scenes
    W, H = 48, 40
    v = scenes.volume_scene(n=20, width=W, height=H)
    lights = [dict(type="quad", position=(-1.0, 2.5, -1.0), edge1=(0.5, 0.0, 0.0), edge2=(0.0, 0.0, 0.5),
                   intensity=6.0, visible=False),
              dict(type="ambient", intensity=0.25, color=(1.0, 1.0, 1.0), visible=False)]
    ov = oracle.VolumeModel(v["volume"], v["origin"], v["spacing"], v["color"], v["opacity"], v["value_range"])
    c = v["camera"]
    cam = oracle.camera(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=W / H)
    plain = oracle.render_scivis(None, ov, cam, lights, [], W, H, spp=2, shadows=True)["color"]
    assert np.array_equal(plain, oracle.render_scivis_volume(ov, cam, 2, W, H, spp=2))
    ov.set_gradient_shading(1.0)
    shaded = oracle.render_scivis(None, ov, cam, lights, [], W, H, spp=2, shadows=True)["color"]
    assert plain[..., 3].max() > 0.3
    assert np.abs(shaded[..., 3] - plain[..., 3]).max() < 1e-5
    assert shaded[..., :3].mean() < plain[..., :3].mean()


def _heightfield_quads(n=24, seed=3):
    rng = np.random.default_rng(seed)
    xs = np.linspace(0.0, 1.0, n, dtype=np.float32)
    X, Z = np.meshgrid(xs, xs)
    Y = (0.08 * np.sin(7.0 * X + 1.3) * np.cos(5.0 * Z) + 0.01 * rng.standard_normal(X.shape)).astype(np.float32)
    v = np.stack([X, Y, Z], -1).reshape(-1, 3)
    i, j = np.meshgrid(np.arange(n - 1), np.arange(n - 1))
    a = (j * n + i).ravel()
    q = np.stack([a, a + 1, a + n + 1, a + n], 1).astype(np.uint32)
    return v, q


def test_oracle_quad_mesh_is_embree_triangle_pair():
    """A quad (v0, v1, v2, v3) traces as the triangles (v0, v1, v3) and
    (v2, v3, v1), Embree's quad decomposition, and reports the quad's index:
    hit t bit for bit and primID = triangle // 2 against the same mesh given
    as triangles."""
    v, q = _heightfield_quads()
    tri = np.stack([q[:, 0], q[:, 1], q[:, 3], q[:, 2], q[:, 3], q[:, 1]], 1).reshape(-1, 3)
    sq, st = oracle.Scene(), oracle.Scene()
    sq.add_instance(sq.add_quad_mesh(v, q), 0, 0)
    st.add_instance(st.add_mesh(v, tri), 0, 0)
    sq.commit()
    st.commit()
    rng = np.random.default_rng(1)
    n = 20000
    org = np.concatenate([rng.uniform(0, 1, (n, 1)), np.full((n, 1), 0.8), rng.uniform(0, 1, (n, 1))], 1)
    d = np.concatenate([rng.normal(0, 0.3, (n, 1)), -np.ones((n, 1)), rng.normal(0, 0.3, (n, 1))], 1)
    rays = np.concatenate([org, np.zeros((n, 1)), d, np.full((n, 1), np.inf)], 1).astype(np.float32)
    fq, iq = sq.trace(rays)
    ft, it = st.trace(rays)
    hit = np.isfinite(ft[:, 0])
    assert hit.mean() > 0.5
    np.testing.assert_array_equal(fq[:, 0].view(np.uint32), ft[:, 0].view(np.uint32))
    assert np.array_equal(iq[hit, 0], it[hit, 0] // 2)


def _random_boxes(n=60, seed=4):
    rng = np.random.default_rng(seed)
    c = rng.uniform(0.0, 1.0, (n, 3))
    h = rng.uniform(0.01, 0.08, (n, 3))
    return np.concatenate([c - h, c + h], 1).astype(np.float32)


def test_oracle_boxes_match_slab_test():
    """Boxes traced as face triangles report the box hit of intersectBox +
    filterIntersectionBoth (common/Intersect.ih:195-223, FilterIntersect.ih:
    107-116): the entry face in range, else the exit face; checked against a
    float64 slab test (t within 1e-5 relative, primID = box index, the
    normal along the face's axis) away from edges."""
    b = _random_boxes()
    s = oracle.Scene()
    s.add_instance(s.add_boxes(b), 0, 0)
    s.commit()
    rng = np.random.default_rng(7)
    n = 20000
    org = rng.uniform(-0.2, 1.2, (n, 3))
    inside = rng.integers(0, len(b), 500)
    org[:500] = (b[inside, :3] + b[inside, 3:]) / 2  # rays starting inside a box hit its exit face
    d = rng.normal(size=(n, 3))
    rays = np.concatenate([org, np.zeros((n, 1)), d, np.full((n, 1), np.inf)], 1).astype(np.float32)
    f, ids = s.trace(rays)
    o64, d64 = org.astype(np.float32).astype(np.float64), d.astype(np.float32).astype(np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        t0 = (b[None, :, :3] - o64[:, None]) / d64[:, None]
        t1 = (b[None, :, 3:] - o64[:, None]) / d64[:, None]
    tn, tf = np.minimum(t0, t1).max(2), np.maximum(t0, t1).min(2)
    ok = tn < tf
    t = np.where(ok & (tn >= 0), tn, np.where(ok & (tf >= 0), tf, np.inf))
    best = t.min(1)
    prim = t.argmin(1)
    # skip near-ties between boxes and grazing rays
    srt = np.sort(t, 1)
    with np.errstate(invalid="ignore"):
        clear = (srt[:, 1] - srt[:, 0] > 1e-4 * np.maximum(1.0, srt[:, 0])) | ~np.isfinite(srt[:, 1])
    hit = np.isfinite(best)
    assert hit[clear].sum() > 2000 and hit[:500].all()
    m = clear & hit
    np.testing.assert_allclose(f[m, 0], best[m], rtol=1e-5)
    assert np.mean(ids[m, 0] == prim[m]) > 0.999
    assert np.all(~np.isfinite(f[clear & ~hit, 0]))
    ng = f[m, 3:6]
    assert np.all(np.sum(np.abs(ng) > 0, 1) == 1)  # axis-aligned face normals
