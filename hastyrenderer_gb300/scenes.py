"""Seeded procedural render jobs in the reference's job format.

Each generator writes a ``renderJob.json`` (settings + scene path), a scene
JSON (camera, world, mesh), an ``.obj``/``.mtl`` pair and any images, exactly
the inputs ``PathTracingViewer <renderJob.json> <outDir>`` consumes
(core/src/RenderJob.cpp:10-28, core/src/Scene.cpp:12-118). Materials are
expressed through the MTL keys the reference maps to its Principled BRDF
(core/src/Scene.cpp:66-118): Kd albedo, Ns -> roughness = 1 - sqrt(Ns/1000),
Ka[0] metallic, Ks[0] specular, Ni IOR, d -> transmission = 1 - d, Ke
emission (radiance = Ke / pi), map_Kd / map_Ns / map_Pm / map_bump textures.

Workloads (sizes as the benchmark configurations state them):
  * ``cornell_box``   - 5 wall quads, 2 rotated cuboids, 1 quad light (36 tris).
  * ``sphere_field``  - N subdivision-3 icospheres on a ground plane under a
    procedural FP32 sky with a Gaussian sun (1.02M tris at N=800).
  * ``textured_room`` - textured quads (albedo, roughness, metallic, normal maps).
  * ``nested_media``  - concentric glass shells, each its own OBJ shape (the
    medium stack nests deeper than four), and a textured wall without
    texture coordinates (the texture's no-UV colour).
"""
from __future__ import annotations

import json
import math
import os

import numpy as np

__all__ = [
    "write_pfm", "write_pnm", "write_pam", "icosphere", "cornell_box", "sphere_field", "textured_room", "stress_scene",
    "nested_media",
    "sky_environment", "roughness_to_ns",
]


# ----------------------------------------------------------------- files --
def write_pfm(path: str, img: np.ndarray) -> None:
    """Write an HxWx3 (or HxW) float image, row 0 = top, as PFM (bottom row first)."""
    img = np.asarray(img, dtype="<f4")
    h, w = img.shape[:2]
    tag = b"PF" if img.ndim == 3 else b"Pf"
    with open(path, "wb") as f:
        f.write(tag + b"\n%d %d\n-1.0\n" % (w, h))
        f.write(np.ascontiguousarray(img[::-1]).tobytes())


def write_pnm(path: str, img: np.ndarray) -> None:
    """Write an 8-bit HxWx3 (PPM) or HxW (PGM) image, values in [0,1]."""
    a = np.clip(np.rint(np.asarray(img, dtype=np.float64) * 255.0), 0, 255).astype(np.uint8)
    h, w = a.shape[:2]
    tag = b"P6" if a.ndim == 3 else b"P5"
    with open(path, "wb") as f:
        f.write(tag + b"\n%d %d\n255\n" % (w, h))
        f.write(np.ascontiguousarray(a).tobytes())


def write_pam(path: str, img: np.ndarray) -> None:
    """Write an 8-bit HxWx4 RGBA (or HxWx3, alpha 255 added) PAM (P7, RGB_ALPHA), values in [0,1]."""
    a = np.clip(np.rint(np.asarray(img, dtype=np.float64) * 255.0), 0, 255).astype(np.uint8)
    if a.shape[-1] == 3:
        a = np.concatenate([a, np.full(a.shape[:2] + (1,), 255, np.uint8)], -1)
    h, w = a.shape[:2]
    with open(path, "wb") as f:
        f.write(b"P7\nWIDTH %d\nHEIGHT %d\nDEPTH 4\nMAXVAL 255\nTUPLTYPE RGB_ALPHA\nENDHDR\n" % (w, h))
        f.write(np.ascontiguousarray(a).tobytes())


def roughness_to_ns(r: float) -> float:
    """Inverse of roughness = 1 - sqrt(Ns/1000) (core/src/Scene.cpp:96-97)."""
    return 1000.0 * (1.0 - r) ** 2


def _fmt_rows(prefix: str, arr: np.ndarray, fmt: str = "%.9g") -> str:
    arr = np.asarray(arr, dtype=np.float64)
    if arr.size == 0:
        return ""
    line = prefix + " " + " ".join([fmt] * arr.shape[1]) + "\n"
    return (line * arr.shape[0]) % tuple(arr.ravel().tolist())


class _ObjWriter:
    def __init__(self):
        self.v, self.vn, self.vt = [], [], []
        self.nv = self.nvn = self.nvt = 0
        self.chunks: list[str] = []

    def add(self, name, verts, faces, material, normals=None, uvs=None, smooth=False):
        verts = np.asarray(verts, dtype=np.float64)
        faces = np.asarray(faces, dtype=np.int64)
        self.v.append(verts)
        base_v = self.nv
        self.nv += len(verts)
        out = [f"o {name}\nusemtl {material}\ns {'1' if smooth else 'off'}\n"]
        fv = faces + base_v + 1
        if normals is not None:
            self.vn.append(np.asarray(normals, dtype=np.float64))
            fn = faces + self.nvn + 1
            self.nvn += len(normals)
        if uvs is not None:
            self.vt.append(np.asarray(uvs, dtype=np.float64))
            ft = faces + self.nvt + 1
            self.nvt += len(uvs)
        if normals is not None and uvs is not None:
            cols = np.stack([fv[:, 0], ft[:, 0], fn[:, 0], fv[:, 1], ft[:, 1], fn[:, 1], fv[:, 2], ft[:, 2], fn[:, 2]], 1)
            out.append(("f %d/%d/%d %d/%d/%d %d/%d/%d\n" * len(faces)) % tuple(cols.ravel().tolist()))
        elif normals is not None:
            cols = np.stack([fv[:, 0], fn[:, 0], fv[:, 1], fn[:, 1], fv[:, 2], fn[:, 2]], 1)
            out.append(("f %d//%d %d//%d %d//%d\n" * len(faces)) % tuple(cols.ravel().tolist()))
        elif uvs is not None:
            cols = np.stack([fv[:, 0], ft[:, 0], fv[:, 1], ft[:, 1], fv[:, 2], ft[:, 2]], 1)
            out.append(("f %d/%d %d/%d %d/%d\n" * len(faces)) % tuple(cols.ravel().tolist()))
        else:
            out.append(("f %d %d %d\n" * len(faces)) % tuple(fv.ravel().tolist()))
        self.chunks.append("".join(out))

    def write(self, path, mtl_name):
        with open(path, "w") as f:
            f.write(f"mtllib {mtl_name}\n")
            for a in self.v:
                f.write(_fmt_rows("v", a))
            for a in self.vn:
                f.write(_fmt_rows("vn", a))
            for a in self.vt:
                f.write(_fmt_rows("vt", a))
            for c in self.chunks:
                f.write(c)


def _mtl_entry(name, kd=(0.8, 0.8, 0.8), ks=0.0, roughness=1.0, metallic=0.0, ior=1.5, dissolve=1.0,
               ke=None, map_kd=None, map_ns=None, map_pm=None, map_bump=None, aniso=None):
    s = [f"newmtl {name}", "Kd %.9g %.9g %.9g" % tuple(kd), "Ks %.9g %.9g %.9g" % (ks, ks, ks),
         "Ka %.9g %.9g %.9g" % (metallic, metallic, metallic), "Ns %.9g" % roughness_to_ns(roughness),
         "Ni %.9g" % ior, "d %.9g" % dissolve]
    if ke is not None:
        s.append("Ke %.9g %.9g %.9g" % tuple(ke))
    if aniso is not None:
        s.append("aniso %.9g" % aniso)
    for key, val in (("map_Kd", map_kd), ("map_Ns", map_ns), ("map_Pm", map_pm), ("map_bump", map_bump)):
        if val:
            s.append(f"{key} {val}")
    return "\n".join(s) + "\n\n"


def _write_job(out_dir, scene, settings, seed, mtl_text, obj: _ObjWriter, name="scene"):
    os.makedirs(out_dir, exist_ok=True)
    with open(os.path.join(out_dir, f"{name}.mtl"), "w") as f:
        f.write(mtl_text)
    obj.write(os.path.join(out_dir, f"{name}.obj"), f"{name}.mtl")
    scene = dict(scene)
    scene["mesh"] = f"{name}.obj"
    with open(os.path.join(out_dir, f"{name}.json"), "w") as f:
        json.dump(scene, f, indent=1)
    job = {"settings": settings, "scene": f"{name}.json", "gb300": {"seed": int(seed)}}
    path = os.path.join(out_dir, "renderJob.json")
    with open(path, "w") as f:
        json.dump(job, f, indent=1)
    return path


# -------------------------------------------------------------- geometry --
def icosphere(subdiv: int):
    """Unit icosphere: 10*4^s+2 vertices, 20*4^s faces (CCW seen from outside)."""
    t = (1.0 + 5 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, dtype=np.float64) / np.linalg.norm(p) for p in v]
    faces = list(f)
    for _ in range(subdiv):
        cache = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return np.array(verts), np.array(faces, dtype=np.int64)


def _quad(p0, p1, p2, p3):
    """Two triangles (p0,p1,p2),(p0,p2,p3); Ng = (p1-p0)x(p2-p0)."""
    return np.array([p0, p1, p2, p3], dtype=np.float64), np.array([[0, 1, 2], [0, 2, 3]])


def _cuboid(center, size, angle):
    sx, sy, sz = np.asarray(size, dtype=np.float64) / 2.0
    c = np.array([[-sx, -sy, -sz], [sx, -sy, -sz], [sx, sy, -sz], [-sx, sy, -sz],
                  [-sx, -sy, sz], [sx, -sy, sz], [sx, sy, sz], [-sx, sy, sz]])
    ca, sa = math.cos(angle), math.sin(angle)
    rot = np.array([[ca, 0, sa], [0, 1, 0], [-sa, 0, ca]])
    c = c @ rot.T + np.asarray(center, dtype=np.float64)
    # outward-facing, CCW from outside
    f = np.array([[0, 2, 1], [0, 3, 2], [4, 5, 6], [4, 6, 7], [0, 1, 5], [0, 5, 4],
                  [3, 6, 2], [3, 7, 6], [0, 4, 7], [0, 7, 3], [1, 2, 6], [1, 6, 5]])
    return c, f


# ---------------------------------------------------------------- scenes --
def cornell_box(out_dir, seed=0, width=256, height=256, spp=64, max_depth=8, roulette_start_depth=3,
                roulette_q=0.3, use_mis=True, light_radiance=15.0):
    """Procedural Cornell box: 5 wall quads (10 tris), 2 cuboids rotated by
    seeded angles in [0, pi/4] (24 tris), 1 quad light of the given radiance
    (2 tris, Ke = radiance*pi). Walls: Lambert 0.75 gray, red, green. Cuboids:
    GGX with roughness U[0.05, 1], metallic in {0, 1}, Ks 0.5."""
    rng = np.random.default_rng(seed)
    ow = _ObjWriter()
    L, H = 1.0, 2.0
    walls = [
        ("floor", "white", (-L, 0, -L), (-L, 0, L), (L, 0, L), (L, 0, -L)),
        ("ceiling", "white", (-L, H, -L), (L, H, -L), (L, H, L), (-L, H, L)),
        ("back", "white", (-L, 0, -L), (L, 0, -L), (L, H, -L), (-L, H, -L)),
        ("left", "red", (-L, 0, -L), (-L, H, -L), (-L, H, L), (-L, 0, L)),
        ("right", "green", (L, 0, -L), (L, 0, L), (L, H, L), (L, H, -L)),
    ]
    for name, mat, *pts in walls:
        v, f = _quad(*pts)
        ow.add(name, v, f, mat)
    a0, a1 = rng.uniform(0.0, math.pi / 4, size=2)
    r0, r1 = rng.uniform(0.05, 1.0, size=2)
    m0, m1 = rng.integers(0, 2, size=2)
    v, f = _cuboid((-0.35, 0.6, -0.3), (0.55, 1.2, 0.55), a0)
    ow.add("tall_box", v, f, "box0")
    v, f = _cuboid((0.38, 0.3, 0.35), (0.55, 0.6, 0.55), a1)
    ow.add("short_box", v, f, "box1")
    ls = 0.25
    v, f = _quad((-ls, H - 0.01, -ls), (ls, H - 0.01, -ls), (ls, H - 0.01, ls), (-ls, H - 0.01, ls))
    ow.add("light", v, f, "light")
    ke = light_radiance * math.pi
    mtl = (_mtl_entry("white", kd=(0.75, 0.75, 0.75)) + _mtl_entry("red", kd=(0.63, 0.06, 0.04))
           + _mtl_entry("green", kd=(0.14, 0.45, 0.09))
           + _mtl_entry("box0", kd=(0.8, 0.7, 0.5), ks=0.5, roughness=float(r0), metallic=float(m0))
           + _mtl_entry("box1", kd=(0.6, 0.7, 0.8), ks=0.5, roughness=float(r1), metallic=float(m1))
           + _mtl_entry("light", kd=(0, 0, 0), ke=(ke, ke, ke)))
    scene = {"camera": {"position": [0.0, 1.0, 3.4], "look_at": [0.0, 1.0, 0.0]},
             "world": {"background_color": [0.0, 0.0, 0.0]}}
    settings = {"num_samples": spp, "num_threads": 8, "width": width, "height": height,
                "roulette_start_depth": roulette_start_depth, "roulette_q": roulette_q,
                "max_depth": max_depth, "use_mis": use_mis}
    return _write_job(out_dir, scene, settings, seed, mtl, ow)


def sky_environment(width=2048, height=1024, sun_elevation_deg=35.0, sun_azimuth_deg=60.0,
                    sun_radius_deg=0.5, sun_intensity=1e4):
    """Lat-long FP32 sky (row 0 = zenith): vertical gradient plus a Gaussian sun
    of the given angular radius (1 sigma) and peak intensity. Directions follow
    the reference's convention theta = acos(d.y), phi = atan2(d.z, d.x)
    (core/include/Hasty/VMath.h:672-700)."""
    ys = (np.arange(height) + 0.5) / height
    xs = (np.arange(width) + 0.5) / width
    theta = ys[:, None] * math.pi
    phi = xs[None, :] * 2.0 * math.pi
    d = np.stack([np.sin(theta) * np.cos(phi), np.cos(theta) * np.ones_like(phi), np.sin(theta) * np.sin(phi)], -1)
    elev = np.clip(d[..., 1], -1.0, 1.0)
    horizon = np.array([0.85, 0.9, 1.0])
    zenith = np.array([0.15, 0.35, 0.85])
    ground = np.array([0.12, 0.1, 0.08])
    t = np.clip(elev, 0.0, 1.0)[..., None] ** 0.5
    sky = horizon * (1 - t) + zenith * t
    sky = np.where(elev[..., None] < 0.0, ground, sky)
    se, sa = math.radians(sun_elevation_deg), math.radians(sun_azimuth_deg)
    sun = np.array([math.cos(se) * math.cos(sa), math.sin(se), math.cos(se) * math.sin(sa)])
    ang = np.arccos(np.clip(d @ sun, -1.0, 1.0))
    sigma = math.radians(sun_radius_deg)
    s = sun_intensity * np.exp(-0.5 * (ang / sigma) ** 2)
    img = sky + s[..., None] * np.array([1.0, 0.95, 0.85])
    return img.astype(np.float32)


def sphere_field(out_dir, seed=0, n_spheres=800, subdiv=3, width=1920, height=1080, spp=256, max_depth=12,
                 env_size=(2048, 1024), aperture=0.15, num_blades=6, blade_rotation=0.3, box=20.0,
                 vary_glass_ior=False, roulette_start_depth=1, roulette_q=0.3, use_mis=True, sky_path=None):
    """N icospheres (radius log-uniform in [0.05, 0.5], centres uniform in a
    box of the given size above a 2-triangle ground plane). Materials: 40%
    Lambert, 40% GGX (roughness U[0.02, 1], metallic 0/1), 20% dielectric
    (transmission 1, roughness 0, IOR U[1.3, 1.7]). Procedural FP32 sky with a
    Gaussian sun, importance sampled; thin-lens camera with aperture blades.
    sky_path: use this existing sky PFM (it does not depend on the seed)
    instead of writing one into out_dir."""
    rng = np.random.default_rng(seed)
    ow = _ObjWriter()
    sv, sf = icosphere(subdiv)
    radii = np.exp(rng.uniform(math.log(0.05), math.log(0.5), size=n_spheres))
    half = box / 2.0
    centers = np.stack([rng.uniform(-half, half, n_spheres), rng.uniform(0.0, box, n_spheres),
                        rng.uniform(-half, half, n_spheres)], 1)
    centers[:, 1] = np.maximum(centers[:, 1], radii)
    kinds = rng.uniform(0.0, 1.0, n_spheres)
    mtl = [_mtl_entry("ground", kd=(0.45, 0.45, 0.42))]
    g = 60.0
    v, f = _quad((-g, 0, -g), (-g, 0, g), (g, 0, g), (g, 0, -g))
    ow.add("ground", v, f, "ground")
    for i in range(n_spheres):
        name = f"m{i}"
        col = rng.uniform(0.1, 0.9, 3)
        if kinds[i] < 0.4:
            mtl.append(_mtl_entry(name, kd=col))
        elif kinds[i] < 0.8:
            mtl.append(_mtl_entry(name, kd=col, ks=0.5, roughness=float(rng.uniform(0.02, 1.0)),
                                  metallic=float(rng.integers(0, 2))))
        else:
            tint = 1.0 - rng.uniform(0.0, 0.3, 3)
            mtl.append(_mtl_entry(name, kd=tint, ks=0.5, roughness=0.0, ior=float(rng.uniform(1.3, 1.7)), dissolve=0.0))
        ow.add(f"sphere{i}", sv * radii[i] + centers[i], sf, name, normals=sv, smooth=True)
    os.makedirs(out_dir, exist_ok=True)
    ew, eh = env_size
    if sky_path is None:
        write_pfm(os.path.join(out_dir, "sky.pfm"), sky_environment(ew, eh))
        sky_ref = "sky.pfm"
    else:
        sky_ref = os.path.abspath(sky_path)
    look = np.array([0.0, box * 0.25, 0.0])
    pos = np.array([0.0, box * 0.45, box * 1.35])
    scene = {"camera": {"position": pos.tolist(), "look_at": look.tolist(), "aperture": aperture,
                        "focal_distance": float(np.linalg.norm(pos - look)), "num_blades": num_blades,
                        "blade_rotation": blade_rotation},
             "world": {"environment_texture": sky_ref, "vary_glass_ior": bool(vary_glass_ior)}}
    settings = {"num_samples": spp, "num_threads": 8, "width": width, "height": height,
                "roulette_start_depth": roulette_start_depth, "roulette_q": roulette_q,
                "max_depth": max_depth, "use_mis": use_mis}
    return _write_job(out_dir, scene, settings, seed, "".join(mtl), ow)


def stress_scene(out_dir, seed=0, n_spheres=8000, n_cuboids=10000, tex_size=4096, width=3840, height=2160,
                 spp=1024, max_depth=32, box=60.0, roulette_start_depth=3, roulette_q=0.3):
    """Stress workload: n_spheres subdivision-3 icospheres (1280 tris each;
    10.24M at 8000) plus n_cuboids rotated cuboids (12 tris each) on a ground
    plane; 50% dispersive glass (Cauchy n = 1.5 + 0.0042 / lambda^2, um) and
    50% GGX (roughness U[0.01, 0.3]); four quads with tex_size^2 RGBA8
    value-noise albedo and normal maps; the procedural sky plus three area
    lights; thin lens; depth max_depth."""
    rng = np.random.default_rng(seed)
    os.makedirs(out_dir, exist_ok=True)
    ow = _ObjWriter()
    mtl = [_mtl_entry("ground", kd=(0.45, 0.45, 0.42))]
    g = box
    v, f = _quad((-g, 0, -g), (-g, 0, g), (g, 0, g), (g, 0, -g))
    ow.add("ground", v, f, "ground")

    def material(name):
        if rng.uniform() < 0.5:
            tint = 1.0 - rng.uniform(0.0, 0.2, 3)
            return _mtl_entry(name, kd=tint, ks=0.5, roughness=0.0, ior=1.5, dissolve=0.0)
        return _mtl_entry(name, kd=rng.uniform(0.1, 0.9, 3), ks=0.5, roughness=float(rng.uniform(0.01, 0.3)),
                          metallic=float(rng.integers(0, 2)))

    sv, sf = icosphere(3)
    half = box / 2.0
    for i in range(n_spheres):
        r = math.exp(rng.uniform(math.log(0.1), math.log(0.8)))
        c = np.array([rng.uniform(-half, half), rng.uniform(r, box * 0.4), rng.uniform(-half, half)])
        mtl.append(material(f"s{i}"))
        ow.add(f"sphere{i}", sv * r + c, sf, f"s{i}", normals=sv, smooth=True)
    for i in range(n_cuboids):
        size = rng.uniform(0.2, 1.5, 3)
        c = np.array([rng.uniform(-half, half), size[1] / 2.0, rng.uniform(-half, half)])
        cv, cf = _cuboid(c, size, float(rng.uniform(0.0, math.pi)))
        mtl.append(material(f"c{i}"))
        ow.add(f"cuboid{i}", cv, cf, f"c{i}")
    n = tex_size
    uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], dtype=np.float64)
    for k in range(4):
        alb = np.stack([_value_noise(rng, n, 32) * 0.8 + 0.1 for _ in range(3)], -1)
        h = _value_noise(rng, n, 64)
        gy, gx = np.gradient(h)
        nm = np.stack([-gx * 40.0, -gy * 40.0, np.ones_like(h)], -1)
        nm /= np.linalg.norm(nm, axis=-1, keepdims=True)
        write_pam(os.path.join(out_dir, f"albedo{k}.pam"), alb)
        write_pam(os.path.join(out_dir, f"normal{k}.pam"), nm * 0.5 + 0.5)
        x0 = -half + k * box / 4.0
        v, f = _quad((x0, 0.0, -half), (x0 + box / 4.5, 0.0, -half), (x0 + box / 4.5, box / 5.0, -half),
                     (x0, box / 5.0, -half))
        ow.add(f"panel{k}", v, f, f"tex{k}", uvs=uv)
        mtl.append(_mtl_entry(f"tex{k}", kd=(1, 1, 1), ks=0.4, roughness=0.4, map_kd=f"albedo{k}.pam",
                              map_bump=f"normal{k}.pam"))
    for k in range(3):
        x = (k - 1) * box / 3.0
        v, f = _quad((x - 2, box * 0.6, -2), (x + 2, box * 0.6, -2), (x + 2, box * 0.6, 2), (x - 2, box * 0.6, 2))
        ow.add(f"light{k}", v, f, f"light{k}")       # Ng = (p1 - p0) x (p2 - p0) points down, at the scene
        mtl.append(_mtl_entry(f"light{k}", kd=(0, 0, 0), ke=(60.0, 55.0, 50.0)))
    write_pfm(os.path.join(out_dir, "sky.pfm"), sky_environment(2048, 1024))
    look = np.array([0.0, box * 0.1, 0.0])
    pos = np.array([0.0, box * 0.35, box * 0.9])
    scene = {"camera": {"position": pos.tolist(), "look_at": look.tolist(), "aperture": 0.1,
                        "focal_distance": float(np.linalg.norm(pos - look)), "num_blades": 6},
             "world": {"environment_texture": "sky.pfm", "vary_glass_ior": True,
                       "dispersion": {"model": "cauchy", "b": 0.0042}}}
    settings = {"num_samples": spp, "num_threads": 8, "width": width, "height": height,
                "roulette_start_depth": roulette_start_depth, "roulette_q": roulette_q,
                "max_depth": max_depth, "use_mis": True}
    return _write_job(out_dir, scene, settings, seed, "".join(mtl), ow)


def _value_noise(rng, size, cells):
    grid = rng.uniform(0.0, 1.0, (cells + 1, cells + 1))
    t = np.linspace(0.0, cells, size, endpoint=False)
    i = np.floor(t).astype(int)
    fr = t - i
    fr = fr * fr * (3 - 2 * fr)
    a = grid[i][:, i]
    b = grid[i][:, i + 1]
    c = grid[i + 1][:, i]
    d = grid[i + 1][:, i + 1]
    fx = fr[None, :]
    fy = fr[:, None]
    return (a * (1 - fx) + b * fx) * (1 - fy) + (c * (1 - fx) + d * fx) * fy


def textured_room(out_dir, seed=0, width=64, height=48, spp=16, max_depth=8, tex_size=64, use_mis=True,
                  roulette_start_depth=2, roulette_q=0.3, rgba8=False, dispersion=None):
    """Textured quads (albedo map in sRGB, roughness/metallic maps, normal map),
    a smooth sphere without UVs (magenta fallback for its albedo map), an
    anisotropic GGX panel and an area light over a dim constant background.
    rgba8: write the albedo and normal maps as RGBA8 PAM files (same texel
    values as the PPM ones). dispersion: the world's "dispersion" object
    (e.g. {"model": "cauchy", "b": 0.0042}) for the dispersive glass."""
    rng = np.random.default_rng(seed)
    os.makedirs(out_dir, exist_ok=True)
    n = tex_size
    alb = np.stack([_value_noise(rng, n, 4) * 0.8 + 0.1 for _ in range(3)], -1)
    alb_name, nrm_name = ("albedo.pam", "normal.pam") if rgba8 else ("albedo.ppm", "normal.ppm")
    (write_pam if rgba8 else write_pnm)(os.path.join(out_dir, alb_name), alb)
    write_pnm(os.path.join(out_dir, "rough.pgm"), _value_noise(rng, n, 3) * 0.8 + 0.1)
    write_pnm(os.path.join(out_dir, "metal.pgm"), (_value_noise(rng, n, 2) > 0.6).astype(np.float64))
    h = _value_noise(rng, n, 6)
    gy, gx = np.gradient(h)
    nm = np.stack([-gx * 4.0, -gy * 4.0, np.ones_like(h)], -1)
    nm /= np.linalg.norm(nm, axis=-1, keepdims=True)
    (write_pam if rgba8 else write_pnm)(os.path.join(out_dir, nrm_name), nm * 0.5 + 0.5)
    ow = _ObjWriter()
    uv = np.array([[0, 0], [2, 0], [2, 2], [0, 2]], dtype=np.float64)
    v, f = _quad((-2, 0, -2), (-2, 0, 2), (2, 0, 2), (2, 0, -2))
    ow.add("floor", v, f, "tex_floor", uvs=uv[[0, 3, 2, 1]])
    v, f = _quad((-2, 0, -2), (2, 0, -2), (2, 3, -2), (-2, 3, -2))
    ow.add("wall", v, f, "tex_wall", uvs=uv)
    v, f = _quad((1.9, 0.2, -1.5), (1.9, 0.2, 1.0), (1.9, 2.0, 1.0), (1.9, 2.0, -1.5))
    ow.add("panel", v, f, "aniso")
    sv, sf = icosphere(2)
    ow.add("ball", sv * 0.6 + np.array([-0.6, 0.6, 0.2]), sf, "ball", normals=sv, smooth=True)
    gv, gf = icosphere(1)
    ow.add("glass", gv * 0.4 + np.array([0.7, 0.4, 0.6]), gf, "glass", normals=gv, smooth=True)
    v, f = _quad((-0.5, 2.9, -0.5), (0.5, 2.9, -0.5), (0.5, 2.9, 0.5), (-0.5, 2.9, 0.5))
    ow.add("light", v, f, "light")
    mtl = (_mtl_entry("tex_floor", kd=(1, 1, 1), ks=0.5, map_kd=alb_name, map_ns="rough.pgm",
                      map_pm="metal.pgm", map_bump=nrm_name)
           + _mtl_entry("tex_wall", kd=(1, 1, 1), ks=0.3, roughness=0.6, map_kd=alb_name, map_bump=nrm_name)
           + _mtl_entry("aniso", kd=(0.9, 0.6, 0.3), ks=0.5, roughness=0.35, metallic=1.0, aniso=0.8)
           + _mtl_entry("ball", kd=(0.9, 0.9, 0.9), ks=0.5, roughness=0.3, map_kd=alb_name)
           + _mtl_entry("glass", kd=(0.95, 0.97, 1.0), ks=0.5, roughness=0.0, ior=1.5, dissolve=0.0)
           + _mtl_entry("light", kd=(0, 0, 0), ke=(40.0, 38.0, 34.0)))
    scene = {"camera": {"position": [0.3, 1.6, 4.2], "look_at": [0.0, 0.8, 0.0], "aperture": 0.05,
                        "focal_distance": 4.0, "num_blades": 5},
             "world": {"background_color": [0.05, 0.06, 0.08], "vary_glass_ior": True}}
    if dispersion is not None:
        scene["world"]["dispersion"] = dict(dispersion)
    settings = {"num_samples": spp, "num_threads": 8, "width": width, "height": height,
                "roulette_start_depth": roulette_start_depth, "roulette_q": roulette_q,
                "max_depth": max_depth, "use_mis": use_mis}
    return _write_job(out_dir, scene, settings, seed, mtl, ow)


def nested_media(out_dir, seed=0, width=32, height=24, spp=4, max_depth=24, shells=6, roulette_start_depth=6,
                 roulette_q=0.2):
    """Concentric smooth-glass icosphere shells (subdivision 2), each its own
    OBJ shape and material (seeded IOR in [1.3, 1.7] and tint, which is the
    medium's transmittance), so a path reaching the core nests `shells` media
    (the medium stack of core/src/LightRayInfo.cpp:8-38 keyed by shape). A
    ground plane, a quad light, and a back wall whose material has an albedo
    texture but whose mesh has no texture coordinates (the texture's no-UV
    colour, core/include/Hasty/Texture.h:98-101)."""
    rng = np.random.default_rng(seed)
    os.makedirs(out_dir, exist_ok=True)
    ow = _ObjWriter()
    mtl = [_mtl_entry("ground", kd=(0.6, 0.6, 0.55)),
           _mtl_entry("wall", kd=(0.5, 0.5, 0.5), map_kd="wall.ppm"),
           _mtl_entry("light", kd=(0, 0, 0), ke=(40.0, 40.0, 40.0))]
    write_pnm(os.path.join(out_dir, "wall.ppm"), rng.uniform(0.2, 0.9, (8, 8, 3)))
    g = 6.0
    v, f = _quad((-g, 0, -g), (-g, 0, g), (g, 0, g), (g, 0, -g))
    ow.add("ground", v, f, "ground")
    v, f = _quad((-g, 0, -2.5), (g, 0, -2.5), (g, 4, -2.5), (-g, 4, -2.5))
    ow.add("wall", v, f, "wall")
    ls = 0.8
    v, f = _quad((-ls, 3.5, -ls), (ls, 3.5, -ls), (ls, 3.5, ls), (-ls, 3.5, ls))
    ow.add("light", v, f, "light")
    sv, sf = icosphere(2)
    c = np.array([0.0, 1.1, 0.0])
    r = 1.0
    for k in range(shells):
        name = f"glass{k}"
        tint = 1.0 - rng.uniform(0.0, 0.25, 3)
        mtl.append(_mtl_entry(name, kd=tint, ks=0.5, roughness=0.0, ior=float(rng.uniform(1.3, 1.7)), dissolve=0.0))
        ow.add(f"shell{k}", sv * r + c, sf, name, normals=sv, smooth=True)
        r *= 0.8
    scene = {"camera": {"position": [0.0, 1.4, 4.2], "look_at": [0.0, 1.0, 0.0]},
             "world": {"background_color": [0.05, 0.05, 0.08]}}
    settings = {"num_samples": spp, "num_threads": 8, "width": width, "height": height,
                "roulette_start_depth": roulette_start_depth, "roulette_q": roulette_q, "max_depth": max_depth,
                "use_mis": True}
    return _write_job(out_dir, scene, settings, seed, "".join(mtl), ow)
