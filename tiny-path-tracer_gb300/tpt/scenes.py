"""Seeded scene generators emitting scene-description (SD) text.

The SD format (one statement per line) is the interchange the product loader
(`tpt_scene_from_text`), the CPU oracle and the reference harness all read, so
the three build identical scenes.  Values are rounded to float32 before they
are written and printed with 9 significant digits, so every reader parses the
exact same floats.

Workloads (sizes from the benchmark definitions):
  one_weekend      random-sphere scene, 488 spheres, BVH, 400x400 16 spp
  cornell          book Cornell box, 600x600 1024 spp
  cornell_guiding  Cornell box with a 40x40 light and a second box
  next_week        the 'next week' final scene (boxes, media, textures)
  batch_scenes     64 random-sphere scenes of 50..5000 spheres
The reference builds the same kinds of scenes in src/utils.cc:96-414.
"""
from __future__ import annotations

import numpy as np

F32 = np.float32


def fmt(v: float) -> str:
    return "%.9g" % float(F32(v))


class SD:
    """Accumulates SD statements; ids are assigned per kind in order."""

    def __init__(self) -> None:
        self.lines: list[str] = []
        self.n_tex = 0
        self.n_mat = 0
        self.n_node = 0
        self.meta: dict = {}

    # textures -----------------------------------------------------------
    def const(self, r, g, b) -> int:
        i = self.n_tex
        self.n_tex += 1
        self.lines.append(f"tex {i} const {fmt(r)} {fmt(g)} {fmt(b)}")
        return i

    def checker(self, odd: int, even: int) -> int:
        i = self.n_tex
        self.n_tex += 1
        self.lines.append(f"tex {i} checker {odd} {even}")
        return i

    def perlin(self, scale) -> int:
        i = self.n_tex
        self.n_tex += 1
        self.lines.append(f"tex {i} perlin {fmt(scale)}")
        return i

    def image(self, w: int, h: int, seed: int) -> int:
        i = self.n_tex
        self.n_tex += 1
        self.lines.append(f"tex {i} image {w} {h} {seed}")
        return i

    def perlin_tables(self, rng: np.random.Generator) -> None:
        """256 unit gradients and three permutations of 0..255 (the tables the
        reference fills in perlin_noise.cc:3-21, here from a seed)."""
        g = rng.uniform(-1.0, 1.0, size=(256, 3)).astype(F32)
        n = np.sqrt((g * g).sum(axis=1, dtype=F32)).astype(F32)
        g = (g / n[:, None]).astype(F32)
        perms = [rng.permutation(256) for _ in range(3)]
        parts = [fmt(v) for v in g.reshape(-1)] + [str(int(v)) for p in perms for v in p]
        self.lines.append("perlin_tables " + " ".join(parts))

    # materials ----------------------------------------------------------
    def _mat(self, body: str) -> int:
        i = self.n_mat
        self.n_mat += 1
        self.lines.append(f"mat {i} {body}")
        return i

    def lambertian(self, tex: int) -> int:
        return self._mat(f"lambertian {tex}")

    def metal(self, r, g, b, fuzz) -> int:
        return self._mat(f"metal {fmt(r)} {fmt(g)} {fmt(b)} {fmt(fuzz)}")

    def dielectric(self, ior) -> int:
        return self._mat(f"dielectric {fmt(ior)}")

    def diffuse_light(self, tex: int) -> int:
        return self._mat(f"diffuse_light {tex}")

    def isotropic(self, tex: int) -> int:
        return self._mat(f"isotropic {tex}")

    # hitables -----------------------------------------------------------
    def _node(self, body: str) -> int:
        i = self.n_node
        self.n_node += 1
        self.lines.append(f"node {i} {body}")
        return i

    def sphere(self, c, r, mat: int) -> int:
        return self._node(f"sphere {fmt(c[0])} {fmt(c[1])} {fmt(c[2])} {fmt(r)} {mat}")

    def moving_sphere(self, c0, c1, t0, t1, r, mat: int) -> int:
        return self._node("moving_sphere " + " ".join(fmt(v) for v in (*c0, *c1, t0, t1, r)) + f" {mat}")

    def rect(self, kind: str, a0, a1, b0, b1, k, mat: int) -> int:
        return self._node(f"{kind} {fmt(a0)} {fmt(a1)} {fmt(b0)} {fmt(b1)} {fmt(k)} {mat}")

    def flip(self, child: int) -> int:
        return self._node(f"flip_normal {child}")

    def box(self, p0, p1, mat: int) -> int:
        return self._node("box " + " ".join(fmt(v) for v in (*p0, *p1)) + f" {mat}")

    def translate(self, child: int, off) -> int:
        return self._node(f"translate {child} {fmt(off[0])} {fmt(off[1])} {fmt(off[2])}")

    def rotate_y(self, child: int, angle) -> int:
        return self._node(f"rotate_y {child} {fmt(angle)}")

    def medium(self, boundary: int, density, tex: int) -> int:
        return self._node(f"constant_medium {boundary} {fmt(density)} {tex}")

    def hlist(self, items) -> int:
        return self._node(f"hitable_list {len(items)} " + " ".join(str(i) for i in items))

    def bvh(self, items, t0=0.0, t1=0.0) -> int:
        return self._node(f"bvh_node {fmt(t0)} {fmt(t1)} {len(items)} " + " ".join(str(i) for i in items))

    def world(self, node: int) -> None:
        self.lines.append(f"world {node}")

    def lights(self, node: int) -> None:
        self.lines.append(f"lights {node}")

    def camera(self, lookfrom, lookat, vup, vfov, aspect, aperture, focus, t0=0.0, t1=0.0) -> None:
        vals = (*lookfrom, *lookat, *vup, vfov, aspect, aperture, focus, t0, t1)
        self.lines.append("camera " + " ".join(fmt(v) for v in vals))

    def text(self) -> str:
        return "\n".join(self.lines) + "\n"


def _main_cpp_lights(sd: SD) -> int:
    """The light list the reference's main() passes for every scene
    (main.cpp:99-106): xz_rect(-100,100,-150,-50,298) and
    sphere((120,-50,40),120); their materials are never used."""
    dummy = sd.lambertian(sd.const(0, 0, 0))
    a = sd.rect("xz_rect", -100, 100, -150, -50, 298, dummy)
    b = sd.sphere((120, -50, 40), 120, dummy)
    return sd.hlist([a, b])


def one_weekend(seed: int = 1, grid: tuple[int, int] = (-11, 11), n_small: int | None = None,
                main_lights: bool = True) -> SD:
    """Random-sphere scene: ground r=1000 lambertian 0.5; a sphere r=0.2 per
    grid cell at (a+0.9u, 0.2, b+0.9u) with lambertian (albedo u*u), metal
    (albedo 0.5(1+u), fuzz 0.5u) or dielectric 1.5 for m<0.8, <0.95, else;
    three r=1 spheres; BVH over all (t0=0, t1=1 as utils.cc:138)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sd = SD()
    items = [sd.sphere((0, -1000, 0), 1000, sd.lambertian(sd.const(0.5, 0.5, 0.5)))]
    cells = [(a, b) for a in range(grid[0], grid[1]) for b in range(grid[0], grid[1])]
    if n_small is not None:
        cells = cells[:n_small]
    for a, b in cells:
        m = rng.random()
        cx = a + 0.9 * rng.random()
        cz = b + 0.9 * rng.random()
        if m < 0.8:
            alb = [rng.random() * rng.random() for _ in range(3)]
            mat = sd.lambertian(sd.const(*alb))
        elif m < 0.95:
            alb = [0.5 * (1 + rng.random()) for _ in range(3)]
            mat = sd.metal(*alb, 0.5 * rng.random())
        else:
            mat = sd.dielectric(1.5)
        items.append(sd.sphere((cx, 0.2, cz), 0.2, mat))
    items.append(sd.sphere((0, 1, 0), 1.0, sd.dielectric(1.5)))
    items.append(sd.sphere((-4, 1, 0), 1.0, sd.lambertian(sd.const(0.4, 0.2, 0.1))))
    items.append(sd.sphere((4, 1, 0), 1.0, sd.metal(0.7, 0.6, 0.5, 0.0)))
    world = sd.bvh(items, 0.0, 1.0)
    sd.world(world)
    if main_lights:
        sd.lights(_main_cpp_lights(sd))
    sd.camera((13, 2, 3), (0, 0, 0), (0, 1, 0), 20.0, 1.0, 0.1, 10.0, 0.0, 0.0)
    sd.meta = dict(width=400, height=400, spp=16, max_depth=50, background=1, sky_scale=1.0,
                   n_spheres=len(items))
    return sd


def cornell(light=(213, 343, 227, 332), emission=15.0, short_box=False, aspect=1.0) -> SD:
    """Book Cornell box (the layout of utils.cc:276-281 with the light
    flipped so it emits downward): red yz_rect x=0, green yz_rect x=555,
    white floor/ceiling/back, tall box 165x330x165 rotated +15 at
    (265,0,295), glass sphere r=90 at (190,90,190); BVH over the items like
    the reference's cornell_box() (utils.cc:287-319).  light_shape = the
    light rect and the glass sphere, as main.cpp:99-106 pairs them."""
    sd = SD()
    red = sd.lambertian(sd.const(0.65, 0.05, 0.05))
    white = sd.lambertian(sd.const(0.73, 0.73, 0.73))
    green = sd.lambertian(sd.const(0.12, 0.45, 0.15))
    lightm = sd.diffuse_light(sd.const(emission, emission, emission))
    x0, x1, z0, z1 = light
    items = [
        sd.flip(sd.rect("yz_rect", 0, 555, 0, 555, 555, green)),
        sd.rect("yz_rect", 0, 555, 0, 555, 0, red),
        sd.flip(sd.rect("xz_rect", x0, x1, z0, z1, 554, lightm)),
        sd.flip(sd.rect("xz_rect", 0, 555, 0, 555, 555, white)),
        sd.rect("xz_rect", 0, 555, 0, 555, 0, white),
        sd.flip(sd.rect("xy_rect", 0, 555, 0, 555, 555, white)),
    ]
    tall = sd.box((0, 0, 0), (165, 330, 165), white)
    items.append(sd.translate(sd.rotate_y(tall, 15.0), (265, 0, 295)))
    if short_box:
        sb = sd.box((0, 0, 0), (165, 165, 165), white)
        items.append(sd.translate(sd.rotate_y(sb, -18.0), (130, 0, 65)))
    items.append(sd.sphere((190, 90, 190), 90, sd.dielectric(1.5)))
    world = sd.bvh(items, 0.0, 0.0)
    sd.world(world)
    dummy = sd.lambertian(sd.const(0, 0, 0))
    ls = sd.rect("xz_rect", x0, x1, z0, z1, 554, dummy)
    gs = sd.sphere((190, 90, 190), 90, dummy)
    sd.lights(sd.hlist([ls, gs]))
    sd.camera((278, 278, -800), (278, 278, 0), (0, 1, 0), 40.0, aspect, 0.0, 10.0, 0.0, 0.0)
    sd.meta = dict(width=600, height=600, spp=1024, max_depth=50, background=0, sky_scale=1.0)
    return sd


def cornell_guiding() -> SD:
    """Cornell box with the light shrunk to 40x40 around the original light
    centre (278, 279.5) and a 165^3 box rotated -18 at (130,0,65)."""
    sd = cornell(light=(258, 298, 259.5, 299.5), short_box=True)
    return sd


def next_week(seed: int = 4, image_size=(2048, 1024)) -> SD:
    """'Next week' final scene (utils.cc:359-414 layout): 20x20 ground boxes
    width 100, height 100*(u+0.01); light xz_rect [123,423]x[147,412] y=554
    emission 7 (flipped to emit downward, as the one-sided emission of
    material.cc:79-86 requires); glass sphere r=50; metal sphere r=50 fuzz
    1.0; medium density 0.2 inside a glass sphere r=70; a sphere with a
    procedural image texture; a perlin sphere scale 0.1; 1000 spheres r=10
    in a 165^3 cube, rotated 15 and translated (-100,270,395).  The moving
    sphere and the r=5000 mist of the reference scene are left out."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sd = SD()
    white = sd.lambertian(sd.const(0.73, 0.73, 0.73))
    ground = sd.lambertian(sd.const(0.48, 0.83, 0.53))
    boxes = []
    for i in range(20):
        for j in range(20):
            w = 100.0
            x0 = -1000 + i * w
            z0 = -1000 + j * w
            y1 = 100 * (rng.random() + 0.01)
            boxes.append(sd.box((x0, 0, z0), (x0 + w, y1, z0 + w), ground))
    items = [sd.bvh(boxes, 0.0, 1.0)]
    lightm = sd.diffuse_light(sd.const(7, 7, 7))
    items.append(sd.flip(sd.rect("xz_rect", 123, 423, 147, 412, 554, lightm)))
    items.append(sd.sphere((260, 150, 45), 50, sd.dielectric(1.5)))
    items.append(sd.sphere((0, 150, 145), 50, sd.metal(0.8, 0.8, 0.9, 1.0)))
    boundary = sd.sphere((360, 150, 145), 70, sd.dielectric(1.5))
    items.append(boundary)
    items.append(sd.medium(boundary, 0.2, sd.const(0.2, 0.4, 0.9)))
    img = sd.image(image_size[0], image_size[1], seed * 7919 + 17)
    items.append(sd.sphere((400, 200, 400), 100, sd.lambertian(img)))
    sd.perlin_tables(rng)
    items.append(sd.sphere((220, 280, 300), 80, sd.lambertian(sd.perlin(0.1))))
    balls = []
    for _ in range(1000):
        c = (165 * rng.random(), 165 * rng.random(), 165 * rng.random())
        balls.append(sd.sphere(c, 10, white))
    inst = sd.translate(sd.rotate_y(sd.bvh(balls, 0.0, 1.0), 15.0), (-100, 270, 395))
    items.append(inst)
    sd.world(sd.hlist(items))
    dummy = sd.lambertian(sd.const(0, 0, 0))
    sd.lights(sd.hlist([sd.rect("xz_rect", 123, 423, 147, 412, 554, dummy)]))
    sd.camera((478, 278, -600), (278, 278, 0), (0, 1, 0), 40.0, 1.0, 0.0, 10.0, 0.0, 1.0)
    sd.meta = dict(width=800, height=800, spp=256, max_depth=50, background=0, sky_scale=1.0)
    return sd


def batch_scenes(seed: int = 2, count: int = 64) -> list[SD]:
    """64 random-sphere scenes (one_weekend layout) with a sphere count
    uniform in [50, 5000], resolution uniform in {256,512,768,1024}^2 and spp
    uniform in [8, 64], each from its own seed."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for k in range(count):
        n = int(rng.integers(50, 5001))
        res = int(rng.choice([256, 512, 768, 1024]))
        spp = int(rng.integers(8, 65))
        side = int(np.ceil(np.sqrt(n - 4)))
        lo = -(side // 2)
        sd = one_weekend(seed=1000 + k, grid=(lo, lo + side), n_small=n - 4)
        sd.meta.update(width=res, height=res, spp=spp, n_spheres=n)
        out.append(sd)
    return out


def tie_scene() -> SD:
    """Exact-tie known-answer cases: coincident spheres inside a BVH (the
    right subtree wins, hitable.cc:71-78), coincident spheres inside a list
    (the earlier wins: strict '<', sphere.cc:21) and coincident rects inside a
    list (the later wins: rect t may equal t_max, rect_box.cc:54)."""
    sd = SD()
    m = [sd.lambertian(sd.const(0.1 * (i + 1), 0.5, 0.5)) for i in range(8)]
    a = sd.sphere((0, 0, -5), 1, m[0])
    b = sd.sphere((0, 0, -5), 1, m[1])
    bv = sd.bvh([a, b], 0, 0)
    c = sd.sphere((3, 0, -5), 1, m[2])
    d = sd.sphere((3, 0, -5), 1, m[3])
    li = sd.hlist([c, d])
    e = sd.rect("xy_rect", -7, -5, -1, 1, -5, m[4])
    f = sd.rect("xy_rect", -7, -5, -1, 1, -5, m[5])
    lr = sd.hlist([e, f])
    sd.world(sd.hlist([bv, li, lr]))
    sd.camera((0, 0, 5), (0, 0, 0), (0, 1, 0), 90.0, 1.0, 0.0, 1.0)
    return sd


def instance_scene() -> SD:
    """Small scene mixing every hitable kind: BVH, list, flip, box,
    translate/rotate instances of a box and of a BVH, a medium, a moving
    sphere."""
    rng = np.random.Generator(np.random.PCG64(7))
    sd = SD()
    w = sd.lambertian(sd.const(0.7, 0.7, 0.7))
    r = sd.lambertian(sd.const(0.7, 0.1, 0.1))
    light = sd.diffuse_light(sd.const(4, 4, 4))
    items = [
        sd.rect("xz_rect", -10, 10, -10, 10, 0, w),
        sd.flip(sd.rect("xz_rect", -2, 2, -2, 2, 8, light)),
        sd.translate(sd.rotate_y(sd.box((0, 0, 0), (2, 3, 2), r), 30.0), (-4, 0, -1)),
        sd.moving_sphere((3, 1, 0), (3, 1.5, 0), 0.0, 1.0, 0.8, w),
    ]
    balls = [sd.sphere(tuple(rng.uniform(0, 2, 3)), 0.3, w) for _ in range(17)]
    items.append(sd.translate(sd.rotate_y(sd.bvh(balls, 0, 1), -40.0), (0, 1, 3)))
    bnd = sd.sphere((0, 2, -3), 1.5, sd.dielectric(1.5))
    items.append(bnd)
    items.append(sd.medium(bnd, 0.5, sd.const(0.9, 0.9, 0.9)))
    sd.world(sd.bvh(items[:5], 0, 1) if False else sd.hlist([sd.bvh(items[:5], 0, 1)] + items[5:]))
    sd.lights(sd.hlist([sd.rect("xz_rect", -2, 2, -2, 2, 8, w)]))
    sd.camera((0, 4, 14), (0, 1, 0), (0, 1, 0), 45.0, 1.0, 0.05, 14.0, 0.0, 1.0)
    sd.meta = dict(width=64, height=64, spp=16, max_depth=20, background=1, sky_scale=0.5)
    return sd


def _room(sd: SD, floor_mat: int | None = None) -> tuple[list[int], int]:
    """The Cornell room of cornell() without its box and sphere: five walls
    and the flipped light rect (emission 15).  Returns the items and the
    light list (the light rect alone)."""
    red = sd.lambertian(sd.const(0.65, 0.05, 0.05))
    white = sd.lambertian(sd.const(0.73, 0.73, 0.73))
    green = sd.lambertian(sd.const(0.12, 0.45, 0.15))
    lightm = sd.diffuse_light(sd.const(15, 15, 15))
    items = [
        sd.flip(sd.rect("yz_rect", 0, 555, 0, 555, 555, green)),
        sd.rect("yz_rect", 0, 555, 0, 555, 0, red),
        sd.flip(sd.rect("xz_rect", 213, 343, 227, 332, 554, lightm)),
        sd.flip(sd.rect("xz_rect", 0, 555, 0, 555, 555, white)),
        sd.rect("xz_rect", 0, 555, 0, 555, 0, white if floor_mat is None else floor_mat),
        sd.flip(sd.rect("xy_rect", 0, 555, 0, 555, 555, white)),
    ]
    dummy = sd.lambertian(sd.const(0, 0, 0))
    lights = sd.hlist([sd.rect("xz_rect", 213, 343, 227, 332, 554, dummy)])
    return items, lights


def _room_camera(sd: SD, t0=0.0, t1=0.0) -> None:
    sd.camera((278, 278, -800), (278, 278, 0), (0, 1, 0), 40.0, 1.0, 0.0, 10.0, t0, t1)
    sd.meta = dict(width=48, height=48, spp=64, max_depth=50, background=0, sky_scale=1.0)


def metals() -> SD:
    """Metal scatter (material.cc:88-98) in the Cornell room: mirror (fuzz
    0), fuzzy (0.35) and over-range fuzz 1.6, which the metal constructor
    clamps to 1 (material.h:41-46), on spheres, plus a fuzzy metal box."""
    sd = SD()
    items, lights = _room(sd)
    items.append(sd.sphere((130, 90, 170), 90, sd.metal(0.85, 0.85, 0.9, 0.0)))
    items.append(sd.sphere((300, 90, 360), 90, sd.metal(0.9, 0.6, 0.3, 0.35)))
    items.append(sd.sphere((440, 90, 170), 90, sd.metal(0.7, 0.8, 0.7, 1.6)))
    mbox = sd.box((0, 0, 0), (120, 200, 120), sd.metal(0.8, 0.8, 0.8, 0.2))
    items.append(sd.translate(sd.rotate_y(mbox, -25.0), (330, 0, 80)))
    sd.world(sd.bvh(items, 0.0, 0.0))
    sd.lights(lights)
    _room_camera(sd)
    return sd


def textures() -> SD:
    """Textures (texture.h:15-24, texture.cc:4-42) in the Cornell room: a
    checker floor and a checker sphere (the sign of sin(10x)sin(10y)sin(10z)),
    two perlin-turbulence spheres (seeded tables; scale 0.1 and 2), and a
    sphere with a procedural 64x32 RGB image texture (nearest texel)."""
    rng = np.random.Generator(np.random.PCG64(11))
    sd = SD()
    odd, even = sd.const(0.2, 0.3, 0.1), sd.const(0.9, 0.9, 0.9)
    floor = sd.lambertian(sd.checker(odd, even))
    items, lights = _room(sd, floor_mat=floor)
    items.append(sd.sphere((130, 90, 170), 90, sd.lambertian(sd.checker(sd.const(0.8, 0.1, 0.1), even))))
    sd.perlin_tables(rng)
    items.append(sd.sphere((300, 90, 360), 90, sd.lambertian(sd.perlin(0.1))))
    items.append(sd.sphere((440, 70, 170), 70, sd.lambertian(sd.perlin(2.0))))
    items.append(sd.sphere((250, 300, 250), 70, sd.lambertian(sd.image(64, 32, 4242))))
    sd.world(sd.bvh(items, 0.0, 0.0))
    sd.lights(lights)
    _room_camera(sd)
    return sd


def motion() -> SD:
    """Moving spheres (sphere.cc:45-85) under the reference's own BVH in the
    Cornell room: the camera's shutter is [0, 1] (camera.cc:26), the BVH
    boxes span the motion (bvh_node t0 = 0, t1 = 1), and one sphere's
    motion spans only [0.25, 0.75] of the shutter, so its centre is
    extrapolated outside that range as the reference does."""
    sd = SD()
    items, lights = _room(sd)
    w = sd.lambertian(sd.const(0.73, 0.73, 0.73))
    items.append(sd.moving_sphere((130, 90, 170), (130, 190, 170), 0.0, 1.0, 80, w))
    items.append(sd.moving_sphere((300, 90, 360), (420, 90, 360), 0.0, 1.0, 70, sd.metal(0.9, 0.8, 0.6, 0.1)))
    items.append(sd.moving_sphere((440, 120, 150), (440, 160, 120), 0.25, 0.75, 60,
                                  sd.lambertian(sd.const(0.2, 0.4, 0.8))))
    items.append(sd.sphere((200, 60, 100), 60, sd.dielectric(1.5)))
    sd.world(sd.bvh(items, 0.0, 1.0))
    sd.lights(lights)
    _room_camera(sd, 0.0, 1.0)
    return sd


def media() -> SD:
    """Constant-density media (hitable.cc:98-128) in the Cornell room: smoke
    in a rotated box (density 0.01, as in the reference's
    cornell_box_smoke) and a denser medium (0.05) inside a glass sphere, as
    the 'next week' scene nests them.  In reference semantics the isotropic
    phase function never scatters (material.h:74-80): media absorb."""
    sd = SD()
    items, lights = _room(sd)
    b = sd.translate(sd.rotate_y(sd.box((0, 0, 0), (165, 330, 165), sd.lambertian(sd.const(1, 1, 1))), 15.0),
                     (265, 0, 295))
    items.append(sd.medium(b, 0.01, sd.const(0.0, 0.0, 0.0)))
    glass = sd.sphere((150, 100, 150), 100, sd.dielectric(1.5))
    items.append(glass)
    items.append(sd.medium(glass, 0.05, sd.const(0.2, 0.4, 0.9)))
    sd.world(sd.hlist([sd.bvh(items[:6], 0.0, 0.0)] + items[6:]))
    sd.lights(lights)
    _room_camera(sd)
    return sd


PRESETS = {
    "one_weekend": one_weekend,
    "cornell": cornell,
    "cornell_guiding": cornell_guiding,
    "next_week": next_week,
    "ties": tie_scene,
    "instances": instance_scene,
    "metals": metals,
    "textures": textures,
    "motion": motion,
    "media": media,
}
