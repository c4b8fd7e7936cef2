"""Seeded synthetic piecewise-planar scenes in the reference's file layout.

There is no public dataset for this path; these scenes stand in for it:

* ``small_scene`` — 3 planes (back wall, floor, a tilted slab) with
  procedural value-noise texture, 1 reference + 4 source pinhole views at
  320x256 on an 8-degree arc, fx = fy = 0.8 W, depth range [0.5, 5];
* ``room_scene`` — 6 walls of a room plus 12 randomly oriented textured
  slabs (per-plane noise octaves 1-4), views on a 360-degree ring looking
  inwards, source views chosen by triangulation angle (peak 5-15 degrees).

Images are rendered by ray casting, rounded to 8-bit gray after adding
Gaussian noise (sigma = 2 DN).  Superpixels are the true plane id
intersected with a 16x16 grid, labelled into 1..255.  All draws come from
``numpy.random.default_rng(seed)``; rendering runs in torch on any device.

``write_scene`` writes ``images/{id:04}.jpg`` (PNG content, which
cv2.imread also reads), ``cams/{id:04}_cam.txt`` (colmap2mvs.py:531-549),
``pair.txt`` (colmap2mvs.py:551-557) and ``superpixels/{id:04}.npy``.
"""

from __future__ import annotations

import math
import os
from dataclasses import dataclass, field
from typing import List, Optional, Tuple

import numpy as np
import torch

from .imageio import write_png


@dataclass
class Plane:
    center: np.ndarray       # world point on the plane
    normal: np.ndarray       # unit normal
    u: np.ndarray            # in-plane axes (texture coordinates)
    v: np.ndarray
    half: Tuple[float, float]  # half extents along u, v (inf = unbounded)
    tex_seed: int
    octaves: int
    freq: float              # lattice cells per metre of the first octave
    lo: float = 30.0
    hi: float = 225.0


@dataclass
class Scene:
    images: np.ndarray            # uint8 [V, H, W]
    K: List[np.ndarray]           # 3x3
    R: List[np.ndarray]           # 3x3 world -> camera
    t: List[np.ndarray]           # 3
    depth_range: Tuple[float, float]
    depths: np.ndarray            # float32 [V, H, W] ground truth
    normals: np.ndarray           # float32 [V, H, W, 3] world frame, facing the camera
    plane_ids: np.ndarray         # int32 [V, H, W] (-1 = no surface)
    superpixels: np.ndarray       # uint8 [V, H, W]
    problems: List[Tuple[int, List[int]]] = field(default_factory=list)
    planes: List[Plane] = field(default_factory=list)

    @property
    def num_views(self) -> int:
        return int(self.images.shape[0])

    @property
    def hw(self) -> Tuple[int, int]:
        return int(self.images.shape[1]), int(self.images.shape[2])


def _unit(v) -> np.ndarray:
    v = np.asarray(v, np.float64)
    return v / np.linalg.norm(v)


def _plane(center, normal, half, rng, octaves, freq) -> Plane:
    n = _unit(normal)
    a = np.array([0.0, 1.0, 0.0]) if abs(n[1]) < 0.9 else np.array([1.0, 0.0, 0.0])
    u = _unit(np.cross(n, a))
    v = np.cross(n, u)
    return Plane(np.asarray(center, np.float64), n, u, v, half, int(rng.integers(1, 2**31 - 1)), octaves, freq)


def look_at(C, target, down_hint=(0.0, 1.0, 0.0)) -> Tuple[np.ndarray, np.ndarray]:
    """World->camera R, t for a camera at C looking at target (y down)."""
    C = np.asarray(C, np.float64)
    f = _unit(np.asarray(target, np.float64) - C)
    r = _unit(np.cross(np.asarray(down_hint, np.float64), f))
    d = np.cross(f, r)
    R = np.stack([r, d, f])
    return R, -R @ C


def _hash2(ix: torch.Tensor, iy: torch.Tensor, seed: int) -> torch.Tensor:
    """Integer lattice hash -> uniform [0, 1) (xorshift-multiply mixing)."""
    m = (1 << 32) - 1
    h = (ix * 0x27D4EB2F + iy * 0x165667B1 + seed * 0x61C88647) & m
    h = h ^ (h >> 15)
    h = (h * 0x2C1B3C6D) & m
    h = h ^ (h >> 12)
    h = (h * 0x297A2D39) & m
    h = h ^ (h >> 15)
    return h.to(torch.float64) / float(1 << 32)


def value_noise(s: torch.Tensor, t: torch.Tensor, seed: int, octaves: int, freq: float) -> torch.Tensor:
    """Sum of `octaves` smooth value-noise octaves in [0, 1]."""
    acc = torch.zeros_like(s)
    amp, norm, f = 1.0, 0.0, freq
    for o in range(octaves):
        x, y = s * f, t * f
        x0, y0 = torch.floor(x), torch.floor(y)
        fx, fy = x - x0, y - y0
        fx = fx * fx * (3 - 2 * fx)
        fy = fy * fy * (3 - 2 * fy)
        ix, iy = x0.to(torch.int64), y0.to(torch.int64)
        so = seed + 7919 * o
        v00, v10 = _hash2(ix, iy, so), _hash2(ix + 1, iy, so)
        v01, v11 = _hash2(ix, iy + 1, so), _hash2(ix + 1, iy + 1, so)
        top = v00 + (v10 - v00) * fx
        bot = v01 + (v11 - v01) * fx
        acc = acc + amp * (top + (bot - top) * fy)
        norm += amp
        amp *= 0.55
        f *= 2.0
    return acc / norm


def render(planes: List[Plane], K, R, t, H: int, W: int, rng: np.random.Generator, noise_sigma: float = 2.0,
           device: Optional[torch.device] = None):
    """Ray-cast one view: (uint8 image, depth, world normal, plane id)."""
    dev = device or torch.device("cpu")
    dt = torch.float64
    Rt = torch.tensor(R, dtype=dt, device=dev)
    tt = torch.tensor(t, dtype=dt, device=dev)
    C = -(Rt.T @ tt)
    ys, xs = torch.meshgrid(torch.arange(H, dtype=dt, device=dev), torch.arange(W, dtype=dt, device=dev),
                            indexing="ij")
    Kinv = torch.tensor(np.linalg.inv(np.asarray(K, np.float64)), dtype=dt, device=dev)
    pc = torch.stack([xs, ys, torch.ones_like(xs)], -1) @ Kinv.T  # camera rays, z = 1
    dw = pc @ Rt                                                                  # world directions
    best = torch.full((H, W), float("inf"), dtype=dt, device=dev)
    pid = torch.full((H, W), -1, dtype=torch.int64, device=dev)
    for k, pl in enumerate(planes):
        n = torch.tensor(pl.normal, dtype=dt, device=dev)
        c = torch.tensor(pl.center, dtype=dt, device=dev)
        den = dw @ n
        tk = ((c - C) @ n) / den
        ok = (den.abs() > 1e-9) & (tk > 1e-6)
        if math.isfinite(pl.half[0]) or math.isfinite(pl.half[1]):
            X = C + tk[..., None] * dw
            du = (X - c) @ torch.tensor(pl.u, dtype=dt, device=dev)
            dv = (X - c) @ torch.tensor(pl.v, dtype=dt, device=dev)
            ok = ok & (du.abs() <= pl.half[0]) & (dv.abs() <= pl.half[1])
        upd = ok & (tk < best)
        best = torch.where(upd, tk, best)
        pid = torch.where(upd, torch.full_like(pid, k), pid)
    depth = torch.where(pid >= 0, best, torch.zeros_like(best))  # camera z (rays have z = 1)
    img = torch.zeros((H, W), dtype=dt, device=dev)
    nrm = torch.zeros((H, W, 3), dtype=dt, device=dev)
    X = C + depth[..., None] * dw
    for k, pl in enumerate(planes):
        m = pid == k
        if not bool(m.any()):
            continue
        c = torch.tensor(pl.center, dtype=dt, device=dev)
        s = (X[m] - c) @ torch.tensor(pl.u, dtype=dt, device=dev)
        q = (X[m] - c) @ torch.tensor(pl.v, dtype=dt, device=dev)
        img[m] = pl.lo + (pl.hi - pl.lo) * value_noise(s, q, pl.tex_seed, pl.octaves, pl.freq)
        n = torch.tensor(pl.normal, dtype=dt, device=dev)
        flip = (dw[m] @ n) > 0
        nk = n.expand(int(m.sum()), 3).clone()
        nk[flip] = -nk[flip]
        nrm[m] = nk
    noise = torch.from_numpy(rng.normal(0.0, noise_sigma, size=(H, W))).to(dev)
    img8 = torch.clamp(torch.round(img + noise), 0, 255).to(torch.uint8)
    return (img8.cpu().numpy(), depth.to(torch.float32).cpu().numpy(), nrm.to(torch.float32).cpu().numpy(),
            pid.to(torch.int32).cpu().numpy())


def superpixels_of(plane_ids: np.ndarray, cell: int = 16) -> np.ndarray:
    """True plane id intersected with a cell x cell grid, labels in 1..255."""
    H, W = plane_ids.shape
    ys, xs = np.mgrid[0:H, 0:W]
    ncx = (W + cell - 1) // cell
    cell_id = (ys // cell) * ncx + (xs // cell)
    lab = ((plane_ids.astype(np.int64) + 1) * 7919 + cell_id) % 255 + 1
    return lab.astype(np.uint8)


def _intrinsics(H: int, W: int) -> np.ndarray:
    f = 0.8 * W
    return np.array([[f, 0.0, W / 2.0], [0.0, f, H / 2.0], [0.0, 0.0, 1.0]])


def small_scene(seed: int = 0, H: int = 256, W: int = 320, device=None) -> Scene:
    """3 planes, 1 reference + 4 sources on an 8-degree arc, depth [0.5, 5]."""
    rng = np.random.default_rng(seed)
    planes = [
        _plane((0.0, 0.0, 4.0), (0.0, 0.0, -1.0), (math.inf, math.inf), rng, 3, 14.0),   # back wall
        _plane((0.0, 0.8, 2.0), (0.0, -1.0, 0.0), (math.inf, math.inf), rng, 2, 12.0),   # floor
        _plane((-0.35, -0.05, 2.3), (math.sin(math.radians(35)), 0.15, -math.cos(math.radians(35))),
               (0.75, 0.55), rng, 4, 16.0),                                             # tilted slab
    ]
    K = _intrinsics(H, W)
    target = np.array([0.0, 0.0, 2.6])
    Ks, Rs, ts, ims, ds, ns, ps = [], [], [], [], [], [], []
    for k in (0, -1, 1, -2, 2):
        th = math.radians(8.0 * k)
        C = target + 2.6 * np.array([math.sin(th), 0.0, -math.cos(th)])
        R, t = look_at(C, target)
        im, d, n, p = render(planes, K, R, t, H, W, rng, device=device)
        Ks.append(K.copy()), Rs.append(R), ts.append(t), ims.append(im), ds.append(d), ns.append(n), ps.append(p)
    pid = np.stack(ps)
    sc = Scene(np.stack(ims), Ks, Rs, ts, (0.5, 5.0), np.stack(ds), np.stack(ns), pid,
               np.stack([superpixels_of(p) for p in pid]), planes=planes)
    sc.problems = [(i, [j for j in range(5) if j != i]) for i in range(5)]
    return sc


def select_sources(sc: Scene, num_src: int, rng: np.random.Generator, lo_deg: float = 5.0,
                   hi_deg: float = 15.0, samples: int = 1500) -> List[Tuple[int, List[int]]]:
    """Per reference view, the num_src sources whose triangulation angle on
    shared ground-truth points is best centred in [lo_deg, hi_deg]."""
    V = sc.num_views
    H, W = sc.hw
    Cs = [-(R.T @ t) for R, t in zip(sc.R, sc.t)]
    mid, sig = 0.5 * (lo_deg + hi_deg), 0.5 * (hi_deg - lo_deg)
    problems = []
    for i in range(V):
        ys = rng.integers(0, H, samples)
        xs = rng.integers(0, W, samples)
        d = sc.depths[i, ys, xs].astype(np.float64)
        ok = d > 0
        ys, xs, d = ys[ok], xs[ok], d[ok]
        pc = np.stack([(xs - sc.K[i][0, 2]) / sc.K[i][0, 0] * d, (ys - sc.K[i][1, 2]) / sc.K[i][1, 1] * d, d], 1)
        Xw = (pc - sc.t[i]) @ sc.R[i]
        scores = []
        for j in range(V):
            if j == i:
                continue
            q = Xw @ sc.R[j].T + sc.t[j]
            z = q[:, 2]
            u = sc.K[j][0, 0] * q[:, 0] / np.maximum(z, 1e-9) + sc.K[j][0, 2]
            v = sc.K[j][1, 1] * q[:, 1] / np.maximum(z, 1e-9) + sc.K[j][1, 2]
            inside = (z > 1e-6) & (u >= 0) & (u < W - 1) & (v >= 0) & (v < H - 1)
            vis = np.zeros_like(inside)
            if inside.any():
                zj = sc.depths[j, v[inside].astype(int), u[inside].astype(int)]
                vis[inside] = np.abs(zj - z[inside]) < 0.02 * z[inside]
            if not vis.any():
                scores.append((0.0, j))
                continue
            a = Xw[vis] - Cs[i]
            b = Xw[vis] - Cs[j]
            cosang = np.sum(a * b, 1) / np.linalg.norm(a, axis=1) / np.linalg.norm(b, axis=1)
            ang = np.degrees(np.arccos(np.clip(cosang, -1, 1)))
            scores.append((float(np.sum(np.exp(-0.5 * ((ang - mid) / sig) ** 2))), j))
        scores.sort(key=lambda s: (-s[0], s[1]))
        problems.append((i, [j for s, j in scores[:num_src] if s > 0]))
    return problems


def room_scene(seed: int = 0, H: int = 1200, W: int = 1600, num_views: int = 20, num_src: int = 10,
               num_slabs: int = 12, device=None) -> Scene:
    """A room of 6 textured walls plus `num_slabs` randomly oriented textured
    slabs, viewed from a 360-degree ring of cameras looking inwards."""
    rng = np.random.default_rng(seed)
    walls = [
        ((0.0, 0.0, 6.0), (0.0, 0.0, -1.0)), ((0.0, 0.0, -6.0), (0.0, 0.0, 1.0)),
        ((6.0, 0.0, 0.0), (-1.0, 0.0, 0.0)), ((-6.0, 0.0, 0.0), (1.0, 0.0, 0.0)),
        ((0.0, 1.5, 0.0), (0.0, -1.0, 0.0)), ((0.0, -2.5, 0.0), (0.0, 1.0, 0.0)),
    ]
    planes = [_plane(c, n, (math.inf, math.inf), rng, int(rng.integers(1, 5)), float(rng.uniform(6.0, 12.0)))
              for c, n in walls]
    for _ in range(num_slabs):
        r = rng.uniform(0.0, 2.2)
        a = rng.uniform(0, 2 * math.pi)
        c = (r * math.cos(a), rng.uniform(-1.2, 0.8), r * math.sin(a))
        n = rng.normal(size=3)
        planes.append(_plane(c, n, (rng.uniform(0.3, 0.9), rng.uniform(0.3, 0.9)), rng, int(rng.integers(1, 5)),
                             float(rng.uniform(10.0, 20.0))))
    K = _intrinsics(H, W)
    Ks, Rs, ts, ims, ds, ns, ps = [], [], [], [], [], [], []
    for k in range(num_views):
        th = 2 * math.pi * k / num_views
        C = np.array([4.2 * math.cos(th), -0.3 + 0.1 * math.sin(3 * th), 4.2 * math.sin(th)])
        target = np.array([0.3 * math.cos(th + 1.0), 0.0, 0.3 * math.sin(th + 1.0)])
        R, t = look_at(C, target)
        im, d, n, p = render(planes, K, R, t, H, W, rng, device=device)
        Ks.append(K.copy()), Rs.append(R), ts.append(t), ims.append(im), ds.append(d), ns.append(n), ps.append(p)
    pid = np.stack(ps)
    sc = Scene(np.stack(ims), Ks, Rs, ts, (0.5, 12.0), np.stack(ds), np.stack(ns), pid,
               np.stack([superpixels_of(p) for p in pid]), planes=planes)
    sc.problems = select_sources(sc, num_src, rng)
    return sc


def camera_args(sc: Scene, i: int):
    """(K, R, t, h, w, dmin, dmax) as the reference's read_camera + load_camera."""
    H, W = sc.hw
    return (sc.K[i].reshape(9).tolist(), sc.R[i].reshape(9).tolist(), np.asarray(sc.t[i]).tolist(), H, W,
            float(sc.depth_range[0]), float(sc.depth_range[1]))


def write_scene(sc: Scene, root: str) -> None:
    """Write the reference's input layout under `root`."""
    for sub in ("images", "cams", "superpixels"):
        os.makedirs(os.path.join(root, sub), exist_ok=True)
    dmin, dmax = sc.depth_range
    for i in range(sc.num_views):
        write_png(os.path.join(root, "images", f"{i:04}.jpg"), sc.images[i])
        E = np.eye(4)
        E[:3, :3] = sc.R[i]
        E[:3, 3] = sc.t[i]
        with open(os.path.join(root, "cams", f"{i:04}_cam.txt"), "w") as f:
            f.write("extrinsic\n")
            for r in range(4):
                f.write(" ".join(repr(float(E[r, c])) for c in range(4)) + " \n")
            f.write("\nintrinsic\n")
            for r in range(3):
                f.write(" ".join(repr(float(sc.K[i][r, c])) for c in range(3)) + " \n")
            f.write("\n%f %f %f %f\n" % (dmin, (dmax - dmin) / 192.0, 192.0, dmax))
        np.save(os.path.join(root, "superpixels", f"{i:04d}.npy"), sc.superpixels[i])
    with open(os.path.join(root, "pair.txt"), "w") as f:
        f.write("%d\n" % sc.num_views)
        for ref, src in sc.problems:
            f.write("%d\n%d " % (ref, len(src)))
            for j in src:
                f.write("%d %d " % (j, 100))
            f.write("\n")


def superpixel_case(rows: int, cols: int, seed: int, cell=(24, 20)):
    """Inputs of the fusion scripts' superpixel statistics: blocky superpixel
    ids 1..K (1 % id-0 holes, gaps in the id range), a planar mask, unit
    normals and a variance map.  Segments are drawn as textureless (10 %
    non-planar pixels), objects (90 %, scattered normals), consistent
    surfaces (90 %, one normal) or mixed (50 %), so every branch of
    fusion_planar_mask is reached.  Returns (seg int32, planar int32,
    normals float32 [rows, cols, 3], var float32)."""
    rng = np.random.default_rng(seed)
    ys, xs = np.mgrid[0:rows, 0:cols]
    jy = rng.integers(0, cell[0], size=(rows // cell[0] + 2,))
    gy = (ys + jy[np.minimum(xs // cell[1], len(jy) - 1)]) // cell[0]
    gx = xs // cell[1]
    seg = (gy * (cols // cell[1] + 2) + gx + 1).astype(np.int32)
    seg[rng.random((rows, cols)) < 0.01] = 0
    seg[seg % 17 == 0] = 0
    ns = int(seg.max()) + 1
    kind = rng.integers(0, 4, ns)
    frac = np.array([0.1, 0.9, 0.9, 0.5])[kind]
    planar = (rng.random((rows, cols)) >= frac[seg]).astype(np.int32)
    base = rng.normal(size=(ns, 3))
    base /= np.linalg.norm(base, axis=1, keepdims=True)
    spread = np.where(kind == 1, 1.5, 0.05)[seg][..., None]
    n = base[seg] + spread * rng.normal(size=(rows, cols, 3))
    n = (n / np.linalg.norm(n, axis=-1, keepdims=True)).astype(np.float32)
    var = rng.random((rows, cols)).astype(np.float32) * np.where(kind % 2 == 0, 0.4, 1.0)[seg].astype(np.float32)
    return seg, planar, n, var


def indoor_image(rows: int, cols: int, seed: int = 0, textured: int = 3):
    """A BGR uint8 [rows, cols, 3] picture of flat-coloured walls and boxes
    with mild shading and sensor noise plus `textured` patches of strong
    texture, and its gray uint8 image: segments with low and with high local
    variance for the superpixel extraction.  Returns (bgr, gray)."""
    rng = np.random.default_rng(seed)
    ys, xs = np.mgrid[0:rows, 0:cols].astype(np.float64)
    img = np.empty((rows, cols, 3))
    base = rng.uniform(60, 200, 3)
    img[:] = base + 20.0 * (ys / rows)[..., None]
    horizon = int(rows * rng.uniform(0.55, 0.75))
    img[horizon:] = rng.uniform(40, 160, 3) + 15.0 * (xs[horizon:] / cols)[..., None]
    for _ in range(int(rng.integers(6, 12))):
        h, w = int(rng.integers(rows // 10, rows // 3)), int(rng.integers(cols // 10, cols // 3))
        y0, x0 = int(rng.integers(0, rows - h)), int(rng.integers(0, cols - w))
        img[y0:y0 + h, x0:x0 + w] = rng.uniform(20, 235, 3)
    for _ in range(textured):
        h, w = int(rng.integers(rows // 12, rows // 5)), int(rng.integers(cols // 12, cols // 5))
        y0, x0 = int(rng.integers(0, rows - h)), int(rng.integers(0, cols - w))
        img[y0:y0 + h, x0:x0 + w] += rng.normal(0, 45, (h, w, 3))
    img += rng.normal(0, 1.5, img.shape)
    bgr = np.clip(np.rint(img), 0, 255).astype(np.uint8)
    x = bgr.astype(np.float64)
    gray = np.clip(np.rint(0.114 * x[..., 0] + 0.587 * x[..., 1] + 0.299 * x[..., 2]), 0, 255).astype(np.uint8)
    return bgr, gray
