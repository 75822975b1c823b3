"""Named CT workloads and seeded synthetic phantoms.

The five workloads below are the ones the package is benchmarked and tested on.
No public data set is used: every slice is a sum of random ellipses
(``ellipse_phantom``), generated on the host with ``numpy.random.default_rng``.

Options vectors use the reference's index semantics (src/ctlib.cpp:18,
src/fan_ed_kernel.cu:1165-1175, src/para_kernel.cu:687-695):
fan   ``[views, dets, width, height, dImg, dDet, Ang0, dAng, s2r, d2r, binshift, scan_type]``
para  ``[views, dets, width, height, dImg, dDet, Ang0, dAng, binshift, scan_type]``
(the parallel vector carries binshift at index 8 and scan_type last, so it has
10 entries whenever binshift is not 2.0).
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

FAN_ED, FAN_EA, PARA = 0, 1, 2


def fan_options(views, dets, width, height, dImg, dDet, Ang0, dAng, s2r, d2r, binshift=0.0,
                scan_type=FAN_ED):
    return [float(views), float(dets), float(width), float(height), float(dImg), float(dDet),
            float(Ang0), float(dAng), float(s2r), float(d2r), float(binshift), float(scan_type)]


def para_options(views, dets, width, height, dImg, dDet, Ang0, dAng, binshift=0.0):
    return [float(views), float(dets), float(width), float(height), float(dImg), float(dDet),
            float(Ang0), float(dAng), float(binshift), float(PARA)]


@dataclass
class Slice:
    """One image slice of a workload with its own geometry."""
    options: list
    seed: int
    noise: float = 0.0

    @property
    def scan_type(self) -> int:
        return int(self.options[-1])

    @property
    def shape_image(self):
        return (int(self.options[3]), int(self.options[2]))

    @property
    def shape_sino(self):
        return (int(self.options[0]), int(self.options[1]))


@dataclass
class Workload:
    name: str
    slices: list = field(default_factory=list)

    @property
    def uniform(self) -> bool:
        return all(s.options == self.slices[0].options for s in self.slices)

    def ray_updates(self) -> int:
        """One ray-update = one (slice, view, detector bin, image line); lines are
        rows or columns by view branch, both H or W long for square images."""
        n = 0
        for s in self.slices:
            V, D, W, H = (int(s.options[i]) for i in range(4))
            n += V * D * max(W, H)
        return n


def ellipse_phantom(height: int, width: int, dImg: float, seed: int, noise: float = 0.0,
                    n_ellipses: int = 10) -> np.ndarray:
    """Sum of ``n_ellipses`` random ellipses on the pixel-centre grid (fp32, 1/mm).

    Centres uniform in the disc of radius 0.45*W*dImg, semi-axes uniform in
    [0.05, 0.35]*W*dImg, orientation uniform in [0, pi), attenuation uniform in
    [0, 0.04]. Optional N(0, noise) texture from ``seed + 1``.
    """
    rng = np.random.default_rng(seed)
    fov = width * dImg
    x = (np.arange(width) - width / 2 + 0.5) * dImg
    y = (height / 2 - np.arange(height) - 0.5) * dImg
    X, Y = np.meshgrid(x, y)
    img = np.zeros((height, width), np.float64)
    for _ in range(n_ellipses):
        r = 0.45 * fov * math.sqrt(rng.uniform())
        t = rng.uniform(0, 2 * math.pi)
        cx, cy = r * math.cos(t), r * math.sin(t)
        a, b = rng.uniform(0.05, 0.35, size=2) * fov
        phi = rng.uniform(0, math.pi)
        mu = rng.uniform(0, 0.04)
        c, s = math.cos(phi), math.sin(phi)
        u = ((X - cx) * c + (Y - cy) * s) / a
        v = (-(X - cx) * s + (Y - cy) * c) / b
        img[u * u + v * v <= 1.0] += mu
    if noise > 0:
        img += np.random.default_rng(seed + 1).normal(0.0, noise, size=img.shape)
    return img.astype(np.float32)


def gaussian(shape, seed: int) -> np.ndarray:
    return np.random.default_rng(seed).standard_normal(shape).astype(np.float32)


# --------------------------------------------------------------------------- #
# the five workloads
# --------------------------------------------------------------------------- #

def parallel_256() -> Workload:
    """Parallel beam, 1 x 256^2, 360 views over 180 deg, 367 bins."""
    o = para_options(360, 367, 256, 256, 1.0, 1.0, 0.0, math.pi / 360, 0.0)
    return Workload("parallel_256_v360_d367", [Slice(o, 1000 * 1 + 0)])


def fan_ed_512(batch: int = 16) -> Workload:
    """Fan equal-distance, B x 512^2, 1152 views, 736 bins (the headline workload)."""
    o = fan_options(1152, 736, 512, 512, 0.6641, 1.2858, 0.0, 2 * math.pi / 1152, 595.0, 490.6, 0.0,
                    FAN_ED)
    return Workload(f"fan_ed_512_b{batch}_v1152_d736", [Slice(o, 1000 * 2 + i) for i in range(batch)])


def fan_ea_512(batch: int = 8) -> Workload:
    """Fan equal-angle, B x 512^2, 984 views over 360 deg, 888 bins of 0.0011 rad."""
    o = fan_options(984, 888, 512, 512, 0.7, 0.0011, 0.0, 2 * math.pi / 984, 541.0, 408.0, 0.0, FAN_EA)
    return Workload(f"fan_ea_512_b{batch}_v984_d888", [Slice(o, 1000 * 3 + i) for i in range(batch)])


def ragged_96(n: int = 96, seed: int = 4000) -> Workload:
    """Mixed geometries: sizes 256..768 (step 128), views from
    {64,128,360,720,1152,2304}, 368..1024 bins, scan types 0/1/2."""
    rng = np.random.default_rng(seed)
    sizes = [256, 384, 512, 640, 768]
    view_set = [64, 128, 360, 720, 1152, 2304]
    out = []
    for i in range(n):
        size = int(rng.choice(sizes))
        V = int(rng.choice(view_set))
        D = int(rng.integers(368, 1025))
        st = int(rng.integers(0, 3))
        fov = 340.0
        dImg = fov / size
        if st == PARA:
            dDet = fov * 1.45 / D
            o = para_options(V, D, size, size, dImg, dDet, 0.0, math.pi / V, 0.0)
        elif st == FAN_ED:
            s2r, d2r = 595.0, 490.6
            half = math.asin(0.5 * fov * 1.42 / s2r)  # fan covering the image diagonal
            virt = 2 * s2r * math.tan(half) / D
            dDet = virt * (s2r + d2r) / s2r
            o = fan_options(V, D, size, size, dImg, dDet, 0.0, 2 * math.pi / V, s2r, d2r, 0.0, FAN_ED)
        else:
            s2r, d2r = 541.0, 408.0
            half = math.asin(0.5 * fov * 1.42 / s2r)
            dDet = 2 * half / D
            o = fan_options(V, D, size, size, dImg, dDet, 0.0, 2 * math.pi / V, s2r, d2r, 0.0, FAN_EA)
        out.append(Slice(o, 4000 + i))
    return Workload(f"ragged_{n}", out)


def fan_ed_1024(batch: int = 8) -> Workload:
    """Fan equal-distance stress case, B x 1024^2 with noise texture, 2304 views, 1472 bins."""
    o = fan_options(2304, 1472, 1024, 1024, 0.33, 0.6429, 0.0, 2 * math.pi / 2304, 595.0, 490.6, 0.0,
                    FAN_ED)
    return Workload(f"fan_ed_1024_b{batch}_v2304_d1472",
                    [Slice(o, 1000 * 5 + i, noise=1e-3) for i in range(batch)])


WORKLOADS = {
    "parallel_256": parallel_256,
    "fan_ed_512": fan_ed_512,
    "fan_ea_512": fan_ea_512,
    "ragged_96": ragged_96,
    "fan_ed_1024": fan_ed_1024,
}


def phantoms(w: Workload) -> list:
    """One fp32 phantom per slice of ``w``."""
    return [ellipse_phantom(s.shape_image[0], s.shape_image[1], s.options[4], s.seed, s.noise)
            for s in w.slices]
