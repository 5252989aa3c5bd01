"""Seeded synthetic scenes with the shapes and value distributions of the benchmark configurations.

No public dataset is involved: every input (level set, velocity, applied field) is generated from a seed.
Collider fractions come from the library's host-side Collider (sf_collider_box_fractions), i.e. the
reference's box-wall construction (core/Collider.cpp:8-73) with boundary width 0 (walls on the grid faces).

Scenes:
* ``pool``        -- phi = y - depth + 0.01 n(x, z), n seeded uniform[-1, 1] on an 8x8 lattice, bilinear;
                    uniform applied field H0 = (0, 1, 0); velocity uniform[-1, 1].
* ``pool_sphere`` -- pool of depth 0.2 united (min) with a sphere of radius 0.15 at (0.5, 0.55, 0.5); dipole
                    applied field of moment (0, 1, 0) at (0.5, -0.3, 0.5) with the reference's dipole formula
                    (demo/SimBuilder.cpp:80-98) without its time ramp; velocity N(0, 0.5^2).
* ``random_scene`` -- the learned form's distribution: pool of random depth with 1-8 random spheres.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import StaggeredGrid, _abi


@dataclass
class Scene:
    name: str
    grid: StaggeredGrid
    phi: np.ndarray
    vel: list
    frac: list
    hext: list
    chi: float
    band_width: float
    meta: dict = field(default_factory=dict)


def unit_grid(n) -> StaggeredGrid:
    """Cell-centred n^3 grid on [0, 1]^3 (dx = 1/n), boundary width 0."""
    if isinstance(n, int):
        n = (n, n, n)
    h = 1.0 / n[0]
    return StaggeredGrid.from_origin(h, tuple(n), (0.0, 0.0, 0.0), 0)


def cell_centres(g: StaggeredGrid, axis: int):
    o = g.origin[axis]
    return o + (np.arange(g.shape[axis]) + 0.5) * g.spacing


def face_positions(g: StaggeredGrid, face_axis: int):
    """Per-axis coordinates of the faces of face grid `face_axis` (core/StaggeredGrid.h:16-20)."""
    out = []
    for b in range(3):
        n = g.shape[b] + (1 if b == face_axis else 0)
        off = 0.0 if b == face_axis else 0.5
        out.append(g.origin[b] + (np.arange(n) + off) * g.spacing)
    return out


def box_fractions(g: StaggeredGrid, boundary_width: int = 0):
    """Collider fractions of the domain-box walls (sf_collider_box_fractions, host code)."""
    lib = _abi.load()
    frac = [np.empty(g.face_shape(a)) for a in range(3)]
    s = lib.sf_collider_box_fractions(C.byref(g.c_grid()), int(boundary_width), _abi.p3([f.ctypes.data for f in frac]),
                                      None)
    if s != 0:
        raise RuntimeError(f"sf_collider_box_fractions failed with status {s}")
    return frac


def lattice_noise(xs, zs, rng, lattice: int = 8):
    """Bilinear interpolation of seeded uniform[-1, 1] values on a lattice x lattice grid over [0, 1]^2."""
    lat = rng.uniform(-1.0, 1.0, (lattice, lattice))
    m = lattice - 1

    def split(t):
        t = np.clip(t, 0.0, 1.0) * m
        i0 = np.minimum(np.floor(t).astype(np.int64), m - 1)
        return i0, t - i0

    ix, fx = split(xs)
    iz, fz = split(zs)
    return ((1 - fx)[:, None] * (1 - fz)[None, :] * lat[ix][:, iz] + fx[:, None] * (1 - fz)[None, :] * lat[ix + 1][:, iz]
            + (1 - fx)[:, None] * fz[None, :] * lat[ix][:, iz + 1] + fx[:, None] * fz[None, :] * lat[ix + 1][:, iz + 1])


def uniform_field(g: StaggeredGrid, h0=(0.0, 1.0, 0.0)):
    return [np.full(g.face_shape(a), float(h0[a])) for a in range(3)]


def dipole_field(g: StaggeredGrid, pos=(0.5, -0.3, 0.5), orient=(0.0, 1.0, 0.0), factor=1.0):
    """Applied field of a point dipole on every face, demo/SimBuilder.cpp:87-97 without the time ramp."""
    m = np.asarray(orient, dtype=np.float64)
    m = m / np.linalg.norm(m)
    out = []
    for a in range(3):
        X, Y, Z = np.meshgrid(*face_positions(g, a), indexing="ij")
        r = np.stack([X - pos[0], Y - pos[1], Z - pos[2]], axis=-1)
        rn = np.linalg.norm(r, axis=-1)
        ru = r / rn[..., None]
        cos_t = (r @ m) / rn
        r3 = rn * rn * rn
        hr = factor * ru * (2 * cos_t / r3)[..., None]
        sin_t = np.sqrt(np.maximum(1 - cos_t * cos_t, 0.0))
        tu = (ru @ m)[..., None] * ru - m
        ht = factor * tu * (sin_t / r3)[..., None]
        h = np.where((1 - cos_t)[..., None] < 1e-6, hr, hr + ht)
        out.append(np.ascontiguousarray(h[..., a]))
    return out


def pool(n, seed: int = 0, chi: float = 1.0, depth: float = 0.25, noise: float = 0.01, with_fractions=True) -> Scene:
    g = unit_grid(n)
    rng = np.random.default_rng(seed)
    xs, ys, zs = (cell_centres(g, a) for a in range(3))
    nz = lattice_noise(xs, zs, rng)
    phi = ys[None, :, None] - depth + noise * nz[:, None, :]
    phi = np.ascontiguousarray(np.broadcast_to(phi, g.shape))
    vel = [rng.uniform(-1.0, 1.0, g.face_shape(a)) for a in range(3)]
    frac = box_fractions(g, 0) if with_fractions else None
    return Scene("pool", g, phi, vel, frac, uniform_field(g), chi, 2 * g.spacing,
                 dict(seed=seed, depth=depth, noise=noise))


def pool_sphere(n, seed: int = 0, chi: float = 2.0, depth: float = 0.2, centre=(0.5, 0.55, 0.5), radius=0.15,
                dipole_pos=(0.5, -0.3, 0.5), dipole_orient=(0.0, 1.0, 0.0), with_fractions=True) -> Scene:
    g = unit_grid(n)
    rng = np.random.default_rng(seed)
    xs, ys, zs = (cell_centres(g, a) for a in range(3))
    X, Y, Z = np.meshgrid(xs, ys, zs, indexing="ij")
    phi = np.minimum(Y - depth, np.sqrt((X - centre[0]) ** 2 + (Y - centre[1]) ** 2 + (Z - centre[2]) ** 2) - radius)
    phi = np.ascontiguousarray(phi)
    vel = [rng.normal(0.0, 0.5, g.face_shape(a)) for a in range(3)]
    frac = box_fractions(g, 0) if with_fractions else None
    return Scene("pool_sphere", g, phi, vel, frac, dipole_field(g, dipole_pos, dipole_orient), chi, 2 * g.spacing,
                 dict(seed=seed, depth=depth, centre=centre, radius=radius))


def random_scene(n, seed: int = 0, with_fractions=True) -> Scene:
    """The learned form's scene distribution: a pool of depth U[0.1, 0.3] united with 1-8 spheres of radius
    U[0.05, 0.25] at uniform centres, chi U[0.5, 3], a uniform applied field of random direction and magnitude
    U[0.5, 2], velocity N(0, 0.5^2), walls on the grid faces."""
    g = unit_grid(n)
    rng = np.random.default_rng(seed)
    xs, ys, zs = (cell_centres(g, a) for a in range(3))
    X, Y, Z = np.meshgrid(xs, ys, zs, indexing="ij")
    phi = Y - rng.uniform(0.1, 0.3)
    for _ in range(int(rng.integers(1, 9))):
        cx, cy, cz = rng.uniform(0, 1, 3)
        r = rng.uniform(0.05, 0.25)
        phi = np.minimum(phi, np.sqrt((X - cx) ** 2 + (Y - cy) ** 2 + (Z - cz) ** 2) - r)
    chi = float(rng.uniform(0.5, 3.0))
    d = rng.normal(size=3)
    d = d / np.linalg.norm(d) * rng.uniform(0.5, 2.0)
    vel = [rng.normal(0.0, 0.5, g.face_shape(a)) for a in range(3)]
    frac = box_fractions(g, 0) if with_fractions else None
    return Scene("random", g, np.ascontiguousarray(phi), vel, frac, uniform_field(g, tuple(d)), chi, 2 * g.spacing,
                 dict(seed=seed))


def divergence(g: StaggeredGrid, vel, frac=None):
    """Discrete divergence sum_faces side * w * u per cell (the reference's rhs without the solid term)."""
    d = np.zeros(g.shape)
    for a in range(3):
        w = np.ones(g.face_shape(a)) if frac is None else 1.0 - frac[a]
        f = w * vel[a]
        sl_hi = [slice(None)] * 3
        sl_lo = [slice(None)] * 3
        sl_hi[a] = slice(1, None)
        sl_lo[a] = slice(0, -1)
        d += f[tuple(sl_hi)] - f[tuple(sl_lo)]
    return d


def full_weight_cells(g: StaggeredGrid, frac):
    """Cells whose six face weights w = 1 - fraction are all 0 or 1.  On such a liquid cell the projected
    velocity's weighted divergence is minus the pressure solve's residual; where a face is partly open the
    projection scales the update by w and the divergence weighs it by w again, so it does not vanish there
    (in the reference as well)."""
    whole = np.ones(g.shape, bool)
    for a in range(3):
        f = frac[a]
        ok = (f == 0) | (f == 1)
        lo, hi = [slice(None)] * 3, [slice(None)] * 3
        lo[a], hi[a] = slice(0, -1), slice(1, None)
        whole &= ok[tuple(lo)] & ok[tuple(hi)]
    return whole
