"""Seeded synthetic scenes for the SPH hot path.

The reference builds its scenes in Lua scripts from OBJ meshes
(share/scripts/prtcl-lua.example.lua:288-316, geometry/sample_volume.hpp).
The workloads here are plain lattices instead, generated deterministically:

* ``dam_break``: a block of fluid particles on a cubic lattice in the corner
  of a closed box whose walls are ``layers`` layers of static boundary
  particles on the same lattice.  Defaults give the 30x30x30 = 27,000 fluid
  particle scene (spacing 0.025 m, 2 x 1 x 1 m box, 2 wall layers).
* ``search_points``: N points in the unit cube, uniform or as isotropic
  Gaussian blobs clipped to the cube, for the neighbour-search workload.
* ``mixed_batch``: many dam-break scenes of log-uniform fluid counts.

All coordinates are produced in float64 and rounded once to float32.
"""
from __future__ import annotations

import math

import numpy as np


def _lattice(lo, hi, spacing):
    """Points (i + 0.5) * spacing for integer i in [lo, hi) per axis."""
    axes = [np.arange(lo[a], hi[a], dtype=np.float64) for a in range(3)]
    g = np.meshgrid(*axes, indexing="ij")
    idx = np.stack([c.ravel() for c in g], axis=1)
    return idx


def dam_break(fluid_cells=(30, 30, 30), spacing=0.025, box=(2.0, 1.0, 1.0), layers=2):
    """Fluid block + closed-box wall particles.

    Returns a dict with float32 arrays ``fluid`` (Nf, 3) and ``boundary``
    (Nb, 3), plus ``spacing`` and the box size in lattice cells.
    """
    s = float(spacing)
    nx, ny, nz = (int(round(b / s)) for b in box)
    fl = _lattice((0, 0, 0), fluid_cells, s)
    fluid = ((fl + 0.5) * s).astype(np.float32)
    L = int(layers)
    shell = _lattice((-L, -L, -L), (nx + L, ny + L, nz + L), s)
    inside = (
        (shell[:, 0] >= 0) & (shell[:, 0] < nx)
        & (shell[:, 1] >= 0) & (shell[:, 1] < ny)
        & (shell[:, 2] >= 0) & (shell[:, 2] < nz)
    )
    boundary = ((shell[~inside] + 0.5) * s).astype(np.float32)
    return {"fluid": fluid, "boundary": boundary, "spacing": s, "box_cells": (nx, ny, nz)}


def dam_break_1m():
    """100^3 = 1,000,000 fluid particles, same geometry ratios as the 27k
    scene (fluid block 0.75 m in a 2 x 1 x 1 m box), spacing 0.0075 m;
    about 363k wall particles."""
    return dam_break(fluid_cells=(100, 100, 100), spacing=0.0075, box=(2.0, 1.0, 1.0), layers=2)


def search_points(n, distribution="uniform", seed=1, blobs=64, sigma=0.03):
    """N float32 points in [0, 1)^3."""
    rng = np.random.default_rng(seed)
    if distribution == "uniform":
        pts = rng.random((n, 3))
    elif distribution == "blobs":
        centres = rng.random((blobs, 3))
        which = rng.integers(0, blobs, size=n)
        pts = centres[which] + rng.normal(0.0, sigma, size=(n, 3))
        pts = np.clip(pts, 0.0, np.nextafter(1.0, 0.0))
    else:
        raise ValueError(distribution)
    return pts.astype(np.float32)


def uniform_radius_for_mean_neighbours(n, mean_neighbours=40.0):
    """Radius giving the requested mean neighbour count (self included) for
    n uniform points in the unit cube (boundary effects ignored)."""
    return (mean_neighbours / (n * 4.0 / 3.0 * math.pi)) ** (1.0 / 3.0)


def calibrate_radius(mean_neighbours_at, n, target=40.0, steps=14):
    """Radius (rounded to float32) at which ``mean_neighbours_at(r)`` first
    reaches ``target``: a bracket found in steps of 1.25x from a quarter of
    the uniform estimate, then ``steps`` bisections.  Steps of 1.25x in the
    radius at most double the mean count, so no trial radius builds lists
    far longer than the target's (clustered points can have many times the
    uniform count at the uniform radius).  ``mean_neighbours_at`` counts on
    whatever grid the caller holds (the device's, for the search workload)."""
    r = 0.25 * uniform_radius_for_mean_neighbours(n, target)
    if mean_neighbours_at(r) >= target:
        hi, lo = r, r / 1.25
        while mean_neighbours_at(lo) >= target:
            hi, lo = lo, lo / 1.25
    else:
        lo, hi = r, 1.25 * r
        while mean_neighbours_at(hi) < target:
            lo, hi = hi, 1.25 * hi
    for _ in range(steps):
        mid = 0.5 * (lo + hi)
        if mean_neighbours_at(mid) < target:
            lo = mid
        else:
            hi = mid
    return float(np.float32(hi))


def mixed_batch(count=256, lo=2000, hi=200000, seed=3, spacing=0.025, layers=2):
    """``count`` dam-break scenes with fluid counts log-uniform in [lo, hi],
    block aspect ratios uniform in [0.5, 2] and boxes 2x the fluid extent."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        nf = math.exp(rng.uniform(math.log(lo), math.log(hi)))
        ax, az = rng.uniform(0.5, 2.0, size=2)
        # cells: nx = ax * k, ny = k, nz = az * k with nx*ny*nz ~= nf
        k = (nf / (ax * az)) ** (1.0 / 3.0)
        cells = (max(1, int(round(ax * k))), max(1, int(round(k))), max(1, int(round(az * k))))
        box = tuple(2.0 * c * spacing for c in cells)
        out.append(dam_break(fluid_cells=cells, spacing=spacing, box=box, layers=layers))
    return out
