"""Seeded synthetic voxel scenes: a fluid pool under a wavy height field with solid spheres.

The reference solves scenes exported by a fluid simulator (flags_*.bin,
A_*.bin, div_v_star_*.bin, lib/read_data.py); those are not distributed, so
workloads are generated with the same flag codes and image channels:

* one layer of BOUNDARY (solid wall) cells on every face of the grid;
* SOLID cells inside spheres with centres ~ U(0.2N, 0.8N)^3 and radii ~ U(0.05N, 0.15N);
* FLUID cells below h(x, y) = 0.4N + 0.08N * sum_{k=1..3} sin(2 pi k (x u_k + y v_k) + phi_k),
  u_k, v_k ~ U(0, 1)/N, phi_k ~ U(0, 2 pi), that are not solid;
* AIR (Dirichlet p = 0) everywhere else.

Random draws come from numpy.random.default_rng(seed) in the order u, v, phi,
then (centre, radius) per sphere, then the right-hand side.  The right-hand
side is U(-1, 1) on fluid cells and 0 elsewhere, with its mean removed on every
6-connected fluid component that touches no air cell (those components are
pure-Neumann, so the system is only consistent with a zero-mean rhs).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

BOUNDARY, SOLID, FLUID, AIR = 0, 1, 2, 3


@dataclass
class Scene:
    flags: np.ndarray      # (N1, N2, N3) uint8 flag codes
    rhs: np.ndarray        # (N1, N2, N3) float64, zero off-fluid
    seed: int

    @property
    def shape(self):
        return self.flags.shape

    @property
    def fluid_cells(self) -> np.ndarray:
        return np.flatnonzero(self.flags.ravel() == FLUID)

    def image(self) -> np.ndarray:
        return flags_to_image(self.flags)


def flags_to_image(flags: np.ndarray) -> np.ndarray:
    """[air, fluid, non-solid] float32 channels (convert_to_binary_images, lib/read_data.py:28-39)."""
    f = np.asarray(flags)
    air = (f == AIR)
    fluid = (f == FLUID)
    nonsolid = ~(f <= SOLID)
    return np.stack([air, fluid, nonsolid]).astype(np.float32)


def make_flags(shape, seed: int, n_spheres: int = 3) -> np.ndarray:
    """Flag grid of the scene ``seed`` (see module docstring)."""
    return _flags_and_rng(shape, seed, n_spheres)[0]


def _flags_and_rng(shape, seed: int, n_spheres: int):
    if isinstance(shape, int):
        shape = (shape,) * 3
    n1, n2, n3 = shape
    N = float(n3)
    rng = np.random.default_rng(seed)
    u = rng.uniform(0.0, 1.0, 3) / N
    v = rng.uniform(0.0, 1.0, 3) / N
    phi = rng.uniform(0.0, 2.0 * np.pi, 3)
    spheres = []
    for _ in range(n_spheres):
        c = rng.uniform(0.2, 0.8, 3) * np.array([n1, n2, n3], dtype=np.float64)
        r = rng.uniform(0.05, 0.15) * N
        spheres.append((c, r))
    x = np.arange(n1, dtype=np.float64)[:, None]
    y = np.arange(n2, dtype=np.float64)[None, :]
    h = 0.4 * N + 0.08 * N * sum(
        np.sin(2.0 * np.pi * (k + 1) * (x * u[k] + y * v[k]) + phi[k]) for k in range(3))
    z = np.arange(n3, dtype=np.float64)
    flags = np.where(z[None, None, :] < h[:, :, None], FLUID, AIR).astype(np.uint8)
    ii, jj, kk = np.meshgrid(np.arange(n1), np.arange(n2), np.arange(n3), indexing="ij", sparse=True)
    for c, r in spheres:
        inside = (ii - c[0]) ** 2 + (jj - c[1]) ** 2 + (kk - c[2]) ** 2 <= r * r
        flags[inside] = SOLID
    flags[0, :, :] = flags[-1, :, :] = BOUNDARY
    flags[:, 0, :] = flags[:, -1, :] = BOUNDARY
    flags[:, :, 0] = flags[:, :, -1] = BOUNDARY
    return flags, rng


def _neumann_components(flags):
    """Labels of 6-connected fluid components and a bool per label: touches no air."""
    from scipy import ndimage
    fluid = flags == FLUID
    struct = ndimage.generate_binary_structure(3, 1)
    lab, nlab = ndimage.label(fluid, structure=struct)
    air = flags == AIR
    air_nb = np.zeros_like(air)
    air_nb[1:] |= air[:-1]; air_nb[:-1] |= air[1:]
    air_nb[:, 1:] |= air[:, :-1]; air_nb[:, :-1] |= air[:, 1:]
    air_nb[:, :, 1:] |= air[:, :, :-1]; air_nb[:, :, :-1] |= air[:, :, 1:]
    touches = np.zeros(nlab + 1, dtype=bool)
    touches[np.unique(lab[fluid & air_nb])] = True
    return lab, nlab, ~touches


def make_scene(shape, seed: int, n_spheres: int = 3) -> Scene:
    flags, rng = _flags_and_rng(shape, seed, n_spheres)
    b = rng.uniform(-1.0, 1.0, flags.shape)
    b = np.where(flags == FLUID, b, 0.0)
    lab, nlab, neumann = _neumann_components(flags)
    if nlab:
        sums = np.bincount(lab.ravel(), weights=b.ravel(), minlength=nlab + 1)
        cnts = np.bincount(lab.ravel(), minlength=nlab + 1).astype(np.float64)
        means = np.where(neumann & (cnts > 0), sums / np.maximum(cnts, 1.0), 0.0)
        means[0] = 0.0
        b = b - means[lab]
        b = np.where(flags == FLUID, b, 0.0)
    return Scene(flags=flags, rhs=b, seed=seed)
