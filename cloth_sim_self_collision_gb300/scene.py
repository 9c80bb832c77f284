"""Synthetic cloth scenes: square grids over a sphere.

The grid topology restates ``SetClothShape_Square`` of the reference
(self_contact_sparse/main.cpp:31-106): vertices ix-major, two triangles per
cell split along the same diagonal, and three families of 4-vertex bending
stencils (one per cell diagonal, one per interior x-edge, one per interior
z-edge).  The reference lays the sheet in its xz-plane; the workloads here lay
it in the xy-plane at a given height with gravity along -z, so the cloth drops
onto a solid sphere at the origin.

A tiny deterministic z-jitter (splitmix64 stream, seeded) breaks the symmetry of
a perfectly flat sheet.  The jittered positions are both the rest shape and the
initial shape, as ``aXYZ = aXYZ0`` in the reference (main.cpp:569).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

OBSTACLE_NONE = 0
OBSTACLE_PLANE_Z = 1
OBSTACLE_SPHERE_SOLID = 2
OBSTACLE_SPHERE_HOLLOW = 3

SOLVER_ILU_PCG = 0
SOLVER_CG = 1

_MASK64 = (1 << 64) - 1


def splitmix64(seed: int, n: int) -> np.ndarray:
    """n uint64 draws of the splitmix64 generator started at ``seed``."""
    out = np.empty(n, dtype=np.uint64)
    s = seed & _MASK64
    for i in range(n):
        s = (s + 0x9E3779B97F4A7C15) & _MASK64
        z = s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK64
        out[i] = z ^ (z >> 31)
    return out


def uniform(seed: int, n: int, lo: float, hi: float) -> np.ndarray:
    """n doubles uniform in [lo, hi) from the top 53 bits of splitmix64."""
    u = (splitmix64(seed, n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return lo + (hi - lo) * u


@dataclasses.dataclass
class Params:
    """Physical and solver parameters of one cloth (layout of ``cs_params``)."""
    dt: float = 0.02
    lam: float = 1.0
    myu: float = 1.0
    stiff_bend: float = 1.0e-3
    gravity: tuple = (0.0, 0.0, -9.8)
    mass_point: float = 1.0
    stiff_contact: float = 300.0
    contact_clearance: float = 0.01
    obs_center: tuple = (0.0, 0.0, 0.0)
    obs_radius: float = 0.3
    tol: float = 1.0e-6
    obstacle_kind: int = OBSTACLE_SPHERE_SOLID
    solver_kind: int = SOLVER_ILU_PCG
    maxit: int = 100
    flags: int = 0  # CS_FLAG_EXACT_DOTS = 1: serial inner products (bit-exact FP64 path)


@dataclasses.dataclass
class Cloth:
    """Topology, rest shape and parameters of one cloth instance."""
    X0: np.ndarray      # (np*3,) float64 rest positions, also the initial positions
    tri: np.ndarray     # (nt*3,) int32
    quad: np.ndarray    # (nq*4,) int32 bending stencils
    bc: np.ndarray      # (np,) int32, 1 = fixed
    params: Params
    side: int = 0

    @property
    def np(self) -> int:
        return self.X0.size // 3

    @property
    def nt(self) -> int:
        return self.tri.size // 3

    @property
    def nq(self) -> int:
        return self.quad.size // 4


def grid_topology(side: int):
    """Triangles and bending stencils of a side x side vertex grid
    (self_contact_sparse/main.cpp:58-97), as int32 arrays."""
    nd = side - 1
    n = side
    ix, iz = np.meshgrid(np.arange(nd), np.arange(nd), indexing="ij")
    ix = ix.ravel()
    iz = iz.ravel()
    t = np.stack([ix * n + iz, (ix + 1) * n + iz, ix * n + iz + 1,
                  (ix + 1) * n + iz + 1, ix * n + iz + 1, (ix + 1) * n + iz], axis=1)
    tri = t.reshape(-1).astype(np.int32)
    q0 = np.stack([ix * n + iz, (ix + 1) * n + iz + 1, (ix + 1) * n + iz, ix * n + iz + 1], axis=1)
    jx, jz = np.meshgrid(np.arange(nd), np.arange(nd - 1), indexing="ij")
    jx = jx.ravel()
    jz = jz.ravel()
    q1 = np.stack([(jx + 1) * n + jz, jx * n + jz + 2, (jx + 1) * n + jz + 1, jx * n + jz + 1], axis=1)
    kx, kz = np.meshgrid(np.arange(nd - 1), np.arange(nd), indexing="ij")
    kx = kx.ravel()
    kz = kz.ravel()
    q2 = np.stack([kx * n + kz + 1, (kx + 2) * n + kz, (kx + 1) * n + kz, (kx + 1) * n + kz + 1], axis=1)
    quad = np.concatenate([q0, q1, q2], axis=0).reshape(-1).astype(np.int32)
    return tri, quad


def square_cloth(side: int, size: float, height: float, *, sphere_radius: float = 0.3,
                 clearance: float = 0.01, rotation: float = 0.0, seed: int = 0,
                 jitter: float = 1.0e-4, density: float = 1.0, **overrides) -> Cloth:
    """A side x side vertex sheet of edge ``size`` centred over the origin at
    ``height``, rotated by ``rotation`` about z, above a solid sphere."""
    nd = side - 1
    h = size / nd
    ix, iz = np.meshgrid(np.arange(side), np.arange(side), indexing="ij")
    u = ix.ravel() * h - 0.5 * size
    w = iz.ravel() * h - 0.5 * size
    c, s = math.cos(rotation), math.sin(rotation)
    X = np.empty((side * side, 3), dtype=np.float64)
    X[:, 0] = c * u - s * w
    X[:, 1] = s * u + c * w
    X[:, 2] = height + uniform(seed, side * side, -jitter, jitter)
    tri, quad = grid_topology(side)
    npnt = side * side
    prm = Params(mass_point=size * size * density / npnt, contact_clearance=clearance,
                 obs_radius=sphere_radius)
    for k, v in overrides.items():
        setattr(prm, k, v)
    return Cloth(X0=X.reshape(-1), tri=tri, quad=quad, bc=np.zeros(npnt, dtype=np.int32),
                 params=prm, side=side)


# Workloads of the self_contact_sparse path.  Sizes, heights and radii follow the
# configurations the benchmark is quoted on; solver policy: the reference's ILU(0)
# PCG where it factorises (coarse sheets), its plain CG where ILU(0) meets
# non-positive pivots (element length <= 0.025 m with bending stiffness 1e-3).
def config_small() -> Cloth:
    """21x21 sheet, 1 m, z=0.5 over a sphere of radius 0.3, ILU(0)-PCG tol 1e-6."""
    return square_cloth(21, 1.0, 0.5, sphere_radius=0.3, clearance=0.01,
                        solver_kind=SOLVER_ILU_PCG, tol=1.0e-6, maxit=100)


def config_single_101() -> Cloth:
    """101x101 sheet, 2 m, z=1.0 over a sphere of radius 0.25, CG tol 1e-6."""
    return square_cloth(101, 2.0, 1.0, sphere_radius=0.25, clearance=0.01,
                        solver_kind=SOLVER_CG, tol=1.0e-6, maxit=1000)


def config_single_256() -> Cloth:
    """256x256 sheet, 2 m, z=2.0 over a sphere of radius 0.1, clearance 0.005, CG tol 1e-6."""
    return square_cloth(256, 2.0, 2.0, sphere_radius=0.1, clearance=0.005,
                        solver_kind=SOLVER_CG, tol=1.0e-6, maxit=1000)


def config_batch(count: int = 512, seed: int = 3, side_lo: int = 11, side_hi: int = 81) -> list:
    """``count`` independent sheets: side uniform in [side_lo, side_hi], drop height
    uniform in [0.3, 1.5] m, rotation uniform in [0, 2 pi) about z, sphere radius
    uniform in [0.1, 0.4] m, 1 m cloth, CG tol 1e-6."""
    r = uniform(seed, 4 * count, 0.0, 1.0).reshape(count, 4)
    out = []
    for i in range(count):
        side = side_lo + min(int(r[i, 0] * (side_hi - side_lo + 1)), side_hi - side_lo)
        height = 0.3 + 1.2 * r[i, 1]
        rot = 2.0 * math.pi * r[i, 2]
        rad = 0.1 + 0.3 * r[i, 3]
        out.append(square_cloth(side, 1.0, height, sphere_radius=rad, clearance=0.01,
                                rotation=rot, seed=1000 + i, solver_kind=SOLVER_CG,
                                tol=1.0e-6, maxit=1000))
    return out


def config_serving(count: int, seed: int = 11, n_lo: float = 1.0e2, n_hi: float = 1.0e5) -> list:
    """``count`` serving scenes: vertex count log-uniform in [n_lo, n_hi] as square
    grids (side = round(sqrt(N))), drop height uniform in [0.3, 1.5] m, rotation
    uniform about z, sphere radius uniform in [0.1, 0.4] m, clearance 0.01 m, CG
    tol 1e-6.

    Sheets are 1 m wide up to 61 vertices a side and grow beyond that so their
    edges stay 1/60 m long: when a cell's diagonal spacing (edge / sqrt(2)) is
    below the clearance the reference's proximity test fires between
    neighbouring cells of a flat sheet, and below 1 cm its edge-edge CCD (whose
    distance test is fixed at 1e-2) does.
    Material and time step are the reference demo's (self_contact_sparse/main.cpp:
    lambda 0, mu 30, bending 1e-2, areal density 0.04, dt 0.01, gravity
    (0, 0.05, -10), contact stiffness 300): with the batched sheets' material
    (lambda = mu = 1, density 1) the reference's own frames blow up within a few
    dozen frames of these drops, and a scene here runs 200 frames."""
    r = uniform(seed, 5 * count, 0.0, 1.0).reshape(count, 5)
    out = []
    for i in range(count):
        n = math.exp(math.log(n_lo) + (math.log(n_hi) - math.log(n_lo)) * r[i, 0])
        side = max(3, int(round(math.sqrt(n))))
        out.append(square_cloth(side, max(1.0, (side - 1) / 60.0), 0.3 + 1.2 * r[i, 1],
                                sphere_radius=0.1 + 0.3 * r[i, 3], clearance=0.01,
                                rotation=2.0 * math.pi * r[i, 2], seed=5000 + i, density=0.04, lam=0.0,
                                myu=30.0, stiff_bend=1.0e-2, dt=0.01, gravity=(0.0, 0.05, -10.0),
                                stiff_contact=300.0, solver_kind=SOLVER_CG, tol=1.0e-6, maxit=1000))
    return out
