"""Shared helpers of the parity tests: run the CUDA library and the CPU oracle on one scene."""
import numpy as np

from xrtailor_gb300 import ClothSolver, scenes
from xrtailor_gb300.solver import Mesh


def bits(a):
    """Bit pattern of a float32 array (NaN-safe exact comparison)."""
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def diag(x):
    x = np.asarray(x, np.float64)
    return float(np.linalg.norm(x.max(0) - x.min(0)))


def small_scene(n=16, obstacle="sphere", pins=True, attached=None, seed=1, size=1.0):
    cloth = scenes.grid_cloth(n, size, origin=(0.0, 0.35, 0.0), jitter=1e-3, seed=seed)
    if pins:
        cloth.fixed_indices = scenes.two_corner_pins(n)
    if attached is not None:
        cloth.attached_indices = np.asarray(attached, np.uint32)
    obs = None
    if obstacle == "sphere":
        obs = scenes.icosphere(2, 0.3, center=(0.5 * size, 0.0, 0.5 * size))
    elif obstacle == "plane":
        obs = scenes.ground_plane(8, 3.0, height=0.2, center=(0.5, 0.5))
    return cloth, obs


def make_pair(params, cloths, obstacles=(), particle_diameter=0.0, colors_from_gpu=True,
              inv_mass=None, fem=None, tile_vertices=None):
    """Builds a ClothSolver (GPU) and an OracleSolver (CPU) with the same inputs; `fem`: an
    xrt_fem_material for both (the FEM fabric)."""
    from oracle.oracle import OracleSolver
    g = ClothSolver(params)
    o = OracleSolver(params)
    if tile_vertices is not None:
        g.set_tile_vertices(tile_vertices)
    if fem is not None:
        g.set_fem_material(fem)
        o.set_fem_material(fem)
    for c in cloths:
        g.add_cloth(c, particle_diameter=particle_diameter)
        o.add_cloth(c, particle_diameter=particle_diameter)
    for ob in obstacles:
        if ob is not None:
            g.add_obstacle(ob)
            o.add_obstacle(ob)
    if inv_mass is not None:
        g.set_inv_mass(inv_mass)
        o.set_inv_mass(inv_mass)
    g.start()
    if colors_from_gpu:
        o.set_coloring(0, g.coloring(0))
        o.set_coloring(1, g.coloring(1))
        if fem is not None:
            o.set_coloring(2, g.coloring(2))
            o.set_coloring(3, g.coloring(3))
    o.start()
    return g, o


def prim_soup(n, seed=0, spread=1.0, size=0.05, flat_axis=None):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-spread, spread, size=(n, 1, 3))
    p = c + rng.normal(0, size, size=(n, 3, 3))
    if flat_axis is not None:
        p[:, :, flat_axis] = 0.0
    return p.astype(np.float32).reshape(n, 9)


def tube_mesh(rings=10, slices=12, seed=2):
    b = scenes.TubeBody(rings=rings, slices=slices, height=0.5, radius=0.1, bones=6, seed=seed,
                        base=(0.5, -0.2, 0.5))
    return b
