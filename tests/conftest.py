"""Shared fixtures: builds the native library and the oracle once per session,
registers the `gpu` marker, and provides the parity scenes."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent
if str(REPO) not in sys.path:
    sys.path.insert(0, str(REPO))

import __graft_entry__ as entry  # noqa: E402

GOLDEN = REPO / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests through the C ABI")


def cuda_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def bp():
    """The product package, with libbrasspan.so and the oracle built."""
    entry.build()
    return entry.load_package()


@pytest.fixture(scope="session")
def oracle(bp):
    import oracle as o

    return o


@pytest.fixture(scope="session")
def gpu(bp):
    if not cuda_available():
        pytest.fail("a CUDA device is required for -m gpu tests")
    import torch

    torch.cuda.init()
    return torch


def small_mixed_scene(bp, seed=0, fluid=(10, 10, 10), grid_dim=32):
    """Fluid block, a cloth pinned at two corners (wind, distance constraints),
    two rigid boxes, a rope, five walls; random initial velocities."""
    sc = bp.scenes
    rng = np.random.default_rng(seed)
    s = sc.Scene(name="small_mixed")
    d = 0.1
    s.particle_radius = 0.05
    s.kernel_radius = 0.2
    s.cell_size = 0.2
    s.grid_dim = grid_dim
    s.rest_density = 1000.0
    sc.box_planes(s, (0, 0, 0), (3.0, 4.0, 3.0))
    s.add_fluid_block(fluid, (0.1, 0.1, 0.1), (d, d, d), 1.0, jitter=0.001, rng=rng)
    s.add_cloth((0.2, 1.25, 0.2), (0.1, 0, 0), (0, 0, 0.1), 8, 8, 1.0, corners=(True, False, False, True))
    s.add_rigid_box((3, 3, 3), (0.4, 1.45, 0.5), (d, d, d), 1.0)
    s.add_rigid_box((4, 2, 3), (0.6, 1.9, 0.4), (d, d, d), 1.0)
    s.add_rope((2.5, 3.0, 0.5), (2.5, 2.0, 0.5), 10, 1.0)
    s.velocities = rng.uniform(-0.5, 0.5, (s.num_particles, 3)).astype(np.float32)
    return s


def fluid_scene(bp, n=(12, 12, 12), seed=0, grid_dim=64, box=(2.0, 3.0, 2.0)):
    s = bp.scenes.pbf_scene(*n, spacing=0.1, seed=seed, box=box, grid_dim=grid_dim)
    rng = np.random.default_rng(seed + 100)
    s.velocities = rng.uniform(-0.3, 0.3, (s.num_particles, 3)).astype(np.float32)
    return s


def cloth_bending_scene(bp, seed=0, n=12, grid_dim=16):
    """A horizontal cloth with the reference's dihedral bending quads, pinned
    at two corners, sagging onto itself; random initial velocities."""
    sc = bp.scenes
    rng = np.random.default_rng(seed)
    s = sc.Scene(name="cloth_bending")
    s.particle_radius, s.kernel_radius, s.cell_size, s.grid_dim, s.rest_density = 0.05, 0.2, 0.2, grid_dim, 1000.0
    sc.box_planes(s, (0, 0, 0), (3.0, 4.0, 3.0))
    s.add_cloth((0.2, 1.5, 0.2), (0.1, 0, 0), (0, 0, 0.1), n, n, 0.1, corners=(True, True, False, False),
                stretch=0.25, shear=0.1, bend=0.05, dihedral=True)
    s.velocities = rng.uniform(-0.3, 0.3, (s.num_particles, 3)).astype(np.float32)
    return s
