"""Scene description and builders (host side of the reference's Scene API).

`Scene` holds flat arrays in original particle order, the content of the
reference's `Scene` vectors (brasstower/scene.h:455-535).  The builders follow
the reference's object factories and the way ParticleSolver's add* methods
assign phases and ids (brasstower/particlesolver.cuh:395-710):

* fluids share one negative phase per block (fluidPhaseCounter, -1, -2, ...);
* granulars and self-colliding ropes/cloths get one solid phase per particle
  (setDevArr_counterIncrement), rigid bodies one solid phase per body;
* constraint ids are offset by the particle count before the object.

The benchmark scenes (`dam_break_32k`, `mixed_phase_1m`, `dam_break_ensemble`,
`rigid_body_pile`) are built from the same factories with seeded jitter.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Scene:
    positions: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.float32))
    velocities: np.ndarray | None = None
    masses: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    phases: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    group_ids: np.ndarray | None = field(default_factory=lambda: np.zeros(0, np.int32))
    planes: np.ndarray = field(default_factory=lambda: np.zeros((0, 6), np.float32))
    distance_pairs: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.int32))
    distance_params: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.float32))
    faces: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.int32))
    rigid_ranges: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.int32))
    rigid_rest: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.float32))
    immovables: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    bendings: np.ndarray = field(default_factory=lambda: np.zeros((0, 4), np.int32))
    # counters as in the reference
    solid_phase_counter: int = 1
    fluid_phase_counter: int = -1
    group_counter: int = 0
    # solver parameters that belong to the scene
    particle_radius: float = 0.05
    kernel_radius: float = 0.115
    cell_size: float = 0.115
    grid_dim: int = 512
    rest_density: float = 1200.0
    gravity: tuple = (0.0, -9.8, 0.0)
    name: str = "scene"

    @property
    def num_particles(self) -> int:
        return int(len(self.positions))

    @property
    def num_distance_constraints(self) -> int:
        return int(len(self.distance_pairs))

    # -- internal append -------------------------------------------------------
    def _append(self, pos, mass, phases, rest=None):
        pos = np.asarray(pos, np.float32).reshape(-1, 3)
        n0 = self.num_particles
        k = len(pos)
        self.positions = np.concatenate([self.positions, pos]).astype(np.float32)
        self.masses = np.concatenate([self.masses, np.full(k, mass, np.float32)])
        self.phases = np.concatenate([self.phases, np.asarray(phases, np.int32)])
        self.group_ids = np.concatenate([self.group_ids, np.full(k, self.group_counter, np.int32)])
        self.group_counter += 1
        r = np.zeros((k, 3), np.float32) if rest is None else np.asarray(rest, np.float32)
        self.rigid_rest = np.concatenate([self.rigid_rest, r]).astype(np.float32)
        if self.velocities is not None:
            self.velocities = np.concatenate([self.velocities, np.zeros((k, 3), np.float32)])
        return n0

    def _solid_phases(self, k, self_collide=True):
        if self_collide:
            ph = np.arange(self.solid_phase_counter, self.solid_phase_counter + k, dtype=np.int32)
            self.solid_phase_counter += k
        else:
            ph = np.full(k, self.solid_phase_counter, np.int32)
            self.solid_phase_counter += 1
        return ph

    # -- builders ----------------------------------------------------------------
    def add_plane(self, origin, normal):
        """Plane(origin, normal) (scene.h:13-37); the normal is used as given."""
        row = np.array([*origin, *normal], np.float32).reshape(1, 6)
        self.planes = np.concatenate([self.planes, row])

    @staticmethod
    def _block(dim, start, step):
        """CreateFluidBlock / CreateGranularsBlock / CreateRigidBox lattice order:
        i (x) outer, k (z) inner (scene.h:62-67, 104-110, 131-137)."""
        dim = np.asarray(dim, int)
        i, j, k = np.meshgrid(np.arange(dim[0]), np.arange(dim[1]), np.arange(dim[2]), indexing="ij")
        ijk = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1).astype(np.float32)
        return np.asarray(start, np.float32) + np.asarray(step, np.float32) * ijk

    def add_fluid_block(self, dim, start, step, mass, jitter=0.0, rng=None):
        pos = self._block(dim, start, step)
        if jitter:
            pos = pos + rng.uniform(-jitter, jitter, pos.shape).astype(np.float32)
        n0 = self._append(pos, mass, np.full(len(pos), self.fluid_phase_counter, np.int32))
        self.fluid_phase_counter -= 1  # particlesolver.cuh:505
        return n0, self.num_particles

    def add_granulars_block(self, dim, start, step, mass):
        pos = self._block(dim, start, step)
        n0 = self._append(pos, mass, self._solid_phases(len(pos), True))
        return n0, self.num_particles

    def add_rigid_body(self, pos, mass):
        """RigidBody + addRigidBody (scene.h:39-89, particlesolver.cuh:424-478):
        rest shape = positions minus their (unweighted) centre of mass."""
        pos = np.asarray(pos, np.float32).reshape(-1, 3)
        cm = pos.mean(axis=0, dtype=np.float64).astype(np.float32)
        rest = pos - cm
        n0 = self._append(pos, mass, self._solid_phases(len(pos), False), rest=rest)
        self.rigid_ranges = np.concatenate([self.rigid_ranges, np.array([[n0, self.num_particles]], np.int32)])
        return n0, self.num_particles

    def add_rigid_box(self, dim, start, step, mass):
        return self.add_rigid_body(self._block(dim, start, step), mass)

    def add_rope(self, start, end, num_joint, mass, self_collide=True):
        """Rope::CreateRope + addNoodles (scene.h:141-179, particlesolver.cuh:510-573)."""
        start = np.asarray(start, np.float32)
        diff = np.asarray(end, np.float32) - start
        d = float(np.linalg.norm(diff)) / float(num_joint - 1)
        t = (np.arange(num_joint, dtype=np.float32) / np.float32(num_joint - 1))[:, None]
        pos = start + t * diff
        n0 = self._append(pos, mass, self._solid_phases(num_joint, self_collide))
        pairs = [(i, i + 1) for i in range(num_joint - 1)] + [(i - 1, i + 1) for i in range(1, num_joint - 1)]
        params = [(d, 1.0)] * (num_joint - 1) + [(2.0 * d, 0.1)] * (num_joint - 2)
        self._add_pairs(np.array(pairs, np.int32) + n0, np.array(params, np.float32))
        return n0, self.num_particles

    def _add_pairs(self, pairs, params):
        self.distance_pairs = np.concatenate([self.distance_pairs, pairs.reshape(-1, 2).astype(np.int32)])
        self.distance_params = np.concatenate([self.distance_params, params.reshape(-1, 2).astype(np.float32)])

    def add_cloth(self, start, offset_x, offset_y, nx, ny, mass, corners=(False, False, False, False),
                  stretch=0.2, shear=None, bend=0.1, self_collide=True, dihedral=False):
        """Cloth::CreateCloth + addCloth (scene.h:226-330, particlesolver.cuh:576-710).

        Positions are pushed x-outer / y-inner as start + y*offset_x + x*offset_y
        while constraint ids use y*nx + x; for square cloths that only
        transposes the lattice, exactly as the reference does.  Pairs:
        horizontal and vertical (stretch), both diagonals (shear), and the
        skip-one "hack bending" pairs of the 3x3 stencil (bend), with the
        reference's repetitions.  dihedral=True adds the reference's
        commented-out dihedral bending quads (scene.h:308-320): per lattice
        quad (p3, p2, p1, p4) when x + y is odd, else (p1, p4, p3, p2)."""
        shear = stretch if shear is None else shear
        ox = np.asarray(offset_x, np.float32)
        oy = np.asarray(offset_y, np.float32)
        lx = float(np.linalg.norm(ox))
        ly = float(np.linalg.norm(oy))
        ld = float(np.linalg.norm(ox + oy))
        pos, faces, pairs, params, imm, quads = [], [], [], [], [], []
        if corners[0]:
            imm.append(0)
        if corners[1]:
            imm.append(nx - 1)
        if corners[2]:
            imm.append(nx * (ny - 1))
        if corners[3]:
            imm.append(nx * ny - 1)
        for x in range(nx):
            for y in range(ny):
                pos.append(np.asarray(start, np.float32) + np.float32(y) * ox + np.float32(x) * oy)
                p1 = y * nx + x
                p2 = y * nx + x + 1
                p3 = (y + 1) * nx + x
                p4 = (y + 1) * nx + x + 1
                if x < nx - 1 and y < ny - 1:
                    faces.append((p1, p2, p3))
                    faces.append((p2, p3, p4))
                    if dihedral:
                        quads.append((p3, p2, p1, p4) if (x + y) % 2 else (p1, p4, p3, p2))
                if x < nx - 1:
                    pairs.append((p1, p2)); params.append((lx, stretch))
                if y < ny - 1:
                    pairs.append((p1, p3)); params.append((ly, stretch))
                if x < nx - 1 and y < ny - 1:
                    pairs.append((p1, p4)); params.append((ld, shear))
                    pairs.append((p2, p3)); params.append((ld, shear))
                if 0 < x < nx - 1 and 0 < y < ny - 1:
                    q = [[(y + i) * nx + x + j for j in (-1, 0, 1)] for i in (-1, 0, 1)]
                    for i in range(3):
                        pairs.append((q[i][0], q[i][2])); params.append((lx * 2, bend))
                    for i in range(3):
                        pairs.append((q[0][i], q[2][i])); params.append((ly * 2, bend))
        pos = np.array(pos, np.float32)
        n0 = self._append(pos, mass, self._solid_phases(len(pos), self_collide))
        self._add_pairs(np.array(pairs, np.int32) + n0, np.array(params, np.float32))
        if faces:
            self.faces = np.concatenate([self.faces, np.array(faces, np.int32) + n0])
        if imm:
            self.immovables = np.concatenate([self.immovables, np.array(imm, np.int32) + n0])
        if quads:
            self.bendings = np.concatenate([self.bendings, np.array(quads, np.int32) + n0])
        return n0, self.num_particles

    def make_immovable(self, ids):
        self.immovables = np.concatenate([self.immovables, np.asarray(ids, np.int32).ravel()])


def box_planes(scene: Scene, lo, hi, ceiling=False):
    """Floor and four walls of the axis-aligned box [lo, hi] (normals inward)."""
    lo = np.asarray(lo, np.float32)
    hi = np.asarray(hi, np.float32)
    scene.add_plane((0, lo[1], 0), (0, 1, 0))
    scene.add_plane((lo[0], 0, 0), (1, 0, 0))
    scene.add_plane((hi[0], 0, 0), (-1, 0, 0))
    scene.add_plane((0, 0, lo[2]), (0, 0, 1))
    scene.add_plane((0, 0, hi[2]), (0, 0, -1))
    if ceiling:
        scene.add_plane((0, hi[1], 0), (0, -1, 0))


def pbf_scene(nx, ny, nz, spacing=0.1, seed=0, box=None, jitter_frac=0.01, grid_dim=64, mass=None):
    """A fluid block on a cubic lattice in the corner of a box: the dam break
    of the benchmark configuration.  h = 2*spacing, cell = h, rho0 = m/d^3."""
    rng = np.random.default_rng(seed)
    d = np.float32(spacing)
    s = Scene(name=f"pbf_{nx}x{ny}x{nz}")
    s.particle_radius = float(d / 2)
    s.kernel_radius = float(2 * d)
    s.cell_size = float(2 * d)
    s.grid_dim = grid_dim
    m = float(mass) if mass is not None else float(1000.0 * d ** 3)
    s.rest_density = m / float(d) ** 3
    if box is None:
        box = (max(4.0, nx * d + 1.0), max(4.0, ny * d + 1.0), max(4.0, nz * d + 1.0))
    box_planes(s, (0, 0, 0), box)
    s.add_fluid_block((nx, ny, nz), (d, d, d), (d, d, d), m, jitter=jitter_frac * d, rng=rng)
    return s


def dam_break_32k(seed=0):
    """32^3 = 32,768 fluid particles, d = 0.1, jitter +-0.01d, box [0,4]^3."""
    return pbf_scene(32, 32, 32, 0.1, seed=seed, box=(4.0, 4.0, 4.0), jitter_frac=0.01)


def mixed_phase_1m(seed=0, fluid=(128, 64, 128), cloth=256, cubes=64, cube_dim=8, stiffness=(0.25, 0.1, 0.05)):
    """1,048,576 fluid particles (128x64x128 block, d = 0.1) in the corner of
    the box [0,25.8] x [0,16] x [0,25.8]; a 256x256 cloth at spacing d (the
    contact distance 2r, so the cloth does not fight its own contacts) 2 m
    above the fluid under wind, with stretch/shear/bend stiffness 0.25/0.1/0.05
    (the configuration's 1.0/0.5/0.1 diverge under the Jacobi distance
    projection once the cloth meets the fluid; pass `stiffness` to use them);
    64 rigid 8^3 cubes on an 8x8 lattice 2-4 m above the cloth.  The 2^18-cell
    table (D = 64, cell 0.2 m) wraps every 12.8 m, as in the configuration."""
    rng = np.random.default_rng(seed)
    d = np.float32(0.1)
    s = Scene(name="mixed")
    s.particle_radius = float(d / 2)
    s.kernel_radius = float(2 * d)
    s.cell_size = float(2 * d)
    s.grid_dim = 64
    m = float(1000.0 * d ** 3)
    s.rest_density = m / float(d) ** 3
    side = max(fluid[0], fluid[2], cloth) * float(d) + 0.2
    box = (side, 16.0, side)
    box_planes(s, (0, 0, 0), box)
    s.add_fluid_block(fluid, (d, d, d), (d, d, d), m, jitter=0.01 * d, rng=rng)
    y = float(fluid[1] * d + 2.0)
    if cloth:
        s.add_cloth((0.15, y, 0.15), (d, 0, 0), (0, 0, d), cloth, cloth, m, stretch=stiffness[0], shear=stiffness[1],
                    bend=stiffness[2])
    ncube = int(round(cubes ** 0.5))
    for c in range(cubes):
        cx, cz = c % ncube, c // ncube
        start = (0.5 + cx * (box[0] - 1.0) / ncube, y + 2.0 + (c % 3) * 1.0, 0.5 + cz * (box[2] - 1.0) / ncube)
        s.add_rigid_box((cube_dim,) * 3, start, (d, d, d), m)
    return s


def ensemble_member(n_target, spacing=0.1, seed=0, rest_scale=1.0, gravity=9.8):
    """One scene of the batched ensemble: a dam break of about n_target fluid
    particles (an a x b x a block, b = a/2) in the corner of a box 1.5 times the
    block's footprint and twice its height; the grid covers the box (D the next
    power of two of its cells per axis).  Returns the scene and the
    rest-density and gravity of the member."""
    d = float(np.float32(spacing))
    a = max(2, int(round((2.0 * n_target) ** (1.0 / 3.0))))
    b = max(1, int(round(n_target / (a * a))))
    box = (1.5 * a * d + 0.2, 2.0 * b * d + 0.2, 1.5 * a * d + 0.2)
    cells = int(np.ceil(max(box) / (2 * d)))
    D = 16
    while D < cells:
        D *= 2
    s = pbf_scene(a, b, a, spacing=spacing, seed=seed, box=box, grid_dim=D)
    s.name = f"ensemble_{a}x{b}x{a}"
    s.rest_density = s.rest_density * float(rest_scale)
    s.gravity = (0.0, -float(gravity), 0.0)
    return s


def dam_break_ensemble(seed=0, num_scenes=256, lo=4096, hi=262144):
    """The batched ensemble: num_scenes dam breaks whose particle counts are
    drawn log-uniform in [lo, hi], rest density scaled uniform in [0.8, 1.2],
    gravity magnitude uniform in [5, 15], boxes scaled to the particle count."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(num_scenes):
        n = float(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        out.append(ensemble_member(n, seed=seed * 100003 + k, rest_scale=rng.uniform(0.8, 1.2),
                                   gravity=rng.uniform(5.0, 15.0)))
    return out


def flag_scene(n=128, spacing=0.1, angle_deg=20.0, seed=0, mass=1.0, stretch=0.25, shear=0.1, bend=0.05,
               floor=-30.0):
    """A cloth flag of n x n particles pinned along its vertical edge (the
    pole), its plane turned by angle_deg about the vertical so that a wind
    along +x meets it, over a distant floor.  Returns the scene; the pole's
    particles are immovable.  The distance constraints are projected Jacobi
    style (all corrections from the same positions, summed), so the summed
    stiffness around a particle must stay small: a pinned flag with the
    stiffnesses 1.0 / 0.5 / 0.1 diverges within a few frames."""
    d = float(np.float32(spacing))
    s = Scene(name=f"flag_{n}x{n}")
    s.particle_radius = d / 2
    s.kernel_radius = 2 * d
    s.cell_size = 2 * d
    s.grid_dim = 64
    s.rest_density = 1000.0
    a = np.deg2rad(angle_deg)
    s.add_plane((0.0, floor, 0.0), (0.0, 1.0, 0.0))
    ox = (d * float(np.cos(a)), 0.0, d * float(np.sin(a)))
    s.add_cloth((0.0, n * d + 1.0, 0.0), ox, (0.0, -d, 0.0), n, n, mass, stretch=stretch, shear=shear, bend=bend)
    s.make_immovable(np.arange(n) * n)  # y = 0 of every row: the pole
    rng = np.random.default_rng(seed)
    s.velocities = rng.uniform(-0.05, 0.05, (s.num_particles, 3)).astype(np.float32)
    return s


def _random_rotation(rng):
    """Uniformly random rotation matrix (from a uniform unit quaternion)."""
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]], np.float32)


def rigid_shape(count, kind, spacing):
    """A lattice of about `count` particles at `spacing`: a cube, a ball or a rod
    (7 x 7 cross-section), centred on the origin; at most about 2 m across for
    1000 particles at 0.1 m."""
    d = spacing
    if kind == "cube":
        a = max(3, int(round(count ** (1.0 / 3.0))))
        g = np.stack(np.meshgrid(*[np.arange(a)] * 3, indexing="ij"), -1).reshape(-1, 3)
    elif kind == "ball":
        r = max(1.5, (3.0 * count / (4.0 * np.pi)) ** (1.0 / 3.0))
        m = int(np.ceil(r))
        g = np.stack(np.meshgrid(*[np.arange(-m, m + 1)] * 3, indexing="ij"), -1).reshape(-1, 3)
        g = g[np.sum(g.astype(np.float64) ** 2, axis=1) <= r * r]
    else:  # rod
        length = max(2, int(round(count / 49.0)))
        g = np.stack(np.meshgrid(np.arange(length), np.arange(7), np.arange(7), indexing="ij"), -1).reshape(-1, 3)
    g = g.astype(np.float32) * np.float32(d)
    return g - g.mean(axis=0, dtype=np.float64).astype(np.float32)


def rigid_body_pile(seed=0, bodies=4096, lo=27, hi=1000, spacing=0.1, lattice=(32, 4, 32), pitch=2.5):
    """The shape-matching stress test: `bodies` rigid bodies whose particle
    counts are drawn uniform in [lo, hi] (cube, ball or rod lattices at
    `spacing`, chosen at random), each with a uniformly random orientation,
    one per site of a lattice of the given pitch in x and z with layers whose
    heights spread over [1, 20] m above a ground plane (bodies do not
    overlap at the start).  The bodies are built in bulk (one array per
    field) rather than body by body."""
    rng = np.random.default_rng(seed)
    s = Scene(name="shape_stress")
    d = float(np.float32(spacing))
    s.particle_radius = d / 2
    s.kernel_radius = 2 * d
    s.cell_size = 2 * d
    s.rest_density = 1000.0
    nx, ny, nz = lattice
    extent = max(nx, nz) * pitch
    # the largest table whose period fits inside the scene: the period is
    # shorter than the scene, so a table cell holds up to two real cells
    # (their particles fail the walks' distance test), and the dense offset
    # table is 8 times smaller than one covering the scene (GB300, 2,090,710
    # particles: 1150 M particle-substeps/s with D = 256 against 1072 M
    # with D = 512 and 919 M with D = 128)
    D = 16
    while 2 * D * s.cell_size <= extent:
        D *= 2
    s.grid_dim = D
    s.add_plane((0.0, 0.0, 0.0), (0.0, 1.0, 0.0))
    pos, rest, ranges, phases = [], [], [], []
    n0 = 0
    for b in range(bodies):
        ix, iy, iz = b % nx, (b // nx) % ny, b // (nx * ny)
        shape = rigid_shape(int(rng.integers(lo, hi + 1)), ("cube", "ball", "rod")[int(rng.integers(0, 3))], d)
        body_rest = shape @ _random_rotation(rng).T
        centre = np.array([(ix + 0.5) * pitch, 1.2 + (18.8 - 2.4) * (iy + rng.uniform(0.0, 0.2)) / max(ny - 1, 1),
                           (iz + 0.5) * pitch], np.float32)
        pos.append(body_rest + centre)
        rest.append(body_rest - body_rest.mean(axis=0, dtype=np.float64).astype(np.float32))
        ranges.append((n0, n0 + len(shape)))
        phases.append(np.full(len(shape), b + 1, np.int32))
        n0 += len(shape)
    s.positions = np.concatenate(pos).astype(np.float32)
    s.rigid_rest = np.concatenate(rest).astype(np.float32)
    s.masses = np.ones(n0, np.float32) * np.float32(1000.0 * d ** 3)
    s.phases = np.concatenate(phases)
    s.group_ids = np.zeros(n0, np.int32)
    s.rigid_ranges = np.asarray(ranges, np.int32)
    s.solid_phase_counter = bodies + 1
    s.velocities = np.zeros((n0, 3), np.float32)
    return s
