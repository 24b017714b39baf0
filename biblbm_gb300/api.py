"""Python mirror of the reference's interface for the coupled IB-LBM step.

Names follow the reference: a ``Lattice`` plays Palabos' ``MultiBlockLattice3D`` with
its ``CoProcessor3D`` offload (``addDomain / send / receive / collideAndStream``,
src/coProcessors/coProcessor3D.h:57-115); ``ParticleShapeLibrary.store_mesh`` is
src/fsi/ParticleShapeFactory.h:26; ``ImmersedBoundaryDynamics3D`` exposes
``add_particle / init / get_particle / compute_total_volume`` and the coupled step of
progs/capsule_in_shear/capsule_in_shear.cpp:187-227.  Every call goes through the C
ABI of ``include/bib/bib.h`` into the CUDA library; errors raise ``BibError``.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import BatchTuning, BibError, Growth, IbParams, LatticeParams, Potential, Tuning

STORAGE = {"f64": 0, "f32": 1, "f16": 2}
COLLISION = {"bgk_guo_vof": 0, "bgk": 1, "trt": 2}
WALL = {"none": 0, "fd_velocity": 1, "halfway_bb": 2}
DIRAC = {"roma": 0, "peskin": 1}
MODEL = {"capsule_neohookean": 0, "capsule_skalak": 1, "rbc_wlcpow": 2, "skalak_bending": 3}
LAYOUT = {"soa": 0, "palabos": 1, "coprocessor": 2}
SPREAD = {"atomic": 0, "deterministic": 1}
KERNEL = {"auto": 0, "rows": 1, "staged": 2}
PARAM_KEYS = ["G", "C", "nu_s", "kb", "shear_modulus", "L0", "k_area_global", "k_area_local",
              "k_volume", "vol_desired", "k_bend", "theta0"]
Q = 19


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


@dataclass
class CapsuleParameters:
    """CapsuleParameters of src/fsi/DeformableCapsule.h:22-31."""
    G: float = 0.0
    C: float = 1.0
    nu_s: float = 1.0
    kb: float = 0.0


@dataclass
class RBCParameters:
    """RBCParameters of src/fsi/RBCParticle.h:21-58 (the fields used by compute_forces)."""
    shear_modulus: float = 0.0
    L0: float = 1.0
    k_area_global: float = 0.0
    k_area_local: float = 0.0
    k_volume: float = 0.0
    vol_desired: float = 1.0
    k_bend: float = 0.0
    theta0: float = 0.0


def membrane_params(capsule: CapsuleParameters | None = None, rbc: RBCParameters | None = None, **kw) -> np.ndarray:
    """The 12-double parameter vector of the C ABI (BIB_P_*)."""
    v = dict(zip(PARAM_KEYS, [0.0, 1.0, 1.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0]))
    if capsule is not None:
        v.update(G=capsule.G, C=capsule.C, nu_s=capsule.nu_s, kb=capsule.kb)
    if rbc is not None:
        v.update(shear_modulus=rbc.shear_modulus, L0=rbc.L0, k_area_global=rbc.k_area_global,
                 k_area_local=rbc.k_area_local, k_volume=rbc.k_volume, vol_desired=rbc.vol_desired,
                 k_bend=rbc.k_bend, theta0=rbc.theta0)
    v.update(kw)
    return np.array([v[k] for k in PARAM_KEYS], dtype=np.float64)


class Context:
    """A CUDA context, stream and the device objects of one user (bib_create)."""

    def __init__(self, device: int = 0):
        self.lib = _lib.load()
        cfg = _lib.Config(device, 0)
        h = C.c_void_p()
        st = self.lib.bib_create(C.byref(cfg), C.byref(h))
        if st != 0:
            raise BibError(st, "bib_create failed (is a CUDA GPU visible?)")
        self.h = h

    def check(self, st):
        if st != 0:
            buf = C.create_string_buffer(1024)
            self.lib.bib_last_error(self.h, buf, 1024)
            raise BibError(st, buf.value.decode())
        return st

    def close(self):
        if getattr(self, "h", None):
            self.lib.bib_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sync(self):
        self.check(self.lib.bib_sync(self.h))

    def set_graph_mode(self, on: bool):
        self.check(self.lib.bib_set_graph_mode(self.h, int(bool(on))))

    def set_profiling(self, on: bool):
        self.check(self.lib.bib_set_profiling(self.h, int(bool(on))))

    def profile(self):
        out = np.zeros(5)
        self.check(self.lib.bib_profile_read(self.h, _d(out), 5))
        return dict(zip(["membrane", "spread", "collide_stream", "walls", "interpolate_update"], out))

    def add_domain(self, nx, ny, nz, **kw) -> "Lattice":
        return Lattice(self, nx, ny, nz, **kw)


def lattice_params(periodic=(1, 1, 1), collision="bgk_guo_vof", storage="f64", omega=1.0, omega_inner=None,
                   trt_magic=0.25, wall_y="none", wall_z="none", wall_u=None, body_force=(0, 0, 0), use_phase=False,
                   f16_scale=0.0) -> LatticeParams:
    """Lattice description of bib_lattice_add_domain.  storage: "f64" (the reference's arithmetic),
    "f32" or "f16" (FP32 collision; "f16" halves the population bytes and pays on lattices of
    millions of cells; below ~1 M cells "f32" is as fast and two orders more accurate)."""
    p = LatticeParams()
    for k in range(3):
        p.periodic[k] = int(bool(periodic[k]))
    p.collision = COLLISION[collision]
    p.storage = STORAGE[storage]
    p.wall_y, p.wall_z = WALL[wall_y], WALL[wall_z]
    p.use_phase = int(bool(use_phase))
    p.omega = float(omega)
    p.omega_inner = float(omega if omega_inner is None else omega_inner)
    p.trt_magic = float(trt_magic)
    wu = np.zeros((4, 3)) if wall_u is None else np.asarray(wall_u, dtype=np.float64).reshape(4, 3)
    for a in range(4):
        for b in range(3):
            p.wall_u[a][b] = float(wu[a, b])
    for a in range(3):
        p.body_force[a] = float(body_force[a])
    p.f16_scale = float(f16_scale)
    return p


class Lattice:
    """A D3Q19 lattice on the device (MultiBlockLattice3D + CoProcessor3D::addDomain)."""

    def __init__(self, ctx: Context, nx, ny, nz, **kw):
        self.ctx, self.nx, self.ny, self.nz = ctx, int(nx), int(ny), int(nz)
        self.n = self.nx * self.ny * self.nz
        self.params = lattice_params(**kw)
        h = C.c_int32()
        ctx.check(ctx.lib.bib_lattice_add_domain(ctx.h, self.nx, self.ny, self.nz, C.byref(self.params), C.byref(h)))
        self.h = h.value

    @property
    def shape(self):
        return (self.nz, self.ny, self.nx)

    # CoProcessor3D::send / receive
    def send(self, f, layout="soa"):
        f = _f64(f)
        self.ctx.check(self.ctx.lib.bib_lattice_send(self.ctx.h, self.h, f.ctypes.data, f.nbytes, LAYOUT[layout]))

    def receive(self, layout="soa"):
        if layout == "soa":
            out = np.empty((Q,) + self.shape)
        else:
            out = np.empty((self.nx, self.ny, self.nz, 23 if layout == "palabos" else Q))
        self.ctx.check(self.ctx.lib.bib_lattice_receive(self.ctx.h, self.h, out.ctypes.data, out.nbytes, LAYOUT[layout]))
        return out

    def collide_and_stream(self, nsteps=1):
        self.ctx.check(self.ctx.lib.bib_lattice_collide_and_stream(self.ctx.h, self.h, int(nsteps)))

    def initialize_at_equilibrium(self, rho, u):
        u = _f64(np.broadcast_to(u, (3,) + self.shape))
        r = None if rho is None else _f64(np.broadcast_to(rho, self.shape))
        self.ctx.check(self.ctx.lib.bib_lattice_init_equilibrium(self.ctx.h, self.h, _d(r) if r is not None else None,
                                                                 _d(u)))

    def set_external_force(self, F):
        F = _f64(np.broadcast_to(F, (3,) + self.shape))
        self.ctx.check(self.ctx.lib.bib_lattice_set_force(self.ctx.h, self.h, _d(F)))

    def get_external_force(self):
        F = np.empty((3,) + self.shape)
        self.ctx.check(self.ctx.lib.bib_lattice_get_force(self.ctx.h, self.h, _d(F)))
        return F

    def set_phase(self, phase):
        ph = _f64(np.broadcast_to(phase, self.shape))
        self.ctx.check(self.ctx.lib.bib_lattice_set_phase(self.ctx.h, self.h, _d(ph)))

    def get_phase(self):
        ph = np.empty(self.shape)
        self.ctx.check(self.ctx.lib.bib_lattice_get_phase(self.ctx.h, self.h, _d(ph)))
        return ph

    def compute_velocity(self):
        u = np.empty((3,) + self.shape)
        self.ctx.check(self.ctx.lib.bib_lattice_get_velocity(self.ctx.h, self.h, _d(u)))
        return u

    def check_health(self):
        self.ctx.check(self.ctx.lib.bib_check_health(self.ctx.h, self.h))

    def save_checkpoint(self, path):
        """Populations, forces, phase, cell types, particles and the iteration counter."""
        self.ctx.check(self.ctx.lib.bib_checkpoint_save(self.ctx.h, self.h, os.fsencode(path)))

    def load_checkpoint(self, path):
        self.ctx.check(self.ctx.lib.bib_checkpoint_load(self.ctx.h, self.h, os.fsencode(path)))

    def save_plb(self, name, folder=""):
        """parallelIO::save(lattice, name, false): Palabos' static-content checkpoint, XML spec
        <folder>/<name>.plb and raw cells <folder>/<name>.dat (io/multiBlockWriter3D.cpp:201-213)."""
        self.ctx.check(self.ctx.lib.bib_lattice_save_plb(self.ctx.h, self.h, os.fsencode(folder), os.fsencode(name)))

    def load_plb(self, name, folder=""):
        """parallelIO::load(name, lattice, false) of a checkpoint written by either library, of any
        block decomposition (io/multiBlockReader3D.cpp:214-268)."""
        self.ctx.check(self.ctx.lib.bib_lattice_load_plb(self.ctx.h, self.h, os.fsencode(folder), os.fsencode(name)))

    def iteration(self) -> int:
        it = C.c_int64()
        self.ctx.check(self.ctx.lib.bib_lattice_iteration(self.ctx.h, self.h, C.byref(it)))
        return it.value

    def set_cell_types(self, types):
        """defineDynamics per cell: 0 the lattice's dynamics, 1 BounceBack, 2 NoDynamics; None resets."""
        if types is None:
            self.ctx.check(self.ctx.lib.bib_lattice_set_cell_types(self.ctx.h, self.h, None))
            return
        t = np.ascontiguousarray(np.broadcast_to(types, self.shape), dtype=np.uint8)
        self.ctx.check(self.ctx.lib.bib_lattice_set_cell_types(self.ctx.h, self.h, t.ctypes.data))

    def set_pipe_walls(self, y0, z0, radius, second_order=False):
        """Walls of a pipe along x as rbc_in_pipe.cpp sets them: BounceBack outside (first order) or
        GuoRigidWallBoundary (second order), NoDynamics beyond radius + 1."""
        self.ctx.check(self.ctx.lib.bib_lattice_set_pipe_walls(self.ctx.h, self.h, float(y0), float(z0), float(radius),
                                                               int(bool(second_order))))

    def set_tuning(self, kernel="auto", tile_cells=0, stages=0, membrane_block=0, force_reset="auto",
                   wait_limit_us=0, withhold_tile=0):
        """Collide-and-stream kernel ("auto", "rows" or "staged"), staged tile size in cells,
        pipeline depth, membrane-kernel block size (0: automatic / default), the reset of the
        previous force field ("auto" = "dense", or "sparse" where the lattice allows it) and the
        bound of the staged kernel's hand-off waits in microseconds (0: 2 s)."""
        t = Tuning()
        t.collide_kernel = KERNEL[kernel]
        t.tile_cells = int(tile_cells)
        t.stages = int(stages)
        t.membrane_block = int(membrane_block)
        t.force_reset = {"auto": 0, "dense": 1, "sparse": 2}[force_reset]
        t.wait_limit_us = int(wait_limit_us)
        t.withhold_tile = int(withhold_tile)  # failure tests only: 1 + a staged tile left uncopied
        self.ctx.check(self.ctx.lib.bib_lattice_set_tuning(self.ctx.h, self.h, C.byref(t)))


class ParticleShapeLibrary:
    """ParticleShapeLibrary (src/fsi/ParticleShapeFactory.h:19-40): rest meshes by tag."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self.by_tag: dict[str, int] = {}
        self.meshes: dict[int, tuple] = {}

    def store_mesh(self, xyz, tri, tag: str) -> int:
        xyz = _f64(xyz)
        tri = np.ascontiguousarray(tri, dtype=np.int64)
        sid = C.c_int32()
        self.ctx.check(self.ctx.lib.bib_shape_store(self.ctx.h, _d(xyz), tri.ctypes.data_as(C.POINTER(C.c_int64)),
                                                    xyz.shape[0], tri.shape[0], C.byref(sid)))
        self.ctx.check(self.ctx.lib.bib_shape_set_tag(self.ctx.h, sid.value, str(tag).encode()))
        self.by_tag[tag] = sid.value
        self.meshes[sid.value] = (xyz, tri)
        return sid.value

    def get_by_tag(self, tag: str) -> int:
        return self.by_tag[tag]

    def info(self, shape: int) -> dict:
        out = np.zeros(6)
        self.ctx.check(self.ctx.lib.bib_shape_info(self.ctx.h, int(shape), _d(out)))
        return dict(area=out[0], volume=out[1], n_links=int(out[2]), n_pairs=int(out[3]), n_vertices=int(out[4]),
                    n_triangles=int(out[5]))


def initial_distribution(box, counts, radii, max_radius, seed, pipe=None, max_tries=5_000_000):
    """The random placement of progs/common/create_particles.h:37-93 (ParticlePositionInitializer
    and random orientations) with the numbers glibc's rand() gives after srand(seed): counts[t]
    non-overlapping spheres of radius radii[t] per type in the integer box (x0, x1, y0, y1, z0, z1),
    inside the pipe (y0, z0, radius) if given.  Returns (positions (n, 3), quaternions (n, 4) as w, x,
    y, z).  Host code of the CUDA library; no device needed."""
    lib = _lib.load()
    box = np.ascontiguousarray(box, dtype=np.int64)
    counts = np.ascontiguousarray(counts, dtype=np.int64)
    radii = _f64(radii)
    n = int(counts.sum())
    pos, quat = np.zeros((n, 3)), np.zeros((n, 4))
    pp = None if pipe is None else _f64(pipe)
    st = lib.bib_initial_distribution(box.ctypes.data_as(C.POINTER(C.c_int64)), _d(pp) if pp is not None else None,
                                      int(counts.shape[0]), counts.ctypes.data_as(C.POINTER(C.c_int64)), _d(radii),
                                      float(max_radius), int(seed), int(max_tries), _d(pos), _d(quat))
    if st != 0:
        raise BibError(st, "initial_distribution: " + _lib.status_string(st))
    return pos, quat


class RBCShapeInitializer:
    """RBCShapeInitializer (progs/common/calibrate_rbc_shape.h:147-198): an RBC on a stored shape,
    its parameters (create_rbc_params), the volume shrink to the discocyte (shrink_rbc_volume, on
    the GPU) with the minor axis turned onto z, and the result stored as a new shape."""

    def __init__(self, shapes: ParticleShapeLibrary, tag: str):
        self.shapes = shapes
        self.ctx = shapes.ctx
        self.shape = shapes.get_by_tag(tag)
        xyz, tri = shapes.meshes[self.shape]
        self.pos = np.array(xyz, dtype=np.float64)
        self.tri = tri
        self.params = np.zeros(12)
        self.damping = None

    def compute_rbc_parameters(self, shear_modulus, k_area, k_bend):
        self.ctx.check(self.ctx.lib.bib_rbc_params(self.ctx.h, self.shape, float(shear_modulus), float(k_area),
                                                   float(k_bend), _d(self.params)))
        return self.params

    def shrink_volume(self, vol_frac, n_it, damping=1.e-2):
        """shrink_rbc_volume to vol_frac of the shape's volume, then the minor axis onto z and
        vol_desired = the shrunk volume."""
        vol0 = self.shapes.info(self.shape)["volume"]
        out = np.empty_like(self.pos)
        used = C.c_double()
        self.ctx.check(self.ctx.lib.bib_rbc_shrink_volume(self.ctx.h, self.shape, _d(self.params),
                                                          float(vol_frac) * vol0, int(n_it), float(damping), _d(out),
                                                          C.byref(used)))
        z = np.array([0.0, 0.0, 1.0])
        self.ctx.check(self.ctx.lib.bib_align_minor_axis(self.ctx.h, self.shape, _d(out), _d(z)))
        self.pos = out
        self.damping = used.value
        # the volume of the relaxed shape, as DeformableParticle3D::update computes it
        self.params[PARAM_KEYS.index("vol_desired")] = _volume(out, self.tri)
        return out

    def store_shape(self, tag: str) -> int:
        """ParticleBase3D::store_shape (ParticleBase.hh:197-212): the current vertices as a new shape."""
        return self.shapes.store_mesh(self.pos, self.tri, tag)


def _volume(pos, tri) -> float:
    """Signed volume of a closed triangulation, sum over triangles of v0 . (v1 x v2) / 6 in order."""
    v = 0.0
    for t in np.asarray(tri):
        a, b, c = pos[t[0]], pos[t[1]], pos[t[2]]
        cx = b[1] * c[2] - b[2] * c[1]
        cy = b[2] * c[0] - b[0] * c[2]
        cz = b[0] * c[1] - b[1] * c[0]
        v += (a[0] * cx + a[1] * cy + a[2] * cz) / 6.
    return v


def MorsePotential(r_min, beta, strength, grid=False) -> Potential:
    """fsi/Potentials.h MorsePotential: 2 beta strength x (x - 1), x = exp(beta (r_min - d)), d <= r_min.
    grid: as a particle-particle force, searched with the reference's collision grid
    (CollisionForces.h) instead of every pair within the cutoff."""
    return Potential(1, 1 if grid else 0, float(r_min), float(beta), float(strength))


def SpringPotential(min_dist, strength, grid=False) -> Potential:
    """fsi/Potentials.h SpringPotential: (min_dist - d) strength, d <= min_dist (grid: see MorsePotential)."""
    return Potential(2, 1 if grid else 0, float(min_dist), 0.0, float(strength))


def _shape_nv(ctx: "Context", shape: int) -> int:
    out = np.zeros(6)
    ctx.check(ctx.lib.bib_shape_info(ctx.h, int(shape), _d(out)))
    return int(out[4])


def grow_particles(ctx: "Context", shapes, com, quat, box, wall=None, periodic=(1, 0, 0), min_dist=1.0,
                   strength=5e-2, initial_scale=0.2, density=1.0, damping=0.1, n_it=40000, rescale_every=10,
                   it_end=None, vertices=False):
    """The growth stage of create_particles (progs/common/create_particles.h:105-161) on the GPU:
    rigid copies of the stored shapes `shapes[k]` at com[k] / quat[k] (w, x, y, z) grow from
    initial_scale to 1 over n_it iterations under spring collision forces (the reference's
    collision grid) and a pipe wall (y0, z0, radius).  Returns (com, quat), plus the vertex positions
    and the last collision forces when `vertices`."""
    sh = np.ascontiguousarray(shapes, dtype=np.int32)
    com, quat = _f64(com).copy(), _f64(quat).copy()
    g = Growth()
    for k in range(6):
        g.box[k] = int(box[k])
    for a in range(3):
        g.periodic[a] = int(periodic[a])
    g.has_wall = 0 if wall is None else 1
    if wall is not None:
        for k in range(3):
            g.wall[k] = float(wall[k])
    g.min_dist, g.strength = float(min_dist), float(strength)
    g.initial_scale, g.density, g.damping = float(initial_scale), float(density), float(damping)
    g.n_it, g.rescale_every = int(n_it), int(rescale_every)
    g.it_end = int(n_it + 1 if it_end is None else it_end)
    nvert = sum(_shape_nv(ctx, int(s)) for s in sh) if vertices else 0
    pos = np.zeros((nvert, 3)) if vertices else None
    frc = np.zeros((nvert, 3)) if vertices else None
    ctx.check(ctx.lib.bib_grow_particles(ctx.h, C.byref(g), len(sh), sh.ctypes.data_as(C.POINTER(C.c_int32)),
                                         _d(com), _d(quat), _d(pos) if vertices else None,
                                         _d(frc) if vertices else None))
    return (com, quat, pos, frc) if vertices else (com, quat)


def place_particle(ctx: "Context", shape: int, com, quat, xyz=None) -> np.ndarray:
    """create_particles' final placement (:193-199): the vertices (default: the shape's rest
    vertices) moved by translate(-centre of mass), rotate(quat), translate(com)."""
    n = _shape_nv(ctx, int(shape))
    v = None if xyz is None else _f64(xyz)
    out = np.zeros((n, 3))
    ctx.check(ctx.lib.bib_place_particle(ctx.h, int(shape), _d(v) if v is not None else None, _d(_f64(com)),
                                         _d(_f64(quat)), _d(out)))
    return out


def create_particles(shapes: ParticleShapeLibrary, types, box, pipe, seed, periodic=(1, 0, 0), n_it=40000,
                     initial_scale=0.2):
    """create_particles (progs/common/create_particles.h:9-212) for particle templates on stored
    shapes: types = [(shape, count), ...], pipe = (y0, z0, radius), srand(seed).  Places the
    particles at initial_scale inside the pipe shrunk by 1.5 (bib_initial_distribution), grows
    rigid copies to full size on the GPU and returns [(shape, vertex positions), ...] of the
    particles at the result, in order, for ImmersedBoundaryDynamics3D.add_particle."""
    ctx = shapes.ctx
    sids = [int(s) for s, _ in types]
    counts = [int(n) for _, n in types]
    radii = []
    for s in sids:
        xyz = shapes.meshes[s][0]
        r = 0.0
        for v in xyz:  # ParticleShape::compute_bounding_volumes (ParticleShape.hh:361-383)
            d = v[0] * v[0] + v[1] * v[1] + v[2] * v[2]
            r = d if d > r else r
        radii.append(initial_scale * float(np.sqrt(r)) + 1.)
    wall = (float(pipe[0]), float(pipe[1]), float(pipe[2]) - 1.5)
    com, quat = initial_distribution(box, counts, radii, max(radii), seed, pipe=wall)
    shape_of = np.repeat(np.array(sids, dtype=np.int32), counts)
    com, quat = grow_particles(ctx, shape_of, com, quat, box, wall=wall, periodic=periodic, n_it=n_it,
                               initial_scale=initial_scale)
    return [(int(s), place_particle(ctx, int(s), com[k], quat[k])) for k, s in enumerate(shape_of)]


class ImmersedBoundaryDynamics3D:
    """The IB module of src/fsi/ImmersedBoundaryDynamics.h:50-217 on one lattice."""

    def __init__(self, lattice: Lattice, shapes: ParticleShapeLibrary, dirac="roma", field_offset=-1.0,
                 spread="atomic"):
        self.lattice, self.shapes, self.ctx = lattice, shapes, lattice.ctx
        p = IbParams(DIRAC[dirac], SPREAD[spread], float(field_offset))
        self.ctx.check(self.ctx.lib.bib_ib_configure(self.ctx.h, lattice.h, C.byref(p)))
        self.nv: list[int] = []

    def add_particle(self, shape: int, model: str, params, positions=None) -> int:
        prm = _f64(params)
        pos = None if positions is None else _f64(positions)
        pid = C.c_int32()
        self.ctx.check(self.ctx.lib.bib_particle_add(self.ctx.h, self.lattice.h, int(shape), MODEL[model], _d(prm),
                                                     _d(pos) if pos is not None else None, C.byref(pid)))
        self.nv.append(self.shapes.info(shape)["n_vertices"])
        return pid.value

    def set_boundary(self, y0, z0, radius):
        """set_boundary(PipeBoundary): near-wall TopHat blending and wall reflection for a pipe
        along x through (y0, z0); radius <= 0 removes it."""
        self.ctx.check(self.ctx.lib.bib_ib_set_pipe_boundary(self.ctx.h, self.lattice.h, float(y0), float(z0),
                                                             float(radius)))

    def add_wall_interaction(self, potential: Potential, axis: int, lo: float, hi: float):
        """add_force_decorator(WallInteraction(ParallelPlatesBoundary(lo, hi), potential)); the
        plates are normal to `axis` (1 = y as in the reference, 2 = z)."""
        self.ctx.check(self.ctx.lib.bib_add_wall_interaction(self.ctx.h, self.lattice.h, int(axis), float(lo),
                                                             float(hi), C.byref(potential)))

    def add_pipe_wall_interaction(self, potential: Potential, y0: float, z0: float, radius: float):
        """add_force_decorator(WallInteraction(PipeBoundary(y0, z0, radius), potential)) for a pipe
        along x (rbc_in_pipe.cpp:154-163)."""
        self.ctx.check(self.ctx.lib.bib_add_pipe_wall_interaction(self.ctx.h, self.lattice.h, float(y0), float(z0),
                                                                  float(radius), C.byref(potential)))

    def add_pp_force(self, potential: Potential):
        """add_pp_force(PPPotentialForce(potential)): repulsion between vertices of different particles."""
        self.ctx.check(self.ctx.lib.bib_add_pp_interaction(self.ctx.h, self.lattice.h, C.byref(potential)))

    def clear_interactions(self):
        self.ctx.check(self.ctx.lib.bib_clear_interactions(self.ctx.h, self.lattice.h))

    def init(self):
        """ImmersedBoundaryDynamics3D::init: upload the particles and voxelize them into the
        phase field (the first step does this by itself)."""
        self.ctx.check(self.ctx.lib.bib_ibm_init(self.ctx.h, self.lattice.h))

    def save_checkpoint(self, path):
        """Lattice, particles and iteration counter in one file (bib_checkpoint_save)."""
        self.ctx.check(self.ctx.lib.bib_checkpoint_save(self.ctx.h, self.lattice.h, os.fsencode(path)))

    def load_checkpoint(self, path):
        """Restore a checkpoint into this lattice; its particles replace the current ones.  The
        shapes must be stored in the same order as in the run that saved it."""
        self.ctx.check(self.ctx.lib.bib_checkpoint_load(self.ctx.h, self.lattice.h, os.fsencode(path)))
        self._refresh_particles()

    def save_particle_checkpoint(self, name, folder=""):
        """The reference's save_checkpoint (ImmersedBoundaryDynamics_io.hh:17-73): the particles in
        its .plb format, header <folder>/<name>.plb and data <folder>/<name>/0.plb."""
        self.ctx.check(self.ctx.lib.bib_particles_save_plb(self.ctx.h, self.lattice.h, os.fsencode(folder),
                                                           os.fsencode(name)))

    def load_particle_checkpoint(self, name, folder=""):
        """The reference's load_checkpoint (ImmersedBoundaryDynamics_io.hh:75-159) of a .plb particle
        checkpoint, written by either library; the particles replace the current ones."""
        self.ctx.check(self.ctx.lib.bib_particles_load_plb(self.ctx.h, self.lattice.h, os.fsencode(folder),
                                                           os.fsencode(name)))
        self._refresh_particles()

    def write_particles_as_vtk(self, iteration, folder=""):
        """One <folder>/obj<id>-<iteration>.vtu per particle (ImmersedBoundaryDynamics_io.hh:161-176)."""
        self.ctx.check(self.ctx.lib.bib_particles_write_vtu(self.ctx.h, self.lattice.h, os.fsencode(folder),
                                                            int(iteration)))

    def write_particle_vtk(self, pid, path):
        """ParticleBase3D::write_vtk of one particle (ParticleBase.hh:270-390)."""
        self.ctx.check(self.ctx.lib.bib_particle_write_vtu(self.ctx.h, self.lattice.h, int(pid), os.fsencode(path)))

    def write_lightweight_particle_data(self, iteration, folder=""):
        """<folder>/objsP0-<iteration>.txt: centre, gyration tensor and volume per particle
        (ImmersedBoundaryDynamics_io.hh:178-199)."""
        self.ctx.check(self.ctx.lib.bib_particles_write_lightweight(self.ctx.h, self.lattice.h, os.fsencode(folder),
                                                                    int(iteration)))

    def _refresh_particles(self):
        n = C.c_int32()
        self.ctx.check(self.ctx.lib.bib_particle_count(self.ctx.h, self.lattice.h, C.byref(n)))
        info = np.zeros(3, dtype=np.int32)
        self.nv = []
        for pid in range(n.value):
            self.ctx.check(self.ctx.lib.bib_particle_info(self.ctx.h, self.lattice.h, pid,
                                                          info.ctypes.data_as(C.POINTER(C.c_int32))))
            self.nv.append(int(info[2]))

    def iteration(self) -> int:
        return self.lattice.iteration()

    def count_particles(self) -> int:
        return len(self.nv)

    def get_particle(self, pid: int) -> dict:
        nv = self.nv[pid]
        pos, vel, frc = np.empty((nv, 3)), np.empty((nv, 3)), np.empty((nv, 3))
        self.ctx.check(self.ctx.lib.bib_particle_get(self.ctx.h, self.lattice.h, pid, _d(pos), _d(vel), _d(frc)))
        st = np.empty(14)
        self.ctx.check(self.ctx.lib.bib_particle_stats(self.ctx.h, self.lattice.h, pid, _d(st)))
        return dict(pos=pos, vel=vel, force=frc, area=st[0], volume=st[1], com=st[2:5], inertia=st[5:14].reshape(3, 3))

    def set_positions(self, pid: int, pos):
        pos = _f64(pos)
        self.ctx.check(self.ctx.lib.bib_particle_set_positions(self.ctx.h, self.lattice.h, pid, _d(pos)))

    def download(self):
        nvt = C.c_int64()
        self.ctx.check(self.ctx.lib.bib_total_vertices(self.ctx.h, self.lattice.h, C.byref(nvt)))
        pos = np.empty((nvt.value, 3))
        stats = np.empty((len(self.nv), 5))
        self.ctx.check(self.ctx.lib.bib_particles_download(self.ctx.h, self.lattice.h, _d(pos), _d(stats)))
        return pos, stats

    def download_async(self, stats, slot, pos=None):
        """Queue the copy of the per-particle area / volume / centre (and optionally all vertex
        positions) behind the steps issued so far; the arrays (C-contiguous float64, pinned for the
        copy to overlap) hold the values once ``wait_download(slot)`` returns."""
        for a in (stats, pos):
            if a is not None and (a.dtype != np.float64 or not a.flags.c_contiguous):
                raise ValueError("download buffers must be C-contiguous float64 arrays")
        self.ctx.check(self.ctx.lib.bib_particles_download_async(self.ctx.h, self.lattice.h,
                                                                 _d(pos) if pos is not None else None,
                                                                 _d(stats) if stats is not None else None, int(slot)))

    def wait_download(self, slot):
        self.ctx.check(self.ctx.lib.bib_download_wait(self.ctx.h, int(slot)))

    def upload_positions(self, pos):
        """All vertex positions (particles in order) into the live device state, no rebuild."""
        pos = _f64(pos)
        self.ctx.check(self.ctx.lib.bib_particles_upload(self.ctx.h, self.lattice.h, _d(pos)))

    def compute_total_volume(self) -> float:
        v = C.c_double()
        self.ctx.check(self.ctx.lib.bib_total_volume(self.ctx.h, self.lattice.h, C.byref(v)))
        return v.value

    def ibm_step(self):
        self.ctx.check(self.ctx.lib.bib_ibm_step(self.ctx.h, self.lattice.h))

    def step(self, nsteps=1):
        """Coupled steps: computeVelocity, setExternalVector, IB step, collideAndStream."""
        self.ctx.check(self.ctx.lib.bib_step(self.ctx.h, self.lattice.h, int(nsteps)))

    def step_timed(self, nsteps=1) -> float:
        """Coupled steps timed with CUDA events on the library's stream; returns milliseconds."""
        ms = C.c_double()
        self.ctx.check(self.ctx.lib.bib_step_timed(self.ctx.h, self.lattice.h, int(nsteps), C.byref(ms)))
        return ms.value

    def kernels_per_step(self) -> int:
        """Kernel launches of one coupled step, counted in the step's captured CUDA graph."""
        n = C.c_int32()
        self.ctx.check(self.ctx.lib.bib_step_kernel_count(self.ctx.h, self.lattice.h, C.byref(n)))
        return n.value


def moments_of_inertia(pos, tri) -> np.ndarray:
    """Moment-of-inertia tensors of closed meshes, vectorised over particles.

    ``pos`` is (n_particles, n_vertices, 3), ``tri`` (n_triangles, 3); the integrals are
    those of DeformableParticle3D::compute_moment_of_intertia (DeformableParticle3D.hh:173-272).
    Host-side post-processing of downloaded vertex positions.
    """
    pos = np.asarray(pos, dtype=np.float64)
    tri = np.asarray(tri)
    v0, v1, v2 = pos[:, tri[:, 0]], pos[:, tri[:, 1]], pos[:, tri[:, 2]]
    N = np.cross(v1 - v0, v2 - v0)
    tmp0 = v0 + v1
    f1 = tmp0 + v2
    tmp1 = v0 * v0
    tmp2 = tmp1 + v1 * tmp0
    f2 = tmp2 + v2 * f1
    f3 = v0 * tmp1 + v1 * tmp2 + v2 * f2
    g0 = f2 + v0 * (f1 + v0)
    g1 = f2 + v1 * (f1 + v1)
    g2 = f2 + v2 * (f1 + v2)
    i0 = (N[..., 0] * f1[..., 0]).sum(-1) / 6.0
    i1 = (N[..., 0] * f2[..., 0]).sum(-1) / 24.0
    i2 = (N[..., 1] * f2[..., 1]).sum(-1) / 24.0
    i3 = (N[..., 2] * f2[..., 2]).sum(-1) / 24.0
    i4 = (N[..., 0] * f3[..., 0]).sum(-1) / 60.0
    i5 = (N[..., 1] * f3[..., 1]).sum(-1) / 60.0
    i6 = (N[..., 2] * f3[..., 2]).sum(-1) / 60.0
    i7 = (N[..., 0] * (v0[..., 1] * g0[..., 0] + v1[..., 1] * g1[..., 0] + v2[..., 1] * g2[..., 0])).sum(-1) / 120.0
    i8 = (N[..., 1] * (v0[..., 2] * g0[..., 1] + v1[..., 2] * g1[..., 1] + v2[..., 2] * g2[..., 1])).sum(-1) / 120.0
    i9 = (N[..., 2] * (v0[..., 0] * g0[..., 2] + v1[..., 0] * g1[..., 2] + v2[..., 0] * g2[..., 2])).sum(-1) / 120.0
    vol = i0
    c = np.stack([i1 / vol, i2 / vol, i3 / vol], -1)
    I = np.empty(pos.shape[:1] + (3, 3))
    I[:, 0, 0] = i5 + i6 - vol * (c[:, 1] ** 2 + c[:, 2] ** 2)
    I[:, 0, 1] = I[:, 1, 0] = -i7 + vol * c[:, 0] * c[:, 1]
    I[:, 0, 2] = I[:, 2, 0] = -i9 + vol * c[:, 2] * c[:, 0]
    I[:, 1, 1] = i4 + i6 - vol * (c[:, 2] ** 2 + c[:, 0] ** 2)
    I[:, 1, 2] = I[:, 2, 1] = -i8 + vol * c[:, 1] * c[:, 2]
    I[:, 2, 2] = i4 + i5 - vol * (c[:, 0] ** 2 + c[:, 1] ** 2)
    return I


def taylor_deformation(inertia) -> float:
    """Taylor index D = (L - B)/(L + B) of the ellipsoid with the same moment of inertia.

    For an ellipsoid with semi-axes a, b, c the principal moments are
    I1 = V(b^2+c^2)/5, ...; so a^2 ∝ (I2 + I3 - I1).  L and B are the largest and
    smallest semi-axes.  Applied identically to the oracle's and the GPU's inertia.
    """
    w = np.linalg.eigvalsh(0.5 * (np.asarray(inertia) + np.asarray(inertia).T))
    s = w.sum()
    ax2 = np.clip(np.array([s - 2 * w[0], s - 2 * w[1], s - 2 * w[2]]), 0, None)
    ax = np.sqrt(ax2)
    L, B = ax.max(), ax.min()
    return float((L - B) / (L + B))


class Batch:
    """Lattices (each with its ImmersedBoundaryDynamics3D) stepped in lockstep: one launch per kernel
    for all of them, replayed as CUDA graphs.  A batch step is a coupled step of every lattice."""

    def __init__(self, ctx: Context, lattices):
        self.ctx = ctx
        self.lattices = list(lattices)
        hs = (C.c_int32 * len(self.lattices))(*[lat.h for lat in self.lattices])
        b = C.c_int32()
        ctx.check(ctx.lib.bib_batch_create(ctx.h, hs, len(self.lattices), C.byref(b)))
        self.h = b.value

    def step(self, nsteps=1):
        self.ctx.check(self.ctx.lib.bib_batch_step(self.ctx.h, self.h, int(nsteps)))

    def step_timed(self, nsteps=1) -> float:
        ms = C.c_double()
        self.ctx.check(self.ctx.lib.bib_batch_step_timed(self.ctx.h, self.h, int(nsteps), C.byref(ms)))
        return ms.value

    def set_tuning(self, tile_cells=0, stages=0, membrane_block=0):
        t = BatchTuning()
        t.tile_cells, t.stages, t.membrane_block = int(tile_cells), int(stages), int(membrane_block)
        self.ctx.check(self.ctx.lib.bib_batch_set_tuning(self.ctx.h, self.h, C.byref(t)))

    def autotune(self, steps=5) -> dict:
        """Times the candidate schedules over `steps` real steps each (the batch advances) and
        keeps the fastest; returns it."""
        t = BatchTuning()
        self.ctx.check(self.ctx.lib.bib_batch_autotune(self.ctx.h, self.h, int(steps), C.byref(t)))
        return {"tile_cells": t.tile_cells, "stages": t.stages, "membrane_block": t.membrane_block}

    def close(self):
        if self.h is not None:
            self.ctx.check(self.ctx.lib.bib_batch_destroy(self.ctx.h, self.h))
            self.h = None
