"""ctypes front end of the CPU oracle (``oracle/_ref/libbib_oracle.so``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()`` and
the CPU-baseline legs of ``bench.py``, never by the product package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libbib_oracle.so")

COLLISION = {"bgk_guo_vof": 0, "bgk": 1, "trt": 2}
WALL = {"none": 0, "fd_velocity": 1, "halfway_bb": 2}
DIRAC = {"roma": 0, "peskin": 1}
MODEL = {"capsule_neohookean": 0, "capsule_skalak": 1, "rbc_wlcpow": 2, "skalak_bending": 3}
POTENTIAL = {"none": 0, "morse": 1, "spring": 2}
PARAM_KEYS = ["G", "C", "nu_s", "kb", "shear_modulus", "L0", "k_area_global", "k_area_local",
              "k_volume", "vol_desired", "k_bend", "theta0"]


class GuoNode(C.Structure):
    _fields_ = [("x", C.c_int64), ("y", C.c_int64), ("z", C.c_int64), ("dir", C.c_int32), ("nodyn", C.c_int32),
                ("delta", C.c_double), ("u", C.c_double * 3)]


class Lattice(C.Structure):
    _fields_ = [
        ("nx", C.c_int64), ("ny", C.c_int64), ("nz", C.c_int64),
        ("periodic", C.c_int32 * 3),
        ("collision", C.c_int32),
        ("wall_y", C.c_int32), ("wall_z", C.c_int32),
        ("omega", C.c_double), ("omega_inner", C.c_double), ("trt_magic", C.c_double),
        ("wall_u", (C.c_double * 3) * 4),
        ("envelope_swap", C.c_int32),
        ("celltype", C.c_void_p),
        ("guo", C.c_void_p),
        ("nguo", C.c_int64),
    ]


class Potential(C.Structure):
    _fields_ = [("kind", C.c_int32), ("r0", C.c_double), ("beta", C.c_double), ("strength", C.c_double)]


class Growth(C.Structure):
    _fields_ = [
        ("box", C.c_int64 * 6), ("periodic", C.c_int32 * 3), ("has_wall", C.c_int32), ("wall", C.c_double * 3),
        ("min_dist", C.c_double), ("strength", C.c_double),
        ("initial_scale", C.c_double), ("density", C.c_double), ("damping", C.c_double),
        ("n_it", C.c_int64), ("rescale_every", C.c_int64), ("it_end", C.c_int64),
    ]


def potential(kind, r0, beta=0.0, strength=0.0) -> Potential:
    """MorsePotential(r_min = r0, beta, strength) or SpringPotential(min_dist = r0, strength)."""
    return Potential(POTENTIAL[kind] if isinstance(kind, str) else int(kind), float(r0), float(beta), float(strength))


def build():
    """Compile the oracle library in place (plain C, seconds)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, "bib_oracle.c")):
            build()
        L = C.CDLL(LIB_PATH)
        dp, ip, i32p = C.POINTER(C.c_double), C.POINTER(C.c_int64), C.POINTER(C.c_int32)
        Lp = C.POINTER(Lattice)
        sig = {
            "orc_collide_cell": (None, [Lp, dp, dp, C.c_double]),
            "orc_collide_stream": (None, [Lp, dp, dp, dp, dp]),
            "orc_apply_fd_walls": (None, [Lp, dp, dp]),
            "orc_compute_velocity": (None, [Lp, dp, dp, dp]),
            "orc_init_equilibrium": (None, [Lp, dp, dp, dp]),
            "orc_shape_connectivity": (C.c_int64, [C.c_int64, dp, C.c_int64, ip, ip, dp, ip, dp, dp, dp, ip]),
            "orc_particle_update": (None, [C.c_int64, dp, C.c_int64, ip, dp]),
            "orc_inertia": (None, [dp, C.c_int64, ip, dp]),
            "orc_membrane_forces": (None, [C.c_int32, dp, C.c_int64, dp, C.c_int64, ip, dp, C.c_double, C.c_int64, ip,
                                           dp, C.c_int64, ip, dp, dp, C.c_double, C.c_double, dp]),
            "orc_rbc_shrink_volume": (C.c_double, [dp, C.c_int64, dp, C.c_int64, ip, dp, C.c_double, C.c_double,
                                                   C.c_int64, ip, dp, C.c_int64, ip, dp, C.c_double, C.c_int64,
                                                   C.c_double, dp, dp]),
            "orc_dirac": (C.c_double, [C.c_int32, C.c_double]),
            "orc_threads": (C.c_int32, []),
            "orc_classify": (None, [Lp, C.c_int32, C.c_int64, dp, i32p]),
            "orc_interpolate": (None, [Lp, C.c_int32, C.c_double, dp, C.c_int64, dp, i32p, dp]),
            "orc_spread": (None, [Lp, C.c_int32, C.c_double, C.c_int64, dp, dp, i32p, dp]),
            "orc_sys_create": (C.c_void_p, [Lp, C.c_int32, C.c_double]),
            "orc_sys_destroy": (None, [C.c_void_p]),
            "orc_sys_f": (dp, [C.c_void_p]),
            "orc_sys_force": (dp, [C.c_void_p]),
            "orc_sys_phase": (dp, [C.c_void_p]),
            "orc_sys_set_body_force": (None, [C.c_void_p, dp]),
            "orc_sys_add_shape": (C.c_int32, [C.c_void_p, C.c_int64, dp, C.c_int64, ip]),
            "orc_sys_add_particle": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, dp, dp]),
            "orc_sys_init": (None, [C.c_void_p]),
            "orc_sys_set_voxelize": (None, [C.c_void_p, C.c_int32]),
            "orc_voxelize": (None, [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
            "orc_sys_step": (None, [C.c_void_p, C.c_int64]),
            "orc_sys_lattice_only_step": (None, [C.c_void_p, C.c_int64]),
            "orc_sys_get_particle": (None, [C.c_void_p, C.c_int32, dp, dp, dp, dp]),
            "orc_pipe_celltypes": (None, [C.c_int64, C.c_int64, C.c_int64, C.c_double, C.c_double, C.c_double,
                                          C.c_void_p]),
            "orc_pipe_guo_nodes": (C.c_int64, [C.c_int64, C.c_int64, C.c_int64, C.c_double, C.c_double, C.c_double,
                                               C.c_void_p, C.c_void_p]),
            "orc_apply_guo": (None, [Lp, dp]),
            "orc_sys_set_pipe": (None, [C.c_void_p, C.c_double, C.c_double, C.c_double]),
            "orc_move_vertices": (None, [C.c_int64, dp, dp, C.c_void_p]),
            "orc_potential_eval": (C.c_double, [C.POINTER(Potential), C.c_double]),
            "orc_wall_forces": (None, [C.POINTER(Potential), C.c_int32, C.c_double, C.c_double, C.c_int64, dp, dp]),
            "orc_pp_forces_grid": (None, [Lp, C.POINTER(Potential), C.c_int64, dp, i32p, dp]),
            "orc_pp_forces": (None, [Lp, C.POINTER(Potential), C.c_int64, dp, i32p, dp]),
            "orc_sys_add_wall_interaction": (C.c_int32, [C.c_void_p, C.POINTER(Potential), C.c_int32, C.c_double,
                                                         C.c_double]),
            "orc_sys_add_pp_interaction": (C.c_int32, [C.c_void_p, C.POINTER(Potential), C.c_int32]),
            "orc_sys_add_pipe_wall_interaction": (C.c_int32, [C.c_void_p, C.POINTER(Potential), C.c_double,
                                                              C.c_double, C.c_double]),
            "orc_sys_velocity": (None, [C.c_void_p, dp]),
            "orc_shape_mass_props": (None, [C.c_int64, ip, dp, dp, dp]),
            "orc_grow_particles": (C.c_int32, [C.POINTER(Growth), C.c_int32, ip, dp, ip, ip, C.c_int32, i32p, dp, dp,
                                               dp, dp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _i(a):
    return a.ctypes.data_as(C.POINTER(C.c_int64))


def _i32(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def i64(a):
    return np.ascontiguousarray(a, dtype=np.int64)


_celltypes_alive = []  # the oracle keeps a pointer to the cell-type array of a lattice


def lattice(dims, periodic=(1, 1, 1), collision="bgk_guo_vof", omega=1.0, omega_inner=None, trt_magic=0.25,
            wall_y="none", wall_z="none", wall_u=None, envelope_swap=False, celltype=None) -> Lattice:
    """celltype: None or a (nz, ny, nx) array, 0 the lattice's dynamics, 1 BounceBack, 2 NoDynamics."""
    L = Lattice()
    if celltype is not None:
        ct = np.ascontiguousarray(celltype, dtype=np.uint8)
        _celltypes_alive.append(ct)
        L.celltype = ct.ctypes.data
    L.nx, L.ny, L.nz = (int(d) for d in dims)
    for k in range(3):
        L.periodic[k] = int(bool(periodic[k]))
    L.collision = COLLISION[collision]
    L.wall_y, L.wall_z = WALL[wall_y], WALL[wall_z]
    L.omega = float(omega)
    L.omega_inner = float(omega if omega_inner is None else omega_inner)
    L.trt_magic = float(trt_magic)
    L.envelope_swap = int(bool(envelope_swap))
    wu = np.zeros((4, 3)) if wall_u is None else np.asarray(wall_u, dtype=np.float64).reshape(4, 3)
    for a in range(4):
        for b in range(3):
            L.wall_u[a][b] = float(wu[a, b])
    return L


def params_vector(**kw) -> np.ndarray:
    p = dict(G=0.0, C=1.0, nu_s=1.0, kb=0.0, shear_modulus=0.0, L0=1.0, k_area_global=0.0, k_area_local=0.0,
             k_volume=0.0, vol_desired=1.0, k_bend=0.0, theta0=0.0)
    p.update(kw)
    return np.array([p[k] for k in PARAM_KEYS], dtype=np.float64)


def threads() -> int:
    return int(lib().orc_threads())


# ------------------------------------------------------------------ lattice ops
def collide_stream(L, f, F=None, phase=None, steps=1):
    f = f64(f).copy()
    tmp = np.empty_like(f)
    Fa = f64(F) if F is not None else None
    ph = f64(phase) if phase is not None else None
    for _ in range(steps):
        lib().orc_collide_stream(C.byref(L), _d(f), _d(tmp), _d(Fa) if Fa is not None else None,
                                 _d(ph) if ph is not None else None)
    return f


def apply_fd_walls(L, f, F):
    f = f64(f).copy()
    lib().orc_apply_fd_walls(C.byref(L), _d(f), _d(f64(F)))
    return f


def compute_velocity(L, f, F=None):
    f = f64(f)
    u = np.empty((3,) + f.shape[1:])
    lib().orc_compute_velocity(C.byref(L), _d(f), _d(f64(F)) if F is not None else None, _d(u))
    return u


def init_equilibrium(L, rho, u):
    u = f64(u)
    f = np.empty((19,) + u.shape[1:])
    lib().orc_init_equilibrium(C.byref(L), _d(f), _d(f64(rho)) if rho is not None else None, _d(u))
    return f


# ------------------------------------------------------------------ shapes / membranes
class Shape:
    def __init__(self, xyz, tri):
        self.rest = f64(xyz)
        self.tri = i64(tri)
        nt = self.tri.shape[0]
        links = np.zeros((3 * nt, 2), np.int64)
        llen = np.zeros(3 * nt)
        pairs = np.zeros((3 * nt, 4), np.int64)
        pcs = np.zeros((3 * nt, 2))
        tarea = np.zeros(nt)
        props = np.zeros(5)
        npairs = np.zeros(1, np.int64)
        nl = lib().orc_shape_connectivity(self.rest.shape[0], _d(self.rest), nt, _i(self.tri), _i(links), _d(llen),
                                          _i(pairs), _d(pcs), _d(tarea), _d(props), _i(npairs))
        npr = int(npairs[0])
        self.links, self.link_len = links[:nl].copy(), llen[:nl].copy()
        self.pairs, self.pair_cs = pairs[:npr].copy(), pcs[:npr].copy()
        self.tri_area = tarea
        self.area, self.volume = float(props[0]), float(props[1])
        self.center = props[2:5].copy()


def particle_update(pos, tri):
    pos, tri = f64(pos), i64(tri)
    out = np.zeros(5)
    lib().orc_particle_update(pos.shape[0], _d(pos), tri.shape[0], _i(tri), _d(out))
    return out


def inertia(pos, tri):
    pos, tri = f64(pos), i64(tri)
    out = np.zeros(9)
    lib().orc_inertia(_d(pos), tri.shape[0], _i(tri), _d(out))
    return out.reshape(3, 3)


def membrane_forces(model, prm, shape: Shape, pos):
    pos = f64(pos)
    st = particle_update(pos, shape.tri)
    out = np.zeros_like(pos)
    lib().orc_membrane_forces(MODEL[model] if isinstance(model, str) else int(model), _d(f64(prm)), pos.shape[0],
                              _d(shape.rest), shape.tri.shape[0], _i(shape.tri), _d(shape.tri_area), shape.area,
                              shape.links.shape[0], _i(shape.links), _d(shape.link_len), shape.pairs.shape[0],
                              _i(shape.pairs), _d(shape.pair_cs), _d(pos), st[0], st[1], _d(out))
    return out


# ------------------------------------------------------------------ immersed boundary
def classify(L, dirac, pos):
    pos = f64(pos)
    cls = np.zeros(pos.shape[0], np.int32)
    lib().orc_classify(C.byref(L), DIRAC[dirac], pos.shape[0], _d(pos), _i32(cls))
    return cls


def interpolate(L, dirac, u, pos, cls=None, offset=0.0):
    pos = f64(pos)
    cls = classify(L, dirac, pos) if cls is None else np.ascontiguousarray(cls, np.int32)
    vel = np.zeros_like(pos)
    lib().orc_interpolate(C.byref(L), DIRAC[dirac], float(offset), _d(f64(u)), pos.shape[0], _d(pos), _i32(cls),
                          _d(vel))
    return vel


def spread(L, dirac, pos, force, cls=None, offset=0.0, F=None):
    pos = f64(pos)
    cls = classify(L, dirac, pos) if cls is None else np.ascontiguousarray(cls, np.int32)
    F = np.zeros((3, L.nz, L.ny, L.nx)) if F is None else f64(F).copy()
    lib().orc_spread(C.byref(L), DIRAC[dirac], float(offset), pos.shape[0], _d(pos), _d(f64(force)), _i32(cls),
                     _d(F))
    return F


# ------------------------------------------------------------------ coupled system
class System:
    """Coupled IB-LBM system with the reference's step order (the oracle's mirror of the C ABI)."""

    def __init__(self, L, dirac="roma", ib_offset=-1.0):
        self.L = L
        self.n = L.nx * L.ny * L.nz
        self.h = lib().orc_sys_create(C.byref(L), DIRAC[dirac], float(ib_offset))
        self.nv = []

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_sys_destroy(self.h)
            self.h = None

    def _view(self, ptr, ncomp):
        shape = (ncomp, self.L.nz, self.L.ny, self.L.nx) if ncomp > 1 else (self.L.nz, self.L.ny, self.L.nx)
        return np.ctypeslib.as_array(ptr, shape=(ncomp * self.n,)).reshape(shape)

    @property
    def f(self):
        return self._view(lib().orc_sys_f(self.h), 19)

    @property
    def force(self):
        return self._view(lib().orc_sys_force(self.h), 3)

    @property
    def phase(self):
        return self._view(lib().orc_sys_phase(self.h), 1)

    def set_body_force(self, b):
        lib().orc_sys_set_body_force(self.h, _d(f64(b)))

    def add_shape(self, xyz, tri):
        xyz, tri = f64(xyz), i64(tri)
        self._shape_nv = getattr(self, "_shape_nv", []) + [xyz.shape[0]]
        return lib().orc_sys_add_shape(self.h, xyz.shape[0], _d(xyz), tri.shape[0], _i(tri))

    def add_particle(self, shape, model, prm, pos=None):
        pid = lib().orc_sys_add_particle(self.h, shape, MODEL[model] if isinstance(model, str) else int(model),
                                         _d(f64(prm)), _d(f64(pos)) if pos is not None else None)
        self.nv.append(self._shape_nv[shape])
        return pid

    def set_voxelize(self, on=True):
        """Revoxelize the membranes into the phase field after every move (and at init)."""
        lib().orc_sys_set_voxelize(self.h, int(bool(on)))

    def add_wall_interaction(self, pot: Potential, axis: int, lo: float, hi: float):
        """add_force_decorator(WallInteraction(ParallelPlatesBoundary(lo, hi) normal to axis, pot))."""
        assert lib().orc_sys_add_wall_interaction(self.h, C.byref(pot), int(axis), float(lo), float(hi)) >= 0

    def add_pipe_wall_interaction(self, pot: Potential, y0: float, z0: float, radius: float):
        """add_force_decorator(WallInteraction(PipeBoundary along x through (y0, z0), pot))."""
        assert lib().orc_sys_add_pipe_wall_interaction(self.h, C.byref(pot), float(y0), float(z0), float(radius)) >= 0

    def add_pp_interaction(self, pot: Potential, grid: bool = False):
        """add_pp_force(PPPotentialForce(pot)); grid=True searches pairs as the reference does."""
        assert lib().orc_sys_add_pp_interaction(self.h, C.byref(pot), int(bool(grid))) >= 0

    def set_pipe(self, y0, z0, radius):
        """set_boundary(PipeBoundary(y0, z0, radius)): near-wall TopHat blend and wall reflection."""
        lib().orc_sys_set_pipe(self.h, float(y0), float(z0), float(radius))

    def init(self):
        """ImmersedBoundaryDynamics3D::init: voxelize the initial positions (when enabled)."""
        lib().orc_sys_init(self.h)

    def step(self, n=1):
        lib().orc_sys_step(self.h, int(n))

    def lattice_step(self, n=1):
        lib().orc_sys_lattice_only_step(self.h, int(n))

    def particle(self, pid):
        nv = self.nv[pid]
        pos, vel, frc, st = np.zeros((nv, 3)), np.zeros((nv, 3)), np.zeros((nv, 3)), np.zeros(5)
        lib().orc_sys_get_particle(self.h, pid, _d(pos), _d(vel), _d(frc), _d(st))
        return dict(pos=pos, vel=vel, force=frc, area=st[0], volume=st[1], com=st[2:5])

    def velocity(self):
        u = np.zeros((3, self.L.nz, self.L.ny, self.L.nx))
        lib().orc_sys_velocity(self.h, _d(u))
        return u


def voxelize(L, pos, tri, phase=None):
    """Phase field (nz, ny, nx) of closed meshes: pos (nvt, 3), tri (ntt, 3) global vertex indices;
    `phase` is updated in place (cells the fill does not reach keep their value)."""
    pos, tri = f64(pos), i64(tri)
    ph = np.zeros((L.nz, L.ny, L.nx)) if phase is None else phase
    lib().orc_voxelize(C.byref(L), pos.shape[0], _d(pos), tri.shape[0], _i(tri), _d(ph))
    return ph


def wall_forces(pot: Potential, axis, lo, hi, pos, force=None):
    pos = f64(pos)
    out = np.zeros_like(pos) if force is None else f64(force).copy()
    lib().orc_wall_forces(C.byref(pot), int(axis), float(lo), float(hi), pos.shape[0], _d(pos), _d(out))
    return out


def pp_forces(L, pot: Potential, pos, owner, force=None, grid=False):
    """Particle-particle forces on the concatenated vertices (owner = particle of each vertex)."""
    pos = f64(pos)
    own = np.ascontiguousarray(owner, dtype=np.int32)
    out = np.zeros_like(pos) if force is None else f64(force).copy()
    fn = lib().orc_pp_forces_grid if grid else lib().orc_pp_forces
    fn(C.byref(L), C.byref(pot), pos.shape[0], _d(pos), _i32(own), _d(out))
    return out


def pipe_celltypes(dims, y0, z0, radius):
    """(nz, ny, nx) uint8 cell types of the reference's first-order pipe walls."""
    nx, ny, nz = dims
    t = np.zeros((nz, ny, nx), dtype=np.uint8)
    lib().orc_pipe_celltypes(nx, ny, nz, float(y0), float(z0), float(radius), t.ctypes.data)
    return t


def pipe_guo_nodes(dims, y0, z0, radius):
    """GuoRigidWallBoundary nodes of a pipe along x and the NoDynamics cells beyond radius + 1:
    (ctypes array of GuoNode, (nz, ny, nx) uint8 cell types)."""
    nx, ny, nz = dims
    cnt = lib().orc_pipe_guo_nodes(nx, ny, nz, float(y0), float(z0), float(radius), None, None)
    nodes = (GuoNode * max(cnt, 1))()
    t = np.zeros((nz, ny, nx), dtype=np.uint8)
    lib().orc_pipe_guo_nodes(nx, ny, nz, float(y0), float(z0), float(radius), C.cast(nodes, C.c_void_p), t.ctypes.data)
    return nodes, int(cnt), t


def set_guo(L, nodes, count):
    """Attach Guo wall nodes to a lattice (the caller keeps `nodes` alive)."""
    L.guo = C.cast(nodes, C.c_void_p)
    L.nguo = count
    return L


def apply_guo(L, f):
    out = f64(f).copy()
    lib().orc_apply_guo(C.byref(L), _d(out))
    return out


def move_vertices(pos, vel, pipe=None):
    """DeformableParticle3D::move_vertices, reflected at the wall of pipe = (y0, z0, radius)."""
    out = f64(pos).copy()
    v = f64(vel)
    pp = None if pipe is None else f64(pipe)
    lib().orc_move_vertices(out.shape[0], _d(out), _d(v), None if pp is None else pp.ctypes.data)
    return out


# ---------------------------------------------------------------- the reference's particle files
# Particle type ids of the reference's particle factory (ParticleFactory.hh:63-66): the order in
# which a program including fsi/headers.hh registers DeformableCapsuleParticle and RBCParticle.
PLB_TYPE_CAPSULE, PLB_TYPE_RBC = 0, 1
SHEAR_SKALAK, SHEAR_NEOHOOKEAN = 0, 1  # enum ShearModel, DeformableCapsule.h:39
CAPSULE_PACK = ["C", "kb", "nu_s", "G"]  # CapsuleParameters::pack, DeformableCapsule.hh:21-29
RBC_PACK = ["L0", "shear_modulus", "k_area_global", "k_area_local", "k_bend", "k_volume", "theta0",
            "vol_desired"]  # RBCParameters::pack, RBCParticle.hh:93-105


def plb_pack(model, shape, pid, pos, vel, force, prm, voxelize=True) -> bytes:
    """One particle's pack: ParticleBase3D::pack (ParticleBase.hh:218-224) type id, shape id,
    particle id, should_voxelize; DeformableParticle3D::pack (DeformableParticle3D.hh:277-287) pos,
    vel, force per vertex; then DeformableCapsuleParticle::pack (shear law + CapsuleParameters,
    DeformableCapsule.hh:217-223) or RBCParticle::pack (RBCParameters, RBCParticle.hh:344-350)."""
    import struct

    prm = dict(zip(PARAM_KEYS, np.asarray(prm, dtype=np.float64)))
    capsule = model in (MODEL["capsule_neohookean"], MODEL["capsule_skalak"])
    if not capsule and model != MODEL["rbc_wlcpow"]:
        raise ValueError("model %d has no particle type in the reference's format" % model)
    out = [struct.pack("<qqq?", PLB_TYPE_CAPSULE if capsule else PLB_TYPE_RBC, shape, pid, voxelize)]
    verts = np.concatenate([f64(pos), f64(vel), f64(force)], axis=1)  # (nv, 9): pos, vel, force
    out.append(verts.astype("<f8").tobytes())
    if capsule:
        law = SHEAR_SKALAK if model == MODEL["capsule_skalak"] else SHEAR_NEOHOOKEAN
        out.append(struct.pack("<i4d", law, *[prm[k] for k in CAPSULE_PACK]))
    else:
        out.append(struct.pack("<8d", *[prm[k] for k in RBC_PACK]))
    return b"".join(out)


def plb_unpack(buf: bytes, at: int, shape_nv):
    """Inverse of plb_pack at byte offset `at`: (particle dict, offset after it)."""
    import struct

    type_id, shape, pid, vox = struct.unpack_from("<qqq?", buf, at)
    at += 25
    nv = shape_nv[shape]
    verts = np.frombuffer(buf, dtype="<f8", count=9 * nv, offset=at).reshape(nv, 9)
    at += 72 * nv
    prm = dict.fromkeys(PARAM_KEYS, 0.0)
    if type_id == PLB_TYPE_CAPSULE:
        law, *vals = struct.unpack_from("<i4d", buf, at)
        at += 36
        model = MODEL["capsule_skalak"] if law == SHEAR_SKALAK else MODEL["capsule_neohookean"]
        prm.update(zip(CAPSULE_PACK, vals))
    elif type_id == PLB_TYPE_RBC:
        vals = struct.unpack_from("<8d", buf, at)
        at += 64
        model = MODEL["rbc_wlcpow"]
        prm.update(zip(RBC_PACK, vals))
    else:
        raise ValueError("unknown particle type %d" % type_id)
    p = dict(model=model, shape=shape, id=pid, voxelize=vox, pos=verts[:, 0:3].copy(), vel=verts[:, 3:6].copy(),
             force=verts[:, 6:9].copy(), params=np.array([prm[k] for k in PARAM_KEYS]))
    return p, at


def plb_files(name, particles):
    """ImmersedBoundaryDynamics3D::save_checkpoint (ImmersedBoundaryDynamics_io.hh:17-73) on one
    rank: (header text, bytes of <name>/0.plb).  particles: dicts as plb_unpack returns them."""
    import struct

    header = "%d\n1\n%s/0.plb\n" % (len(particles), name)
    body = struct.pack("<q", len(particles)) + b"".join(
        plb_pack(p["model"], p["shape"], p["id"], p["pos"], p["vel"], p["force"], p["params"], p.get("voxelize", True))
        for p in particles)
    return header, body


def vtu_bytes(pos, force, tri) -> bytes:
    """ParticleBase3D::write_vtk (ParticleBase.hh:270-390): XML UnstructuredGrid with raw appended
    data, UInt32 block sizes, Float32 positions and forces, Int32 connectivity, offsets, types."""
    import struct

    pos, force, tri = f64(pos), f64(force), np.asarray(tri, dtype=np.int64)
    nv, nt = pos.shape[0], tri.shape[0]
    sizes = [12 * nv, 12 * nv, 12 * nt, 4 * nt, 4 * nt]
    offs = [0]
    for s in sizes[:-1]:
        offs.append(offs[-1] + 4 + s)
    head = ('<?xml version="1.0"?>\n'
            '<VTKFile type="UnstructuredGrid" version="0.1" byte_order="LittleEndian" header_type="UInt32" >\n'
            '  <UnstructuredGrid>\n'
            '    <Piece NumberOfPoints="%d" NumberOfCells="%d" >\n'
            '      <Points>\n'
            '        <DataArray type="Float32" NumberOfComponents="3" format="appended" offset="%d" />\n'
            '      </Points>\n'
            '      <PointData>\n'
            '        <DataArray type="Float32" NumberOfComponents="3" Name="force_tot" format="appended" offset="%d" />\n'
            '      </PointData>\n'
            '      <Cells>\n'
            '        <DataArray type="Int32" Name="connectivity" format="appended" offset="%d" />\n'
            '        <DataArray type="Int32" Name="offsets" format="appended" offset="%d" />\n'
            '        <DataArray type="Int32" Name="types" format="appended" offset="%d" />\n'
            '      </Cells>\n'
            '    </Piece>\n'
            '  </UnstructuredGrid>\n'
            '  <AppendedData encoding="raw">\n'
            '_') % (nv, nt, *offs)
    blocks = [pos.astype("<f4"), force.astype("<f4"), tri.astype("<i4"), 3 * np.arange(1, nt + 1, dtype="<i4"),
              np.full(nt, 5, dtype="<i4")]
    data = b"".join(struct.pack("<I", s) + b.tobytes() for s, b in zip(sizes, blocks))
    return head.encode() + data + b"\n  </AppendedData>\n</VTKFile>\n"


def _stream_double(x: float) -> str:
    """A double as std::ostream writes it with default flags (%g, 6 significant digits)."""
    return "%g" % x


def lightweight_text(iteration, rows) -> str:
    """write_lightweight_particle_data (ImmersedBoundaryDynamics_io.hh:178-199) with
    DeformableParticle3D::write_lightweight (DeformableParticle3D.hh:318-333) per particle.
    rows: (tag, id, positions, centre, volume) per particle; the gyration tensor follows
    compute_tensor_of_gyration (DeformableParticle3D.hh:111-125)."""
    lines = ["iteration:%d" % iteration]
    for tag, pid, pos, com, vol in rows:
        pos, com = f64(pos), f64(com)
        g = np.zeros((3, 3))
        for v in range(pos.shape[0]):
            for i in range(3):
                for j in range(i, 3):
                    g[i, j] += (pos[v, i] - com[i]) * (pos[v, j] - com[j])
        vals = list(com) + [g[i, j] / pos.shape[0] for i in range(3) for j in range(i, 3)] + [vol]
        lines.append("%s:%d:" % (tag, pid) + ":".join(_stream_double(float(v)) for v in vals))
    return "\n".join(lines) + "\n"


def plb_lattice_files(name, fbar, force, phase, vof=True):
    """parallelIO::save(lattice, name, false) of a one-block ForcedPhaseD3Q19 lattice
    (io/multiBlockWriter3D.cpp:53-137, 201-213): (XML spec text, raw .dat bytes).  fbar (19, nz,
    ny, nx), force (3, nz, ny, nx), phase (nz, ny, nx); cells x-major with z fastest, 23 doubles
    each (BlockLattice3D::send, blockLattice3D.hh:671-689)."""
    fbar, force, phase = f64(fbar), f64(force), f64(phase)
    nz, ny, nx = phase.shape
    cells = np.concatenate([fbar, force, phase[None]], axis=0)  # (23, nz, ny, nx)
    dat = np.ascontiguousarray(np.transpose(cells, (3, 2, 1, 0))).astype("<f8").tobytes()
    box = "0 %d 0 %d 0 %d" % (nx - 1, ny - 1, nz - 1)
    lines = ['<?xml version="1.0" ?>', "<Block3D>", "    <General>",
             "        <Family> BlockLattice3D </Family>", "        <Datatype> double </Datatype>",
             "        <Descriptor> ForcedPhaseD3Q19 </Descriptor>", "        <cellDim> 23 </cellDim>",
             "        <dynamicContent> False </dynamicContent>", "        <globalId> 0 </globalId>",
             "    </General>", "    <Structure>", "        <BoundingBox> %s </BoundingBox>" % box,
             "        <EnvelopeWidth> 1 </EnvelopeWidth>", "        <GridLevel> 0 </GridLevel>",
             "        <NumComponents> 1 </NumComponents>", "    </Structure>", "    <Data>",
             "        <File> %s.dat </File>" % name, "        <Component> %s </Component>" % box,
             "        <Offsets> %d </Offsets>" % len(dat)]
    if vof:
        lines += ["        <DynamicsDict>", "            <Guo_VOF_dynamics> 3 </Guo_VOF_dynamics>",
                  "        </DynamicsDict>"]
    lines += ["    </Data>", "</Block3D>"]
    return "\n".join(lines) + "\n", dat


def plb_lattice_read(xml: str, dat: bytes):
    """parallelIO::load's reading of a static-content checkpoint (io/multiBlockReader3D.cpp:135-268)
    of any block decomposition: (fbar, force, phase) on the whole bounding box; phase is None for
    22 values per cell (ForcedD3Q19)."""
    import re

    def leaves(tag):
        return [m.group(1) for m in re.finditer(r"<%s(?:\s[^>]*)?>(.*?)</%s>" % (tag, tag), xml, re.S)]

    def ints(text):
        return [int(v) for v in text.split()]

    per = ints(leaves("cellDim")[0])[0]
    x0, x1, y0, y1, z0, z1 = ints(leaves("BoundingBox")[0])
    nx, ny, nz = x1 - x0 + 1, y1 - y0 + 1, z1 - z0 + 1
    cells = np.zeros((nx, ny, nz, per))
    offsets = ints(leaves("Offsets")[0])
    start = 0
    for comp, end in zip(leaves("Component"), offsets):
        a0, a1, b0, b1, c0, c1 = ints(comp)
        block = np.frombuffer(dat[start:end], dtype="<f8").reshape(a1 - a0 + 1, b1 - b0 + 1, c1 - c0 + 1, per)
        cells[a0 - x0:a1 - x0 + 1, b0 - y0:b1 - y0 + 1, c0 - z0:c1 - z0 + 1] = block
        start = end
    cells = np.transpose(cells, (3, 2, 1, 0))
    return cells[:19].copy(), cells[19:22].copy(), (cells[22].copy() if per == 23 else None)


# ---------------------------------------------------------------- RBC shape calibration
def rbc_shrink_volume(shape: Shape, prm, vol_final, n_it, damping=1.e-2):
    """shrink_rbc_volume (progs/common/calibrate_rbc_shape.h:12-69): (relaxed vertices, damping used)."""
    pos = np.zeros_like(shape.rest)
    d = lib().orc_rbc_shrink_volume(_d(f64(prm)), shape.rest.shape[0], _d(shape.rest), shape.tri.shape[0], _i(shape.tri),
                                    _d(shape.tri_area), shape.area, shape.volume, shape.links.shape[0], _i(shape.links),
                                    _d(shape.link_len), shape.pairs.shape[0], _i(shape.pairs), _d(shape.pair_cs),
                                    float(vol_final), int(n_it), float(damping), _d(pos), None)
    return pos, d


def rbc_params(shape: Shape, shear_modulus, k_area, k_bend):
    """create_rbc_params (progs/common/calibrate_rbc_shape.h:72-110) as a BIB_P_* vector."""
    import math

    lavg = 0.0
    for l in shape.link_len:
        lavg += float(l)
    lavg /= shape.link_len.shape[0]
    p = dict.fromkeys(PARAM_KEYS, 0.0)
    p.update(shear_modulus=shear_modulus, L0=lavg, vol_desired=shape.volume)
    dk = k_area - (2 * shear_modulus + 0.0 + 0.0)  # RBCParameters::K() with both area stiffnesses 0
    p.update(k_area_global=dk * 0.8, k_area_local=dk * 0.2)
    r2 = 0.0
    for x, y, z in shape.rest:
        d2 = x * x + y * y + z * z
        if d2 > r2:
            r2 = d2
    p["k_volume"] = 1000. * shear_modulus / math.sqrt(r2)
    p["k_bend"] = k_bend
    nv = shape.rest.shape[0]
    p["theta0"] = math.acos((math.sqrt(3.) * (nv - 2.) - 5 * math.pi) / (math.sqrt(3.) * (nv - 2.) - 3. * math.pi))
    return np.array([p[k] for k in PARAM_KEYS])


def _jacobi3(A):
    """Cyclic Jacobi eigen decomposition of a symmetric 3x3 matrix (J. Kopp, "Efficient numerical
    diagonalization of hermitian 3x3 matrices", 2008; the method of linalg::diagonalize,
    fsi/linalg.h:21-138): (eigenvalues, eigenvectors as columns).  Uses the upper triangle."""
    import math

    A = [list(map(float, r)) for r in A]
    Q = [[1.0 if i == j else 0.0 for j in range(3)] for i in range(3)]
    w = [A[i][i] for i in range(3)]
    for sweep in range(50):
        so = 0.0
        for p in range(3):
            for q in range(p + 1, 3):
                so += abs(A[p][q])
        if so == 0.0:
            break
        thresh = 0.2 * so / 9 if sweep < 4 else 0.0
        for p in range(3):
            for q in range(p + 1, 3):
                g = 100.0 * abs(A[p][q])
                if sweep > 4 and abs(w[p]) + g == abs(w[p]) and abs(w[q]) + g == abs(w[q]):
                    A[p][q] = 0.0
                    continue
                if not abs(A[p][q]) > thresh:
                    continue
                h = w[q] - w[p]
                if abs(h) + g == abs(h):
                    t = A[p][q] / h
                else:
                    theta = 0.5 * h / A[p][q]
                    t = -1.0 / (math.sqrt(1.0 + theta * theta) - theta) if theta < 0.0 else \
                        1.0 / (math.sqrt(1.0 + theta * theta) + theta)
                c = 1.0 / math.sqrt(1.0 + t * t)
                s = t * c
                z = t * A[p][q]
                A[p][q] = 0.0
                w[p] -= z
                w[q] += z
                for r in range(p):
                    t2 = A[r][p]
                    A[r][p] = c * t2 - s * A[r][q]
                    A[r][q] = s * t2 + c * A[r][q]
                for r in range(p + 1, q):
                    t2 = A[p][r]
                    A[p][r] = c * t2 - s * A[r][q]
                    A[r][q] = s * t2 + c * A[r][q]
                for r in range(q + 1, 3):
                    t2 = A[p][r]
                    A[p][r] = c * t2 - s * A[q][r]
                    A[q][r] = s * t2 + c * A[q][r]
                for r in range(3):
                    t2 = Q[r][p]
                    Q[r][p] = c * t2 - s * Q[r][q]
                    Q[r][q] = s * t2 + c * Q[r][q]
    return w, Q


def align_minor_axis(pos, tri, pref=(0.0, 0.0, 1.0)):
    """DeformableParticle3D::set_minor_axis_orientation (DeformableParticle3D.hh:85-144): the
    eigenvector of the tensor of gyration with the smallest |eigenvalue| rotated onto pref about
    the centre of mass (Quaternion.h:28-40, 144-155; Transform.hh:36-84)."""
    import math

    pos = f64(pos).copy()
    com = particle_update(pos, tri)[2:5]
    nv = pos.shape[0]
    A = [[0.0] * 3 for _ in range(3)]
    for v in range(nv):
        for i in range(3):
            for j in range(i, 3):
                A[i][j] += (pos[v, i] - com[i]) * (pos[v, j] - com[j])
    for i in range(3):
        for j in range(i, 3):
            A[i][j] /= nv
    w, Q = _jacobi3(A)
    a = [abs(x) for x in w]
    k = 0 if (a[0] < a[1] and a[0] < a[2]) else (1 if a[1] < a[2] else 2)
    d = [Q[0][k], Q[1][k], Q[2][k]]
    dn = math.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
    d = [x / dn for x in d]
    p = [float(x) for x in pref]
    ax = [d[1] * p[2] - d[2] * p[1], d[2] * p[0] - d[0] * p[2], d[0] * p[1] - d[1] * p[0]]
    an = math.sqrt(ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2])
    angle = math.asin(an / (math.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) *
                            math.sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2])))
    ax = [x / an for x in ax]
    if p[0] * d[0] + p[1] * d[1] + p[2] * d[2] < 0:
        ax = [-x for x in ax]
    sh = math.sin(angle / 2)
    q0, q1, q2, q3 = math.cos(angle / 2), sh * ax[0], sh * ax[1], sh * ax[2]
    R = [[1 - 2 * (q2 * q2 + q3 * q3), 2 * (q1 * q2 - q0 * q3), 2 * (q0 * q2 + q1 * q3)],
         [2 * (q1 * q2 + q0 * q3), 1 - 2 * (q1 * q1 + q3 * q3), 2 * (q2 * q3 - q0 * q1)],
         [2 * (q1 * q3 - q0 * q2), 2 * (q0 * q1 + q2 * q3), 1 - 2 * (q1 * q1 + q2 * q2)]]
    # Transform::translate(-com).rotate(R).translate(com): columns 0-2 = R, column 3 = R (-com) + com
    t = [R[i][0] * -com[0] + R[i][1] * -com[1] + R[i][2] * -com[2] + com[i] for i in range(3)]
    out = np.empty_like(pos)
    for v in range(nv):
        x, y, z = pos[v]
        for i in range(3):
            out[v, i] = x * R[i][0] + y * R[i][1] + z * R[i][2] + t[i]
    return out


# ---------------------------------------------------------------- random initial placement
class GlibcRand:
    """glibc's rand() after srand(seed) (TYPE_3): x_i = x_{i-3} + x_{i-31} mod 2^32, output
    x_i >> 1; x_1 .. x_30 from the Lehmer generator 16807 x mod (2^31 - 1); 310 outputs discarded."""

    def __init__(self, seed):
        seed = seed or 1
        r = [seed]
        for i in range(1, 31):
            r.append((16807 * r[i - 1]) % 2147483647)
        r += r[0:3]
        for i in range(34, 344):
            r.append((r[i - 31] + r[i - 3]) & 0xFFFFFFFF)
        self.r = r[-34:]

    def __call__(self):
        v = (self.r[-31] + self.r[-3]) & 0xFFFFFFFF
        self.r = self.r[1:] + [v]
        return v >> 1


def initial_distribution(box, counts, radii, seed, pipe=None):
    """ParticlePositionInitializer::generate_points (ParticlePositionInitializer.hh:17-80) per type
    and the random orientations of progs/common/create_particles.h:80-93, as the reference draws
    them from rand(): (positions (n, 3), quaternions (n, 4))."""
    import math

    rand = GlibcRand(int(seed))
    RM = 2147483647.0
    pos, rad = [], []
    for t, n in enumerate(counts):
        r = float(radii[t])
        for _ in range(int(n)):
            while True:
                p = [float(box[2 * a]) + r + (rand() / RM) * (float(box[2 * a + 1] - box[2 * a]) - 2 * r) for a in range(3)]
                if pipe is not None:
                    dy, dz = p[1] - pipe[0], p[2] - pipe[1]
                    if not (dy * dy + dz * dz) < (pipe[2] - r) * (pipe[2] - r):
                        continue
                ok = True
                for q, rq in zip(pos, rad):
                    dx, dy, dz = q[0] - p[0], q[1] - p[1], q[2] - p[2]
                    if dx * dx + dy * dy + dz * dz < (rq + r) * (rq + r):
                        ok = False
                        break
                if ok:
                    break
            pos.append(p)
            rad.append(r)
    quats = []
    for _ in pos:
        d2, d1, d0 = rand() / RM, rand() / RM, rand() / RM  # g++ evaluates the three arguments last to first
        dn = math.sqrt(d0 * d0 + d1 * d1 + d2 * d2)
        if dn > 2.220446049250313e-16:
            theta = 2. * math.pi * rand() / RM
            s = math.sin(theta / 2)
            quats.append([math.cos(theta / 2), s * (d0 / dn), s * (d1 / dn), s * (d2 / dn)])
        else:
            quats.append([1.0, 0.0, 0.0, 0.0])
    return np.array(pos), np.array(quats)


def growth(box, wall=None, periodic=(1, 0, 0), pot=(1.0, 5e-2), initial_scale=0.2, density=1.0, damping=0.1,
           n_it=40000, it_end=None, rescale_every=10) -> Growth:
    """Parameters of create_particles' growth stage (progs/common/create_particles.h:105-161)."""
    g = Growth()
    for k in range(6):
        g.box[k] = int(box[k])
    for a in range(3):
        g.periodic[a] = int(periodic[a])
    g.has_wall = 0 if wall is None else 1
    if wall is not None:
        for k in range(3):
            g.wall[k] = float(wall[k])
    g.min_dist, g.strength = float(pot[0]), float(pot[1])
    g.initial_scale, g.density, g.damping = float(initial_scale), float(density), float(damping)
    g.n_it, g.rescale_every = int(n_it), int(rescale_every)
    g.it_end = int(n_it + 1 if it_end is None else it_end)
    return g


def grow_particles(g: Growth, shapes, shape_of, com, quat):
    """The growth stage on rigid copies of shapes [(xyz, tri), ...]: particle k on shape_of[k]
    from com[k], quat[k].  Returns (com, quat, vertex positions, vertex forces of the last
    collision step)."""
    nv = np.array([len(x) for x, _ in shapes], dtype=np.int64)
    nt = np.array([len(t) for _, t in shapes], dtype=np.int64)
    verts = f64(np.concatenate([np.asarray(x, dtype=np.float64) for x, _ in shapes]))
    tris = i64(np.concatenate([np.asarray(t, dtype=np.int64) for _, t in shapes]))
    sh = np.ascontiguousarray(shape_of, dtype=np.int32)
    com, quat = f64(com).copy(), f64(quat).copy()
    ntot = int(nv[sh].sum())
    pos, frc = np.zeros((ntot, 3)), np.zeros((ntot, 3))
    st = lib().orc_grow_particles(C.byref(g), len(shapes), _i(nv), _d(verts), _i(nt), _i(tris), len(sh), _i32(sh),
                                  _d(com), _d(quat), _d(pos), _d(frc))
    if st != 0:
        raise ValueError("orc_grow_particles: bad input")
    return com, quat, pos, frc


def shape_radius(xyz):
    """ParticleShape::compute_bounding_volumes (ParticleShape.hh:361-383): the largest vertex
    distance from the origin."""
    r = 0.0
    for v in np.asarray(xyz, dtype=np.float64):
        d = v[0] * v[0] + v[1] * v[1] + v[2] * v[2]
        if d > r:
            r = d
    return float(np.sqrt(r))


def place_particle(xyz, tri, pos, quat):
    """The final placement of create_particles (:193-199): the template's vertices moved by
    Transform().translate(-com).rotate(quat).translate(pos) (Transform.hh:28-85), com the
    template's centre (DeformableParticle3D::update)."""
    xyz = f64(xyz)
    c = particle_update(xyz, tri)[2:5]
    q = [float(v) for v in quat]
    R = [[1 - 2 * (q[2] * q[2] + q[3] * q[3]), 2 * (q[1] * q[2] - q[0] * q[3]), 2 * (q[0] * q[2] + q[1] * q[3])],
         [2 * (q[1] * q[2] + q[0] * q[3]), 1 - 2 * (q[1] * q[1] + q[3] * q[3]), 2 * (q[2] * q[3] - q[0] * q[1])],
         [2 * (q[1] * q[3] - q[0] * q[2]), 2 * (q[0] * q[1] + q[2] * q[3]), 1 - 2 * (q[1] * q[1] + q[2] * q[2])]]
    m3 = [R[i][0] * -c[0] + R[i][1] * -c[1] + R[i][2] * -c[2] + float(pos[i]) for i in range(3)]
    out = np.empty_like(xyz)
    for i in range(3):
        out[:, i] = xyz[:, 0] * R[i][0] + xyz[:, 1] * R[i][1] + xyz[:, 2] * R[i][2] + m3[i]
    return out


def create_particles(box, pipe, types, seed, n_it=40000, periodic=(1, 0, 0)):
    """create_particles (progs/common/create_particles.h:9-212) for capsule templates: types =
    [(xyz, tri, count), ...], pipe = (y0, z0, radius); srand(seed) placement at 20 % scale inside
    the pipe shrunk by 1.5, growth, placement of the templates.  Returns the vertex positions of
    all particles in order."""
    shapes = [(x, t) for x, t, _ in types]
    counts = [int(n) for _, _, n in types]
    radii = np.array([0.2 * shape_radius(x) + 1.0 for x, _ in shapes])
    wall = (float(pipe[0]), float(pipe[1]), float(pipe[2]) - 1.5)
    com, quat = initial_distribution(box, counts, radii, seed, pipe=wall)
    shape_of = np.repeat(np.arange(len(shapes)), counts)
    com, quat, _, _ = grow_particles(growth(box, wall, periodic, n_it=n_it), shapes, shape_of, com, quat)
    return [place_particle(shapes[s][0], shapes[s][1], com[k], quat[k]) for k, s in enumerate(shape_of)]
