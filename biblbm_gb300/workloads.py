"""Seeded synthetic instances of the benchmark configurations.

The reference publishes no dataset; its drivers place particles with std::rand
(progs/common/create_particles.h:80-82).  These generators are seeded and
deterministic so that the CUDA path, the CPU oracle and the reference harness can be
fed the same instance.

``channel_suspension``: the dense red-cell suspension in a channel (512 x 128 x 128,
bounce-back walls on y and z, periodic x, body force 1e-6, 400 Evans-Fung cells of 642
vertices at 20 % haematocrit, random non-overlapping positions and orientations).
``capsule_shear``: one spherical capsule in simple shear between finite-difference
velocity walls (progs/capsule_in_shear/capsule_in_shear.cpp).
``batched_capsules``: independent capsule-in-shear instances of uneven sizes (cubic edges
drawn from {32, 48, 64, 80, 96}, radius edge/6, 162- or 642-vertex meshes, capillary number
log-uniform in [0.01, 1]), stepped together as one batch.
"""
from __future__ import annotations

import numpy as np

from . import meshes

# parameter vector order of the C ABI (BIB_P_*)
_KEYS = ["G", "C", "nu_s", "kb", "shear_modulus", "L0", "k_area_global", "k_area_local", "k_volume", "vol_desired",
         "k_bend", "theta0"]


def params_vector(**kw) -> np.ndarray:
    v = dict(zip(_KEYS, [0.0, 1.0, 1.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0]))
    v.update(kw)
    return np.array([v[k] for k in _KEYS], dtype=np.float64)


def mesh_area_volume(xyz, tri):
    a, b, c = xyz[tri[:, 0]], xyz[tri[:, 1]], xyz[tri[:, 2]]
    area = 0.5 * np.linalg.norm(np.cross(b - a, c - a), axis=1).sum()
    vol = np.einsum("ij,ij->i", a, np.cross(b, c)).sum() / 6.0
    return float(area), float(vol)


def _place_cells(rng, dims, rest, n_cells, margin, max_tries=20000):
    """Random sequential addition of rigid copies of ``rest`` (centred at 0, symmetry axis z).

    Overlap test: each cell is approximated by its enclosing oblate spheroid
    (R, R, h); a candidate is rejected if any of its vertices falls inside a
    neighbour's spheroid or vice versa (x periodic), or if a vertex comes within
    ``margin`` of the y / z walls.
    """
    nx, ny, nz = dims
    R = np.sqrt((rest[:, 0] ** 2 + rest[:, 1] ** 2).max())
    h = np.abs(rest[:, 2]).max()
    scale = np.array([R, R, h]) * 1.04
    centers, rots, verts = [], [], []
    lo = np.array([0.0, margin, margin])
    hi = np.array([nx, ny - 1.0 - margin, nz - 1.0 - margin])
    for _ in range(n_cells):
        for _try in range(max_tries):
            c = np.array([rng.uniform(0, nx), rng.uniform(lo[1], hi[1]), rng.uniform(lo[2], hi[2])])
            Rm = meshes.random_rotation(rng)
            v = rest @ Rm.T + c
            if v[:, 1].min() < lo[1] or v[:, 1].max() > hi[1] or v[:, 2].min() < lo[2] or v[:, 2].max() > hi[2]:
                continue
            ok = True
            near = []
            if centers:
                dc = c - np.asarray(centers)
                dc[:, 0] -= nx * np.round(dc[:, 0] / nx)
                near = np.nonzero(np.einsum("ij,ij->i", dc, dc) < (2.0 * R * 1.04) ** 2)[0]
            for j in near:
                cj, Rj, vj = centers[j], rots[j], verts[j]
                d = c - cj
                d[0] -= nx * np.round(d[0] / nx)
                shift = np.array([c[0] - cj[0] - d[0], 0.0, 0.0])
                p = ((v - shift - cj) @ Rj) / scale
                if (np.einsum("ij,ij->i", p, p) < 1.0).any():
                    ok = False
                    break
                q = ((vj + shift - c) @ Rm) / scale
                if (np.einsum("ij,ij->i", q, q) < 1.0).any():
                    ok = False
                    break
            if ok:
                centers.append(c)
                rots.append(Rm)
                verts.append(v)
                break
        else:
            raise RuntimeError("could not place cell %d of %d" % (len(centers) + 1, n_cells))
    return np.array(centers), np.array(verts)


def channel_suspension(nx=512, ny=128, nz=128, n_cells=400, level=3, hct=0.20, tau=1.0, body=1e-6, Ca=0.1,
                       seed=3):
    rng = np.random.default_rng(seed)
    unit, tri = meshes.evans_fung(level, 1.0)
    _, v1 = mesh_area_volume(unit, tri)
    R = (hct * nx * ny * nz / (n_cells * v1)) ** (1.0 / 3.0)
    rest, tri = meshes.evans_fung(level, R)
    rest = rest - rest.mean(axis=0)
    A0, V0 = mesh_area_volume(rest, tri)
    centers, verts = _place_cells(rng, (nx, ny, nz), rest, n_cells, margin=1.0)
    nu = (tau - 0.5) / 3.0
    gamma = body * ny / (2.0 * nu)  # wall shear rate of plane Poiseuille flow across y
    G = nu * gamma * R / Ca
    prm = params_vector(G=G, C=1.0, k_area_global=1.0, k_volume=1.0, vol_desired=V0, k_bend=0.01 * G * A0)
    return dict(
        name="channel_%dx%dx%d_%drbc_%dv" % (nx, ny, nz, n_cells, rest.shape[0]),
        dims=(nx, ny, nz),
        lattice=dict(periodic=(1, 0, 0), collision="bgk_guo_vof", omega=1.0 / tau, wall_y="halfway_bb",
                     wall_z="halfway_bb", body_force=(body, 0.0, 0.0)),
        rest=rest, tri=tri, positions=verts, centers=centers, model="skalak_bending", params=prm,
        radius=R, hct=n_cells * V0 / (nx * ny * nz), A0=A0, V0=V0, Ca=Ca, seed=seed,
        initial_velocity=None,
    )


def capsule_shear(n=64, level=3, radius=10.0, U=0.01, tau=1.0, Ca=0.1, seed=1):
    rest, tri = meshes.icosphere(level, radius)
    nu = (tau - 0.5) / 3.0
    gamma = 2.0 * U / (n - 1)
    G = nu * gamma * radius / Ca
    c = 0.5 * (n - 1)
    pos = meshes.place(rest, None, (c, c, c))
    y = np.arange(n)
    u0 = np.zeros((3, n, n, n))
    u0[0] = (U * (2.0 * y / (n - 1) - 1))[None, :, None]
    return dict(
        name="capsule_shear_%d_%dv" % (n, rest.shape[0]),
        dims=(n, n, n),
        lattice=dict(periodic=(1, 0, 1), collision="bgk_guo_vof", omega=1.0 / tau, wall_y="fd_velocity",
                     wall_u=[[-U, 0, 0], [U, 0, 0], [0, 0, 0], [0, 0, 0]]),
        rest=rest, tri=tri, positions=pos[None], model="capsule_skalak", params=params_vector(G=G, C=1.0),
        radius=radius, initial_velocity=u0, seed=seed,
    )


def batched_capsules(n_inst=64, seed=4, edges=(32, 48, 64, 80, 96), U=0.01, tau=1.0):
    rng = np.random.default_rng(seed)
    inst = []
    for _ in range(n_inst):
        n = int(rng.choice(edges))
        level = 2 if rng.uniform() < 0.5 else 3  # 162 or 642 vertices
        Ca = float(np.exp(rng.uniform(np.log(0.01), np.log(1.0))))
        inst.append(capsule_shear(n=n, level=level, radius=n / 6.0, U=U, tau=tau, Ca=Ca, seed=seed))
    cells = sum(w["dims"][0] ** 3 for w in inst)
    verts = sum(w["rest"].shape[0] for w in inst)
    return dict(name="batched_capsules_%d" % n_inst, instances=inst, cells=cells, vertices=verts, seed=seed)


def rbc_shear(nx=128, ny=64, nz=64, level=4, radius=8.0, U=0.01, tau=1.0, Ca=0.1, seed=2):
    """One Evans-Fung red cell (major radius 8, 2562 vertices) in simple shear between
    finite-difference velocity walls, Skalak + bending (kb = 0.01 G A0) + global area and
    volume penalties, random orientation."""
    rng = np.random.default_rng(seed)
    rest, tri = meshes.evans_fung(level, radius)
    rest = rest - rest.mean(axis=0)
    A0, V0 = mesh_area_volume(rest, tri)
    nu = (tau - 0.5) / 3.0
    gamma = 2.0 * U / (ny - 1)
    G = nu * gamma * radius / Ca
    c = np.array([0.5 * (nx - 1), 0.5 * (ny - 1), 0.5 * (nz - 1)])
    pos = rest @ meshes.random_rotation(rng).T + c
    y = np.arange(ny)
    u0 = np.zeros((3, nz, ny, nx))
    u0[0] = (U * (2.0 * y / (ny - 1) - 1))[None, :, None]
    prm = params_vector(G=G, C=1.0, k_area_global=1.0, k_volume=1.0, vol_desired=V0, k_bend=0.01 * G * A0)
    return dict(
        name="rbc_shear_%dx%dx%d_%dv" % (nx, ny, nz, rest.shape[0]),
        dims=(nx, ny, nz),
        lattice=dict(periodic=(1, 0, 1), collision="bgk_guo_vof", omega=1.0 / tau, wall_y="fd_velocity",
                     wall_u=[[-U, 0, 0], [U, 0, 0], [0, 0, 0], [0, 0, 0]]),
        rest=rest, tri=tri, positions=pos[None], model="skalak_bending", params=prm, radius=radius, A0=A0, V0=V0,
        initial_velocity=u0, seed=seed,
    )
