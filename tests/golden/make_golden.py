"""Generate the golden fixtures in this folder by running the REFERENCE's own code.

The reference (niclasberg/biblbm: Palabos + src/fsi, FP64 C++) is compiled from
its sources by ``make -C oracle ref`` into ``oracle/_ref/ref_harness``; this
script writes seeded inputs, runs the harness and stores inputs and outputs as
small ``.npz`` files.  The fixtures pin both the CPU oracle restatement and the
CUDA path.  Run from the repository root:

    make -C oracle ref REF=<path to the reference checkout>
    python tests/golden/make_golden.py

Only this script needs the reference; the tests read the committed ``.npz``.
"""
from __future__ import annotations

import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from biblbm_gb300 import meshes  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")

# D3Q19 velocity set in the reference's order (src/latticeBoltzmann/nearestNeighborLattices3D.hh:165-197)
C = np.array(
    [[0, 0, 0], [-1, 0, 0], [0, -1, 0], [0, 0, -1], [-1, -1, 0], [-1, 1, 0], [-1, 0, -1], [-1, 0, 1],
     [0, -1, -1], [0, -1, 1], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 0], [1, -1, 0], [1, 0, 1],
     [1, 0, -1], [0, 1, 1], [0, 1, -1]], dtype=np.int64)
W = np.array([1 / 3] + [1 / 18] * 3 + [1 / 36] * 6 + [1 / 18] * 3 + [1 / 36] * 6)


# ---------------------------------------------------------------- record files
def write_rec(path, arrays: dict):
    with open(path, "wb") as f:
        for name, a in arrays.items():
            a = np.asarray(a)
            if a.dtype.kind in "iub":
                a, dt = a.astype("<i8"), b"i"
            else:
                a, dt = a.astype("<f8"), b"d"
            f.write(name.encode().ljust(32, b"\0"))
            f.write(dt)
            f.write(struct.pack("<i", a.ndim))
            f.write(struct.pack("<%dq" % a.ndim, *a.shape))
            f.write(np.ascontiguousarray(a).tobytes())


def read_rec(path) -> dict:
    out = {}
    with open(path, "rb") as f:
        while True:
            name = f.read(32)
            if len(name) < 32:
                break
            dt = f.read(1)
            (nd,) = struct.unpack("<i", f.read(4))
            shape = struct.unpack("<%dq" % nd, f.read(8 * nd))
            n = int(np.prod(shape)) if nd else 1
            a = np.frombuffer(f.read(8 * n), dtype="<f8" if dt == b"d" else "<i8").reshape(shape)
            out[name.rstrip(b"\0").decode()] = a.copy()
    return out


def run(case, inputs):
    with tempfile.TemporaryDirectory() as d:
        fin, fout = os.path.join(d, "in.rec"), os.path.join(d, "out.rec")
        write_rec(fin, inputs)
        subprocess.run([HARNESS, case, fin, fout], check=True, cwd=d,
                       stdout=subprocess.DEVNULL)
        out = read_rec(fout)
        if os.path.exists(fout + ".step0"):
            out.update(read_rec(fout + ".step0"))
        return out


def run_with_files(case, inputs, files):
    """run() plus the bytes of the files the harness wrote (paths relative to its working
    directory), as uint8 arrays keyed by the given names."""
    with tempfile.TemporaryDirectory() as d:
        fin, fout = os.path.join(d, "in.rec"), os.path.join(d, "out.rec")
        write_rec(fin, inputs)
        subprocess.run([HARNESS, case, fin, fout], check=True, cwd=d, stdout=subprocess.DEVNULL)
        out = read_rec(fout)
        for key, rel in files.items():
            with open(os.path.join(d, rel), "rb") as f:
                out[key] = np.frombuffer(f.read(), dtype=np.uint8).copy()
        return out


def save(name, inputs, outputs, **extra):
    path = os.path.join(HERE, name + ".npz")
    payload = {"in_" + k: np.asarray(v) for k, v in inputs.items()}
    payload.update({"out_" + k: np.asarray(v) for k, v in outputs.items()})
    payload.update({k: np.asarray(v) for k, v in extra.items()})
    np.savez_compressed(path, **payload)
    print("wrote", os.path.relpath(path, ROOT), "%.1f KB" % (os.path.getsize(path) / 1024))


# ---------------------------------------------------------------- helpers
def equilibrium(rho, u):
    """Palabos D3Q19 equilibrium in f-bar form (dynamicsTemplates3D.h:675-678)."""
    rhobar = rho - 1.0
    j = rho[None] * u
    jsq = (j * j).sum(0)
    inv = 1.0 / rho
    f = np.empty((19,) + rho.shape)
    for i in range(19):
        cj = C[i, 0] * j[0] + C[i, 1] * j[1] + C[i, 2] * j[2]
        f[i] = W[i] * (rhobar + 3.0 * cj + inv * (4.5 * cj * cj - 1.5 * jsq))
    return f


def random_state(rng, nx, ny, nz, amp_u=0.03, amp_rho=0.01, noise=2e-4):
    shape = (nz, ny, nx)
    rho = 1.0 + amp_rho * rng.uniform(-1, 1, shape)
    u = amp_u * rng.uniform(-1, 1, (3,) + shape)
    return equilibrium(rho, u) + noise * rng.uniform(-1, 1, (19,) + shape)


def particle_params(model, **kw):
    p = dict(G=0.0, C=1.0, nu_s=1.0, kb=0.0, shear_modulus=0.0, L0=1.0, k_area_global=0.0,
             k_area_local=0.0, k_volume=0.0, vol_desired=1.0, k_bend=0.0, theta0=0.0)
    p.update(kw)
    keys = ["G", "C", "nu_s", "kb", "shear_modulus", "L0", "k_area_global", "k_area_local",
            "k_volume", "vol_desired", "k_bend", "theta0"]
    return np.array([p[k] for k in keys], dtype=np.float64)


# ---------------------------------------------------------------- cases
def case_lbm_periodic():
    rng = np.random.default_rng(101)
    nx, ny, nz = 9, 7, 6
    tau, lam = 0.8, 5.0
    omega = 1 / tau
    omega_in = 1 / (0.5 + lam * (tau - 0.5))
    inp = dict(dims=[nx, ny, nz], omega=[omega, omega_in], walls=0, steps=3,
               fbar=random_state(rng, nx, ny, nz),
               force=1e-3 * rng.uniform(-1, 1, (3, nz, ny, nx)),
               phase=(rng.random((nz, ny, nx)) < 0.4).astype(np.float64))
    out = run("lbm", inp)
    save("lbm_periodic", inp, out)


def case_lbm_shear():
    rng = np.random.default_rng(102)
    nx, ny, nz = 8, 9, 7
    omega = 1 / 0.9
    force = 2e-4 * rng.uniform(-1, 1, (3, nz, ny, nx))
    inp = dict(dims=[nx, ny, nz], omega=[omega, omega], walls=1, U=0.01, steps=4,
               force=force, phase=np.zeros((nz, ny, nx)))
    out = run("lbm", inp)
    save("lbm_shear", inp, out)


def case_lbm_bounceback():
    """Per-cell BounceBack and NoDynamics nodes (defineDynamics) in a periodic box, lambda = 1."""
    rng = np.random.default_rng(103)
    nx, ny, nz = 10, 8, 6
    omega = 1 / 0.85
    ct = np.zeros((nz, ny, nx), dtype=np.int64)
    ct[1:4, 2:5, 3:6] = 1          # a solid block
    ct[2, 0:3, 0] = 1              # solid cells on the periodic seam
    ct[:, :, 8] = 2                # a NoDynamics slab
    ct[4, 5, 8] = 1
    inp = dict(dims=[nx, ny, nz], omega=[omega, omega], walls=0, steps=4,
               fbar=random_state(rng, nx, ny, nz),
               force=1e-3 * rng.uniform(-1, 1, (3, nz, ny, nx)),
               phase=np.zeros((nz, ny, nx)), celltype=ct)
    out = run("lbm", inp)
    save("lbm_bounceback", inp, out)


def case_interp():
    for dirac, dname in ((0, "roma"), (1, "peskin")):
        for per, pname in (((1, 1, 1), "ppp"), ((1, 0, 1), "pwp"), ((1, 0, 0), "pww")):
            rng = np.random.default_rng(200 + 10 * dirac + len(pname) + sum(per))
            nx, ny, nz = 10, 9, 8
            u = 0.05 * rng.uniform(-1, 1, (3, nz, ny, nx))
            npts = 48
            pos = rng.uniform(0, 1, (npts, 3)) * np.array([nx, ny, nz]) - 0.5
            # a few nodes hugging the periodic seams and the non-periodic faces
            pos[:6, 0] = [-0.45, 0.1, 0.7, nx - 1.3, nx - 0.7, nx - 0.55]
            pos[6:12, 1] = [-0.3, 0.2, 0.9, ny - 1.9, ny - 1.2, ny - 0.6]
            pos[12:18, 2] = [-0.2, 0.4, 1.2, nz - 1.6, nz - 1.1, nz - 0.7]
            nforce = rng.uniform(-1, 1, (npts, 3))
            inp = dict(dims=[nx, ny, nz], periodic=list(per), dirac=dirac, u=u, pos=pos, nforce=nforce)
            out = run("interp", inp)
            save("interp_%s_%s" % (dname, pname), inp, out)


def mesh_sets():
    ico_xyz, ico_tri = meshes.icosphere(2, 4.0)
    ef_xyz, ef_tri = meshes.evans_fung(2, 5.0)
    return {"ico2": (ico_xyz, ico_tri), "ef2": (ef_xyz, ef_tri)}


def case_shape():
    for name, (xyz, tri) in mesh_sets().items():
        inp = dict(rest=xyz, tri=tri)
        out = run("shape", inp)
        save("shape_" + name, inp, out)


def deform(rng, xyz, amp):
    """A smooth stretch plus small noise: a prestressed, non-degenerate state."""
    s = np.diag([1.0 + 2 * amp, 1.0 - amp, 1.0 - 0.5 * amp])
    c = xyz.mean(0)
    return (xyz - c) @ s.T + c + 0.02 * amp * rng.uniform(-1, 1, xyz.shape) + np.array([3.1, -2.2, 7.4])


def case_forces():
    sets = mesh_sets()
    rng = np.random.default_rng(303)
    xyz, tri = sets["ico2"]
    ef, eft = sets["ef2"]
    A_ef = None
    cases = []
    cases.append(("capsule_neohookean", xyz, tri, 0, particle_params(0, G=0.01, C=1.0)))
    cases.append(("capsule_skalak", xyz, tri, 1, particle_params(1, G=0.02, C=1.0)))
    shape_out = run("shape", dict(rest=ef, tri=eft))
    A_ef, V_ef = float(shape_out["area"][0]), float(shape_out["volume"][0])
    lmean = float(shape_out["link_length"].mean())
    cases.append(("rbc_wlcpow", ef, eft, 2, particle_params(2, shear_modulus=0.01, L0=lmean, k_area_global=0.5,
                                                             k_area_local=0.2, k_volume=0.7, vol_desired=V_ef,
                                                             k_bend=0.05)))
    cases.append(("skalak_bending", ef, eft, 3, particle_params(3, G=0.01, C=1.0, k_area_global=1.0, k_volume=1.0,
                                                                 vol_desired=V_ef, k_bend=0.01 * 0.01 * A_ef)))
    for name, rest, t, model, prm in cases:
        pos = deform(rng, rest, 0.06)
        inp = dict(rest=rest, tri=t, pos=pos, model=model, params=prm)
        out = run("forces", inp)
        save("forces_" + name, inp, out)


def case_inertia():
    rng = np.random.default_rng(404)
    xyz, tri = meshes.evans_fung(2, 6.0)
    pos = meshes.place(xyz, meshes.random_rotation(rng), (10.3, 12.1, 9.7))
    inp = dict(rest=xyz, tri=tri, pos=pos)
    out = run("inertia", inp)
    save("inertia_ef2", inp, out)


def case_ibm_capsule_shear():
    n = 20
    xyz, tri = meshes.icosphere(2, 4.0)
    tau = 1.0
    nu = (tau - 0.5) / 3
    U = 0.04
    gamma = 2 * U / (n - 1)
    G = nu * gamma * 4.0 / 0.2
    pos = meshes.place(xyz, None, (0.5 * (n - 1) + 0.13, 0.5 * (n - 1) - 0.21, 0.5 * (n - 1) + 0.07))
    inp = dict(dims=[n, n, n], tau=tau, walls=1, U=U, steps=6, rest=xyz, tri=tri, pos=pos, model=1,
               params=particle_params(1, G=G, C=1.0))
    out = run("ibm", inp)
    keep = {k: out[k] for k in ("pos", "vel", "force", "volume", "area", "com", "inertia")}
    keep["u_end"] = out["u_end"]
    keep["fbar_end_planes"] = out["fbar_end"][:, :, [0, 1, n // 2, n - 2, n - 1], :]
    keep["fbar_end_sum"] = out["fbar_end"].sum(axis=(1, 2, 3))
    keep["force_spread"] = out["force_spread"]
    keep["phase_0"], keep["phase_end"] = out["phase_0"], out["phase_end"]
    save("ibm_capsule_shear", inp, keep)


def case_ibm_rbc_periodic():
    n = 16
    xyz, tri = meshes.evans_fung(2, 4.5)
    shape_out = run("shape", dict(rest=xyz, tri=tri))
    A0, V0 = float(shape_out["area"][0]), float(shape_out["volume"][0])
    rng = np.random.default_rng(505)
    pos = meshes.place(deform(rng, xyz, 0.05), meshes.random_rotation(rng), (n - 1.2, 6.3, 0.4))
    G = 0.004
    inp = dict(dims=[n, n, n], tau=1.0, walls=0, steps=5, rest=xyz, tri=tri, pos=pos, model=3,
               params=particle_params(3, G=G, C=1.0, k_area_global=1.0, k_volume=1.0, vol_desired=V0,
                                      k_bend=0.01 * G * A0),
               body=[2e-5, 0.0, 0.0])
    out = run("ibm", inp)
    keep = {k: out[k] for k in ("pos", "vel", "force", "volume", "area", "com", "inertia")}
    keep["u_end"] = out["u_end"]
    keep["fbar_end_sum"] = out["fbar_end"].sum(axis=(1, 2, 3))
    keep["fbar_end_planes"] = out["fbar_end"][:, :, [0, 5, 10], :]
    keep["force_spread"] = out["force_spread"]
    keep["phase_0"], keep["phase_end"] = out["phase_0"], out["phase_end"]
    save("ibm_rbc_periodic", inp, keep)


def case_ibm_capsule_lambda():
    """Viscosity ratio 5 inside a capsule in shear: the voxelized phase enters omega."""
    n = 20
    xyz, tri = meshes.icosphere(2, 4.5)
    tau, U = 0.9, 0.04
    nu = (tau - 0.5) / 3
    G = nu * (2 * U / (n - 1)) * 4.5 / 0.3
    pos = meshes.place(xyz, None, (0.5 * (n - 1) + 0.31, 0.5 * (n - 1) - 0.17, 0.5 * (n - 1) + 0.23))
    inp = dict(dims=[n, n, n], tau=tau, lam=5.0, walls=1, U=U, steps=6, rest=xyz, tri=tri, pos=pos, model=1,
               params=particle_params(1, G=G, C=1.0))
    inp["lambda"] = inp.pop("lam")
    out = run("ibm", inp)
    keep = {k: out[k] for k in ("pos", "vel", "force", "volume", "area", "com")}
    keep["u_end"] = out["u_end"]
    keep["fbar_end"] = out["fbar_end"]
    keep["phase_0"], keep["phase_end"] = out["phase_0"], out["phase_end"]
    save("ibm_capsule_lambda", inp, keep)


def interact_geometry(n=24, radius=3.0, cut_pp=0.6, cut_wall=0.5):
    """Two capsules almost touching along x and a pair of y plates just outside them, placed so
    that every vertex pair within the cutoff lies in cells the reference's grid search pairs
    (checked with the oracle: the grid search and the all-pairs search give the same forces)."""
    from oracle import oracle as O

    xyz, tri = meshes.icosphere(2, radius)
    L = O.lattice((n, n, n), (1, 1, 1))
    pot = O.potential("spring", cut_pp, 0.0, 1.0)
    a = xyz + np.array([8.3, 10.2, 11.6])
    owner = np.repeat([0, 1], xyz.shape[0])
    gap_x = a[:, 0].max() - a[:, 0].min()
    for dy in np.linspace(-0.45, 0.45, 19):
        for dz in np.linspace(-0.45, 0.45, 19):
            for d in (0.25, 0.3, 0.35):
                b = xyz + np.array([8.3 + gap_x + d, 10.2 + dy, 11.6 + dz])
                pos = np.concatenate([a, b])
                f_all = O.pp_forces(L, pot, pos, owner)
                f_grid = O.pp_forces(L, pot, pos, owner, grid=True)
                n_pairs = int((np.abs(f_all).sum(axis=1) > 0).sum())
                if n_pairs >= 6 and np.abs(f_all - f_grid).max() <= 1e-15 * np.abs(f_all).max():
                    lo = a[:, 1].min() - 0.6 * cut_wall
                    hi = max(a[:, 1].max(), b[:, 1].max()) + 0.8 * cut_wall
                    return xyz, tri, a, b, (lo, hi)
    raise RuntimeError("no configuration where the grid search finds every pair")


def case_interact():
    """Particle-particle (PPPotentialForce) and wall (WallInteraction on parallel y plates)
    forces of one IB step on a lattice at rest: Morse pairs + spring walls, and the reverse."""
    n = 24
    xyz, tri, a, b, wy = interact_geometry(n)
    prm = particle_params(1, G=1e-3, C=1.0)
    for name, ppk, ppq, wk, wq in (("interact_morse_spring", 1, [0.6, 3.0, 2e-3], 2, [0.5, 0.0, 1e-2]),
                                   ("interact_spring_morse", 2, [0.6, 0.0, 5e-3], 1, [0.5, 2.0, 1e-3])):
        inp = dict(dims=[n, n, n], rest=xyz, tri=tri, pos_a=a, pos_b=b, model=1, params=prm, pp_kind=ppk,
                   pp_params=ppq, wall_kind=wk, wall_params=wq, wall_y=list(wy))
        out = run("interact", inp)
        assert np.abs(out["force_a"]).max() > 1e-4 and np.abs(out["force_b"]).max() > 1e-4
        save(name, inp, {"force_a": out["force_a"], "force_b": out["force_b"]})
    # the wall interaction on a pipe along x (rbc_in_pipe.cpp:154-163) through the capsules' axis,
    # its wall just outside the outermost vertices
    y0, z0 = 10.2, 11.6
    rmax = max(np.hypot(a[:, 1] - y0, a[:, 2] - z0).max(), np.hypot(b[:, 1] - y0, b[:, 2] - z0).max())
    inp = dict(dims=[n, n, n], rest=xyz, tri=tri, pos_a=a, pos_b=b, model=1, params=prm, pp_kind=1,
               pp_params=[0.6, 3.0, 2e-3], wall_kind=2, wall_params=[0.5, 0.0, 1e-2], wall_y=list(wy),
               pipe=[y0, z0, rmax + 0.3])
    out = run("interact", inp)
    save("interact_pipe_wall", inp, {"force_a": out["force_a"], "force_b": out["force_b"]})


def case_lbm_pipe():
    """Body-force flow in a pipe along x with the reference's first-order pipe walls
    (BounceBack outside PipeBoundary, NoDynamics beyond radius + 1), periodic box."""
    inp = dict(dims=[12, 21, 21], pipe=[10.0, 10.2, 7.3], omega=1.0 / 0.8, body=[1e-4, 0.0, 0.0], steps=40)
    out = run("pipe", inp)
    save("lbm_pipe", inp, {"mask": out["mask"], "fbar_end": out["fbar_end"], "u_end": out["u_end"]})


def case_lbm_pipe_guo():
    """The same pipe flow with the reference's second-order walls (GuoRigidWallBoundary)."""
    inp = dict(dims=[12, 21, 21], pipe=[10.0, 10.2, 7.3], omega=1.0 / 0.8, body=[1e-4, 0.0, 0.0], steps=40)
    out = run("pipe_guo", inp)
    save("lbm_pipe_guo", inp, {k: out[k] for k in ("wall_loc", "wall_dir", "wall_delta", "fbar_0", "fbar_1",
                                                     "fbar_end", "u_end")})


def case_ibm_pipe():
    """A prestressed capsule next to the wall of a pipe with second-order walls and body-force
    flow: the near-wall TopHat blend of interpolation and spreading, 8 coupled steps."""
    n, R = 21, 8.3
    rng = np.random.default_rng(606)
    xyz, tri = meshes.icosphere(2, 2.6)
    pos = meshes.place(deform(rng, xyz, 0.04), meshes.random_rotation(rng), (7.5, 10.0 + 5.0, 10.2 + 0.3))
    inp = dict(dims=[16, n, n], pipe=[10.0, 10.2, R], tau=1.0, body=[2e-5, 0.0, 0.0], steps=8, rest=xyz, tri=tri,
               pos=pos, model=1, params=particle_params(1, G=2e-3, C=1.0))
    out = run("ibm_pipe", inp)
    keep = {k: out[k] for k in ("pos", "vel", "force")}
    keep["fbar_end_planes"] = out["fbar_end"][:, :, :, [0, 7]]
    keep["fbar_end_sum"] = out["fbar_end"].sum(axis=(1, 2, 3))
    keep["force_spread"] = out["force_spread"][:, :, :, 4:12]  # the capsule's x range
    save("ibm_pipe", inp, keep)


def case_reflect():
    """DeformableParticle3D::move_vertices with a pipe boundary: vertices whose step crosses
    the wall are reflected about the wall normal at the crossing."""
    rng = np.random.default_rng(707)
    xyz, tri = meshes.icosphere(1, 2.0)
    pos = meshes.place(xyz, None, (5.0, 10.0 + 5.9, 10.2 + 0.4))
    vel = np.array([0.05, 1.0, 0.1]) + 0.05 * rng.standard_normal(pos.shape)
    inp = dict(pipe=[10.0, 10.2, 8.3], rest=xyz, tri=tri, pos=pos, vel=vel, model=1,
               params=particle_params(1, G=1e-3, C=1.0))
    out = run("reflect", inp)
    r_new = np.hypot(out["pos"][:, 1] - 10.0, out["pos"][:, 2] - 10.2)
    r_free = np.hypot(pos[:, 1] + vel[:, 1] - 10.0, pos[:, 2] + vel[:, 2] - 10.2)
    assert (r_free > 8.3).sum() >= 3 and r_new.max() <= 8.3 + 1e-12
    save("reflect_pipe", inp, {"pos": out["pos"]})


def case_plb():
    """The reference's particle output formats: save_checkpoint (a text header naming one
    binary file per rank holding each particle's pack), write_particles_as_vtk (one VTU file
    per particle, appended raw data) and write_lightweight_particle_data (text), for two
    capsules of either shear law and a red blood cell on a second shape."""
    rng = np.random.default_rng(808)
    ico, ico_t = meshes.icosphere(1, 3.0)
    ef, ef_t = meshes.evans_fung(1, 4.0)
    shape_out = run("shape", dict(rest=ef, tri=ef_t))
    V_ef = float(shape_out["volume"][0])
    lmean = float(shape_out["link_length"].mean())
    specs = [(0, 0, particle_params(0, G=0.01, C=1.0, kb=0.002, nu_s=0.3), (6.2, 7.1, 8.3)),
             (1, 0, particle_params(1, G=0.02, C=2.5), (14.5, 6.0, 12.2)),
             (2, 1, particle_params(2, shear_modulus=0.01, L0=lmean, k_area_global=0.5, k_area_local=0.2,
                                    k_volume=0.7, vol_desired=V_ef, k_bend=0.05, theta0=0.1), (9.0, 15.0, 7.0))]
    pos, vel, frc = [], [], []
    for model, shape, prm, centre in specs:
        rest = ico if shape == 0 else ef
        p = meshes.place(deform(rng, rest, 0.05), meshes.random_rotation(rng), centre)
        pos.append(p)
        vel.append(1e-3 * rng.standard_normal(p.shape))
        frc.append(1e-4 * rng.standard_normal(p.shape))
    inp = dict(dims=np.array([24, 24, 24]), rest=ico, tri=ico_t, rest_b=ef, tri_b=ef_t,
               models=np.array([s[0] for s in specs]), shapes=np.array([s[1] for s in specs]),
               params=np.stack([s[2] for s in specs]), pos=np.concatenate(pos), vel=np.concatenate(vel),
               force=np.concatenate(frc), iter=1234)
    files = {"file_header": "out/ckpt.plb", "file_rank0": "out/ckpt/0.plb", "file_light": "out/objsP0-1234.txt"}
    files.update({"file_vtu%d" % k: "out/obj%d-1234.vtu" % k for k in range(len(specs))})
    out = run_with_files("plb", inp, files)
    save("plb_particles", inp, out)


def case_lattice_plb():
    """parallelIO::save of a lattice with random populations, forces and phase: the default
    one-block lattice and the same data on 3 x 2 x 1 blocks (a multi-rank run's layout).  The
    reference's parallelIO::load reads the oracle's restatement of the one-block files back."""
    from oracle import oracle as O

    rng = np.random.default_rng(909)
    nx, ny, nz = 7, 5, 4
    f = random_state(rng, nx, ny, nz)
    F = 1e-4 * rng.standard_normal((3, nz, ny, nx))
    ph = (rng.uniform(size=(nz, ny, nx)) > 0.5).astype(np.float64)
    inp = dict(dims=np.array([nx, ny, nz]), fbar=f, force=F, phase=ph, blocks=np.array([3, 2, 1]))
    out = run_with_files("lattice_save", inp, {"file_xml": "out/ckpt.plb", "file_dat": "out/ckpt.dat",
                                               "file_blocks_xml": "out/blocks.plb", "file_blocks_dat": "out/blocks.dat"})
    assert int(out["nblocks"][0]) == 6
    # the reference reads the oracle's files
    xml, dat = O.plb_lattice_files("ckpt", f, F, ph)
    with tempfile.TemporaryDirectory() as d:
        os.makedirs(os.path.join(d, "in"))
        with open(os.path.join(d, "in", "ckpt.plb"), "w") as fh:
            fh.write(xml)
        with open(os.path.join(d, "in", "ckpt.dat"), "wb") as fh:
            fh.write(dat)
        fin, fout = os.path.join(d, "in.rec"), os.path.join(d, "out.rec")
        write_rec(fin, dict(dims=np.array([nx, ny, nz])))
        subprocess.run([HARNESS, "lattice_load", fin, fout], check=True, cwd=d, stdout=subprocess.DEVNULL)
        back = read_rec(fout)
    assert np.array_equal(back["fbar_loaded"], f) and np.array_equal(back["force_loaded"], F)
    assert np.array_equal(back["phase_loaded"], ph)
    save("lattice_plb", inp, out)


def case_calibrate():
    """RBC shape calibration (progs/common/calibrate_rbc_shape.h): create_rbc_params on a rotated
    ellipsoid mesh, shrink_rbc_volume to 65 % of its volume (it flattens into a disc), minor axis
    onto z.  The moduli and damping keep the explicit relaxation contracting, so that rounding
    differences do not grow over the 801 iterations."""
    rng = np.random.default_rng(5)
    xyz, tri = meshes.icosphere(2, 3.9)
    xyz = (xyz * np.array([1.15, 1.0, 0.85])) @ meshes.random_rotation(rng).T
    inp = dict(rest=xyz, tri=tri, moduli=np.array([1e-3, 0.1, 4e-4]), vol_frac=0.65, n_it=400, damping=0.05)
    out = run("calibrate", inp)
    short = run("calibrate", dict(inp, n_it=5))  # 11 iterations
    out["short_shrunk"] = short["shrunk"]
    save("calibrate_rbc", inp, out)


def case_initial():
    """The random initial placement of progs/common/create_particles.h: two particle types at 20 %
    scale (radius 0.2 R + 1) in a pipe of radius 12 (the driver's pipe radius - 1.5), seeded."""
    inp = dict(box=np.array([0, 79, 0, 29, 0, 29]), pipe=np.array([14.5, 14.5, 12.0]), counts=np.array([60, 25]),
               radii=np.array([0.2 * 7.8 + 1.0, 0.2 * 4.0 + 1.0]), max_radius=0.2 * 7.8 + 1.0, seed=12345)
    out = run("initial", inp)
    assert out["pos"].shape == (85, 3)
    save("initial_distribution", inp, out)


def case_coprocessor():
    """Palabos' example co-processor (D3Q19ExampleCoProcessor3D, BGK): a seeded 14 x 11 x 9 block
    of f-bar in the CoProcessor3D byte order (19 populations per cell, z fastest, x slowest)
    sent, collided and streamed twice, received; the one-cell outer layer is undefined by the
    interface (coProcessor3D.h:105-107)."""
    rng = np.random.default_rng(21)
    nx, ny, nz = 14, 11, 9
    rho = 1.0 + rng.uniform(-0.02, 0.02, (nx, ny, nz))
    u = rng.uniform(-0.03, 0.03, (nx, ny, nz, 3))
    j = rho[..., None] * u
    jsq = (j * j).sum(-1)
    fbar = np.empty((nx, ny, nz, 19))
    for i in range(19):  # BGK equilibrium plus a seeded non-equilibrium part
        cj = C[i, 0] * j[..., 0] + C[i, 1] * j[..., 1] + C[i, 2] * j[..., 2]
        fbar[..., i] = W[i] * ((rho - 1.0) + 3 * cj + (4.5 * cj * cj - 1.5 * jsq) / rho)
    fbar += rng.uniform(-1e-3, 1e-3, fbar.shape) * W[None, None, None, :]
    inp = dict(dims=np.array([nx, ny, nz]), omega=1.0 / 0.83, steps=2, data=fbar)
    out = run("coprocessor", inp)
    save("coprocessor_bgk", inp, out)



# ---------------------------------------------------------------- growth of the initial distribution
# A pipe along x through (0, 0) of radius 7.5 and length 24 on the lattice of
# PipeBoundary::get_bounding_box(2) (Boundary.h:141-146), as progs/rbc_in_pipe_distribution sets it up.
GROW_BOX = np.array([0, 24, -9, 9, -9, 9])
GROW_PIPE = np.array([0.0, 0.0, 7.5, 24.0])


def growth_shapes():
    """Two particle types: a sphere of radius 2.5 and an oblate ellipsoid (162 vertices each)."""
    s0 = meshes.icosphere(2, 2.5)
    x1, t1 = meshes.icosphere(2, 2.8)
    return [s0, (x1 * np.array([1.25, 1.25, 0.6]), t1)]


def shape_radius(xyz):
    """ParticleShape::compute_bounding_volumes (ParticleShape.hh:361-383)."""
    r = 0.0
    for v in xyz:
        d = v[0] * v[0] + v[1] * v[1] + v[2] * v[2]
        if d > r:
            r = d
    return float(np.sqrt(r))


def case_create():
    """The reference's own create_particles (progs/common/create_particles.h) for 8 spheres and 3
    ellipsoids in the pipe: placement at 20 % scale, 40001 growth iterations of rigid copies
    under spring collisions with the pipe wall at radius 6, capsules placed at the result."""
    inp = dict(box=GROW_BOX, pipe=GROW_PIPE, counts=np.array([8, 3]), seed=7)
    for t, (x, tri) in enumerate(growth_shapes()):
        inp["rest%d" % t], inp["tri%d" % t] = x, tri
    out = run("create", inp)
    assert int(out["count"][0]) == 11
    save("create_particles_pipe", inp, out)


def case_grow():
    """The growth loop of create_particles from the reference's own random placement of the same
    call (seed 7), the scale reaching 1 after 300 iterations: states after 1, 2, 11 and 301
    iterations."""
    shapes = growth_shapes()
    radii = np.array([0.2 * shape_radius(x) + 1.0 for x, _ in shapes])
    counts = np.array([8, 3])
    init = run("initial", dict(box=GROW_BOX, pipe=np.array([0.0, 0.0, 6.0]), counts=counts, radii=radii,
                               max_radius=radii.max(), seed=7))
    inp = dict(box=GROW_BOX, wall=np.array([0.0, 0.0, 6.0]), pot=np.array([1.0, 5e-2]), growth=np.array([0.2, 1.0, 0.1]),
               n_it=300, ntypes=2, shape=np.repeat(np.arange(2), counts), com=init["pos"], quat=init["quat"],
               dump=np.array([1, 2, 11, 301]))
    for t, (x, tri) in enumerate(shapes):
        inp["rest%d" % t], inp["tri%d" % t] = x, tri
    out = run("grow", inp)
    save("grow_pipe", inp, out)

CASES = [case_lbm_periodic, case_lbm_shear, case_lbm_bounceback, case_interp, case_shape, case_forces, case_inertia,
         case_ibm_capsule_shear, case_ibm_rbc_periodic, case_ibm_capsule_lambda, case_interact, case_lbm_pipe, case_lbm_pipe_guo, case_ibm_pipe,
         case_reflect, case_plb, case_lattice_plb, case_calibrate, case_initial, case_coprocessor,
         case_create, case_grow]

if __name__ == "__main__":
    if not os.path.exists(HARNESS):
        sys.exit("build the reference harness first: make -C oracle ref REF=<reference checkout>")
    sel = sys.argv[1:]
    for fn in CASES:
        if not sel or fn.__name__.replace("case_", "") in sel:
            fn()
