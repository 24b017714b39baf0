"""Wall-interaction decorators and particle-particle interaction forces on the CUDA path.

Against the reference fixtures (two capsules almost touching, parallel y plates: Morse pairs
with spring walls and the reverse) and against the oracle's all-pairs search on a dense
periodic packing where pairs cross the periodic faces and cells of every offset.  FP64 forces
agree to 1e-12 of the largest component (FMA contraction, exp and the summation order).
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import golden

pytestmark = pytest.mark.gpu

bib = pytest.importorskip("biblbm_gb300")
from biblbm_gb300 import meshes  # noqa: E402


@pytest.fixture(scope="module")
def ctx():
    c = bib.Context(0)
    yield c
    c.close()


def potential(kind, q):
    return bib.MorsePotential(q[0], q[1], q[2]) if int(kind) == 1 else bib.SpringPotential(q[0], q[2])


@pytest.mark.parametrize("name", ["interact_morse_spring", "interact_spring_morse", "interact_pipe_wall"])
@pytest.mark.parametrize("spread,storage", [("atomic", "f64"), ("deterministic", "f64"), ("atomic", "f32")])
def test_interaction_forces_match_reference(ctx, name, spread, storage):
    d = golden(name)
    n = int(d["in_dims"][0])
    lat = ctx.add_domain(n, n, n, periodic=(1, 1, 1), omega=1.0, storage=storage)
    shapes = bib.ParticleShapeLibrary(ctx)
    sid = shapes.store_mesh(d["in_rest"], d["in_tri"], "c")
    fsi = bib.ImmersedBoundaryDynamics3D(lat, shapes, spread=spread)
    pa = fsi.add_particle(sid, "capsule_skalak", d["in_params"], d["in_pos_a"])
    pb = fsi.add_particle(sid, "capsule_skalak", d["in_params"], d["in_pos_b"])
    if "in_pipe" in d.files:  # WallInteraction on a PipeBoundary along x
        fsi.add_pipe_wall_interaction(potential(d["in_wall_kind"], d["in_wall_params"]), *d["in_pipe"])
    else:
        lo, hi = d["in_wall_y"]
        fsi.add_wall_interaction(potential(d["in_wall_kind"], d["in_wall_params"]), 1, lo, hi)
    fsi.add_pp_force(potential(d["in_pp_kind"], d["in_pp_params"]))
    fsi.ibm_step()
    fa, fb = fsi.get_particle(pa)["force"], fsi.get_particle(pb)["force"]
    scale = max(np.abs(d["out_force_a"]).max(), np.abs(d["out_force_b"]).max())
    tol = 1e-12 if storage == "f64" else 1e-6
    assert np.abs(fa - d["out_force_a"]).max() <= tol * scale
    assert np.abs(fb - d["out_force_b"]).max() <= tol * scale


def packed_capsules(n=20, k=3, radius=3.1, seed=8):
    """k^3 capsules on a jittered lattice that fills a periodic box, closer than the cutoff."""
    rng = np.random.default_rng(seed)
    xyz, tri = meshes.icosphere(2, radius)
    step = n / k
    pos = []
    for i in range(k):
        for j in range(k):
            for m in range(k):
                c = (np.array([i, j, m]) + 0.5) * step + rng.uniform(-0.2, 0.2, 3) + np.array([6.3, 0.0, 0.0])
                pos.append(meshes.place(xyz, meshes.random_rotation(rng), c))
    return xyz, tri, pos


@pytest.mark.parametrize("kind", ["spring", "morse"])
def test_dense_packing_against_oracle(ctx, kind):
    """27 capsules packed so that neighbours overlap the cutoff across the periodic faces,
    spring or Morse pairs, one wall pair on z: forces of one step and positions after 5."""
    n = 20
    xyz, tri, pos = packed_capsules(n)
    prm = bib.membrane_params(G=2e-3, C=1.0)
    pot_pp = ("spring", 1.0, 0.0, 2e-3) if kind == "spring" else ("morse", 1.0, 1.5, 1e-4)
    pot_w = ("morse", 0.8, 2.0, 1e-4)
    L = O.lattice((n, n, n), (1, 1, 1), "bgk_guo_vof", 1.0, 1.0)
    S = O.System(L, "roma", -1.0)
    sid = S.add_shape(xyz, tri)
    for p in pos:
        S.add_particle(sid, "capsule_skalak", prm, p)
    S.add_wall_interaction(O.potential(*pot_w), 2, -0.4, 20.4)
    S.add_pp_interaction(O.potential(*pot_pp))
    lat = ctx.add_domain(n, n, n, periodic=(1, 1, 1), omega=1.0)
    shapes = bib.ParticleShapeLibrary(ctx)
    gsid = shapes.store_mesh(xyz, tri, "c")
    fsi = bib.ImmersedBoundaryDynamics3D(lat, shapes)
    pids = [fsi.add_particle(gsid, "capsule_skalak", prm, p) for p in pos]
    fsi.add_wall_interaction(bib.MorsePotential(*pot_w[1:]), 2, -0.4, 20.4)
    fsi.add_pp_force(bib.SpringPotential(pot_pp[1], pot_pp[3]) if kind == "spring"
                     else bib.MorsePotential(*pot_pp[1:]))
    S.step(1)
    fsi.step(1)
    fo = np.concatenate([S.particle(i)["force"] for i in range(len(pos))])
    fg = np.concatenate([fsi.get_particle(i)["force"] for i in pids])
    # the packing is dense enough that many vertices feel pairs, some across the periodic faces
    pp_only = O.pp_forces(L, O.potential(*pot_pp), np.concatenate(pos), np.repeat(np.arange(len(pos)), xyz.shape[0]))
    assert (np.abs(pp_only).sum(axis=1) > 0).sum() > 100
    assert np.abs(fg - fo).max() <= 1e-12 * np.abs(fo).max()
    S.step(4)
    fsi.step(4)
    po = np.concatenate([S.particle(i)["pos"] for i in range(len(pos))])
    pg = np.concatenate([fsi.get_particle(i)["pos"] for i in pids])
    assert np.abs(pg - po).max() < 1e-11


def test_interaction_arguments_are_checked(ctx):
    lat = ctx.add_domain(16, 16, 16, periodic=(1, 1, 1), omega=1.0)
    shapes = bib.ParticleShapeLibrary(ctx)
    fsi = bib.ImmersedBoundaryDynamics3D(lat, shapes)
    with pytest.raises(bib.BibError, match="cutoff"):
        fsi.add_pp_force(bib.SpringPotential(1.2, 1e-3))  # beyond Roma's half support - 1/2
    with pytest.raises(bib.BibError):
        fsi.add_wall_interaction(bib.SpringPotential(0.5, 1e-3), 1, 5.0, 2.0)
    fsi.add_pp_force(bib.SpringPotential(0.8, 1e-3))
    rest, tri = meshes.icosphere(1, 3.0)
    sid = shapes.store_mesh(rest, tri, "b")
    fsi.add_particle(sid, "capsule_skalak", bib.membrane_params(G=1e-3), rest + 8.0)
    lat2 = ctx.add_domain(16, 16, 16, periodic=(1, 1, 1), omega=1.0)
    with pytest.raises(bib.BibError, match="particle-particle"):
        b = bib.Batch(ctx, [lat, lat2])
        b.step(2)
    fsi.clear_interactions()
    fsi.step(2)
