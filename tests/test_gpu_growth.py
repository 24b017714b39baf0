"""The reference's collision grid and the growth stage of the initial distribution on the GPU
(bib_grow_particles, bib_place_particle, BIB_PAIR_SEARCH_GRID) against the oracle, which matches
the reference's own runs bit for bit (tests/test_oracle_growth.py).

The grid forces follow the reference's accumulation order without contraction: one force step
equals the oracle's bit for bit.  The rigid-body move uses CUDA's sin / cos for the rotation, so
longer runs agree to rounding.
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


def fixture_shapes(ctx, d):
    lib = bib.ParticleShapeLibrary(ctx)
    return lib, [lib.store_mesh(d["in_rest%d" % t], d["in_tri%d" % t], "type%d" % t) for t in range(2)]


def oracle_grow(d, shapes, com, quat, it_end, **kw):
    gr = d["in_growth"]
    args = dict(pot=d["in_pot"], initial_scale=gr[0], density=gr[1], damping=gr[2], n_it=int(d["in_n_it"]))
    args.update(kw)
    g = O.growth(d["in_box"], d["in_wall"], it_end=it_end, **args)
    return O.grow_particles(g, shapes, d["in_shape"], com, quat)


def test_grid_forces_bit_for_bit_with_contacts(ctx):
    """Full-size rigid copies at the packed state the reference reached after 301 iterations: the
    spring forces between vertices (grid search, periodic x) and against the wall at radius 6
    equal the oracle's exactly."""
    d = golden("grow_pipe")
    _, sids = fixture_shapes(ctx, d)
    shapes = [(d["in_rest%d" % t], d["in_tri%d" % t]) for t in range(2)]
    com, quat = d["out_com_301"], d["out_quat_301"]
    sh = np.array(sids, dtype=np.int32)[d["in_shape"]]
    c, q, pos, frc = bib.grow_particles(ctx, sh, com, quat, d["in_box"], wall=d["in_wall"], initial_scale=1.0,
                                        n_it=300, it_end=1, vertices=True)
    oc, oq, opos, ofrc = oracle_grow(d, shapes, com, quat, 1, initial_scale=1.0)
    assert (np.abs(ofrc).sum(1) > 0).sum() > 100  # many contacts
    assert np.array_equal(frc, ofrc)
    assert np.abs(c - oc).max() < 1e-13 and np.abs(q - oq).max() < 1e-13
    assert np.abs(pos - opos).max() < 1e-12


def test_grid_forces_all_periodic_bit_for_bit(ctx):
    """27 rigid spheres packed in a box periodic on all three axes, no wall: the face, edge and
    corner layer passes of the grid pair vertices across the periodic faces."""
    rng = np.random.default_rng(11)
    xyz, tri = meshes.icosphere(2, 3.05)
    n, k = 20, 3
    com = np.array([(np.array([i, j, m]) + 0.5) * (n / k) + rng.uniform(-0.25, 0.25, 3)
                    for i in range(k) for j in range(k) for m in range(k)])
    quat = rng.normal(size=(k ** 3, 4))
    quat /= np.linalg.norm(quat, axis=1)[:, None]
    box = np.array([0, n - 1, 0, n - 1, 0, n - 1])
    lib = bib.ParticleShapeLibrary(ctx)
    sid = lib.store_mesh(xyz, tri, "s")
    sh = np.full(k ** 3, sid, dtype=np.int32)
    _, _, _, frc = bib.grow_particles(ctx, sh, com, quat, box, wall=None, periodic=(1, 1, 1), initial_scale=1.0,
                                      n_it=10, it_end=1, vertices=True)
    g = O.growth(box, None, (1, 1, 1), initial_scale=1.0, n_it=10, it_end=1)
    _, _, opos, ofrc = O.grow_particles(g, [(xyz, tri)], np.zeros(k ** 3, dtype=np.int32), com, quat)
    touched = np.abs(ofrc).sum(1) > 0
    assert touched.sum() > 200
    # some pairs only meet across a periodic face
    near_face = (opos < 1.0) | (opos > n - 2.0)
    assert (touched & near_face.any(1)).any()
    assert np.array_equal(frc, ofrc)


@pytest.mark.parametrize("k", [1, 2, 11, 301])
def test_growth_loop_against_reference(ctx, k):
    """The growth loop from the reference's own placement, scale reaching 1 after 300 iterations."""
    d = golden("grow_pipe")
    _, sids = fixture_shapes(ctx, d)
    sh = np.array(sids, dtype=np.int32)[d["in_shape"]]
    gr = d["in_growth"]
    c, q, pos, frc = bib.grow_particles(ctx, sh, d["in_com"], d["in_quat"], d["in_box"], wall=d["in_wall"],
                                        min_dist=d["in_pot"][0], strength=d["in_pot"][1], initial_scale=gr[0],
                                        density=gr[1], damping=gr[2], n_it=int(d["in_n_it"]), it_end=k, vertices=True)
    if k <= 11:  # no contact yet: no rotation, the arithmetic is the reference's exactly
        assert np.array_equal(c, d["out_com_%d" % k]) and np.array_equal(q, d["out_quat_%d" % k])
        assert np.array_equal(pos, d["out_pos_%d" % k]) and np.array_equal(frc, d["out_force_%d" % k])
    else:
        assert np.abs(c - d["out_com_%d" % k]).max() < 1e-12
        assert np.abs(q - d["out_quat_%d" % k]).max() < 1e-12
        assert np.abs(pos - d["out_pos_%d" % k]).max() < 1e-11
        f_ref = d["out_force_%d" % k]
        assert np.abs(frc - f_ref).max() < 1e-9 * np.abs(f_ref).max()


def test_create_particles_against_reference(ctx):
    """The reference's create_particles end to end: 8 spheres and 3 ellipsoids, srand(7)
    placement, 40001 growth iterations on the GPU, capsules placed at the result."""
    d = golden("create_particles_pipe")
    lib, sids = fixture_shapes(ctx, d)
    parts = bib.create_particles(lib, [(sids[0], int(d["in_counts"][0])), (sids[1], int(d["in_counts"][1]))],
                                 d["in_box"], d["in_pipe"][:3], int(d["in_seed"]))
    pos = np.concatenate([p for _, p in parts])
    err = np.abs(pos - d["out_pos"]).max()
    assert err < 1e-8, err
    assert [s for s, _ in parts] == [sids[0]] * 8 + [sids[1]] * 3


def test_place_particle_matches_oracle(ctx):
    rng = np.random.default_rng(2)
    xyz, tri = meshes.icosphere(2, 2.7)
    xyz = xyz * np.array([1.2, 1.0, 0.7]) + np.array([0.3, -0.2, 0.1])
    lib = bib.ParticleShapeLibrary(ctx)
    sid = lib.store_mesh(xyz, tri, "e")
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    com = np.array([4.5, -1.25, 2.0])
    assert np.array_equal(bib.place_particle(ctx, sid, com, q), O.place_particle(xyz, tri, com, q))


def test_coupled_step_with_the_reference_grid_search(ctx):
    """A coupled IB step with SpringPotential(grid=True) particle-particle forces on a dense
    periodic packing: the vertex forces equal the oracle's grid search (to the membrane forces'
    rounding) and differ from the every-pair search where the grid misses pairs."""
    n = 20
    rng = np.random.default_rng(8)
    xyz, tri = meshes.icosphere(2, 3.1)
    step = n / 3
    pos = [meshes.place(xyz, meshes.random_rotation(rng),
                        (np.array([i, j, m]) + 0.5) * step + rng.uniform(-0.2, 0.2, 3) + np.array([6.3, 0.0, 0.0]))
           for i in range(3) for j in range(3) for m in range(3)]
    prm = bib.membrane_params(G=2e-3, C=1.0)
    forces = {}
    for grid in (True, False):
        L = O.lattice((n, n, n), (1, 1, 1), "bgk_guo_vof", 1.0, 1.0)
        S = O.System(L, "roma", -1.0)
        osid = S.add_shape(xyz, tri)
        for p in pos:
            S.add_particle(osid, "capsule_skalak", prm, p)
        S.add_pp_interaction(O.potential("spring", 1.0, 0.0, 2e-3), grid=grid)
        lat = ctx.add_domain(n, n, n, periodic=(1, 1, 1), omega=1.0)
        shapes = bib.ParticleShapeLibrary(ctx)
        gsid = shapes.store_mesh(xyz, tri, "c")
        fsi = bib.ImmersedBoundaryDynamics3D(lat, shapes)
        pids = [fsi.add_particle(gsid, "capsule_skalak", prm, p) for p in pos]
        fsi.add_pp_force(bib.SpringPotential(1.0, 2e-3, grid=grid))
        S.step(1)
        fsi.step(1)
        fo = np.concatenate([S.particle(i)["force"] for i in range(len(pos))])
        fg = np.concatenate([fsi.get_particle(i)["force"] for i in pids])
        assert np.abs(fg - fo).max() <= 1e-12 * np.abs(fo).max()
        forces[grid] = fg
        del fsi, lat
    assert np.abs(forces[True] - forces[False]).max() > 1e-6 * np.abs(forces[False]).max()


def test_growth_arguments_are_checked(ctx):
    lib = bib.ParticleShapeLibrary(ctx)
    xyz, tri = meshes.icosphere(1, 2.0)
    sid = lib.store_mesh(xyz, tri, "b")
    box = np.array([0, 15, -8, 8, -8, 8])
    com, quat = np.array([[5.0, 0.0, 0.0]]), np.array([[1.0, 0.0, 0.0, 0.0]])
    with pytest.raises(bib.BibError):
        bib.grow_particles(ctx, [sid], com, quat, box, wall=(0, 0, 6), min_dist=1.5)
    with pytest.raises(bib.BibError):
        bib.grow_particles(ctx, [sid + 7], com, quat, box, wall=(0, 0, 6))
    with pytest.raises(bib.BibError):
        bib.grow_particles(ctx, [sid], com, quat, np.array([0, 0, -8, 8, -8, 8]), wall=(0, 0, 6))
    with pytest.raises(bib.BibError):
        bib.grow_particles(ctx, [sid], np.array([[np.nan, 0, 0]]), quat, box, wall=(0, 0, 6))
    lat = ctx.add_domain(16, 16, 16, periodic=(1, 1, 1), omega=1.0)
    fsi = bib.ImmersedBoundaryDynamics3D(lat, lib)
    fsi.add_pp_force(bib.SpringPotential(0.8, 1e-3, grid=True))
    with pytest.raises(bib.BibError, match="one pair search"):
        fsi.add_pp_force(bib.SpringPotential(0.8, 1e-3))
