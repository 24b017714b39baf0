"""Batched lockstep stepping (several lattices, one launch per kernel for all of them)
against stepping every lattice on its own through bib_step.

The batched kernels do the same per-cell and per-vertex arithmetic; only the order of the
atomic additions in spreading and in the membrane accumulation may differ, so FP64
lattices agree to 1e-13 relative (positions) / 1e-15 absolute (populations)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

bib = pytest.importorskip("biblbm_gb300")
from biblbm_gb300 import meshes, workloads  # noqa: E402


@pytest.fixture(scope="module")
def ctx():
    c = bib.Context(0)
    yield c
    c.close()


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


def capsule_instance(ctx, n, level, storage="f64", Ca=0.1, seed=0, fd=True, lam=1.0):
    """Capsule in shear (periodic x, z; FD velocity walls on y) of edge n, radius n/6; lam != 1: a
    viscosity ratio, with the membranes voxelized into the phase field every step."""
    U = 0.01
    radius = n / 6.0
    wall_u = [[-U, 0, 0], [U, 0, 0], [0, 0, 0], [0, 0, 0]]
    phase_kw = {} if lam == 1.0 else dict(use_phase=True, omega_inner=1.0 / (0.5 + lam * 0.5))
    if fd:
        lat = ctx.add_domain(n, n, n, periodic=(1, 0, 1), omega=1.0, wall_y="fd_velocity", wall_u=wall_u,
                             storage=storage, **phase_kw)
        y = np.arange(n)
        u0 = np.zeros((3, n, n, n))
        u0[0] = (U * (2.0 * y / (n - 1) - 1))[None, :, None]
        lat.initialize_at_equilibrium(None, u0)
    else:
        lat = ctx.add_domain(n, n, n, periodic=(1, 1, 1), omega=1.0, storage=storage, body_force=(1e-5, 0, 0),
                             **phase_kw)
    rest, tri = meshes.icosphere(level, radius)
    rng = np.random.default_rng(seed)
    c = 0.5 * (n - 1) + rng.uniform(-0.5, 0.5, 3)
    shapes = bib.ParticleShapeLibrary(ctx)
    sid = shapes.store_mesh(rest, tri, "capsule")
    fsi = bib.ImmersedBoundaryDynamics3D(lat, shapes)
    G = (1.0 / 6.0) * (2 * U / (n - 1)) * radius / Ca
    pid = fsi.add_particle(sid, "capsule_skalak", workloads.params_vector(G=G, C=1.0), meshes.place(rest, None, c))
    return lat, fsi, pid


SPECS = [(32, 2, 0.1, True), (48, 3, 0.05, True), (40, 2, 0.5, False)]


def make_set(ctx, storage):
    return [capsule_instance(ctx, n, lvl, storage, Ca, seed=i, fd=fd) for i, (n, lvl, Ca, fd) in enumerate(SPECS)]


@pytest.mark.parametrize("storage", ["f64", "f32"])
def test_batch_equals_individual_steps(ctx, storage):
    solo = make_set(ctx, storage)
    grouped = make_set(ctx, storage)
    batch = bib.Batch(ctx, [g[0] for g in grouped])
    batch.step(5)  # odd: graph pairs plus one plain step
    batch.step(4)
    for lat, fsi, pid in solo:
        fsi.step(9)
    # single lattices with few particles split the membrane and update kernels over several
    # CTAs per particle: the same sums, grouped differently (FP32 partial sums in FP32 storage)
    tol_p, tol_f, tol_v = (1e-13, 1e-15, 1e-9) if storage == "f64" else (2e-6, 2e-7, 1e-7)
    for (ls, fs, ps), (lg, fg, pg) in zip(solo, grouped):
        a, b = fs.get_particle(ps), fg.get_particle(pg)
        assert rel(b["pos"], a["pos"]) < tol_p
        assert abs(b["volume"] - a["volume"]) < tol_v * a["volume"]
        assert np.abs(lg.receive() - ls.receive()).max() < tol_f
    batch.close()


@pytest.mark.parametrize("storage", ["f64", "f32"])
def test_batch_with_phase_fields_equals_individual_steps(ctx, storage):
    """Capsules with viscosity ratios 3 and 5 (GuoExternalForceVOFDynamics with the membranes
    voxelized into the phase field after every move) and one lattice without: the batch moves
    first, voxelizes per lattice, then collides, as a single lattice does."""
    specs = [(32, 2, 0.1, True, 3.0), (40, 2, 0.5, False, 5.0), (32, 2, 0.1, True, 1.0)]
    solo = [capsule_instance(ctx, n, l, storage, Ca, seed=i, fd=fd, lam=lam) for i, (n, l, Ca, fd, lam) in enumerate(specs)]
    grouped = [capsule_instance(ctx, n, l, storage, Ca, seed=i, fd=fd, lam=lam)
               for i, (n, l, Ca, fd, lam) in enumerate(specs)]
    batch = bib.Batch(ctx, [g[0] for g in grouped])
    batch.step(5)
    batch.step(4)
    for lat, fsi, pid in solo:
        fsi.step(9)
    tol_p, tol_f = (1e-13, 1e-15) if storage == "f64" else (2e-6, 2e-7)
    for k, ((ls, fs, ps), (lg, fg, pg)) in enumerate(zip(solo, grouped)):
        assert rel(fg.get_particle(pg)["pos"], fs.get_particle(ps)["pos"]) < tol_p
        assert np.abs(lg.receive() - ls.receive()).max() < tol_f
        if specs[k][4] != 1.0:
            ph = lg.get_phase()
            assert np.array_equal(ph, ls.get_phase()) and ph.sum() > 100  # the capsule's interior
    batch.close()


def test_batch_follows_individual_steps_in_between(ctx):
    """A lattice stepped on its own between batch steps: the batch rebuilds its tables."""
    solo = make_set(ctx, "f64")
    grouped = make_set(ctx, "f64")
    batch = bib.Batch(ctx, [g[0] for g in grouped])
    batch.step(3)
    grouped[1][1].step(1)  # only the second lattice
    batch.step(2)
    for i, (lat, fsi, pid) in enumerate(solo):
        fsi.step(6 if i == 1 else 5)
    for (ls, fs, ps), (lg, fg, pg) in zip(solo, grouped):
        assert rel(fg.get_particle(pg)["pos"], fs.get_particle(ps)["pos"]) < 1e-13
        assert np.abs(lg.receive() - ls.receive()).max() < 1e-15
    batch.close()


def test_batch_autotune_keeps_the_physics(ctx):
    solo = make_set(ctx, "f32")
    grouped = make_set(ctx, "f32")
    batch = bib.Batch(ctx, [g[0] for g in grouped])
    chosen = batch.autotune(steps=2)
    assert chosen["stages"] in (2, 3, 4) and chosen["membrane_block"] in (64, 128, 256, 512)
    # 6 tile x stage candidates + 4 block sizes, each one untimed + 2 timed steps
    steps = (6 + 4) * 3
    batch.step(4)
    for lat, fsi, pid in solo:
        fsi.step(steps + 4)
    for (ls, fs, ps), (lg, fg, pg) in zip(solo, grouped):
        assert rel(fg.get_particle(pg)["pos"], fs.get_particle(ps)["pos"]) < 2e-6
    batch.close()


def test_batch_rejects_mixed_or_unsupported_lattices(ctx):
    a = capsule_instance(ctx, 32, 2, "f64")
    b = capsule_instance(ctx, 32, 2, "f32")
    with pytest.raises(bib.BibError):
        bib.Batch(ctx, [a[0], b[0]])
    lat = ctx.add_domain(32, 32, 32, periodic=(1, 1, 1), omega=1.0)
    bib.ImmersedBoundaryDynamics3D(lat, bib.ParticleShapeLibrary(ctx), spread="deterministic")
    with pytest.raises(bib.BibError):
        bib.Batch(ctx, [lat])
    with pytest.raises(bib.BibError):
        bib.Batch(ctx, [a[0], a[0]])
