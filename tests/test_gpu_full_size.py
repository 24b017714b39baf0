"""The bench's full-size workload checked through size-independent properties: the 512 x 128 x 128
channel (periodic x, halfway bounce-back on y and z, body force) with 400 cells of 642 vertices
(Skalak + bending + area / volume penalties).  Over the same steps from the same state: total mass
is conserved by the FP64 path to rounding and by FP16 storage within its quantisation; FP16 and FP32
cell volumes, centres and velocities follow the FP64 path; the state stays finite."""
import numpy as np
import pytest

from biblbm_gb300 import workloads

pytestmark = pytest.mark.gpu

bib = pytest.importorskip("biblbm_gb300")
STEPS = 20


@pytest.fixture(scope="module")
def ctx():
    c = bib.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def wl():
    return workloads.channel_suspension()


def run(ctx, wl, storage):
    nx, ny, nz = wl["dims"]
    lat = ctx.add_domain(nx, ny, nz, storage=storage, **wl["lattice"])
    lat.initialize_at_equilibrium(None, np.zeros((3, nz, ny, nx)))
    shapes = bib.ParticleShapeLibrary(ctx)
    sid = shapes.store_mesh(wl["rest"], wl["tri"], "rbc")
    fsi = bib.ImmersedBoundaryDynamics3D(lat, shapes)
    for p in wl["positions"]:
        fsi.add_particle(sid, wl["model"], wl["params"], p)
    m0 = float(lat.receive().sum())
    fsi.step(STEPS)
    lat.check_health()
    f = lat.receive()
    u = lat.compute_velocity()
    pos, stats = fsi.download()
    out = dict(mass0=m0, mass=float(f.sum()), u=u, pos=pos, stats=stats)
    return out


@pytest.fixture(scope="module")
def runs(ctx, wl):
    return {st: run(ctx, wl, st) for st in ("f64", "f32", "f16")}


def test_mass_is_conserved(runs, wl):
    n = int(np.prod(wl["dims"]))
    # the mass is n + the sum of f-bar; bounce-back walls and Guo forcing conserve it
    # (measured: 2e-21 n, 1e-13 n, 1e-10 n)
    assert abs(runs["f64"]["mass"] - runs["f64"]["mass0"]) < 1e-15 * n
    assert abs(runs["f32"]["mass"] - runs["f32"]["mass0"]) < 1e-11 * n
    assert abs(runs["f16"]["mass"] - runs["f16"]["mass0"]) < 1e-8 * n


@pytest.mark.parametrize("storage,tol_v,tol_u", [("f32", 5e-7, 5e-3), ("f16", 5e-7, 5e-3)])
def test_reduced_storage_follows_fp64(runs, storage, tol_v, tol_u):
    ref, got = runs["f64"], runs[storage]
    assert np.isfinite(got["pos"]).all() and np.isfinite(got["u"]).all()
    # cell volumes and centres (measured after 20 steps: 5e-8 / 6e-8 and 2e-7; velocity 6.7e-4 / 6.9e-4)
    assert np.abs(got["stats"][:, 1] / ref["stats"][:, 1] - 1).max() < tol_v
    assert np.abs(got["stats"][:, 2:5] - ref["stats"][:, 2:5]).max() < 2e-6
    # velocity field, relative L2
    du = np.sqrt(((got["u"] - ref["u"]) ** 2).sum() / (ref["u"] ** 2).sum())
    assert du < tol_u


def test_cells_keep_their_volume(runs, wl):
    V0 = wl["V0"]
    assert np.abs(runs["f64"]["stats"][:, 1] / V0 - 1).max() < 1e-7
