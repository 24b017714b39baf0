"""bib_spread_forces_noalloc: deterministic spreading with its sort scratch in the library's
static device array, called through the C ABI, against the deterministic spreading that
bib_ibm_step performs with the lattice's own buffers.

Both run the same key, sort and per-cell reduce kernels in the same order on the same
inputs, so the fields agree to 1e-15 of the largest force component; two calls in a row
must give identical fields (the shared scratch carries nothing from one call to the next).
The fields are also checked against the CPU oracle's spreading (the reference's
spread_forces_impl, ImmersedBoundaryDynamics_forces.hh:22-163, restated).
This file is collected last and also passes on its own in a fresh process.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

bib = pytest.importorskip("biblbm_gb300")
torch = pytest.importorskip("torch")
from biblbm_gb300 import meshes, workloads  # noqa: E402
from oracle import oracle as O  # noqa: E402

MAX_ENTRIES = 1 << 20  # BIB_SPREAD_NOALLOC_MAX_ENTRIES


@pytest.fixture(scope="module")
def ctx():
    c = bib.Context(0)
    yield c
    c.close()


def capsule_after_ibm_step(ctx, storage, dirac, n=24):
    """One deformed capsule; bib_ibm_step resets the force field to the body force and
    spreads the membrane forces at the initial positions into it."""
    body = np.array([2e-5, -1e-5, 3e-6])
    lat = ctx.add_domain(n, n, n, periodic=(1, 1, 1), omega=1.0, storage=storage, body_force=tuple(body))
    shapes = bib.ParticleShapeLibrary(ctx)
    rest, tri = meshes.icosphere(3, 6.0)
    sid = shapes.store_mesh(rest, tri, "capsule")
    fsi = bib.ImmersedBoundaryDynamics3D(lat, shapes, dirac=dirac, spread="deterministic")
    rng = np.random.default_rng(17)
    pos = rest * np.array([1.25, 0.85, 1.0]) + np.array([11.7, 12.3, 12.6]) + 0.05 * rng.standard_normal(rest.shape)
    pid = fsi.add_particle(sid, "capsule_skalak", workloads.params_vector(G=0.02, C=1.0), pos)
    fsi.ibm_step()
    ctx.sync()
    forces = fsi.get_particle(pid)["force"]
    return lat, pos, forces, body, lat.get_external_force()


def noalloc_spread(ctx, lat, pos_d, force_d, nvert, field_d):
    torch.cuda.synchronize()  # inputs written on torch's stream; the library runs on its own
    ctx.check(ctx.lib.bib_spread_forces_noalloc(ctx.h, lat.h, pos_d.data_ptr(), force_d.data_ptr(), int(nvert),
                                                field_d.data_ptr()))
    ctx.sync()


@pytest.mark.parametrize("storage,dirac", [("f64", "roma"), ("f64", "peskin"), ("f32", "roma"), ("f16", "roma")])
def test_noalloc_spreading_matches_ibm_step(ctx, storage, dirac):
    """FP16-storage lattices spread into a float field, as FP32 ones do."""
    lat, pos, forces, body, F_ref = capsule_after_ibm_step(ctx, storage, dirac)
    assert np.abs(forces).max() > 0 and np.abs(F_ref - body[:, None, None, None]).max() > 0
    dev = torch.device("cuda", 0)
    pos_d = torch.tensor(pos.reshape(-1), dtype=torch.float64, device=dev)
    force_d = torch.tensor(forces.reshape(-1), dtype=torch.float64, device=dev)
    ft = torch.float64 if storage == "f64" else torch.float32
    field_d = torch.empty((3,) + lat.shape, dtype=ft, device=dev)
    body_d = torch.tensor(body, dtype=ft, device=dev)[:, None, None, None]
    tol = 1e-15 * np.abs(F_ref).max()
    outs = []
    for _ in range(2):  # two calls in a row share the one scratch array
        field_d.copy_(body_d.expand_as(field_d))
        noalloc_spread(ctx, lat, pos_d, force_d, pos.shape[0], field_d)
        out = field_d.double().cpu().numpy()
        assert np.abs(out - F_ref).max() <= tol
        outs.append(out)
    assert np.array_equal(outs[0], outs[1])
    # and against the CPU oracle's spreading of the same forces onto the body force (FP64
    # weights and sums; the FP32 field of reduced-precision lattices rounds each of them)
    n = lat.shape[0]
    L = O.lattice((n, n, n), (1, 1, 1))
    F_orc = O.spread(L, dirac, pos, forces, offset=-1.0, F=np.broadcast_to(body[:, None, None, None], (3, n, n, n)))
    rel = np.abs(outs[0] - F_orc).max() / np.abs(F_orc - body[:, None, None, None]).max()
    assert rel < (1e-13 if storage == "f64" else 1e-5), rel


def test_noalloc_spreading_rejects_too_many_entries(ctx):
    lat = ctx.add_domain(16, 16, 16, periodic=(1, 1, 1), omega=1.0)
    bib.ImmersedBoundaryDynamics3D(lat, bib.ParticleShapeLibrary(ctx), dirac="roma")
    dev = torch.device("cuda", 0)
    small = torch.zeros(3 * 8, dtype=torch.float64, device=dev)
    field_d = torch.zeros((3,) + lat.shape, dtype=torch.float64, device=dev)
    too_many = MAX_ENTRIES // 27 + 1  # rejected before any work touches the (short) arrays
    with pytest.raises(bib.BibError, match="BIB_SPREAD_NOALLOC_MAX_ENTRIES"):
        noalloc_spread(ctx, lat, small, small, too_many, field_d)
    assert float(field_d.abs().max()) == 0.0
