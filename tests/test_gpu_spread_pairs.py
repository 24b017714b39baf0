"""FP32 atomic spreading (two lanes per vertex, with the general path where a support wraps around
the periodic x axis) against the deterministic spreading of the same lattice.

The deterministic path (keys, radix sort, one sum per node in vertex order) shares no code with the
atomic one; both spread the same membrane forces into an FP32 field.  Their fields may differ by the
order of the FP32 sums (and the membrane kernels' own summation order), ~1e-6 of the largest spread
force; a word sent to the wrong 16-byte block, or a straddling window's second word dropped, moves a
whole node's share, ~1e-2 .. 1 of it.
"""
import numpy as np
import pytest

from biblbm_gb300 import workloads

pytestmark = pytest.mark.gpu

bib = pytest.importorskip("biblbm_gb300")


@pytest.fixture(scope="module")
def ctx():
    c = bib.Context(0)
    yield c
    c.close()


def instance():
    """Eight Evans-Fung cells of 162 vertices in a 64 x 32 x 32 channel; the first is moved so that
    its centre sits 0.3 cells from x = 0 (its supports wrap around the periodic x axis)."""
    wl = workloads.channel_suspension(nx=64, ny=32, nz=32, n_cells=8, level=2, hct=0.08, seed=11)
    pos = np.array(wl["positions"], dtype=float)
    c = pos[0].mean(axis=0)
    pos[0][:, 0] += 0.3 - c[0]
    wl["positions"] = pos
    return wl


def spread_field(ctx, wl, storage, spread, dirac):
    nx, ny, nz = wl["dims"]
    lat = ctx.add_domain(nx, ny, nz, storage=storage, **wl["lattice"])
    shapes = bib.ParticleShapeLibrary(ctx)
    sid = shapes.store_mesh(wl["rest"], wl["tri"], "cell")
    fsi = bib.ImmersedBoundaryDynamics3D(lat, shapes, dirac=dirac, spread=spread)
    for p in wl["positions"]:
        # slightly inflated: the membranes start strained, so the spread forces are not ~0
        fsi.add_particle(sid, wl["model"], wl["params"], 1.02 * (p - p.mean(axis=0)) + p.mean(axis=0))
    fsi.step(1)
    lat.check_health()
    F = lat.get_external_force()
    body = np.asarray(wl["lattice"]["body_force"], dtype=float)[:, None, None, None]
    del fsi, lat
    return F - body


@pytest.mark.parametrize("dirac", ["roma", "peskin"])
@pytest.mark.parametrize("storage", ["f32", "f16"])
def test_atomic_spreading_matches_deterministic(ctx, storage, dirac):
    wl = instance()
    a = spread_field(ctx, wl, storage, "atomic", dirac)
    d = spread_field(ctx, wl, storage, "deterministic", dirac)
    scale = np.abs(d).max()
    assert scale > 0
    # the wrapped cell's supports reach both ends of the x axis
    assert np.abs(d[:, :, :, :2]).max() > 1e-3 * scale and np.abs(d[:, :, :, -2:]).max() > 1e-3 * scale
    err = np.abs(a - d).max() / scale
    assert err < 2e-5, err
