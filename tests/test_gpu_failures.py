"""Failure detection in the forms that fault, trap and hang no GPU.

- A bounded device wait that runs out: the staged collide-and-stream's producer withholds the copies
  of one tile (the failure-testing tuning field), so the consumers wait for a barrier phase that
  nothing completes.  Their wait gives up after the tuned bound, the launch ends, bib_check_health
  reports BIB_ETIMEOUT, and the context keeps working.  The reference's only failure handling is
  exit(-1) (fsi/ImmersedBoundaryDynamics.hh:51-54).
- Device allocations that fail: the N-th allocation of a context is made to fail
  (BIB_FAIL_DEVICE_ALLOC); every path returns BIB_ENOMEM and leaves the context usable, and a retry
  gives the same result as a run without the failure.
- Non-finite or out-of-range parameters are rejected with BIB_EINVAL before any state changes.
"""
import os
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

bib = pytest.importorskip("biblbm_gb300")
from biblbm_gb300 import _lib, meshes  # noqa: E402

EINVAL, ENOMEM, ETIMEOUT = -1, -2, -5


@pytest.fixture(scope="module")
def ctx():
    c = bib.Context(0)
    yield c
    c.close()


def seeded_populations(nx, ny, nz, seed=1):
    rng = np.random.default_rng(seed)
    w = np.array([1 / 3] + [1 / 18] * 3 + [1 / 36] * 6 + [1 / 18] * 3 + [1 / 36] * 6)
    return rng.uniform(-0.02, 0.02, (19, nz, ny, nx)) * w[:, None, None, None]


@pytest.mark.parametrize("storage", ["f16", "f32"])
def test_withheld_tile_times_out_and_the_context_recovers(ctx, storage):
    nx, ny, nz = 64, 24, 16
    f0 = seeded_populations(nx, ny, nz)
    lat = ctx.add_domain(nx, ny, nz, storage=storage, periodic=(1, 1, 1), omega=1.3)
    lat.set_tuning(kernel="staged", wait_limit_us=2000, withhold_tile=7)
    lat.send(f0)
    t0 = time.perf_counter()
    lat.collide_and_stream(1)
    with pytest.raises(_lib.BibError) as e:
        lat.check_health()
    # the consumers gave up after 2 ms and the producer drained only the copies it issued
    assert e.value.status == ETIMEOUT and time.perf_counter() - t0 < 1.0
    lat.check_health()  # the report clears the flag
    # the same lattice, untuned, from the same state: identical to a lattice that never failed
    lat.set_tuning(kernel="staged")
    lat.send(f0)
    lat.collide_and_stream(3)
    lat.check_health()
    ref = ctx.add_domain(nx, ny, nz, storage=storage, periodic=(1, 1, 1), omega=1.3)
    ref.send(f0)
    ref.collide_and_stream(3)
    assert np.array_equal(lat.receive(), ref.receive())


def test_withheld_tile_in_a_coupled_step(ctx):
    n = 32
    lat = ctx.add_domain(n, n, n, storage="f16", periodic=(1, 1, 1), omega=1.0)
    lat.set_tuning(kernel="staged", wait_limit_us=2000, withhold_tile=3)
    shapes = bib.ParticleShapeLibrary(ctx)
    xyz, tri = meshes.icosphere(2, 5.0)
    sid = shapes.store_mesh(xyz, tri, "capsule")
    fsi = bib.ImmersedBoundaryDynamics3D(lat, shapes)
    fsi.add_particle(sid, "capsule_skalak", bib.membrane_params(G=0.01, C=1.0), meshes.place(xyz, None, (15.5,) * 3))
    fsi.step(2)
    with pytest.raises(_lib.BibError) as e:
        lat.check_health()
    assert e.value.status == ETIMEOUT
    lat.set_tuning(kernel="staged")
    fsi.step(2)  # steps again (the state of the failed step is not meaningful)
    assert np.isfinite(lat.receive()).all()


def coupled_run(ctx):
    """A small coupled run touching most allocation paths: lattice buffers, shape tables,
    particle buffers, deterministic-spreading sort buffers and the transfer staging area."""
    n = 24
    lat = ctx.add_domain(n, n, n, storage="f64", periodic=(1, 1, 1), omega=1.0, body_force=(1e-5, 0, 0))
    shapes = bib.ParticleShapeLibrary(ctx)
    xyz, tri = meshes.icosphere(2, 4.0)
    sid = shapes.store_mesh(xyz, tri, "capsule")
    fsi = bib.ImmersedBoundaryDynamics3D(lat, shapes, spread="deterministic")
    fsi.add_particle(sid, "capsule_skalak", bib.membrane_params(G=0.01, C=1.0), meshes.place(xyz, None, (11.3, 12.1, 11.7)))
    fsi.step(3)
    return lat.receive(), fsi.download()[0]


def test_every_device_allocation_failure_returns_enomem():
    ref_ctx = bib.Context(0)
    f_ref, pos_ref = coupled_run(ref_ctx)
    ref_ctx.close()
    failures = 0
    for k in range(60):
        os.environ["BIB_FAIL_DEVICE_ALLOC"] = str(k)
        try:
            c = bib.Context(0)
        finally:
            del os.environ["BIB_FAIL_DEVICE_ALLOC"]
        try:
            out = None
            try:
                out = coupled_run(c)
            except _lib.BibError as e:
                assert e.status == ENOMEM and "allocation" in str(e), e
                failures += 1
                # the context stays usable: the same run again (no further allocation fails)
                out = coupled_run(c)
            f, pos = out
            assert np.array_equal(f, f_ref) and np.array_equal(pos, pos_ref)
        finally:
            c.close()
    assert failures >= 20  # the run makes at least that many device allocations


def test_non_finite_parameters_are_rejected(ctx):
    bad = [dict(body_force=(np.nan, 0, 0)), dict(wall_y="halfway_bb", periodic=(1, 0, 1), wall_u=[[np.inf, 0, 0]] + [[0] * 3] * 3),
           dict(omega=np.nan), dict(omega=2.5), dict(trt_magic=np.nan), dict(storage="f16", f16_scale=-1.0),
           dict(storage="f16", f16_scale=1e6)]
    for kw in bad:
        args = dict(periodic=(1, 1, 1), omega=1.0)
        args.update(kw)
        with pytest.raises(_lib.BibError) as e:
            ctx.add_domain(16, 16, 16, **args)
        assert e.value.status == EINVAL, kw
    lat = ctx.add_domain(16, 16, 16, periodic=(1, 1, 1))
    shapes = bib.ParticleShapeLibrary(ctx)
    xyz, tri = meshes.icosphere(1, 3.0)
    sid = shapes.store_mesh(xyz, tri, "capsule")
    fsi = bib.ImmersedBoundaryDynamics3D(lat, shapes)
    pos = meshes.place(xyz, None, (8.0, 8.0, 8.0))
    prm = bib.membrane_params(G=0.01, C=1.0)
    for p, x in ((np.where(np.arange(prm.size) == 0, np.nan, prm), pos), (prm, np.where(pos > 8.5, np.inf, pos))):
        with pytest.raises(_lib.BibError) as e:
            fsi.add_particle(sid, "capsule_skalak", p, x)
        assert e.value.status == EINVAL
    # nothing was added: the valid particle is particle 0 and steps
    assert fsi.add_particle(sid, "capsule_skalak", prm, pos) == 0
    fsi.step(2)
    lat.check_health()
