"""Population transfers of bib_lattice_send / bib_lattice_receive (the CoProcessor3D send /
receive of coProcessor3D.h:57-115 and the Palabos static-content order of blockLattice3D.hh:644-689).

Page-locked host buffers are read and written by the import / export kernels directly;
pageable buffers go through the double-buffered staging pipeline.  Both must give the same
lattice state and the same bytes back, in every wire layout, on lattices large enough for several
staging chunks, with finite-difference wall rows (their own buffer) and halfway bounce-back faces.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

bib = pytest.importorskip("biblbm_gb300")
torch = pytest.importorskip("torch")

LAYOUT = {"soa": 0, "palabos": 1, "coprocessor": 2}
_dp = ctypes.POINTER(ctypes.c_double)
PER = {"soa": 19, "palabos": 23, "coprocessor": 19}


@pytest.fixture(scope="module")
def ctx():
    c = bib.Context(0)
    yield c
    c.close()


def pinned_like(a):
    p = torch.empty(a.shape, dtype=torch.float64, pin_memory=True).numpy()
    p[...] = a
    return p


def wire(layout, f, F=None, phase=None):
    """Host buffer in wire order from SoA populations (19, nz, ny, nx)."""
    if layout == "soa":
        return np.ascontiguousarray(f)
    nz, ny, nx = f.shape[1:]
    cells = np.transpose(f, (3, 2, 1, 0)).reshape(nx * ny * nz, 19)  # x slowest, z fastest
    if layout == "coprocessor":
        return np.ascontiguousarray(cells)
    ext = np.zeros((nx * ny * nz, 4))
    ext[:, :3] = np.transpose(F, (3, 2, 1, 0)).reshape(-1, 3)
    ext[:, 3] = np.transpose(phase, (2, 1, 0)).reshape(-1)
    return np.ascontiguousarray(np.concatenate([cells, ext], axis=1))


WALLS = {
    # finite-difference velocity walls on y (their nodes live in the wall buffer), periodic x and z
    "fd": dict(periodic=(1, 0, 1), wall_y="fd_velocity", wall_u=[[-0.01, 0, 0], [0.01, 0, 0], [0, 0, 0], [0, 0, 0]]),
    # halfway bounce-back on y and z (a moving wall on z-), periodic x
    "bb": dict(periodic=(1, 0, 0), wall_y="halfway_bb", wall_z="halfway_bb",
               wall_u=[[0, 0, 0], [0, 0, 0], [0.01, 0, 0], [0, 0, 0]]),
}


@pytest.mark.parametrize("walls", ["fd", "bb"])
@pytest.mark.parametrize("storage", ["f64", "f32", "f16"])
@pytest.mark.parametrize("layout", ["soa", "palabos", "coprocessor"])
def test_pinned_and_pageable_transfers_agree(ctx, storage, layout, walls):
    # 128 x 64 x 40: 6.2 M doubles of populations, two staging chunks of each order
    nx, ny, nz = 128, 64, 40
    rng = np.random.default_rng(7)
    f = rng.uniform(-0.01, 0.01, (19, nz, ny, nx))
    F = rng.uniform(-1e-4, 1e-4, (3, nz, ny, nx))
    phase = (rng.uniform(size=(nz, ny, nx)) < 0.3).astype(np.float64)
    kw = dict(storage=storage, omega=1.0, use_phase=layout == "palabos", **WALLS[walls])
    buf = wire(layout, f, F, phase)
    results = {}
    for kind, host in (("pageable", buf.copy()), ("pinned", pinned_like(buf))):
        lat = ctx.add_domain(nx, ny, nz, **kw)
        ctx.check(ctx.lib.bib_lattice_send(ctx.h, lat.h, host.ctypes.data, host.nbytes, LAYOUT[layout]))
        lat.collide_and_stream(1)
        out = np.zeros_like(buf) if kind == "pageable" else pinned_like(np.zeros_like(buf))
        ctx.check(ctx.lib.bib_lattice_receive(ctx.h, lat.h, out.ctypes.data, out.nbytes, LAYOUT[layout]))
        results[kind] = (np.array(out), lat.receive())
        del lat
    (a_wire, a_soa), (b_wire, b_soa) = results["pageable"], results["pinned"]
    assert np.isfinite(a_wire).all()
    # the same kernels convert either way: the states and the bytes agree exactly
    assert np.array_equal(a_wire, b_wire)
    assert np.array_equal(a_soa, b_soa)
    # and the wire order is the SoA state transposed
    if layout == "soa":
        assert np.array_equal(a_wire, a_soa)
    else:
        assert np.array_equal(a_wire[:, :19], wire("coprocessor", a_soa))
    if layout == "palabos":  # the force and the phase come back as sent (FP32 force field below FP64)
        F_back = np.transpose(a_wire[:, 19:22].reshape(nx, ny, nz, 3), (3, 2, 1, 0))
        assert np.abs(F_back - F).max() <= (0.0 if storage == "f64" else 1e-11)
        assert np.array_equal(np.transpose(a_wire[:, 22].reshape(nx, ny, nz), (2, 1, 0)), phase)


@pytest.mark.parametrize("storage", ["f64", "f16"])
def test_pinned_round_trip_is_exact_where_storage_is(ctx, storage):
    nx, ny, nz = 64, 32, 24
    rng = np.random.default_rng(3)
    f = rng.uniform(-0.01, 0.01, (19, nz, ny, nx))
    if storage == "f16":  # values the FP16 storage holds exactly (multiples of 1/scale)
        f = np.round(f * 8192.0) / 8192.0
    lat = ctx.add_domain(nx, ny, nz, periodic=(1, 1, 1), storage=storage)
    host = pinned_like(f)
    lat.send(host)
    out = pinned_like(np.zeros_like(f))
    ctx.check(ctx.lib.bib_lattice_receive(ctx.h, lat.h, out.ctypes.data, out.nbytes, 0))
    assert np.array_equal(out, f)


@pytest.mark.parametrize("storage", ["f64", "f16"])
def test_equilibrium_and_velocity_through_pinned_buffers(ctx, storage):
    """bib_lattice_init_equilibrium and bib_lattice_get_velocity read / write page-locked host
    arrays directly; the result must equal the staged path's for pageable arrays."""
    nx, ny, nz = 48, 20, 12
    rng = np.random.default_rng(5)
    u = rng.uniform(-0.02, 0.02, (3, nz, ny, nx))
    rho = 1.0 + rng.uniform(-0.01, 0.01, (nz, ny, nx))
    outs = []
    for kind in ("pageable", "pinned"):
        lat = ctx.add_domain(nx, ny, nz, storage=storage, **WALLS["fd"])
        uu, rr = (u.copy(), rho.copy()) if kind == "pageable" else (pinned_like(u), pinned_like(rho))
        ctx.check(ctx.lib.bib_lattice_init_equilibrium(ctx.h, lat.h, rr.ctypes.data_as(_dp), uu.ctypes.data_as(_dp)))
        lat.collide_and_stream(2)
        vel = np.zeros_like(u) if kind == "pageable" else pinned_like(np.zeros_like(u))
        ctx.check(ctx.lib.bib_lattice_get_velocity(ctx.h, lat.h, vel.ctypes.data_as(_dp)))
        outs.append((lat.receive(), np.array(vel)))
        del lat
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])
    assert np.abs(outs[1][1]).max() > 1e-3
