"""The benchmark workloads themselves, CUDA path against the CPU oracle on the same instance.

Headline: the 512 x 128 x 128 channel (periodic x, halfway bounce-back on y and z, body force 1e-6)
with 400 Evans-Fung cells of 642 vertices (Skalak + bending + area / volume penalties), the instance
``workloads.channel_suspension()`` that bench.py times.  Both sides take two coupled steps in the
driver order of progs/rbcs_in_channel/rbcs_in_channel.cpp:209-235 (computeVelocity,
setExternalVector with the body force, the immersed-boundary functional, collideAndStream).  The
capsule in shear (64^3, finite-difference velocity walls, 642-vertex Skalak capsule,
``workloads.capsule_shear()``) takes 20 steps in the order of
progs/capsule_in_shear/capsule_in_shear.cpp:187-227.

The bench instance starts with every cell in its stress-free rest shape, so its membrane forces
are round-off of sums that cancel (|F| ~ 1e-12 in FP64, ~ 1e-7 in FP32 element arithmetic); a
second instance, the same 400 cells inflated by 2 % about their centres, checks the membrane forces
at full size where they are not.  Forces are compared in units of G R (shear modulus x cell radius,
the model's force scale).

Bounds (about 5x the errors measured on a GB300) are in ``TOL`` below.  Not bit-exact: nvcc
contracts multiply-adds into FMAs and the spreading atomics sum in varying order; the reduced
storage runs are compared with the same FP64 oracle state.
"""
import numpy as np
import pytest

from biblbm_gb300 import workloads
from oracle import oracle as O

pytestmark = pytest.mark.gpu

bib = pytest.importorskip("biblbm_gb300")

# (populations abs, positions abs in lu, forces abs in units of G R, volumes rel)
TOL = {
    # rest-shape channel, 2 steps (measured f64 1.9e-13 / 2.8e-14 / 8e-12 / 1.1e-12; f32 and f16
    # 5.4e-8 / 8.3e-8 / 2.4e-6 / 7.4e-8: the FP32 round-off forces move vertices by F/2 per step)
    "channel": {"f64": (1e-12, 2e-13, 5e-11, 1e-11), "f32": (3e-7, 5e-7, 1.5e-5, 5e-7),
                "f16": (3e-7, 5e-7, 1.5e-5, 5e-7)},
    # the same cells inflated by 2 %, 2 steps (f16 positions measured 1.1e-5: FP16 storage keeps the
    # velocity field in FP16 too, 11 significant bits, so a vertex moving at u ~ 0.01 is off by up to
    # ~5e-6 per step)
    "channel_prestrained": {"f64": (1e-12, 1e-12, 1e-10, 1e-11), "f32": (1e-5, 1e-5, 1e-3, 1e-5),
                            "f16": (1e-5, 5e-5, 1e-3, 1e-5)},
    # capsule in shear, 20 steps (measured f64 5.5e-18 / 7.1e-15 / 1.2e-12 rel. / 3.1e-15; f32 9.1e-10
    # / 2.4e-8 / 1.7e-4 rel. / 2.9e-8; f16 7.5e-7 / 6.9e-6 / 6.4e-4 rel. / 3.9e-7)
    "capsule": {"f64": (1e-16, 5e-14, 1e-10, 2e-14), "f32": (5e-9, 1.5e-7, 1e-3, 1.5e-7),
                "f16": (4e-6, 4e-5, 4e-3, 2e-6)},
}


def oracle_run(wl, steps):
    nx, ny, nz = wl["dims"]
    lp = wl["lattice"]
    L = O.lattice((nx, ny, nz), lp["periodic"], lp["collision"], lp["omega"], lp["omega"],
                  wall_y=lp.get("wall_y", "none"), wall_z=lp.get("wall_z", "none"), wall_u=lp.get("wall_u"))
    S = O.System(L, "roma", -1.0)
    if wl.get("initial_velocity") is not None:
        f0 = O.init_equilibrium(L, None, wl["initial_velocity"])
        if lp.get("wall_y") == "fd_velocity":
            f0 = O.apply_fd_walls(L, f0, np.zeros((3, nz, ny, nx)))
        S.f[...] = f0
    S.set_body_force(np.asarray(lp.get("body_force", (0, 0, 0)), dtype=np.float64))
    sid = S.add_shape(wl["rest"], wl["tri"])
    pids = [S.add_particle(sid, wl["model"], wl["params"], p) for p in wl["positions"]]
    S.step(steps)
    parts = [S.particle(p) for p in pids]
    return dict(f=np.array(S.f), pos=np.concatenate([p["pos"] for p in parts]),
                force=np.concatenate([p["force"] for p in parts]),
                volume=np.array([p["volume"] for p in parts]))


def gpu_run(ctx, wl, storage, steps):
    nx, ny, nz = wl["dims"]
    lat = ctx.add_domain(nx, ny, nz, storage=storage, **wl["lattice"])
    if wl.get("initial_velocity") is not None:
        lat.initialize_at_equilibrium(None, wl["initial_velocity"])
    shapes = bib.ParticleShapeLibrary(ctx)
    sid = shapes.store_mesh(wl["rest"], wl["tri"], "cell")
    fsi = bib.ImmersedBoundaryDynamics3D(lat, shapes)
    pids = [fsi.add_particle(sid, wl["model"], wl["params"], p) for p in wl["positions"]]
    fsi.step(steps)
    lat.check_health()
    parts = [fsi.get_particle(p) for p in pids]
    out = dict(f=lat.receive(), pos=np.concatenate([p["pos"] for p in parts]),
               force=np.concatenate([p["force"] for p in parts]),
               volume=np.array([p["volume"] for p in parts]))
    del fsi, lat
    return out


def compare(got, ref, wl, storage, case):
    tf, tp, tF, tV = TOL[case][storage]
    GR = wl["params"][0] * wl["radius"]
    df = np.abs(got["f"] - ref["f"]).max()
    dp = np.abs(got["pos"] - ref["pos"]).max()
    dF = np.abs(got["force"] - ref["force"]).max() / GR
    dV = np.abs(got["volume"] / ref["volume"] - 1).max()
    print("%s %s: |df| %.3e  |dpos| %.3e  |dforce|/GR %.3e (|F|max/GR %.3e)  rel|dV| %.3e"
          % (case, storage, df, dp, dF, np.abs(ref["force"]).max() / GR, dV))
    assert np.isfinite(got["f"]).all() and np.isfinite(got["pos"]).all()
    assert df < tf, (storage, df)
    assert dp < tp, (storage, dp)
    assert dF < tF, (storage, dF)
    assert dV < tV, (storage, dV)


@pytest.fixture(scope="module")
def ctx():
    c = bib.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def channel():
    wl = workloads.channel_suspension()
    return wl, oracle_run(wl, 2)


@pytest.fixture(scope="module")
def channel_prestrained():
    wl = dict(workloads.channel_suspension())
    c = wl["centers"][:, None, :]
    wl["positions"] = c + 1.02 * (wl["positions"] - c)
    return wl, oracle_run(wl, 2)


@pytest.fixture(scope="module")
def capsule():
    wl = workloads.capsule_shear()
    return wl, oracle_run(wl, 20)


@pytest.mark.parametrize("storage", ["f64", "f32", "f16"])
def test_channel_400_cells_two_steps_match_oracle(ctx, channel, storage):
    wl, ref = channel
    assert wl["dims"] == (512, 128, 128) and wl["positions"].shape == (400, 642, 3)
    compare(gpu_run(ctx, wl, storage, 2), ref, wl, storage, "channel")


@pytest.mark.parametrize("storage", ["f64", "f32", "f16"])
def test_channel_400_prestrained_cells_match_oracle(ctx, channel_prestrained, storage):
    wl, ref = channel_prestrained
    assert np.abs(ref["force"]).max() > 1e-3 * wl["params"][0] * wl["radius"]
    compare(gpu_run(ctx, wl, storage, 2), ref, wl, storage, "channel_prestrained")


@pytest.mark.parametrize("storage", ["f64", "f32", "f16"])
def test_capsule_in_shear_twenty_steps_match_oracle(ctx, capsule, storage):
    wl, ref = capsule
    assert wl["dims"] == (64, 64, 64) and wl["positions"].shape == (1, 642, 3)
    compare(gpu_run(ctx, wl, storage, 20), ref, wl, storage, "capsule")
