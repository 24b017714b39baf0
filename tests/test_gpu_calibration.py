"""RBC shape calibration on the GPU through the C ABI (bib_rbc_params, bib_rbc_shrink_volume,
bib_align_minor_axis) and the RBCShapeInitializer mirror, against the reference's own run
(tests/golden/calibrate_rbc.npz) and the oracle."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import golden

pytestmark = pytest.mark.gpu

bib = pytest.importorskip("biblbm_gb300")


@pytest.fixture(scope="module")
def ctx():
    c = bib.Context(0)
    yield c
    c.close()


def dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def test_calibration_against_the_reference(ctx):
    d = golden("calibrate_rbc")
    shapes = bib.ParticleShapeLibrary(ctx)
    sid = shapes.store_mesh(d["in_rest"], d["in_tri"], "sphere")
    prm = np.zeros(12)
    ctx.check(ctx.lib.bib_rbc_params(ctx.h, sid, *[float(v) for v in d["in_moduli"]], dp(prm)))
    np.testing.assert_allclose(prm, d["out_params"], rtol=1e-15, atol=0)
    vol0 = shapes.info(sid)["volume"]
    pos = np.empty_like(d["in_rest"])
    used = C.c_double()
    ctx.check(ctx.lib.bib_rbc_shrink_volume(ctx.h, sid, dp(prm), float(d["in_vol_frac"]) * vol0, int(d["in_n_it"]),
                                            float(d["in_damping"]), dp(pos), C.byref(used)))
    assert used.value == float(d["in_damping"])
    # 801 explicit iterations in FP64 (force sums by atomics, an amplification of about 10 over the
    # run): within 1e-10 of the reference's positions
    assert np.abs(pos - d["out_shrunk"]).max() < 1e-10
    aligned = pos.copy()
    ctx.check(ctx.lib.bib_align_minor_axis(ctx.h, sid, dp(aligned), dp(np.array([0.0, 0.0, 1.0]))))
    # the alignment of these positions as the oracle restates the reference's
    np.testing.assert_allclose(aligned, O.align_minor_axis(pos, d["in_tri"]), rtol=0, atol=1e-12)
    assert np.abs(aligned - d["out_aligned"]).max() < 1e-10


def test_shape_initializer_flow(ctx):
    """compute_rbc_parameters -> shrink_volume -> store_shape, then the calibrated RBC steps."""
    d = golden("calibrate_rbc")
    shapes = bib.ParticleShapeLibrary(ctx)
    shapes.store_mesh(d["in_rest"], d["in_tri"], "sphere")
    init = bib.RBCShapeInitializer(shapes, "sphere")
    init.compute_rbc_parameters(*d["in_moduli"])
    init.shrink_volume(float(d["in_vol_frac"]), int(d["in_n_it"]), float(d["in_damping"]))
    assert init.params[9] == pytest.approx(float(d["out_vol_desired"][0]), rel=1e-9)
    rbc = init.store_shape("rbc")
    info = shapes.info(rbc)
    assert info["volume"] == pytest.approx(float(d["out_vol_desired"][0]), rel=1e-9)
    lat = ctx.add_domain(24, 24, 24, periodic=(1, 1, 1), omega=1.0)
    lat.initialize_at_equilibrium(None, np.zeros((3, 24, 24, 24)))
    fsi = bib.ImmersedBoundaryDynamics3D(lat, shapes)
    pid = fsi.add_particle(rbc, "rbc_wlcpow", init.params, shapes.meshes[rbc][0] + 12.0)
    fsi.step(20)
    p = fsi.get_particle(pid)
    assert np.isfinite(p["pos"]).all()
    assert p["volume"] == pytest.approx(info["volume"], rel=1e-3)


def test_divergent_calibration_is_an_error(ctx):
    d = golden("calibrate_rbc")
    shapes = bib.ParticleShapeLibrary(ctx)
    sid = shapes.store_mesh(d["in_rest"], d["in_tri"], "sphere")
    prm = np.zeros(12)
    ctx.check(ctx.lib.bib_rbc_params(ctx.h, sid, 0.5, 50.0, 2e-3, dp(prm)))
    pos = np.empty_like(d["in_rest"])
    st = ctx.lib.bib_rbc_shrink_volume(ctx.h, sid, dp(prm), 0.65 * shapes.info(sid)["volume"], 100, 1e-2, dp(pos), None)
    assert st == -4  # BIB_ENAN after 64 restarts


def test_calibration_arguments_are_checked(ctx):
    d = golden("calibrate_rbc")
    shapes = bib.ParticleShapeLibrary(ctx)
    sid = shapes.store_mesh(d["in_rest"], d["in_tri"], "sphere")
    prm = np.zeros(12)
    ctx.check(ctx.lib.bib_rbc_params(ctx.h, sid, 1e-3, 0.1, 4e-4, dp(prm)))
    pos = np.empty_like(d["in_rest"])
    lib, h = ctx.lib, ctx.h
    assert lib.bib_rbc_params(h, 999, 1e-3, 0.1, 4e-4, dp(prm)) == -1          # unknown shape
    assert lib.bib_rbc_shrink_volume(h, sid, dp(prm), 100.0, 0, 0.05, dp(pos), None) == -1      # n_it < 1
    assert lib.bib_rbc_shrink_volume(h, sid, dp(prm), 100.0, 10, 0.0, dp(pos), None) == -1      # damping <= 0
    assert lib.bib_rbc_shrink_volume(h, sid, dp(prm), -1.0, 10, 0.05, dp(pos), None) == -1      # vol_final <= 0
    bad = prm.copy()
    bad[9] = 0.0
    assert lib.bib_rbc_shrink_volume(h, sid, dp(bad), 100.0, 10, 0.05, dp(pos), None) == -1     # vol_desired 0
    assert lib.bib_align_minor_axis(h, sid, dp(pos), dp(np.zeros(3))) == -1                      # zero direction
    # the context still works
    ctx.check(lib.bib_rbc_shrink_volume(h, sid, dp(prm), 0.9 * shapes.info(sid)["volume"], 2, 0.05, dp(pos), None))
    assert np.isfinite(pos).all()
