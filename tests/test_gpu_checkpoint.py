"""Checkpoints through the C ABI: a run resumed from bib_checkpoint_save / _load continues bit
for bit (deterministic spreading), including finite-difference walls, FP16 storage, a
voxelized phase field with viscosity ratio 5 and per-cell dynamics; a file of another
configuration, a corrupted or truncated file and missing shapes are rejected and leave the
lattice as it was."""
import numpy as np
import pytest

from tests.conftest import golden
from tests.test_gpu_parity import run_coupled_gpu

pytestmark = pytest.mark.gpu

bib = pytest.importorskip("biblbm_gb300")


@pytest.fixture(scope="module")
def ctx():
    c = bib.Context(0)
    yield c
    c.close()


def state(lat, fsi, pid):
    p = fsi.get_particle(pid)
    return lat.receive(), p["pos"], p["vel"], p["force"], p["volume"], lat.get_external_force()


@pytest.mark.parametrize("name,storage,graph", [("ibm_capsule_shear", "f64", False), ("ibm_capsule_shear", "f16", True),
                                                ("ibm_rbc_periodic", "f32", True), ("ibm_capsule_lambda", "f64", True)])
def test_resumed_run_is_bit_identical(ctx, tmp_path, name, storage, graph):
    d = golden(name)
    lat_a, fsi_a, pa = run_coupled_gpu(ctx, d, storage=storage, graph=graph, spread="deterministic")
    fsi_a.step(3)
    path = tmp_path / "run.bibckpt"
    fsi_a.save_checkpoint(path)
    fsi_a.step(4)
    ref = state(lat_a, fsi_a, pa)
    assert fsi_a.iteration() == 7
    # a second lattice built the same way (its particle is replaced by the checkpoint's)
    lat_b, fsi_b, pb = run_coupled_gpu(ctx, d, storage=storage, graph=graph, spread="deterministic")
    fsi_b.load_checkpoint(path)
    assert fsi_b.iteration() == 3 and fsi_b.count_particles() == 1
    fsi_b.step(4)
    got = state(lat_b, fsi_b, pb)
    for a, b in zip(ref, got):
        assert np.array_equal(a, b)
    if "in_lambda" in d.files:
        assert np.array_equal(lat_a.get_phase(), lat_b.get_phase())
    assert fsi_b.iteration() == 7


def test_lattice_only_checkpoint_with_cell_types(ctx, tmp_path):
    n = 16
    rng = np.random.default_rng(5)
    kw = dict(periodic=(1, 1, 1), omega=1.2, collision="trt", storage="f32")
    types = (rng.random((n, n, n)) < 0.05).astype(np.uint8)
    a = ctx.add_domain(n, n, n, **kw)
    a.initialize_at_equilibrium(None, 0.01 * rng.standard_normal((3, n, n, n)))
    a.set_cell_types(types)
    a.collide_and_stream(5)
    a.save_checkpoint(tmp_path / "lat.bibckpt")
    a.collide_and_stream(5)
    b = ctx.add_domain(n, n, n, **kw)
    b.load_checkpoint(tmp_path / "lat.bibckpt")
    assert b.iteration() == 5
    b.collide_and_stream(5)
    assert np.array_equal(a.receive(), b.receive())


def test_bad_checkpoints_are_rejected(ctx, tmp_path):
    d = golden("ibm_capsule_shear")
    lat, fsi, pid = run_coupled_gpu(ctx, d, spread="deterministic")
    fsi.step(2)
    path = tmp_path / "good.bibckpt"
    fsi.save_checkpoint(path)
    fsi.step(1)
    before = state(lat, fsi, pid)
    raw = path.read_bytes()

    def rejected(blob, match):
        bad = tmp_path / "bad.bibckpt"
        bad.write_bytes(blob)
        with pytest.raises(bib.BibError, match=match):
            fsi.load_checkpoint(bad)
        for x, y in zip(before, state(lat, fsi, pid)):
            assert np.array_equal(x, y)

    corrupt = bytearray(raw)
    corrupt[len(raw) // 2] ^= 0x40
    rejected(bytes(corrupt), "checksum")
    rejected(raw[: len(raw) - 100], "truncated|checksum")
    rejected(b"not a checkpoint" + raw[16:], "not a biblbm_gb300 checkpoint")
    # a lattice of another size
    n = int(d["in_dims"][0])
    other = ctx.add_domain(n + 2, n, n, periodic=(1, 0, 1), omega=1.0, wall_y="fd_velocity",
                           wall_u=[[-0.01, 0, 0], [0.01, 0, 0], [0, 0, 0], [0, 0, 0]])
    with pytest.raises(bib.BibError, match="another configuration"):
        other.load_checkpoint(path)
    # a context that does not hold the particle's shape
    U = float(d["in_U"])
    c3 = bib.Context(0)
    try:
        l3 = c3.add_domain(n, n, n, periodic=(1, 0, 1), omega=1.0 / float(d["in_tau"]), wall_y="fd_velocity",
                           wall_u=[[-U, 0, 0], [U, 0, 0], [0, 0, 0], [0, 0, 0]])
        with pytest.raises(bib.BibError, match="shape"):
            l3.load_checkpoint(path)
    finally:
        c3.close()
