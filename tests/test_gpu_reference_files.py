"""The reference's own files through the C ABI: particle files (bib_particles_save_plb / _load_plb,
bib_particles_write_vtu, bib_particles_write_lightweight) and Palabos' lattice checkpoint
(bib_lattice_save_plb / _load_plb).

The files the reference itself wrote (tests/golden/plb_particles.npz) are loaded into a lattice;
saving that state again reproduces them byte for byte, and so do the VTU and lightweight outputs
of the loaded state.  A run's particles survive a save / load through the format exactly; a
checkpoint split over two rank files (a two-rank reference run) loads by particle id; bad input
is rejected.  The lattice checkpoints the reference wrote (one block, and six blocks as a
multi-rank run writes them) load exactly; saving reproduces the reference's bytes; a coupled run
saved in both reference formats and resumed continues bit for bit."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import golden
from tests.test_reference_files import TAGS, fixture_particles

pytestmark = pytest.mark.gpu

bib = pytest.importorskip("biblbm_gb300")


@pytest.fixture(scope="module")
def ctx():
    c = bib.Context(0)
    yield c
    c.close()


def fixture_lattice(ctx, d):
    lat = ctx.add_domain(*(int(v) for v in d["in_dims"]), periodic=(1, 1, 1), omega=1.0)
    lat.initialize_at_equilibrium(None, np.zeros((3,) + tuple(int(v) for v in d["in_dims"][::-1])))
    shapes = bib.ParticleShapeLibrary(ctx)
    ids = [shapes.store_mesh(d["in_rest"], d["in_tri"], TAGS[0]), shapes.store_mesh(d["in_rest_b"], d["in_tri_b"], TAGS[1])]
    fsi = bib.ImmersedBoundaryDynamics3D(lat, shapes)
    return lat, fsi, ids


def write_reference_files(d, folder):
    os.makedirs(os.path.join(folder, "ckpt"), exist_ok=True)
    with open(os.path.join(folder, "ckpt.plb"), "wb") as f:
        f.write(bytes(d["out_file_header"]))
    with open(os.path.join(folder, "ckpt", "0.plb"), "wb") as f:
        f.write(bytes(d["out_file_rank0"]))


def read(path):
    with open(path, "rb") as f:
        return f.read()


@pytest.fixture(scope="module")
def loaded(ctx, tmp_path_factory):
    d = golden("plb_particles")
    ref = str(tmp_path_factory.mktemp("ref"))
    write_reference_files(d, ref)
    lat, fsi, ids = fixture_lattice(ctx, d)
    assert ids == [0, 1]  # shape ids as the reference's library numbers them
    fsi.load_particle_checkpoint("ckpt", folder=ref)
    return d, lat, fsi


def test_load_reference_checkpoint(ctx, loaded):
    d, lat, fsi = loaded
    parts, _, _ = fixture_particles(d)
    assert fsi.count_particles() == len(parts)
    info = np.zeros(3, dtype=np.int32)
    import ctypes as C

    for p in parts:
        ctx.check(ctx.lib.bib_particle_info(ctx.h, lat.h, p["id"], info.ctypes.data_as(C.POINTER(C.c_int32))))
        assert (int(info[0]), int(info[1])) == (p["shape"], p["model"])
        got = fsi.get_particle(p["id"])
        for key in ("pos", "vel", "force"):
            assert np.array_equal(got[key], p[key]), key


def test_save_reproduces_the_reference_checkpoint(loaded, tmp_path):
    d, lat, fsi = loaded
    fsi.save_particle_checkpoint("ckpt", folder=str(tmp_path))
    assert read(tmp_path / "ckpt.plb") == bytes(d["out_file_header"])
    assert read(tmp_path / "ckpt" / "0.plb") == bytes(d["out_file_rank0"])
    # FileName semantics: the name's own folder and extension are dropped
    fsi.save_particle_checkpoint("somewhere/ckpt.bin", folder=str(tmp_path / "x" / "y"))
    assert read(tmp_path / "x" / "y" / "ckpt" / "0.plb") == bytes(d["out_file_rank0"])


def test_vtu_and_lightweight_outputs_match_the_reference(loaded, tmp_path):
    d, lat, fsi = loaded
    fsi.write_particles_as_vtk(1234, folder=str(tmp_path))
    for k in range(3):
        assert read(tmp_path / ("obj%d-1234.vtu" % k)) == bytes(d["out_file_vtu%d" % k]), k
    fsi.write_particle_vtk(2, str(tmp_path / "one.vtu"))
    assert read(tmp_path / "one.vtu") == bytes(d["out_file_vtu2"])
    fsi.write_lightweight_particle_data(1234, folder=str(tmp_path))
    assert read(tmp_path / "objsP0-1234.txt").decode() == bytes(d["out_file_light"]).decode()


def test_run_state_survives_the_format(ctx, tmp_path):
    """Particles of a coupled run (velocities and forces of its last step included) go through
    save / load unchanged; the reloaded lattice writes the same files again."""
    d = golden("plb_particles")
    lat, fsi, ids = fixture_lattice(ctx, d)
    parts, _, _ = fixture_particles(d)
    for p in parts:
        model = {0: "capsule_neohookean", 1: "capsule_skalak", 2: "rbc_wlcpow"}[p["model"]]
        fsi.add_particle(ids[p["shape"]], model, p["params"], p["pos"])
    fsi.step(3)
    before = [fsi.get_particle(k) for k in range(3)]
    assert np.abs(before[0]["force"]).max() > 0 and np.abs(before[0]["vel"]).max() > 0
    fsi.save_particle_checkpoint("run", folder=str(tmp_path))
    lat2, fsi2, _ = fixture_lattice(ctx, d)
    fsi2.load_particle_checkpoint("run", folder=str(tmp_path))
    for k in range(3):
        after = fsi2.get_particle(k)
        for key in ("pos", "vel", "force"):
            assert np.array_equal(after[key], before[k][key]), (k, key)
        assert after["volume"] == pytest.approx(before[k]["volume"], rel=1e-13)
    fsi2.save_particle_checkpoint("again", folder=str(tmp_path))
    assert read(tmp_path / "again" / "0.plb") == read(tmp_path / "run" / "0.plb")
    # the reloaded particles step like the originals' copies (same lattice state: at rest)
    fsi2.step(1)
    assert np.isfinite(fsi2.get_particle(0)["pos"]).all()


def test_two_rank_checkpoint_loads_by_id(ctx, tmp_path):
    d = golden("plb_particles")
    parts, _, _ = fixture_particles(d)
    import struct

    (tmp_path / "ckpt").mkdir()
    (tmp_path / "ckpt.plb").write_text("3\n2\nckpt/0.plb\nckpt/1.plb\n")
    pack = [O.plb_pack(p["model"], p["shape"], p["id"], p["pos"], p["vel"], p["force"], p["params"]) for p in parts]
    (tmp_path / "ckpt" / "0.plb").write_bytes(struct.pack("<q", 1) + pack[1])
    (tmp_path / "ckpt" / "1.plb").write_bytes(struct.pack("<q", 2) + pack[2] + pack[0])
    lat, fsi, _ = fixture_lattice(ctx, d)
    fsi.load_particle_checkpoint("ckpt", folder=str(tmp_path))
    for p in parts:
        assert np.array_equal(fsi.get_particle(p["id"])["pos"], p["pos"])


def test_bad_particle_files_are_rejected(ctx, tmp_path):
    d = golden("plb_particles")
    parts, _, _ = fixture_particles(d)
    lat, fsi, ids = fixture_lattice(ctx, d)
    # a model without a reference particle type: error, no file written
    fsi.add_particle(ids[1], "skalak_bending", d["in_params"][2], parts[2]["pos"])
    with pytest.raises(bib.BibError):
        fsi.save_particle_checkpoint("nope", folder=str(tmp_path))
    assert not (tmp_path / "nope.plb").exists()
    # ids that are not 0 .. n-1
    import struct

    (tmp_path / "gap").mkdir()
    (tmp_path / "gap.plb").write_text("3\n1\ngap/0.plb\n")
    pk = [O.plb_pack(p["model"], p["shape"], 2 * p["id"], p["pos"], p["vel"], p["force"], p["params"]) for p in parts[:2]]
    (tmp_path / "gap" / "0.plb").write_bytes(struct.pack("<q", 2) + b"".join(pk))
    with pytest.raises(bib.BibError):
        fsi.load_particle_checkpoint("gap", folder=str(tmp_path))
    # a truncated rank file, a missing header
    (tmp_path / "cut").mkdir()
    (tmp_path / "cut.plb").write_text("1\n1\ncut/0.plb\n")
    (tmp_path / "cut" / "0.plb").write_bytes(bytes(d["out_file_rank0"])[:500])
    with pytest.raises(bib.BibError):
        fsi.load_particle_checkpoint("cut", folder=str(tmp_path))
    with pytest.raises(bib.BibError):
        fsi.load_particle_checkpoint("missing", folder=str(tmp_path))
    # the failed loads left the lattice's particle as it was
    assert fsi.count_particles() == 1
    assert np.array_equal(fsi.get_particle(0)["pos"], parts[2]["pos"])


# ---------------------------------------------------------------- lattice checkpoint (parallelIO)
def lattice_fixture(ctx, d):
    nx, ny, nz = (int(v) for v in d["in_dims"])
    return ctx.add_domain(nx, ny, nz, periodic=(1, 1, 1), omega=1.0, use_phase=True, omega_inner=0.5)


def write_lattice_files(d, folder, which=""):
    name = "blocks" if which else "ckpt"
    with open(os.path.join(folder, name + ".plb"), "wb") as f:
        f.write(bytes(d["out_file_%sxml" % which]))
    with open(os.path.join(folder, name + ".dat"), "wb") as f:
        f.write(bytes(d["out_file_%sdat" % which]))
    return name


@pytest.mark.parametrize("which", ["", "blocks_"])
def test_lattice_checkpoint_of_the_reference_loads_exactly(ctx, tmp_path, which):
    d = golden("lattice_plb")
    name = write_lattice_files(d, str(tmp_path), which)
    lat = lattice_fixture(ctx, d)
    lat.load_plb(name, folder=str(tmp_path))
    assert np.array_equal(lat.receive(), d["in_fbar"])
    assert np.array_equal(lat.get_external_force(), d["in_force"])
    assert np.array_equal(lat.get_phase(), d["in_phase"])


def test_lattice_checkpoint_save_reproduces_the_reference(ctx, tmp_path):
    d = golden("lattice_plb")
    write_lattice_files(d, str(tmp_path), "blocks_")
    lat = lattice_fixture(ctx, d)
    lat.load_plb("blocks", folder=str(tmp_path))
    lat.save_plb("ckpt", folder=str(tmp_path / "out"))
    assert read(tmp_path / "out" / "ckpt.plb") == bytes(d["out_file_xml"])
    assert read(tmp_path / "out" / "ckpt.dat") == bytes(d["out_file_dat"])


def test_lattice_checkpoint_without_phase_keeps_the_phase(ctx, tmp_path):
    """ForcedD3Q19 checkpoints (22 values per cell) load; the lattice's phase field stays."""
    d = golden("lattice_plb")
    xml = bytes(d["out_file_xml"]).decode().replace("ForcedPhaseD3Q19", "ForcedD3Q19").replace(
        "<cellDim> 23 </cellDim>", "<cellDim> 22 </cellDim>")
    cells = np.frombuffer(bytes(d["out_file_dat"]), dtype="<f8").reshape(-1, 23)[:, :22]
    xml = xml.replace("<Offsets> %d </Offsets>" % (cells.shape[0] * 184), "<Offsets> %d </Offsets>" % (cells.shape[0] * 176))
    (tmp_path / "f22.plb").write_text(xml.replace("ckpt.dat", "f22.dat"))
    (tmp_path / "f22.dat").write_bytes(np.ascontiguousarray(cells).tobytes())
    lat = lattice_fixture(ctx, d)
    phase = 1.0 - d["in_phase"]
    lat.set_phase(phase)
    lat.load_plb("f22", folder=str(tmp_path))
    assert np.array_equal(lat.receive(), d["in_fbar"])
    assert np.array_equal(lat.get_external_force(), d["in_force"])
    assert np.array_equal(lat.get_phase(), phase)


def test_bad_lattice_checkpoints_are_rejected(ctx, tmp_path):
    d = golden("lattice_plb")
    write_lattice_files(d, str(tmp_path))
    xml = bytes(d["out_file_xml"]).decode()
    lat = lattice_fixture(ctx, d)
    before = lat.receive()
    # another lattice size
    nx, ny, nz = (int(v) for v in d["in_dims"])
    other = ctx.add_domain(nx + 1, ny, nz, periodic=(1, 1, 1), omega=1.0)
    with pytest.raises(bib.BibError):
        other.load_plb("ckpt", folder=str(tmp_path))
    # dynamic content, a truncated data file, components that leave cells out, no spec
    (tmp_path / "dyn.plb").write_text(xml.replace("False", "True").replace("ckpt.dat", "ckpt.dat"))
    (tmp_path / "cut.plb").write_text(xml.replace("ckpt.dat", "cut.dat"))
    (tmp_path / "cut.dat").write_bytes(bytes(d["out_file_dat"])[:1000])
    box = "0 %d 0 %d 0 %d" % (nx - 1, ny - 1, nz - 1)
    small = "0 %d 0 %d 0 %d" % (nx - 1, ny - 1, nz - 2)
    (tmp_path / "hole.plb").write_text(xml.replace("<Component> %s </Component>" % box, "<Component> %s </Component>" % small)
                                       .replace("<Offsets> %d </Offsets>" % (nx * ny * nz * 184),
                                                "<Offsets> %d </Offsets>" % (nx * ny * (nz - 1) * 184)))
    for name in ("dyn", "cut", "hole", "missing"):
        with pytest.raises(bib.BibError):
            lat.load_plb(name, folder=str(tmp_path))
    assert np.array_equal(lat.receive(), before)


@pytest.mark.parametrize("name", ["ibm_capsule_shear", "ibm_capsule_lambda"])
def test_run_resumed_from_reference_formats_is_bit_identical(ctx, tmp_path, name):
    """A coupled FP64 run (deterministic spreading) saved in the reference's two formats, the
    lattice (parallelIO::save) and the particles (save_checkpoint), and resumed in a fresh lattice
    continues exactly like the uninterrupted run: finite-difference walls, and a voxelized phase
    field with viscosity ratio 5."""
    from tests.test_gpu_parity import run_coupled_gpu

    g = golden(name)
    lat_a, fsi_a, pa = run_coupled_gpu(ctx, g, spread="deterministic")
    fsi_a.step(3)
    lat_a.save_plb("lbm", folder=str(tmp_path))
    fsi_a.save_particle_checkpoint("fsi", folder=str(tmp_path))
    fsi_a.step(4)
    lat_b, fsi_b, pb = run_coupled_gpu(ctx, g, spread="deterministic")
    lat_b.load_plb("lbm", folder=str(tmp_path))
    fsi_b.load_particle_checkpoint("fsi", folder=str(tmp_path))
    fsi_b.step(4)
    assert np.array_equal(lat_b.receive(), lat_a.receive())
    assert np.array_equal(fsi_b.get_particle(0)["pos"], fsi_a.get_particle(pa)["pos"])
    ctx.set_graph_mode(True)
