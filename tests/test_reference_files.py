"""The reference's own files, CPU side: the oracle's restatement of the .plb particle
checkpoint (save_checkpoint, ImmersedBoundaryDynamics_io.hh:17-73), the VTU particle output
(ParticleBase3D::write_vtk, ParticleBase.hh:270-390) and the lightweight text output
(DeformableParticle3D::write_lightweight, DeformableParticle3D.hh:318-333), and of Palabos'
static-content lattice checkpoint (parallelIO::save / load, io/multiBlockWriter3D.cpp:53-213,
io/multiBlockReader3D.cpp:135-268), against the files the reference itself wrote
(tests/golden/plb_particles.npz, tests/golden/lattice_plb.npz), byte for byte."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import golden

TAGS = ["shape", "shape_b"]


def fixture_particles(d):
    tri = [d["in_tri"], d["in_tri_b"]]
    nv = [d["in_rest"].shape[0], d["in_rest_b"].shape[0]]
    parts, off = [], 0
    for k, (m, s) in enumerate(zip(d["in_models"], d["in_shapes"])):
        n = nv[int(s)]
        parts.append(dict(model=int(m), shape=int(s), id=k, pos=d["in_pos"][off:off + n],
                          vel=d["in_vel"][off:off + n], force=d["in_force"][off:off + n], params=d["in_params"][k]))
        off += n
    return parts, tri, nv


def test_reference_type_ids_are_the_oracles():
    d = golden("plb_particles")
    assert list(d["out_type_ids"]) == [O.PLB_TYPE_CAPSULE, O.PLB_TYPE_RBC]


def test_plb_checkpoint_bytes_match_the_reference():
    d = golden("plb_particles")
    parts, _, _ = fixture_particles(d)
    header, body = O.plb_files("ckpt", parts)
    assert header.encode() == bytes(d["out_file_header"])
    assert body == bytes(d["out_file_rank0"])


def test_plb_unpack_inverts_the_reference_file():
    d = golden("plb_particles")
    parts, _, nv = fixture_particles(d)
    buf = bytes(d["out_file_rank0"])
    (count,) = np.frombuffer(buf[:8], dtype="<i8")
    assert count == len(parts)
    at = 8
    for ref in parts:
        p, at = O.plb_unpack(buf, at, nv)
        assert (p["model"], p["shape"], p["id"], p["voxelize"]) == (ref["model"], ref["shape"], ref["id"], True)
        for key in ("pos", "vel", "force"):
            assert np.array_equal(p[key], ref[key])
        # the pack holds the parameters of the particle's own class only
        keys = O.CAPSULE_PACK if ref["model"] in (0, 1) else O.RBC_PACK
        for k in keys:
            i = O.PARAM_KEYS.index(k)
            assert p["params"][i] == ref["params"][i]
    assert at == len(buf)


@pytest.mark.parametrize("k", [0, 1, 2])
def test_vtu_bytes_match_the_reference(k):
    d = golden("plb_particles")
    parts, tri, _ = fixture_particles(d)
    p = parts[k]
    assert O.vtu_bytes(p["pos"], p["force"], tri[p["shape"]]) == bytes(d["out_file_vtu%d" % k])


def test_lightweight_text_matches_the_reference():
    d = golden("plb_particles")
    parts, tri, _ = fixture_particles(d)
    rows = []
    for p in parts:
        st = O.particle_update(p["pos"], tri[p["shape"]])
        rows.append((TAGS[p["shape"]], p["id"], p["pos"], st[2:5], st[1]))
    assert O.lightweight_text(1234, rows) == bytes(d["out_file_light"]).decode()


def test_plb_pack_rejects_a_model_without_reference_type():
    with pytest.raises(ValueError):
        O.plb_pack(O.MODEL["skalak_bending"], 0, 0, np.zeros((4, 3)), np.zeros((4, 3)), np.zeros((4, 3)),
                   np.zeros(12))


# ---------------------------------------------------------------- lattice checkpoint (parallelIO)
def test_lattice_checkpoint_bytes_match_the_reference():
    d = golden("lattice_plb")
    xml, dat = O.plb_lattice_files("ckpt", d["in_fbar"], d["in_force"], d["in_phase"])
    assert xml.encode() == bytes(d["out_file_xml"])
    assert dat == bytes(d["out_file_dat"])


@pytest.mark.parametrize("which", ["", "blocks_"])
def test_lattice_checkpoint_read_of_any_block_layout(which):
    """The one-block file and the 3 x 2 x 1 block file the reference wrote both read back to the
    lattice's data."""
    d = golden("lattice_plb")
    f, F, ph = O.plb_lattice_read(bytes(d["out_file_%sxml" % which]).decode(), bytes(d["out_file_%sdat" % which]))
    assert np.array_equal(f, d["in_fbar"]) and np.array_equal(F, d["in_force"]) and np.array_equal(ph, d["in_phase"])
