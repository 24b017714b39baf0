"""The random initial placement of progs/common/create_particles.h:37-93 (ParticlePositionInitializer
and random orientations, drawn from glibc's rand()): the oracle's restatement and the library's
host code against the reference's own run (tests/golden/initial_distribution.npz), exactly."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import golden


def test_oracle_matches_the_reference():
    d = golden("initial_distribution")
    pos, quat = O.initial_distribution(d["in_box"], d["in_counts"], d["in_radii"], int(d["in_seed"]), d["in_pipe"])
    assert np.array_equal(pos, d["out_pos"]) and np.array_equal(quat, d["out_quat"])


@pytest.fixture(scope="module")
def bib():
    """The library's host code needs no GPU; the library is built in place if it is not."""
    from biblbm_gb300 import build

    build.build()
    import biblbm_gb300

    return biblbm_gb300


def test_library_matches_the_reference(bib):
    d = golden("initial_distribution")
    pos, quat = bib.initial_distribution(d["in_box"], d["in_counts"], d["in_radii"], float(d["in_max_radius"]),
                                         int(d["in_seed"]), pipe=d["in_pipe"])
    assert np.array_equal(pos, d["out_pos"]) and np.array_equal(quat, d["out_quat"])
    # a valid packing: inside the pipe by the radius, no two spheres overlapping
    r = np.repeat(d["in_radii"], d["in_counts"])
    y0, z0, R = d["in_pipe"]
    assert (np.hypot(pos[:, 1] - y0, pos[:, 2] - z0) < R - r).all()
    dist = np.linalg.norm(pos[:, None] - pos[None], axis=-1) + np.eye(len(r)) * 1e9
    assert (dist >= r[:, None] + r[None]).all()
    assert np.allclose(np.linalg.norm(quat, axis=1), 1.0)


def test_no_room_is_an_error(bib):
    with pytest.raises(bib.BibError):
        bib.initial_distribution([0, 9, 0, 9, 0, 9], [50], [2.0], 2.0, 7, max_tries=2000)
