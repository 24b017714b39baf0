"""RBC shape calibration (progs/common/calibrate_rbc_shape.h), CPU side: the oracle's
create_rbc_params, shrink_rbc_volume (RBCParticle::relax_nodes iterations) and
set_minor_axis_orientation against the reference's own run of them (tests/golden/calibrate_rbc.npz),
exactly."""
import numpy as np

from oracle import oracle as O
from tests.conftest import golden


def fixture_shape():
    d = golden("calibrate_rbc")
    return d, O.Shape(d["in_rest"], d["in_tri"])


def test_rbc_params_match_the_reference():
    d, S = fixture_shape()
    assert np.array_equal(O.rbc_params(S, *d["in_moduli"]), d["out_params"])


def test_short_shrink_matches_the_reference_exactly():
    d, S = fixture_shape()
    prm = O.rbc_params(S, *d["in_moduli"])
    pos, damping = O.rbc_shrink_volume(S, prm, float(d["in_vol_frac"]) * S.volume, 5, float(d["in_damping"]))
    assert damping == float(d["in_damping"])
    assert np.array_equal(pos, d["out_short_shrunk"])


def test_shrink_and_alignment_match_the_reference():
    """801 iterations: the oracle agrees with the reference to 1e-13.  It is exact over the first 20
    iterations. Later a last-bit difference in some force term appears, and the explicit relaxation
    amplifies a perturbation by about 10 over the run."""
    d, S = fixture_shape()
    prm = O.rbc_params(S, *d["in_moduli"])
    pos, damping = O.rbc_shrink_volume(S, prm, float(d["in_vol_frac"]) * S.volume, int(d["in_n_it"]),
                                       float(d["in_damping"]))
    assert damping == float(d["in_damping"])  # no restart
    assert np.abs(pos - d["out_shrunk"]).max() < 1e-12
    aligned = O.align_minor_axis(pos, d["in_tri"])
    assert np.abs(aligned - d["out_aligned"]).max() < 1e-12
    # the alignment itself is exact on the reference's own shrunk positions
    assert np.array_equal(O.align_minor_axis(d["out_shrunk"], d["in_tri"]), d["out_aligned"])
    st = O.particle_update(d["out_aligned"], d["in_tri"])
    assert st[1] == float(d["out_vol_desired"][0]) and st[0] == float(d["out_area"][0])
    # the minor axis is z now
    ext = aligned.max(0) - aligned.min(0)
    assert ext[2] < ext[0] and ext[2] < ext[1]


def test_divergent_relaxation_gives_up():
    """A membrane too stiff for the explicit relaxation: every doubling of the damping diverges;
    the restatement stops after 64 restarts (the reference would retry forever)."""
    _, S = fixture_shape()
    prm = O.rbc_params(S, 0.5, 50.0, 2e-3)
    _, damping = O.rbc_shrink_volume(S, prm, 0.65 * S.volume, 100, 1e-2)
    assert damping == -1.0
