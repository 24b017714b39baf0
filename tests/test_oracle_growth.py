"""The growth stage of the initial distribution (progs/common/create_particles.h:105-212): the oracle
against runs of the reference's own code.

grow_pipe: the growth loop body (rigid copies, RigidParticle.hh; the collision grid of
CollisionForces.h with the pipe wall pass; SpringPotential) from the reference's own random
placement, states after 1, 2, 11 and 301 iterations.  create_particles_pipe: the reference's
create_particles itself, 40001 iterations, the capsules placed at the result.  Both bit for bit.
"""
import numpy as np
import pytest

from oracle import oracle as O

from tests.conftest import golden


def grow_inputs(d):
    shapes = [(d["in_rest0"], d["in_tri0"]), (d["in_rest1"], d["in_tri1"])]
    gr = d["in_growth"]
    return shapes, dict(pot=d["in_pot"], initial_scale=gr[0], density=gr[1], damping=gr[2], n_it=int(d["in_n_it"]))


@pytest.mark.parametrize("k", [1, 2, 11, 301])
def test_growth_loop_matches_reference(k):
    d = golden("grow_pipe")
    shapes, kw = grow_inputs(d)
    g = O.growth(d["in_box"], d["in_wall"], it_end=k, **kw)
    com, quat, pos, force = O.grow_particles(g, shapes, d["in_shape"], d["in_com"], d["in_quat"])
    assert np.array_equal(com, d["out_com_%d" % k])
    assert np.array_equal(quat, d["out_quat_%d" % k])
    assert np.array_equal(pos, d["out_pos_%d" % k])
    assert np.array_equal(force, d["out_force_%d" % k])


def test_growth_fixture_has_contacts():
    """The fixture exercises both force terms: by iteration 301 vertices of different particles
    touch (equal and opposite pair terms) and vertices press on the wall at radius 6."""
    d = golden("grow_pipe")
    f, x = d["out_force_301"], d["out_pos_301"]
    touched = np.abs(f).sum(1) > 0
    assert touched.sum() > 20
    r = np.hypot(x[:, 1], x[:, 2])
    assert (touched & (r >= 6.0 - 1.0)).any()  # within the spring's reach of the wall
    owner = np.repeat(np.arange(len(d["in_shape"])), 162)
    assert len(np.unique(owner[touched])) >= 3


def test_create_particles_matches_reference():
    """The whole of create_particles: srand(7) placement of 8 spheres and 3 ellipsoids at 20 %
    scale in the pipe shrunk by 1.5, 40001 growth iterations, capsules placed at the result."""
    d = golden("create_particles_pipe")
    types = [(d["in_rest0"], d["in_tri0"], d["in_counts"][0]), (d["in_rest1"], d["in_tri1"], d["in_counts"][1])]
    parts = O.create_particles(d["in_box"], d["in_pipe"][:3], types, int(d["in_seed"]))
    assert np.array_equal(np.concatenate(parts), d["out_pos"])
    # the cells grew to full size inside the pipe without overlapping the wall by much
    r = np.hypot(d["out_pos"][:, 1], d["out_pos"][:, 2])
    assert r.max() < d["in_pipe"][2]


def test_powi_chain_is_what_the_reference_computes():
    """std::pow(T, int) in the reference's C++98 build is __builtin_powi (x^2 x^3 for x^5); libm's
    pow differs in the last bit for some scales of the growth (0.2 + 0.8 * it / 300)."""
    diff = 0
    for it in range(0, 301, 10):
        s = 0.2 + (1.0 - 0.2) * (it / 300.0)
        s2 = s * s
        diff += (s2 * (s * s2)) != s ** 5.0
    assert diff > 0
