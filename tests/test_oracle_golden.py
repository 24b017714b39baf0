"""The CPU oracle against fixtures produced by the reference's own compiled code.

Every comparison here is exact (max |difference| == 0): the oracle restates the
reference's arithmetic operation by operation and both are built without
floating-point contraction.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import golden

SHEAR_WALLS = dict(wall_y="fd_velocity")


def shear_lattice(d, tau=None):
    nx, ny, nz = (int(v) for v in d["in_dims"])
    U = float(d["in_U"])
    om = d["in_omega"] if tau is None else (1 / tau, 1 / tau)
    return O.lattice((nx, ny, nz), (1, 0, 1), "bgk_guo_vof", om[0], om[1], wall_y="fd_velocity",
                     wall_u=[[-U, 0, 0], [U, 0, 0], [0, 0, 0], [0, 0, 0]])


def shear_init(L, U):
    nx, ny, nz = L.nx, L.ny, L.nz
    y = np.arange(ny)
    u = np.zeros((3, nz, ny, nx))
    u[0] = (U * (2.0 * y / (ny - 1) - 1))[None, :, None]
    f = O.init_equilibrium(L, None, u)
    return O.apply_fd_walls(L, f, np.zeros((3, nz, ny, nx)))


@pytest.mark.parametrize("swap", [True, False])
def test_periodic_collide_stream(swap):
    d = golden("lbm_periodic")
    nx, ny, nz = (int(v) for v in d["in_dims"])
    om = d["in_omega"]
    L = O.lattice((nx, ny, nz), (1, 1, 1), "bgk_guo_vof", om[0], om[1], envelope_swap=swap)
    assert np.array_equal(O.compute_velocity(L, d["in_fbar"], d["in_force"]), d["out_u_0"])
    f1 = O.collide_stream(L, d["in_fbar"], d["in_force"], d["in_phase"], 1)
    fe = O.collide_stream(L, d["in_fbar"], d["in_force"], d["in_phase"], 3)
    if swap:
        # with the reference's envelope quirk reproduced the match is exact
        assert np.array_equal(f1, d["out_fbar_1"])
        assert np.array_equal(fe, d["out_fbar_end"])
        assert np.array_equal(O.compute_velocity(L, fe, d["in_force"]), d["out_u_end"])
    else:
        # without it only populations that crossed a periodic face differ
        assert not np.array_equal(f1, d["out_fbar_1"])
        assert np.abs(f1 - d["out_fbar_1"])[0].max() == 0.0


def test_bounce_back_and_no_dynamics_nodes():
    """BounceBack (core/dynamics.hh:763-770) and NoDynamics nodes set per cell with
    defineDynamics; velocity 0 on them (dynamics.hh:796-801)."""
    d = golden("lbm_bounceback")
    nx, ny, nz = (int(v) for v in d["in_dims"])
    om = d["in_omega"]
    L = O.lattice((nx, ny, nz), (1, 1, 1), "bgk_guo_vof", om[0], om[1], celltype=d["in_celltype"])
    f1 = O.collide_stream(L, d["in_fbar"], d["in_force"], d["in_phase"], 1)
    assert np.array_equal(f1, d["out_fbar_1"])
    f_end = O.collide_stream(L, d["in_fbar"], d["in_force"], d["in_phase"], int(d["in_steps"]))
    assert np.array_equal(f_end, d["out_fbar_end"])
    assert np.array_equal(O.compute_velocity(L, f_end, d["in_force"]), d["out_u_end"])


def test_shear_fd_walls():
    d = golden("lbm_shear")
    L = shear_lattice(d)
    assert np.array_equal(shear_init(L, float(d["in_U"])), d["out_fbar_0"])
    f1 = O.collide_stream(L, d["out_fbar_0"], d["in_force"], d["in_phase"], 1)
    assert np.array_equal(f1, d["out_fbar_1"])
    fe = O.collide_stream(L, d["out_fbar_0"], d["in_force"], d["in_phase"], int(d["in_steps"]))
    assert np.array_equal(fe, d["out_fbar_end"])
    assert np.array_equal(O.compute_velocity(L, fe, d["in_force"]), d["out_u_end"])


@pytest.mark.parametrize("dirac", ["roma", "peskin"])
@pytest.mark.parametrize("per", ["ppp", "pwp", "pww"])
def test_interpolation_and_spreading(dirac, per):
    d = golden("interp_%s_%s" % (dirac, per))
    L = O.lattice(d["in_dims"], d["in_periodic"])
    pos, frc = d["in_pos"], d["in_nforce"]
    n = len(pos)
    gen = np.full(n, 2, np.int32)
    ids = d["out_bulk_ids"]
    bulk = np.full(len(ids), 1, np.int32)
    assert np.array_equal(O.interpolate(L, dirac, d["in_u"], pos, gen), d["out_vel_general"])
    assert np.array_equal(O.interpolate(L, dirac, d["in_u"], pos[ids], bulk), d["out_vel_bulk"])
    assert np.array_equal(O.spread(L, dirac, pos, frc, gen), d["out_spread_general"])
    assert np.array_equal(O.spread(L, dirac, pos[ids], frc[ids], bulk), d["out_spread_bulk"])


@pytest.mark.parametrize("name", ["ico2", "ef2"])
def test_shape_connectivity(name):
    d = golden("shape_" + name)
    S = O.Shape(d["in_rest"], d["in_tri"])
    assert np.array_equal(S.links, d["out_links"])
    assert np.array_equal(S.link_len, d["out_link_length"])
    assert np.array_equal(S.pairs, d["out_pairs"])
    assert np.array_equal(S.pair_cs, d["out_pair_cos_sin"])
    assert np.array_equal(S.tri_area, d["out_tri_area"])
    assert S.area == d["out_area"][0] and S.volume == d["out_volume"][0]


@pytest.mark.parametrize("model", ["capsule_neohookean", "capsule_skalak", "rbc_wlcpow", "skalak_bending"])
def test_membrane_forces(model):
    d = golden("forces_" + model)
    S = O.Shape(d["in_rest"], d["in_tri"])
    F = O.membrane_forces(int(d["in_model"]), d["in_params"], S, d["in_pos"])
    assert np.abs(d["out_force"]).max() > 1e-4  # the state is prestressed
    assert np.array_equal(F, d["out_force"])
    st = O.particle_update(d["in_pos"], d["in_tri"])
    assert st[0] == d["out_area"][0] and st[1] == d["out_volume"][0]
    assert np.array_equal(st[2:], d["out_com"])


def test_inertia():
    d = golden("inertia_ef2")
    assert np.array_equal(O.inertia(d["in_pos"], d["in_tri"]), d["out_inertia"])


def coupled_lattice(d, envelope_swap=False):
    nx, ny, nz = (int(v) for v in d["in_dims"])
    tau = float(d["in_tau"])
    lam = float(d["in_lambda"]) if "in_lambda" in d.files else 1.0
    om, om_in = 1 / tau, 1 / (0.5 + lam * (tau - 0.5))
    if int(d["in_walls"]) == 1:
        U = float(d["in_U"])
        return O.lattice((nx, ny, nz), (1, 0, 1), "bgk_guo_vof", om, om_in, wall_y="fd_velocity",
                         wall_u=[[-U, 0, 0], [U, 0, 0], [0, 0, 0], [0, 0, 0]], envelope_swap=envelope_swap)
    return O.lattice((nx, ny, nz), (1, 1, 1), "bgk_guo_vof", om, om_in, envelope_swap=envelope_swap)


def run_coupled(d):
    # the reference rebuilds the periodic-envelope dynamics with the two omegas swapped (see
    # the oracle's collide_stream); with lambda = 1 that is invisible
    L = coupled_lattice(d, envelope_swap=True)
    S = O.System(L, "roma", -1.0)
    S.f[...] = shear_init(L, float(d["in_U"])) if int(d["in_walls"]) == 1 else 0.0
    if "in_body" in d.files:
        S.set_body_force(d["in_body"])
    S.set_voxelize(True)
    pid = S.add_particle(S.add_shape(d["in_rest"], d["in_tri"]), int(d["in_model"]), d["in_params"], d["in_pos"])
    S.init()
    for it in range(int(d["in_steps"])):
        assert np.array_equal(S.particle(pid)["pos"], d["out_pos"][it])
        S.step(1)
        p = S.particle(pid)
        assert np.array_equal(p["vel"], d["out_vel"][it])
        assert np.array_equal(p["force"], d["out_force"][it])
        assert p["volume"] == d["out_volume"][it + 1] and p["area"] == d["out_area"][it + 1]
        if it == 0 and "out_force_spread" in d.files:
            assert np.array_equal(S.force, d["out_force_spread"])
    assert np.array_equal(S.particle(pid)["pos"], d["out_pos"][-1])
    assert np.array_equal(S.velocity(), d["out_u_end"])
    if "out_fbar_end" in d.files:
        assert np.array_equal(S.f, d["out_fbar_end"])
    else:
        assert np.array_equal(S.f.sum(axis=(1, 2, 3)), d["out_fbar_end_sum"])
    # the voxelized phase field of the final positions (ImmersedBoundaryDynamics_voxelization.hh)
    assert np.array_equal(S.phase, d["out_phase_end"])


def test_coupled_capsule_in_shear():
    run_coupled(golden("ibm_capsule_shear"))


def test_coupled_rbc_periodic_body_force():
    run_coupled(golden("ibm_rbc_periodic"))


def test_coupled_capsule_viscosity_ratio():
    """lambda = 5: the voxelized phase enters omega every step."""
    run_coupled(golden("ibm_capsule_lambda"))


def interact_system(d, grid):
    n = int(d["in_dims"][0])
    L = O.lattice((n, n, n), (1, 1, 1), "bgk_guo_vof", 1.0, 1.0)
    S = O.System(L, "roma", -1.0)
    sid = S.add_shape(d["in_rest"], d["in_tri"])
    pa = S.add_particle(sid, int(d["in_model"]), d["in_params"], d["in_pos_a"])
    pb = S.add_particle(sid, int(d["in_model"]), d["in_params"], d["in_pos_b"])
    wq, pq = d["in_wall_params"], d["in_pp_params"]
    if "in_pipe" in d.files:  # WallInteraction on a PipeBoundary along x
        S.add_pipe_wall_interaction(O.potential(int(d["in_wall_kind"]), wq[0], wq[1], wq[2]), *d["in_pipe"])
    else:
        lo, hi = d["in_wall_y"]
        S.add_wall_interaction(O.potential(int(d["in_wall_kind"]), wq[0], wq[1], wq[2]), 1, lo, hi)
    S.add_pp_interaction(O.potential(int(d["in_pp_kind"]), pq[0], pq[1], pq[2]), grid=grid)
    S.init()
    S.step(1)
    return S.particle(pa)["force"], S.particle(pb)["force"]


@pytest.mark.parametrize("name", ["interact_morse_spring", "interact_spring_morse", "interact_pipe_wall"])
def test_interaction_forces(name):
    """Wall decorator + particle-particle forces of one IB step: the reference's grid search
    bit for bit, and the all-pairs search (what the CUDA path evaluates) to the summation
    order on a configuration where the grid finds every pair."""
    d = golden(name)
    fa, fb = interact_system(d, grid=True)
    assert np.array_equal(fa, d["out_force_a"]) and np.array_equal(fb, d["out_force_b"])
    # both particles feel the pair force, particle a also the lower plate (b the pipe wall)
    near = np.abs(d["out_force_a"][:, 0]) > 0
    assert near.any() and (np.abs(d["out_force_b"][:, 0]) > 0).any()
    if "in_pipe" not in d.files:
        assert (d["out_force_a"][:, 1] > 1e-6).any()
    ga, gb = interact_system(d, grid=False)
    scale = max(np.abs(d["out_force_a"]).max(), np.abs(d["out_force_b"]).max())
    assert np.abs(ga - d["out_force_a"]).max() <= 1e-15 * scale
    assert np.abs(gb - d["out_force_b"]).max() <= 1e-15 * scale


def test_grid_search_misses_diagonal_pairs():
    """The reference's grid pairs a cell with 7 of its 13 forward neighbours: two vertices in
    cells offset by (+1, -1, 0) do not interact there; the all-pairs search finds them."""
    L = O.lattice((16, 16, 16), (1, 1, 1))
    pot = O.potential("spring", 0.8, 0.0, 1.0)
    pos = np.array([[7.45, 8.55, 8.0], [7.55, 8.45, 8.0]])  # grid cells (x 8, y 10) and (x 9, y 9)
    owner = np.array([0, 1])
    assert np.abs(O.pp_forces(L, pot, pos, owner, grid=True)).max() == 0.0
    f = O.pp_forces(L, pot, pos, owner)
    d = np.linalg.norm(pos[1] - pos[0])
    expect = -(0.8 - d) / d * (pos[1] - pos[0])
    assert np.allclose(f[0], expect, rtol=1e-14) and np.array_equal(f[1], -f[0])


def test_pipe_first_order_walls():
    """rbc_in_pipe.cpp's first-order pipe walls (BounceBack outside PipeBoundary, NoDynamics
    beyond radius + 1) with a body force: the cell types and the flow after 40 steps."""
    d = golden("lbm_pipe")
    nx, ny, nz = (int(v) for v in d["in_dims"])
    y0, z0, R = d["in_pipe"]
    types = O.pipe_celltypes((nx, ny, nz), y0, z0, R)
    assert np.array_equal(types, d["out_mask"])
    om = float(d["in_omega"])
    L = O.lattice((nx, ny, nz), (1, 1, 1), "bgk_guo_vof", om, om, celltype=types)
    n = nx * ny * nz
    F = np.broadcast_to(np.asarray(d["in_body"])[:, None, None, None], (3, nz, ny, nx))
    f = O.collide_stream(L, np.zeros((19, nz, ny, nx)), F, np.zeros((nz, ny, nx)), int(d["in_steps"]))
    assert np.array_equal(f, d["out_fbar_end"])
    assert np.array_equal(O.compute_velocity(L, f, F), d["out_u_end"])
    assert n > 0 and d["out_u_end"][0].max() > 1e-3


def test_pipe_second_order_walls():
    """GuoRigidWallBoundary on the pipe (rbc_in_pipe.cpp's second-order walls): the wall nodes
    with their lattice vectors and distances, the state after initialize(), after one step and
    after 40 steps of body-force flow."""
    d = golden("lbm_pipe_guo")
    nx, ny, nz = (int(v) for v in d["in_dims"])
    y0, z0, R = d["in_pipe"]
    nodes, cnt, types = O.pipe_guo_nodes((nx, ny, nz), y0, z0, R)
    assert cnt == d["out_wall_loc"].shape[0]
    C = np.array([[0, 0, 0], [-1, 0, 0], [0, -1, 0], [0, 0, -1], [-1, -1, 0], [-1, 1, 0], [-1, 0, -1], [-1, 0, 1],
                  [0, -1, -1], [0, -1, 1], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 0], [1, -1, 0], [1, 0, 1],
                  [1, 0, -1], [0, 1, 1], [0, 1, -1]])
    loc = np.array([[nodes[k].x, nodes[k].y, nodes[k].z] for k in range(cnt)])
    assert np.array_equal(loc, d["out_wall_loc"])
    assert np.array_equal(C[[nodes[k].dir for k in range(cnt)]], d["out_wall_dir"])
    assert np.array_equal(np.array([nodes[k].delta for k in range(cnt)]), d["out_wall_delta"])
    om = float(d["in_omega"])
    L = O.set_guo(O.lattice((nx, ny, nz), (1, 1, 1), "bgk_guo_vof", om, om, celltype=types), nodes, cnt)
    f0 = O.apply_guo(L, np.zeros((19, nz, ny, nx)))  # initializeAtEquilibrium + initialize()
    assert np.array_equal(f0, d["out_fbar_0"])
    F = np.broadcast_to(np.asarray(d["in_body"])[:, None, None, None], (3, nz, ny, nx))
    f1 = O.collide_stream(L, f0, F, np.zeros((nz, ny, nx)), 1)
    assert np.array_equal(f1, d["out_fbar_1"])
    fe = O.collide_stream(L, f0, F, np.zeros((nz, ny, nx)), int(d["in_steps"]))
    assert np.array_equal(fe, d["out_fbar_end"])
    assert np.array_equal(O.compute_velocity(L, fe, F), d["out_u_end"])


def test_move_vertices_reflects_at_pipe_wall():
    d = golden("reflect_pipe")
    assert np.array_equal(O.move_vertices(d["in_pos"], d["in_vel"], d["in_pipe"]), d["out_pos"])
    free = O.move_vertices(d["in_pos"], d["in_vel"])
    assert np.array_equal(free, d["in_pos"] + d["in_vel"]) and not np.array_equal(free, d["out_pos"])


def pipe_ibm_system(d):
    nx, ny, nz = (int(v) for v in d["in_dims"])
    y0, z0, R = d["in_pipe"]
    om = 1.0 / float(d["in_tau"])
    nodes, cnt, types = O.pipe_guo_nodes((nx, ny, nz), y0, z0, R)
    L = O.set_guo(O.lattice((nx, ny, nz), (1, 1, 1), "bgk_guo_vof", om, om, celltype=types), nodes, cnt)
    S = O.System(L, "roma", -1.0)
    S._keep = (nodes, types)
    S.f[...] = O.apply_guo(L, np.zeros((19, nz, ny, nx)))
    S.set_body_force(d["in_body"])
    S.set_pipe(y0, z0, R)
    pid = S.add_particle(S.add_shape(d["in_rest"], d["in_tri"]), int(d["in_model"]), d["in_params"], d["in_pos"])
    S.init()
    return S, pid


def test_capsule_near_pipe_wall():
    """A capsule next to the wall of a pipe with second-order walls: the near-wall TopHat
    blend of interpolation and spreading (set_boundary), step by step against the reference."""
    d = golden("ibm_pipe")
    S, pid = pipe_ibm_system(d)
    for it in range(int(d["in_steps"])):
        assert np.array_equal(S.particle(pid)["pos"], d["out_pos"][it])
        S.step(1)
        p = S.particle(pid)
        assert np.array_equal(p["vel"], d["out_vel"][it]), it
        assert np.array_equal(p["force"], d["out_force"][it]), it
        if it == 0:
            assert np.array_equal(S.force[:, :, :, 4:12], d["out_force_spread"])
    assert np.array_equal(S.particle(pid)["pos"], d["out_pos"][-1])
    assert np.array_equal(S.f[:, :, :, [0, 7]], d["out_fbar_end_planes"])
    assert np.array_equal(S.f.sum(axis=(1, 2, 3)), d["out_fbar_end_sum"])


def test_bending_force_is_the_gradient_of_the_bending_energy():
    """progs/bending_angle_test/bending_angle_test.cpp prints the analytic dihedral-angle gradient
    (tri::grad_angle_between_pair) beside central differences for a human to compare.  Here the
    comparison is a test: the RBC bending force of a deformed membrane (k_bend alone) equals minus the
    central-difference gradient of E = sum over pairs k_bend (1 - cos(t) cos(t0) - sin(t) sin(t0)),
    with cos t, sin t as tri::cos_sin_of_angle_between_pair (TriangleUtils.h:122-136) gives them."""
    from biblbm_gb300 import meshes

    rng = np.random.default_rng(11)
    xyz, tri = meshes.evans_fung(1, 4.0)
    S = O.Shape(xyz, tri)
    pos = xyz + 0.08 * rng.standard_normal(xyz.shape)
    kb = 0.05
    prm = O.params_vector(k_bend=kb, vol_desired=1.0)

    def unit_normal(a, b, c):
        n = np.cross(b - a, c - a)
        return n / np.linalg.norm(n)

    def energy(p):
        e = 0.0
        for (i0, i1, i2, i3), (c0, s0) in zip(S.pairs, S.pair_cs):
            n1, n2 = unit_normal(p[i0], p[i1], p[i2]), unit_normal(p[i0], p[i2], p[i3])
            c = float(n1 @ n2)
            s = (1.0 if float((n1 - n2) @ (p[i1] - p[i3])) > 0 else -1.0) * float(np.linalg.norm(np.cross(n1, n2)))
            e += kb * (1 - c * c0 - s * s0)
        return e

    F = O.membrane_forces("rbc_wlcpow", prm, S, pos)
    dx = 1e-6
    fd = np.zeros_like(pos)
    for i in range(pos.shape[0]):
        for a in range(3):
            pp, pm = pos.copy(), pos.copy()
            pp[i, a] += dx
            pm[i, a] -= dx
            fd[i, a] = -(energy(pp) - energy(pm)) / (2 * dx)
    assert np.abs(F - fd).max() < 1e-6 * np.abs(fd).max()
