"""CUDA path (through the C ABI) against the reference fixtures and the CPU oracle.

Tolerances: the FP64 path is compared with the reference / oracle to 1e-13 absolute on
populations (|f-bar| <= ~1e-2) and 1e-12 relative on vertex data.  It is not bit-exact:
nvcc contracts multiply-adds into FMAs, and spreading uses atomics whose summation order
varies from run to run.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import golden

pytestmark = pytest.mark.gpu

bib = pytest.importorskip("biblbm_gb300")
from biblbm_gb300 import meshes  # noqa: E402


@pytest.fixture(scope="module")
def ctx():
    c = bib.Context(0)
    yield c
    c.close()


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


# collide-and-stream kernels: shared-memory staged (default where the x-row fits) and
# row-vectorised; odd nx runs the per-cell kernel
KERNELS = ["staged", "rows"]


def shear_state(L, U):
    nx, ny, nz = L.nx, L.ny, L.nz
    y = np.arange(ny)
    u = np.zeros((3, nz, ny, nx))
    u[0] = (U * (2.0 * y / (ny - 1) - 1))[None, :, None]
    return u


# ---------------------------------------------------------------- lattice
def test_periodic_collide_stream_matches_oracle(ctx):
    d = golden("lbm_periodic")
    nx, ny, nz = (int(v) for v in d["in_dims"])
    om = d["in_omega"]
    lat = ctx.add_domain(nx, ny, nz, periodic=(1, 1, 1), omega=om[0], omega_inner=om[1], use_phase=True)
    lat.send(d["in_fbar"])
    lat.set_external_force(d["in_force"])
    lat.set_phase(d["in_phase"])
    assert np.abs(lat.compute_velocity() - d["out_u_0"]).max() < 1e-15
    lat.collide_and_stream(1)
    f1 = lat.receive()
    L = O.lattice((nx, ny, nz), (1, 1, 1), "bgk_guo_vof", om[0], om[1])
    ref1 = O.collide_stream(L, d["in_fbar"], d["in_force"], d["in_phase"], 1)
    assert np.abs(f1 - ref1).max() < 1e-15
    # populations that did not cross a periodic face equal the reference's own output
    assert np.abs(f1[0] - d["out_fbar_1"][0]).max() < 1e-15
    lat.collide_and_stream(2)
    ref3 = O.collide_stream(L, d["in_fbar"], d["in_force"], d["in_phase"], 3)
    assert np.abs(lat.receive() - ref3).max() < 1e-14


@pytest.mark.parametrize("kernel", KERNELS)
def test_shear_walls_match_reference(ctx, kernel):
    d = golden("lbm_shear")
    nx, ny, nz = (int(v) for v in d["in_dims"])
    om = d["in_omega"]
    U = float(d["in_U"])
    wall_u = [[-U, 0, 0], [U, 0, 0], [0, 0, 0], [0, 0, 0]]
    lat = ctx.add_domain(nx, ny, nz, periodic=(1, 0, 1), omega=om[0], wall_y="fd_velocity", wall_u=wall_u)
    lat.set_tuning(kernel)
    L = O.lattice((nx, ny, nz), (1, 0, 1), "bgk_guo_vof", om[0], om[1], wall_y="fd_velocity", wall_u=wall_u)
    lat.initialize_at_equilibrium(None, shear_state(L, U))
    assert np.abs(lat.receive() - d["out_fbar_0"]).max() < 1e-16
    lat.set_external_force(d["in_force"])
    lat.collide_and_stream(1)
    assert np.abs(lat.receive() - d["out_fbar_1"]).max() < 1e-15
    assert np.abs(lat.compute_velocity() - d["out_u_1"]).max() < 1e-15
    lat.collide_and_stream(int(d["in_steps"]) - 1)
    assert np.abs(lat.receive() - d["out_fbar_end"]).max() < 1e-15
    assert np.abs(lat.compute_velocity() - d["out_u_end"]).max() < 1e-15


def test_palabos_layout_round_trip(ctx):
    d = golden("lbm_periodic")
    nx, ny, nz = (int(v) for v in d["in_dims"])
    lat = ctx.add_domain(nx, ny, nz, periodic=(1, 1, 1), omega=1.2)
    wire = np.zeros((nx, ny, nz, 23))
    wire[..., :19] = np.transpose(d["in_fbar"], (3, 2, 1, 0))
    wire[..., 19:22] = np.transpose(d["in_force"], (3, 2, 1, 0))
    lat.send(wire, layout="palabos")
    assert np.array_equal(lat.receive(), d["in_fbar"])
    assert np.array_equal(lat.get_external_force(), d["in_force"])
    back = lat.receive(layout="palabos")
    assert np.array_equal(back[..., :22], wire[..., :22])


@pytest.mark.parametrize("nx,kernel", [(16, "staged"), (16, "rows"), (11, "auto")])
@pytest.mark.parametrize("storage", ["f64", "f32", "f16"])
def test_channel_bounce_back_against_oracle(ctx, nx, kernel, storage):
    """Halfway bounce-back on y and z with moving walls, body force, random state."""
    rng = np.random.default_rng(7)
    ny, nz = 7, 6
    wall_u = [[0.01, 0, 0.002], [-0.005, 0, 0], [0, 0.003, 0], [0.004, -0.002, 0]]
    f0 = 1e-3 * rng.uniform(-1, 1, (19, nz, ny, nx))
    F = 1e-4 * rng.uniform(-1, 1, (3, nz, ny, nx))
    lat = ctx.add_domain(nx, ny, nz, periodic=(1, 0, 0), omega=1.3, wall_y="halfway_bb", wall_z="halfway_bb",
                         wall_u=wall_u, storage=storage)
    if kernel != "auto":
        lat.set_tuning(kernel)
    lat.send(f0)
    lat.set_external_force(F)
    lat.collide_and_stream(5)
    L = O.lattice((nx, ny, nz), (1, 0, 0), "bgk_guo_vof", 1.3, 1.3, wall_y="halfway_bb", wall_z="halfway_bb",
                  wall_u=wall_u)
    ref = O.collide_stream(L, f0, F, None, 5)
    tol = {"f64": 1e-15, "f32": 2e-8, "f16": 1e-5}[storage]
    assert np.abs(lat.receive() - ref).max() < tol
    assert np.abs(lat.compute_velocity() - O.compute_velocity(L, ref, F)).max() < 50 * tol


@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("storage,tol", [("f64", 1e-14), ("f32", 5e-6), ("f16", 2e-3)])
def test_taylor_green_trt(ctx, storage, tol, kernel):
    """TRT (magic 1/4) Taylor-Green decay: against the FP64 oracle and the analytic rate."""
    from tests.test_oracle_analytic import tgv_state

    n, u0, tau, steps = 32, 0.02, 0.8, 200
    L = O.lattice((n, n, 4), (1, 1, 1), "trt", 1 / tau, trt_magic=0.25)
    f0, k = tgv_state(n, u0, L)
    lat = ctx.add_domain(n, n, 4, periodic=(1, 1, 1), collision="trt", omega=1 / tau, trt_magic=0.25, storage=storage)
    lat.set_tuning(kernel)
    lat.send(f0)
    lat.collide_and_stream(steps)
    ref = O.collide_stream(L, f0, None, None, steps)
    u_gpu, u_ref = lat.compute_velocity(), O.compute_velocity(L, ref)
    assert np.abs(u_gpu - u_ref).max() < tol * u0
    nu = (tau - 0.5) / 3
    expect = np.exp(-2 * nu * k * k * steps)
    assert abs(np.abs(u_gpu[0]).max() / u0 - expect) / expect < 1.5e-2


# ---------------------------------------------------------------- membranes
@pytest.mark.parametrize("mode", ["atomic", "deterministic"])
@pytest.mark.parametrize("model", ["capsule_neohookean", "capsule_skalak", "rbc_wlcpow", "skalak_bending"])
def test_membrane_forces_match_reference(ctx, model, mode):
    d = golden("forces_" + model)
    n = 40
    lat = ctx.add_domain(n, n, n, periodic=(1, 1, 1), omega=1.0)
    shapes = bib.ParticleShapeLibrary(ctx)
    sid = shapes.store_mesh(d["in_rest"], d["in_tri"], "m")
    fsi = bib.ImmersedBoundaryDynamics3D(lat, shapes, spread=mode)
    pos = d["in_pos"] + np.array([15.0, 18.0, 12.0])  # inside the box, away from the faces
    pid = fsi.add_particle(sid, model, d["in_params"], pos)
    p0 = fsi.get_particle(pid)
    assert abs(p0["area"] - d["out_area"][0]) < 1e-12 * d["out_area"][0]
    assert abs(p0["volume"] - d["out_volume"][0]) < 1e-10 * d["out_volume"][0]
    fsi.ibm_step()  # forces are evaluated at the current positions, before the move
    p = fsi.get_particle(pid)
    assert rel(p["force"], d["out_force"]) < 1e-11


# ---------------------------------------------------------------- coupled steps
def run_coupled_gpu(ctx, d, storage="f64", graph=True, spread="atomic", kernel="auto", use_phase=False):
    """The fixture's coupled case on the GPU; use_phase (implied by a viscosity ratio in the
    fixture) gives the lattice a phase field that the membranes are voxelized into."""
    nx, ny, nz = (int(v) for v in d["in_dims"])
    tau = float(d["in_tau"])
    om = 1.0 / tau
    lam = float(d["in_lambda"]) if "in_lambda" in d.files else 1.0
    phase_kw = {}
    if use_phase or lam != 1.0:
        phase_kw = dict(use_phase=True, omega_inner=1.0 / (0.5 + lam * (tau - 0.5)))
    walls = int(d["in_walls"])
    body = d["in_body"] if "in_body" in d.files else np.zeros(3)
    if walls == 1:
        U = float(d["in_U"])
        wall_u = [[-U, 0, 0], [U, 0, 0], [0, 0, 0], [0, 0, 0]]
        lat = ctx.add_domain(nx, ny, nz, periodic=(1, 0, 1), omega=om, wall_y="fd_velocity", wall_u=wall_u,
                             storage=storage, body_force=body, **phase_kw)
        L = O.lattice((nx, ny, nz), (1, 0, 1), "bgk_guo_vof", om, om, wall_y="fd_velocity", wall_u=wall_u)
        lat.initialize_at_equilibrium(None, shear_state(L, U))
    else:
        lat = ctx.add_domain(nx, ny, nz, periodic=(1, 1, 1), omega=om, storage=storage, body_force=body, **phase_kw)
        lat.initialize_at_equilibrium(None, np.zeros((3, nz, ny, nx)))
    lat.set_tuning(kernel)
    shapes = bib.ParticleShapeLibrary(ctx)
    sid = shapes.store_mesh(d["in_rest"], d["in_tri"], "p")
    fsi = bib.ImmersedBoundaryDynamics3D(lat, shapes, spread=spread)
    model = {0: "capsule_neohookean", 1: "capsule_skalak", 2: "rbc_wlcpow", 3: "skalak_bending"}[int(d["in_model"])]
    pid = fsi.add_particle(sid, model, d["in_params"], d["in_pos"])
    ctx.set_graph_mode(graph)
    return lat, fsi, pid


@pytest.mark.parametrize("name", ["ibm_capsule_shear", "ibm_rbc_periodic"])
@pytest.mark.parametrize("kernel", KERNELS)
def test_coupled_steps_match_reference(ctx, name, kernel):
    d = golden(name)
    lat, fsi, pid = run_coupled_gpu(ctx, d, graph=False, kernel=kernel)
    steps = int(d["in_steps"])
    fscale = np.abs(d["out_force"]).max()  # the first steps start stress-free (forces ~1e-17)
    for it in range(steps):
        p = fsi.get_particle(pid)
        assert rel(p["pos"], d["out_pos"][it]) < 1e-13
        fsi.step(1)
        p = fsi.get_particle(pid)
        assert rel(p["vel"], d["out_vel"][it]) < 1e-11, it
        assert np.abs(p["force"] - d["out_force"][it]).max() < 1e-10 * fscale, it
        assert abs(p["volume"] - d["out_volume"][it + 1]) < 1e-11 * d["out_volume"][it + 1]
        if it == 0:
            assert np.abs(lat.get_external_force() - d["out_force_spread"]).max() < 1e-15
    assert np.abs(lat.compute_velocity() - d["out_u_end"]).max() < 1e-14
    assert rel(fsi.get_particle(pid)["inertia"], d["out_inertia"][-1]) < 1e-12


@pytest.mark.parametrize("name", ["ibm_capsule_shear", "ibm_rbc_periodic"])
@pytest.mark.parametrize("kernel", KERNELS)
def test_voxelized_phase_matches_reference(ctx, name, kernel):
    """Viscosity ratio 1 with a phase field: the step that voxelizes the moved membranes
    before the collision follows the reference's trajectory, and the phase field of the
    final positions is the reference's, cell for cell."""
    d = golden(name)
    lat, fsi, pid = run_coupled_gpu(ctx, d, graph=False, kernel=kernel, use_phase=True)
    steps = int(d["in_steps"])
    fscale = np.abs(d["out_force"]).max()
    for it in range(steps):
        fsi.step(1)
        p = fsi.get_particle(pid)
        assert rel(p["pos"], d["out_pos"][it + 1]) < 1e-13, it
        assert rel(p["vel"], d["out_vel"][it]) < 1e-11, it
        assert np.abs(p["force"] - d["out_force"][it]).max() < 1e-10 * fscale, it
    assert np.abs(lat.compute_velocity() - d["out_u_end"]).max() < 1e-14
    ph = lat.get_phase()
    assert ph.sum() > 0
    assert np.array_equal(ph, d["out_phase_end"])


def oracle_lambda_system(d):
    """The oracle on the fixture's inputs with the reference's intended dynamics (no omega
    swap on the periodic envelope), voxelizing after every move."""
    nx, ny, nz = (int(v) for v in d["in_dims"])
    tau, lam, U = float(d["in_tau"]), float(d["in_lambda"]), float(d["in_U"])
    om, om_in = 1 / tau, 1 / (0.5 + lam * (tau - 0.5))
    wall_u = [[-U, 0, 0], [U, 0, 0], [0, 0, 0], [0, 0, 0]]
    L = O.lattice((nx, ny, nz), (1, 0, 1), "bgk_guo_vof", om, om_in, wall_y="fd_velocity", wall_u=wall_u,
                  envelope_swap=False)
    S = O.System(L, "roma", -1.0)
    S.f[...] = O.apply_fd_walls(L, O.init_equilibrium(L, None, shear_state(L, U)), np.zeros((3, nz, ny, nx)))
    S.set_voxelize(True)
    pid = S.add_particle(S.add_shape(d["in_rest"], d["in_tri"]), int(d["in_model"]), d["in_params"], d["in_pos"])
    S.init()
    return S, pid


@pytest.mark.parametrize("kernel,graph", [("staged", False), ("rows", False), ("staged", True)])
def test_viscosity_ratio_capsule_against_oracle(ctx, kernel, graph):
    """Viscosity ratio 5: the voxelized phase selects omega in every collision.  Positions,
    forces and the phase field follow the oracle step by step, the populations at the end."""
    d = golden("ibm_capsule_lambda")
    S, opid = oracle_lambda_system(d)
    lat, fsi, pid = run_coupled_gpu(ctx, d, graph=graph, kernel=kernel)
    steps = int(d["in_steps"])
    if graph:  # graph replay: compare at the end only
        S.step(steps)
        fsi.step(steps)
    for it in range(0 if graph else steps):
        S.step(1)
        fsi.step(1)
        g, r = fsi.get_particle(pid), S.particle(opid)
        assert rel(g["pos"], r["pos"]) < 1e-13, it
        assert rel(g["vel"], r["vel"]) < 1e-11, it
        assert np.array_equal(lat.get_phase(), S.phase), it
    g, r = fsi.get_particle(pid), S.particle(opid)
    assert rel(g["pos"], r["pos"]) < 1e-13
    assert np.array_equal(lat.get_phase(), S.phase)
    assert lat.get_phase().sum() > 0
    assert np.abs(lat.receive() - S.f).max() < 1e-13
    assert np.abs(lat.compute_velocity() - S.velocity()).max() < 1e-14


# 10-cell rows: 80 bytes in FP64 fit the staged tile, 40 bytes in FP32 do not
@pytest.mark.parametrize("kernel,storage,tol", [("staged", "f64", 1e-15), ("rows", "f64", 1e-15), ("rows", "f32", 1e-7)])
def test_bounce_back_nodes_match_reference(ctx, kernel, storage, tol):
    """BounceBack / NoDynamics nodes set per cell, against the reference's own run."""
    d = golden("lbm_bounceback")
    nx, ny, nz = (int(v) for v in d["in_dims"])
    om = d["in_omega"]
    lat = ctx.add_domain(nx, ny, nz, periodic=(1, 1, 1), omega=om[0], omega_inner=om[1], storage=storage)
    lat.set_tuning(kernel)
    lat.set_cell_types(d["in_celltype"])
    lat.send(d["in_fbar"])
    lat.set_external_force(d["in_force"])
    lat.collide_and_stream(1)
    assert np.abs(lat.receive() - d["out_fbar_1"]).max() < tol
    lat.collide_and_stream(int(d["in_steps"]) - 1)
    assert np.abs(lat.receive() - d["out_fbar_end"]).max() < tol
    assert np.abs(lat.compute_velocity() - d["out_u_end"]).max() < 50 * tol


def test_bounce_back_nodes_odd_rows_and_coupled_steps(ctx):
    """Odd nx (per-cell kernel) against the oracle; coupled steps of the staged and the
    row-vectorised kernels against each other, with solid and NoDynamics cells."""
    rng = np.random.default_rng(23)
    nx, ny, nz = 11, 9, 6
    f0 = 1e-3 * rng.uniform(-1, 1, (19, nz, ny, nx))
    F = 1e-4 * rng.uniform(-1, 1, (3, nz, ny, nx))
    ct = (rng.uniform(size=(nz, ny, nx)) < 0.2).astype(np.uint8) + (rng.uniform(size=(nz, ny, nx)) < 0.05)
    lat = ctx.add_domain(nx, ny, nz, periodic=(1, 0, 1), omega=1.2, wall_y="halfway_bb")
    lat.set_cell_types(ct)
    lat.send(f0)
    lat.set_external_force(F)
    lat.collide_and_stream(3)
    L = O.lattice((nx, ny, nz), (1, 0, 1), "bgk_guo_vof", 1.2, 1.2, wall_y="halfway_bb", celltype=ct)
    ref = O.collide_stream(L, f0, F, None, 3)
    assert np.abs(lat.receive() - ref).max() < 1e-15
    assert np.abs(lat.compute_velocity() - O.compute_velocity(L, ref, F)).max() < 1e-14
    nx = 16
    f0 = 1e-3 * rng.uniform(-1, 1, (19, nz, ny, nx))
    ct = (rng.uniform(size=(nz, ny, nx)) < 0.2).astype(np.uint8) + (rng.uniform(size=(nz, ny, nx)) < 0.05)
    out = {}
    for kernel in ("rows", "staged"):
        lat = ctx.add_domain(nx, ny, nz, periodic=(1, 0, 1), omega=1.2, wall_y="halfway_bb", body_force=(1e-5, 0, 0))
        lat.set_tuning(kernel)
        lat.set_cell_types(ct)
        lat.send(f0)
        fsi = bib.ImmersedBoundaryDynamics3D(lat, bib.ParticleShapeLibrary(ctx))
        fsi.step(4)
        out[kernel] = (lat.receive(), lat.compute_velocity())
    for a, b in zip(out["rows"], out["staged"]):
        assert np.abs(a - b).max() < 1e-16


def random_channel(nx, ny, nz, seed=11):
    rng = np.random.default_rng(seed)
    f0 = 1e-3 * rng.uniform(-1, 1, (19, nz, ny, nx))
    F = 1e-4 * rng.uniform(-1, 1, (3, nz, ny, nx))
    phase = (rng.uniform(size=(nz, ny, nx)) < 0.3).astype(np.float64)
    return f0, F, phase


@pytest.mark.parametrize("storage,tol", [("f64", 1e-15), ("f32", 2e-8), ("f16", 1e-5)])
def test_staged_pipeline_many_tiles(ctx, storage, tol):
    """Thousands of one-row tiles per launch: every CTA runs the double-buffered pipeline
    through many tiles.  Periodic y, moving halfway walls on z, phase field, body force."""
    nx, ny, nz = 32, 64, 48
    f0, F, phase = random_channel(nx, ny, nz)
    wall_u = [[0, 0, 0], [0, 0, 0], [0.003, 0, 0.001], [-0.002, 0.001, 0]]
    kw = dict(periodic=(1, 1, 0), omega=1.3, omega_inner=0.9, use_phase=True, wall_z="halfway_bb", wall_u=wall_u)
    lat = ctx.add_domain(nx, ny, nz, storage=storage, **kw)
    lat.set_tuning("staged", tile_cells=nx)
    lat.send(f0)
    lat.set_external_force(F)
    lat.set_phase(phase)
    lat.collide_and_stream(3)
    L = O.lattice((nx, ny, nz), (1, 1, 0), "bgk_guo_vof", 1.3, 0.9, wall_z="halfway_bb", wall_u=wall_u)
    ref = O.collide_stream(L, f0, F, phase, 3)
    assert np.abs(lat.receive() - ref).max() < tol
    lat.check_health()


@pytest.mark.parametrize("storage", ["f64", "f32", "f16"])
@pytest.mark.parametrize("tile_cells", [32, 160, 0])
def test_staged_coupled_step_equals_rows_kernel(ctx, storage, tile_cells):
    """Coupled lattice step (velocity output, force reset, body force) of the staged kernel
    against the row-vectorised kernel, on 1-, 5- and 16-row tiles."""
    nx, ny, nz = 32, 80, 24
    f0, F, phase = random_channel(nx, ny, nz, seed=5)
    out = {}
    for kernel in ("rows", "staged"):
        lat = ctx.add_domain(nx, ny, nz, periodic=(1, 0, 0), omega=1.1, wall_y="halfway_bb", wall_z="halfway_bb",
                             storage=storage, body_force=(1e-5, -2e-6, 0))
        lat.set_tuning(kernel, tile_cells=tile_cells)
        lat.send(f0)
        lat.set_external_force(F)
        fsi = bib.ImmersedBoundaryDynamics3D(lat, bib.ParticleShapeLibrary(ctx))
        fsi.step(4)
        out[kernel] = (lat.receive(), lat.compute_velocity(), lat.get_external_force())
    tol = {"f64": 1e-16, "f32": 2e-9, "f16": 5e-6}[storage]
    for a, b in zip(out["rows"], out["staged"]):
        assert np.abs(a - b).max() < tol


def test_staged_kernel_rejects_misfit_rows(ctx):
    lat = ctx.add_domain(12, 8, 8, periodic=(1, 1, 1), omega=1.0, storage="f16")  # 24-byte rows
    with pytest.raises(bib.BibError):
        lat.set_tuning("staged")
    lat.set_tuning("auto")
    lat.collide_and_stream(1)


def test_graph_replay_equals_plain_launches(ctx):
    d = golden("ibm_capsule_shear")
    lat_a, fsi_a, pa = run_coupled_gpu(ctx, d, graph=False)
    fsi_a.step(6)
    lat_b, fsi_b, pb = run_coupled_gpu(ctx, d, graph=True)
    fsi_b.step(6)
    ctx.set_graph_mode(True)
    assert rel(fsi_b.get_particle(pb)["pos"], fsi_a.get_particle(pa)["pos"]) < 1e-14
    assert np.abs(lat_b.receive() - lat_a.receive()).max() < 1e-15
    # one step at a time with a read after each: one-step graphs of every parity state
    lat_c, fsi_c, pc = run_coupled_gpu(ctx, d, graph=True)
    for _ in range(6):
        fsi_c.step(1)
        fsi_c.get_particle(pc)
    assert rel(fsi_c.get_particle(pc)["pos"], fsi_a.get_particle(pa)["pos"]) < 1e-14
    assert np.abs(lat_c.receive() - lat_a.receive()).max() < 1e-15
    assert lat_c.iteration() == lat_a.iteration()


def oracle_capsule_system(n, U, xyz, tri, pos, prm, dirac="roma", steps=0):
    om = 1.0
    wall_u = [[-U, 0, 0], [U, 0, 0], [0, 0, 0], [0, 0, 0]]
    L = O.lattice((n, n, n), (1, 0, 1), "bgk_guo_vof", om, om, wall_y="fd_velocity", wall_u=wall_u)
    S = O.System(L, dirac, -1.0)
    S.f[...] = O.apply_fd_walls(L, O.init_equilibrium(L, None, shear_state(L, U)), np.zeros((3, n, n, n)))
    pid = S.add_particle(S.add_shape(xyz, tri), "capsule_skalak", prm, pos)
    S.step(steps)
    return S, pid


@pytest.mark.parametrize("dirac", ["roma", "peskin"])
def test_capsule_in_shear_against_oracle(ctx, dirac):
    n, U = 20, 0.03
    xyz, tri = meshes.icosphere(2, 4.0)
    pos = meshes.place(xyz, None, (9.4, 9.2, 9.6))
    prm = bib.membrane_params(G=0.002, C=1.0)
    S, opid = oracle_capsule_system(n, U, xyz, tri, pos, prm, dirac, steps=20)
    wall_u = [[-U, 0, 0], [U, 0, 0], [0, 0, 0], [0, 0, 0]]
    lat = ctx.add_domain(n, n, n, periodic=(1, 0, 1), omega=1.0, wall_y="fd_velocity", wall_u=wall_u)
    lat.initialize_at_equilibrium(None, shear_state(S.L, U))
    shapes = bib.ParticleShapeLibrary(ctx)
    fsi = bib.ImmersedBoundaryDynamics3D(lat, shapes, dirac=dirac)
    pid = fsi.add_particle(shapes.store_mesh(xyz, tri, "c"), "capsule_skalak", prm, pos)
    fsi.step(20)
    g, r = fsi.get_particle(pid), S.particle(opid)
    assert rel(g["pos"], r["pos"]) < 1e-13
    assert rel(g["force"], r["force"]) < 1e-8
    assert np.abs(lat.receive() - S.f).max() < 1e-13


@pytest.mark.parametrize("storage", ["f64", "f32"])
def test_deterministic_spreading(ctx, storage):
    """Vertex-sorted spreading: identical bits on every run, equal to the atomic path to
    rounding, and to the oracle."""
    d = golden("ibm_rbc_periodic")
    runs = []
    for mode in ["deterministic", "deterministic", "atomic"]:
        lat, fsi, pid = run_coupled_gpu(ctx, d, storage=storage, graph=True, spread=mode)
        fsi.step(7)
        runs.append((lat.receive(), fsi.get_particle(pid)["pos"], lat.get_external_force()))
    assert np.array_equal(runs[0][0], runs[1][0]) and np.array_equal(runs[0][1], runs[1][1])
    assert np.array_equal(runs[0][2], runs[1][2])
    tol = 1e-15 if storage == "f64" else 1e-8
    assert np.abs(runs[0][0] - runs[2][0]).max() < tol
    assert rel(runs[0][1], runs[2][1]) < (1e-14 if storage == "f64" else 1e-7)


# ---------------------------------------------------------------- reduced precision
@pytest.mark.parametrize("storage,tol_pos,tol_u", [("f32", 2e-5, 2e-4), ("f16", 2e-3, 2e-2)])
def test_reduced_precision_capsule(ctx, storage, tol_pos, tol_u):
    """FP32 / FP16 deviation storage against the FP64 oracle on the same inputs.

    Bounds: vertex displacement error relative to the displacement itself, and the
    velocity field relative L2 error, after 40 steps.
    """
    n, U = 20, 0.03
    xyz, tri = meshes.icosphere(2, 4.0)
    pos = meshes.place(xyz, None, (9.4, 9.2, 9.6))
    prm = bib.membrane_params(G=0.002, C=1.0)
    S, opid = oracle_capsule_system(n, U, xyz, tri, pos, prm, steps=40)
    wall_u = [[-U, 0, 0], [U, 0, 0], [0, 0, 0], [0, 0, 0]]
    lat = ctx.add_domain(n, n, n, periodic=(1, 0, 1), omega=1.0, wall_y="fd_velocity", wall_u=wall_u, storage=storage)
    lat.initialize_at_equilibrium(None, shear_state(S.L, U))
    shapes = bib.ParticleShapeLibrary(ctx)
    fsi = bib.ImmersedBoundaryDynamics3D(lat, shapes)
    pid = fsi.add_particle(shapes.store_mesh(xyz, tri, "c"), "capsule_skalak", prm, pos)
    fsi.step(40)
    g, r = fsi.get_particle(pid), S.particle(opid)
    disp = np.abs(r["pos"] - pos).max()
    assert np.abs(g["pos"] - r["pos"]).max() < tol_pos * max(disp, 1e-3) + 1e-6
    u_ref = S.velocity()
    err = np.linalg.norm(lat.compute_velocity() - u_ref) / np.linalg.norm(u_ref)
    assert err < tol_u
    assert abs(g["volume"] - r["volume"]) / r["volume"] < 1e-4


# ---------------------------------------------------------------- errors
def test_invalid_arguments_are_reported(ctx):
    with pytest.raises(bib.BibError) as e:
        ctx.add_domain(2, 8, 8, periodic=(1, 1, 1), omega=1.0)
    assert e.value.status == -1
    with pytest.raises(bib.BibError):
        ctx.add_domain(8, 8, 8, periodic=(1, 1, 1), omega=2.5)
    lat = ctx.add_domain(8, 8, 8, periodic=(1, 1, 1), omega=1.0)
    with pytest.raises(bib.BibError):
        lat.send(np.zeros(10))
    shapes = bib.ParticleShapeLibrary(ctx)
    with pytest.raises(bib.BibError):
        shapes.store_mesh(np.zeros((4, 3)), np.array([[0, 1, 9], [0, 1, 2], [1, 2, 3], [0, 2, 3]]), "bad")


def test_nan_is_detected(ctx):
    lat = ctx.add_domain(8, 8, 8, periodic=(1, 1, 1), omega=1.0)
    f = np.zeros((19, 8, 8, 8))
    f[3, 2, 2, 2] = np.nan
    lat.send(f)
    with pytest.raises(bib.BibError) as e:
        lat.check_health()
    assert e.value.status == -4


@pytest.mark.parametrize("kernel,storage,tol", [("staged", "f64", 1e-15), ("rows", "f64", 1e-15), ("staged", "f32", 1e-7),
                                                ("rows", "f16", 2e-4)])
def test_pipe_walls_match_reference(ctx, kernel, storage, tol):
    """First-order pipe walls (rbc_in_pipe.cpp: BounceBack outside the pipe, NoDynamics beyond
    radius + 1) with a body force, against the reference's populations after 40 steps."""
    d = golden("lbm_pipe")
    nx, ny, nz = (int(v) for v in d["in_dims"])
    y0, z0, R = d["in_pipe"]
    om = float(d["in_omega"])
    lat = ctx.add_domain(nx, ny, nz, periodic=(1, 1, 1), omega=om, storage=storage)
    lat.set_tuning(kernel)
    lat.set_pipe_walls(y0, z0, R)
    lat.initialize_at_equilibrium(None, np.zeros((3, nz, ny, nx)))
    lat.set_external_force(np.asarray(d["in_body"])[:, None, None, None])
    lat.collide_and_stream(int(d["in_steps"]))
    f = lat.receive()
    assert np.abs(f - d["out_fbar_end"]).max() <= tol
    fluid = d["out_mask"] == 0
    u = lat.compute_velocity()
    assert np.abs(u[:, fluid] - d["out_u_end"][:, fluid]).max() <= 10 * tol


# 12-cell rows: FP16 rows (24 bytes) do not fit the staged tile's 16-byte copies
@pytest.mark.parametrize("kernel,storage,tol", [("staged", "f64", 1e-15), ("rows", "f64", 1e-15), ("staged", "f32", 1e-7),
                                                ("rows", "f16", 2e-4)])
def test_second_order_pipe_walls_match_reference(ctx, kernel, storage, tol):
    """GuoRigidWallBoundary on a pipe (rbc_in_pipe.cpp's second-order walls): the state after
    initialize(), one step and 40 steps of body-force flow, against the reference."""
    d = golden("lbm_pipe_guo")
    nx, ny, nz = (int(v) for v in d["in_dims"])
    y0, z0, R = d["in_pipe"]
    om = float(d["in_omega"])
    lat = ctx.add_domain(nx, ny, nz, periodic=(1, 1, 1), omega=om, storage=storage)
    lat.set_tuning(kernel)
    lat.set_pipe_walls(y0, z0, R, second_order=True)
    lat.initialize_at_equilibrium(None, np.zeros((3, nz, ny, nx)))
    assert np.abs(lat.receive() - d["out_fbar_0"]).max() <= tol
    lat.set_external_force(np.asarray(d["in_body"])[:, None, None, None])
    lat.collide_and_stream(1)
    assert np.abs(lat.receive() - d["out_fbar_1"]).max() <= tol
    lat.collide_and_stream(int(d["in_steps"]) - 1)
    assert np.abs(lat.receive() - d["out_fbar_end"]).max() <= tol
    u = lat.compute_velocity()
    assert np.abs(u - d["out_u_end"]).max() <= 10 * tol


def test_pipe_too_narrow_for_second_order_walls(ctx):
    lat = ctx.add_domain(8, 9, 9, periodic=(1, 1, 1), omega=1.0)
    with pytest.raises(bib.BibError, match="narrow"):
        lat.set_pipe_walls(4.0, 4.0, 1.2, second_order=True)
    lat.set_pipe_walls(4.0, 4.0, 1.2)  # first order works at any size


def pipe_capsule_gpu(ctx, d, u0=None, storage="f64"):
    nx, ny, nz = (int(v) for v in d["in_dims"])
    y0, z0, R = d["in_pipe"]
    lat = ctx.add_domain(nx, ny, nz, periodic=(1, 1, 1), omega=1.0 / float(d["in_tau"]), body_force=d["in_body"],
                         storage=storage)
    lat.set_pipe_walls(y0, z0, R, second_order=True)
    lat.initialize_at_equilibrium(None, np.zeros((3, nz, ny, nx)) if u0 is None else u0)
    shapes = bib.ParticleShapeLibrary(ctx)
    fsi = bib.ImmersedBoundaryDynamics3D(lat, shapes)
    fsi.set_boundary(y0, z0, R)
    pid = fsi.add_particle(shapes.store_mesh(d["in_rest"], d["in_tri"], "c"), "capsule_skalak", d["in_params"], d["in_pos"])
    ctx.set_graph_mode(False)
    return lat, fsi, pid


def test_capsule_near_pipe_wall_matches_reference(ctx):
    """set_boundary(PipeBoundary): the TopHat near-wall blend of interpolation and spreading,
    with the second-order pipe walls, step by step against the reference."""
    d = golden("ibm_pipe")
    lat, fsi, pid = pipe_capsule_gpu(ctx, d)
    fscale = np.abs(d["out_force"]).max()
    for it in range(int(d["in_steps"])):
        fsi.step(1)
        p = fsi.get_particle(pid)
        assert rel(p["pos"], d["out_pos"][it + 1]) < 1e-13, it
        assert np.abs(p["vel"] - d["out_vel"][it]).max() < 1e-11 * max(np.abs(d["out_vel"][it]).max(), 1e-30), it
        assert np.abs(p["force"] - d["out_force"][it]).max() < 1e-10 * fscale, it
        if it == 0:
            F = lat.get_external_force()[:, :, :, 4:12]
            assert np.abs(F - d["out_force_spread"]).max() < 1e-15
    f = lat.receive()
    assert np.abs(f[:, :, :, [0, 7]] - d["out_fbar_end_planes"]).max() < 1e-14
    ctx.set_graph_mode(True)


@pytest.mark.parametrize("storage,tol", [("f32", 1e-4), ("f16", 3e-2)])
def test_capsule_near_pipe_wall_reduced_precision(ctx, storage, tol):
    """The same capsule with FP32 / FP16 populations: its vertex displacements over the run follow
    the reference's FP64 ones within the storage's precision."""
    d = golden("ibm_pipe")
    lat, fsi, pid = pipe_capsule_gpu(ctx, d, storage=storage)
    ctx.set_graph_mode(True)
    fsi.step(int(d["in_steps"]))
    disp = fsi.get_particle(pid)["pos"] - d["out_pos"][0]
    ref = d["out_pos"][-1] - d["out_pos"][0]
    assert np.abs(disp - ref).max() < tol * np.abs(ref).max()


def test_wall_reflection_against_oracle(ctx):
    """A capsule against the wall in a strong outward flow: vertices whose step crosses the
    wall are reflected (DeformableParticle3D::move_vertices), as the oracle does."""
    d = golden("ibm_pipe")
    nx, ny, nz = (int(v) for v in d["in_dims"])
    y0, z0, R = d["in_pipe"]
    Y, Z = np.meshgrid(np.arange(ny) - y0, np.arange(nz) - z0, indexing="ij")
    r = np.hypot(Y, Z) + 1e-30
    u0 = np.zeros((3, nz, ny, nx))
    inside = (r < R)[..., None]
    u0[1] = np.where(inside, (0.25 * Y / r)[..., None], 0.0).transpose(1, 0, 2)
    u0[2] = np.where(inside, (0.25 * Z / r)[..., None], 0.0).transpose(1, 0, 2)
    pos = d["in_pos"] + np.array([0.0, 0.55, 0.0])  # outermost vertices 0.2 from the wall
    dd = dict(d)
    dd["in_pos"] = pos
    lat, fsi, pid = pipe_capsule_gpu(ctx, dd, u0)
    nodes, cnt, types = O.pipe_guo_nodes((nx, ny, nz), y0, z0, R)
    L = O.set_guo(O.lattice((nx, ny, nz), (1, 1, 1), "bgk_guo_vof", 1.0, 1.0, celltype=types), nodes, cnt)
    S = O.System(L, "roma", -1.0)
    S.f[...] = O.apply_guo(L, O.init_equilibrium(L, None, u0))
    S.set_body_force(d["in_body"])
    S.set_pipe(y0, z0, R)
    opid = S.add_particle(S.add_shape(d["in_rest"], d["in_tri"]), "capsule_skalak", d["in_params"], pos)
    S.init()
    S.step(1)
    fsi.step(1)
    g, o = fsi.get_particle(pid), S.particle(opid)
    free = pos + o["vel"]
    crossed = np.hypot(free[:, 1] - y0, free[:, 2] - z0) > R
    assert crossed.sum() >= 3  # the step pushes some vertices through the wall
    assert np.hypot(o["pos"][:, 1] - y0, o["pos"][:, 2] - z0).max() <= R
    assert np.abs(g["pos"] - o["pos"]).max() < 1e-12
    ctx.set_graph_mode(True)


def test_async_download_equals_sync_download(ctx):
    """bib_particles_download_async behind each step, waited for one step later, gives the stats
    of every step as the synchronous download does."""
    d = golden("ibm_capsule_shear")
    lat, fsi, pid = run_coupled_gpu(ctx, d, spread="deterministic")
    lat2, fsi2, pid2 = run_coupled_gpu(ctx, d, spread="deterministic")
    bufs = [np.zeros((1, 5)), np.zeros((1, 5))]
    got, ref = [], []
    for k in range(6):
        fsi.step(1)
        fsi.download_async(bufs[k % 2], k % 2)
        if k:
            fsi.wait_download((k - 1) % 2)
            got.append(bufs[(k - 1) % 2].copy())
        fsi2.step(1)
        ref.append(fsi2.download()[1].copy())
    ctx.check(ctx.lib.bib_download_wait(ctx.h, 1))
    got.append(bufs[1].copy())
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("name", ["ibm_capsule_shear", "ibm_capsule_lambda"])
def test_bulk_position_upload_equals_per_particle_positions(ctx, name):
    """bib_particles_upload (all vertices into the live device state) continues like
    bib_particle_set_positions (which rebuilds the particle state from the host), with a
    re-voxelized phase field where the viscosity ratio needs one."""
    d = golden(name)
    lat_a, fsi_a, pa = run_coupled_gpu(ctx, d, spread="deterministic")
    lat_b, fsi_b, pb = run_coupled_gpu(ctx, d, spread="deterministic")
    fsi_a.step(2)
    fsi_b.step(2)
    new = fsi_a.get_particle(pa)["pos"] + np.array([0.3, -0.2, 0.1])
    fsi_a.set_positions(pa, new)
    fsi_b.upload_positions(new)
    pa_b = fsi_b.get_particle(pb)
    assert np.array_equal(pa_b["pos"], new)
    assert pa_b["volume"] == pytest.approx(fsi_a.get_particle(pa)["volume"], rel=1e-13)
    fsi_a.step(3)
    fsi_b.step(3)
    assert rel(fsi_b.get_particle(pb)["pos"], fsi_a.get_particle(pa)["pos"]) < 1e-12
    assert np.abs(lat_b.receive() - lat_a.receive()).max() < 1e-14
    if "lambda" in name:
        assert np.array_equal(lat_b.get_phase(), lat_a.get_phase())
