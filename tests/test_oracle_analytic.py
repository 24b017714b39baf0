"""Pins for the oracle's parts that have no reference counterpart: TRT collision and
halfway (moving-wall) bounce-back, checked against analytic flows.

- Taylor-Green vortex (z-invariant, periodic cube): the velocity amplitude decays as
  exp(-2 nu k^2 t), nu = (1/omega - 1/2)/3, for BGK and for TRT with any magic parameter.
- Plane Poiseuille flow between halfway bounce-back walls at y = -1/2 and y = ny - 1/2
  driven by a body force g (Guo forcing): u(y) = g/(2 nu) (y + 1/2)(ny - 1/2 - y).
- Plane Couette flow between a resting and a moving halfway wall: linear profile.
"""
import numpy as np
import pytest

from oracle import oracle as O


def tgv_state(n, u0, L):
    k = 2 * np.pi / n
    x = np.arange(n)
    X, Y = np.meshgrid(x, x, indexing="xy")  # (y, x)
    ux = u0 * np.sin(k * X) * np.cos(k * Y)
    uy = -u0 * np.cos(k * X) * np.sin(k * Y)
    p = 0.25 * u0 * u0 * (np.cos(2 * k * X) + np.cos(2 * k * Y))
    rho = 1.0 + 3.0 * p
    u = np.zeros((3, 4, n, n))
    u[0] = ux[None]
    u[1] = uy[None]
    return O.init_equilibrium(L, np.broadcast_to(rho[None], (4, n, n)).copy(), u), k


@pytest.mark.parametrize("collision,magic", [("bgk", 0.25), ("trt", 0.25), ("trt", 3.0 / 16.0)])
def test_taylor_green_decay(collision, magic):
    n, u0, tau, steps = 32, 0.02, 0.8, 200
    L = O.lattice((n, n, 4), (1, 1, 1), collision, 1 / tau, trt_magic=magic)
    f, k = tgv_state(n, u0, L)
    u_start = np.abs(O.compute_velocity(L, f)[0]).max()
    f = O.collide_stream(L, f, None, None, steps)
    u_end = np.abs(O.compute_velocity(L, f)[0]).max()
    nu = (tau - 0.5) / 3
    expect = np.exp(-2 * nu * k * k * steps)
    assert abs(u_end / u_start - expect) / expect < 1e-2


def test_poiseuille_between_halfway_walls():
    ny, g, tau = 12, 1e-6, 0.9
    L = O.lattice((4, ny, 4), (1, 0, 1), "bgk_guo_vof", 1 / tau, wall_y="halfway_bb")
    F = np.zeros((3, 4, ny, 4))
    F[0] = g
    f = O.collide_stream(L, np.zeros((19, 4, ny, 4)), F, None, 6000)
    u = O.compute_velocity(L, f, F)[0, 1, :, 1]
    nu = (tau - 0.5) / 3
    y = np.arange(ny)
    exact = g / (2 * nu) * (y + 0.5) * (ny - 0.5 - y)
    assert np.abs(u - exact).max() / exact.max() < 1e-2


def test_couette_moving_halfway_wall():
    ny, U, tau = 10, 0.01, 1.0
    L = O.lattice((4, ny, 4), (1, 0, 1), "bgk_guo_vof", 1 / tau, wall_y="halfway_bb",
                  wall_u=[[0, 0, 0], [U, 0, 0], [0, 0, 0], [0, 0, 0]])
    f = O.collide_stream(L, np.zeros((19, 4, ny, 4)), np.zeros((3, 4, ny, 4)), None, 4000)
    u = O.compute_velocity(L, f)[0, 1, :, 1]
    exact = U * (np.arange(ny) + 0.5) / ny
    assert np.abs(u - exact).max() < 2e-3 * U
