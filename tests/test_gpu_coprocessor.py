"""The co-processor path on the GPU, through the C ABI calls the Palabos adapter
(include/bib/bib_coprocessor3D.h) makes: bib_coprocessor_domain_params + bib_lattice_add_domain
(CoProcessor3D::addDomain), bib_lattice_send with BIB_LAYOUT_COPROCESSOR_F64 (send),
bib_lattice_collide_and_stream (collideAndStream), bib_lattice_receive (receive), on the bytes the
reference's own D3Q19ExampleCoProcessor3D received and returned (tests/golden/coprocessor_bgk.npz).

The outer layer is undefined by the interface (coProcessor3D.h:105-107), one cell per step; the
cells inside it agree with the reference to 1e-15 in FP64 (FMA contraction), and within the storage
precision for FP32 / FP16.
"""
import ctypes as C

import numpy as np
import pytest

from tests.conftest import golden

pytestmark = pytest.mark.gpu

bib = pytest.importorskip("biblbm_gb300")
from biblbm_gb300 import _lib  # noqa: E402

STORAGE = {"f64": 0, "f32": 1, "f16": 2}
BGK, TRT = 1, 2  # BIB_COLLISION_BGK, BIB_COLLISION_TRT


@pytest.fixture(scope="module")
def ctx():
    c = bib.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("storage,tol", [("f64", 1e-15), ("f32", 5e-8), ("f16", 2e-5)])
def test_coprocessor_calls_match_the_reference_coprocessor(ctx, storage, tol):
    g = golden("coprocessor_bgk")
    nx, ny, nz = (int(v) for v in g["in_dims"])
    steps = int(g["in_steps"])
    p = _lib.LatticeParams()
    assert ctx.lib.bib_coprocessor_domain_params(float(g["in_omega"]), STORAGE[storage], BGK, C.byref(p)) == 0
    h = C.c_int32()
    ctx.check(ctx.lib.bib_lattice_add_domain(ctx.h, nx, ny, nz, C.byref(p), C.byref(h)))
    data = np.ascontiguousarray(g["in_data"])  # (x, y, z, 19): the CoProcessor3D byte order
    ctx.check(ctx.lib.bib_lattice_send(ctx.h, h.value, data.ctypes.data, data.nbytes, 2))
    for _ in range(steps):
        ctx.check(ctx.lib.bib_lattice_collide_and_stream(ctx.h, h.value, 1))
    back = np.empty_like(data)
    ctx.check(ctx.lib.bib_lattice_receive(ctx.h, h.value, back.ctypes.data, back.nbytes, 2))
    s = steps
    inner = (slice(s, nx - s), slice(s, ny - s), slice(s, nz - s))
    err = np.abs(back[inner] - g["out_data"][inner]).max()
    assert err < tol, err


def test_domain_params_reject_what_the_interface_does_not_cover(ctx):
    p = _lib.LatticeParams()
    assert ctx.lib.bib_coprocessor_domain_params(1.2, 0, TRT, C.byref(p)) != 0  # TRT: not a co-processor dynamics
    assert ctx.lib.bib_coprocessor_domain_params(2.5, 0, BGK, C.byref(p)) != 0  # omega outside (0, 2)
    assert ctx.lib.bib_coprocessor_domain_params(1.2, 7, BGK, C.byref(p)) != 0  # unknown storage
