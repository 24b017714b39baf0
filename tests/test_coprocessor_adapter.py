"""The Palabos co-processor adapter (include/bib/bib_coprocessor3D.h) and its fixture.

The adapter must compile with the reference's own toolchain settings (-std=gnu++98 -fpermissive
-DPLB_MPI_PARALLEL, its headers), link against the library and answer 0 ("failure", the
interface's convention, coProcessor3D.h:66-74) instead of crashing where no GPU can be opened.
These checks need the reference checkout; set BIB_REFERENCE to it (they are skipped otherwise).

The fixture tests/golden/coprocessor_bgk.npz was written by the reference's own
D3Q19ExampleCoProcessor3D (coProcessors/coProcessor3D.hh:34-78); the oracle's BGK restatement must
reproduce its cells away from the undefined outer layer exactly.
"""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from tests.conftest import ROOT, golden

REF = os.environ.get("BIB_REFERENCE", "")
HAVE_REF = bool(REF) and os.path.isdir(os.path.join(REF, "src", "coProcessors"))
LIB = os.path.join(ROOT, "biblbm_gb300", "lib", "libbib_gb300.so")
PLB = os.path.join(ROOT, "oracle", "_ref", "libplb_ref.a")

DRIVER = r"""
#include "palabos3D.h"
#include "palabos3D.hh"
#include "bib/bib_coprocessor3D.h"
#include <cstdio>
using namespace plb;

int main(int argc, char** argv) {
    plbInit(&argc, &argv);
    BibCoProcessor3D cp;
    CoProcessor3D<double>& base = cp;  // used through the reference's interface
    int handle = -1;
    const int added = base.addDomain(6, 5, 4, 1.2, handle);
    std::vector<char> data(6 * 5 * 4 * 19 * sizeof(double), 0);
    const Box3D box(0, 5, 0, 4, 0, 3);
    int sent = 0, stepped = 0, received = 0;
    if (added) {
        sent = base.send(handle, box, data);
        stepped = base.collideAndStream(handle);
        std::vector<char> back;
        received = base.receive(handle, box, back) && back.size() == data.size();
    }
    std::printf("addDomain=%d send=%d collideAndStream=%d receive=%d\n", added, sent, stepped, received);
    return 0;
}
"""


def compile_flags():
    return ["-std=gnu++98", "-fpermissive", "-DPLB_MPI_PARALLEL", "-O1", "-w",
            "-I", os.path.join(ROOT, "oracle", "mpi_shim"), "-I", os.path.join(REF, "src"),
            "-I", os.path.join(REF, "externalLibraries"), "-I", os.path.join(ROOT, "include")]


@pytest.mark.skipif(not HAVE_REF, reason="set BIB_REFERENCE to the reference checkout")
def test_adapter_compiles_as_cxx98_against_the_reference_headers():
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "driver.cpp")
        with open(src, "w") as f:
            f.write(DRIVER)
        r = subprocess.run(["g++", *compile_flags(), "-c", src, "-o", os.path.join(d, "driver.o")],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-4000:]


@pytest.mark.skipif(not (HAVE_REF and os.path.exists(PLB) and os.path.exists(LIB)),
                    reason="needs BIB_REFERENCE, make -C oracle ref and the built library")
def test_adapter_links_and_reports_failure_without_a_device():
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "driver.cpp"), os.path.join(d, "driver")
        with open(src, "w") as f:
            f.write(DRIVER)
        r = subprocess.run(["g++", *compile_flags(), src, PLB, LIB, "-Wl,-rpath," + os.path.dirname(LIB), "-o", exe],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-4000:]
        r = subprocess.run([exe], capture_output=True, text=True, cwd=d, timeout=120)
        assert r.returncode == 0, r.stderr[-2000:]
        line = [ln for ln in r.stdout.splitlines() if ln.startswith("addDomain=")][0]
        vals = dict(kv.split("=") for kv in line.split())
        import torch

        if not torch.cuda.is_available():
            assert vals == {"addDomain": "0", "send": "0", "collideAndStream": "0", "receive": "0"}
        else:
            assert vals == {"addDomain": "1", "send": "1", "collideAndStream": "1", "receive": "1"}


def test_oracle_bgk_matches_the_reference_coprocessor():
    from oracle import oracle as O

    g = golden("coprocessor_bgk")
    nx, ny, nz = (int(v) for v in g["in_dims"])
    steps = int(g["in_steps"])
    f = np.ascontiguousarray(np.transpose(g["in_data"], (3, 2, 1, 0)))  # (x, y, z, i) -> (i, z, y, x)
    L = O.lattice((nx, ny, nz), (1, 1, 1), "bgk", float(g["in_omega"]))
    out = O.collide_stream(L, f, None, None, steps)
    ref = np.transpose(g["out_data"], (3, 2, 1, 0))
    s = steps  # the undefined layer grows by one cell per step
    inner = (slice(None), slice(s, nz - s), slice(s, ny - s), slice(s, nx - s))
    assert np.array_equal(out[inner], ref[inner])
