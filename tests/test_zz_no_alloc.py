"""gf_min_angle_noalloc (the mesh-quality test for callers that cannot
allocate device memory) against the context entry gf_itest_mesh, through the
C-ABI.  Kept in its own file, collected last, so that it runs both after the
other GPU tests and alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

from geoflac_gb300 import inpgen, new_state
from geoflac_gb300.capi import load_library
from geoflac_gb300.flac import Flac

pytestmark = pytest.mark.gpu

GF_ERR_LIMIT = -9
TOL = 1e-12  # relative; the two kernels evaluate the same FP64 expressions


def _entry():
    lib = load_library()
    f = lib.gf_min_angle_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.POINTER(C.c_double)]
    return f


@pytest.mark.parametrize("name,steps", [("extension_60x20", 300), ("convergence_60x15", 600)])
def test_min_angle_noalloc_matches_itest_mesh(workdir, name, steps):
    torch = pytest.importorskip("torch")
    f = _entry()
    p, c, s = new_state(inpgen.CONFIGS[name]().write(str(workdir / f"{name}_na.inp")))
    g = Flac(p, c, s, "fp64")
    g.step(steps)
    expect = g.itest_mesh()
    g.download()
    cord = np.asfortranarray(g.state["cord"])
    d_cord = torch.from_numpy(cord.ravel(order="F").copy()).cuda()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):  # two calls in a row share the scratch array
        out = C.c_double(-1.0)
        assert f(d_cord.data_ptr(), p.nx, p.nz, stream, C.byref(out)) == 0
        assert abs(out.value - expect) <= TOL * expect, (out.value, expect)
    assert 0.0 < expect < 90.0
    g.close()


def test_min_angle_noalloc_rejects_oversize_mesh():
    torch = pytest.importorskip("torch")
    f = _entry()
    d = torch.zeros(16, dtype=torch.float64, device="cuda")
    out = C.c_double(-1.0)
    # 2049 x 1025 nodes = 2048 * 1024 = 2,097,152 elements is the limit
    assert f(d.data_ptr(), 2050, 1025, None, C.byref(out)) == GF_ERR_LIMIT
    assert f(d.data_ptr(), 3001, 3001, None, C.byref(out)) == GF_ERR_LIMIT
    assert out.value == -1.0
