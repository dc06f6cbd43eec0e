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


def _expected_min_angle(x, y):
    """The smallest angle of the four overlaid triangles of every quad
    (src/rem_test.f90:77-118) in numpy, in the kernel's order of operations:
    the angles at the second and third vertex from acos, the first as 180
    minus both, each quad's minimum clamped at zero."""
    q = [(x[:-1, :-1], y[:-1, :-1]), (x[1:, :-1], y[1:, :-1]), (x[:-1, 1:], y[:-1, 1:]), (x[1:, 1:], y[1:, 1:])]
    raddeg = 180.0 / np.pi
    amin = np.full(x[:-1, :-1].shape, 180.0)
    for tv in ((0, 1, 2), (1, 3, 2), (0, 1, 3), (0, 3, 2)):
        v = (tv[0], tv[1], tv[2], tv[0])
        ang = [None, None, None]
        for k in (1, 2):
            xa, ya = q[v[k + 1]][0] - q[v[k]][0], q[v[k + 1]][1] - q[v[k]][1]
            xb, yb = q[v[k - 1]][0] - q[v[k]][0], q[v[k - 1]][1] - q[v[k]][1]
            la, lb = np.sqrt(xa * xa + ya * ya), np.sqrt(xb * xb + yb * yb)
            ang[k] = raddeg * np.arccos((xa * xb + ya * yb) / (la * lb))
        ang[0] = 180.0 - ang[1] - ang[2]
        amin = np.minimum(amin, np.minimum(ang[0], np.minimum(ang[1], ang[2])))
    return float(np.maximum(amin, 0.0).min())


def test_min_angle_noalloc_largest_mesh_allocates_nothing():
    """The largest accepted mesh, 2049 x 1025 nodes (2,097,152 elements, all
    8,192 blocks of partial minima), with jittered nodes and one node pulled
    towards its neighbour to set a known smallest angle: the result equals
    numpy's, on two calls in a row, and the device's free memory is the same
    before and after them."""
    torch = pytest.importorskip("torch")
    f = _entry()
    nx, nz = 2049, 1025
    rng = np.random.default_rng(11)
    xs, zs = np.meshgrid(np.arange(nx) * 1000.0, np.arange(nz) * -800.0)  # (nz, nx)
    x = xs + rng.uniform(-60.0, 60.0, xs.shape)
    y = zs + rng.uniform(-60.0, 60.0, zs.shape)
    x[700, 1500] += 600.0  # a sliver near node (700, 1500)
    expect = _expected_min_angle(x, y)
    cord = np.stack([x, y], axis=-1)  # (nz, nx, 2); Fortran order = depth fastest
    d_cord = torch.from_numpy(cord.transpose(2, 1, 0).copy().ravel()).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    out = C.c_double(-1.0)
    assert f(d_cord.data_ptr(), nx, nz, stream, C.byref(out)) == 0  # first call: module and address set-up
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(2):
        out = C.c_double(-1.0)
        assert f(d_cord.data_ptr(), nx, nz, stream, C.byref(out)) == 0
        assert abs(out.value - expect) <= TOL * expect, (out.value, expect)
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert 0.0 < expect < 30.0
