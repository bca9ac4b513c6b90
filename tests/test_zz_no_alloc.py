"""The operator entry point that allocates nothing (s4g_op_amul_dot_noalloc)
against the allocating operator entry point (s4g_op_amul) on the same mesh:
the same y = A x to round-off, x.Ax equal to the column sums of x * y, and
two calls in a row giving identical bits (its static scratch is left ready
for the next call).  The file sorts last so that it also runs after every
other test of the session."""
import numpy as np
import pytest

import solids4foam_gb300 as sg
from solids4foam_gb300 import _lib

pytestmark = pytest.mark.gpu
TOL_Y = 1e-14    # relative L2, y against the allocating entry point
TOL_XAX = 1e-12  # relative, per column


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def model_on(ctx, nx, ny, nz, seed=7):
    m = sg.box_mesh(nx, ny, nz, 1.0, 0.9, 0.8, 0.2, seed)
    bcs = {"zmin": ("fixedDisplacement", None, None),
           "zmax": ("solidTraction", None, np.full(int(m["patch_size"][5]), 1e6))}
    return sg.SolidModel(ctx, m, dict(type="linearElastic", E=70e9, nu=0.33), bcs)


@pytest.mark.parametrize("k", [3, 2, 1])
def test_matches_allocating_entry_point_twice(ctx, k):
    model = model_on(ctx, 12, 10, 9)
    model.op_matrix()  # assembles the matrix
    rng = np.random.default_rng(k)
    n = model.n_cells
    x = rng.standard_normal((n, k)) if k > 1 else rng.standard_normal(n)
    y_ref = model.op_amul(x)
    y1, d1 = model.op_amul_dot_noalloc(x)
    y2, d2 = model.op_amul_dot_noalloc(x)
    assert rel(y1, y_ref) < TOL_Y
    d_ref = (x.reshape(n, k) * y_ref.reshape(n, k)).sum(axis=0)
    assert np.all(np.abs(d1 - d_ref) <= TOL_XAX * np.abs(d_ref))
    assert np.array_equal(y1, y2) and np.array_equal(d1, d2)
    model.close()


def test_allocates_no_device_memory(ctx):
    """The property the entry point exists for: a batch of calls leaves the
    device's free memory exactly as it was (cudaMemGetInfo, read through
    torch), while the allocating entry point is free to use the allocator."""
    torch = pytest.importorskip("torch")
    model = model_on(ctx, 12, 10, 9)
    model.op_matrix()
    x = np.random.default_rng(5).standard_normal((model.n_cells, 3))
    model.op_amul_dot_noalloc(x)  # the one-time set-up of the device
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(50):
        model.op_amul_dot_noalloc(x)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    model.close()
    assert free1 == free0


def test_needs_an_assembled_matrix(ctx):
    model = model_on(ctx, 5, 4, 4)
    with pytest.raises(_lib.S4GError, match="not assembled"):
        model.op_amul_dot_noalloc(np.ones((model.n_cells, 3)))
    model.op_matrix()
    y, d = model.op_amul_dot_noalloc(np.ones((model.n_cells, 3)))
    assert np.all(np.isfinite(y)) and np.all(np.isfinite(d))
    model.close()


def test_rejects_meshes_beyond_its_scratch(ctx):
    model = model_on(ctx, 65, 64, 64)  # 266,240 cells > 262,144
    model.op_matrix()
    with pytest.raises(_lib.S4GError, match="at most 262144"):
        model.op_amul_dot_noalloc(np.ones((model.n_cells, 3)))
    model.close()
