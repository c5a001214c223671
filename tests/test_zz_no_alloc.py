"""The no-allocation centre-of-mass entry point (vx3_center_of_mass_noalloc).

It serves callers that cannot allocate device memory themselves — code that
records into a CUDA graph, or that lives inside another framework's device
allocator — by keeping its scratch in a fixed array compiled into the library.
This test gives it device buffers made by the test (the entry point allocates
nothing), calls it twice in a row through the C ABI, and checks both results
against the engine's own centre of mass (vx3_get_result), within the
centre-of-mass tolerance the parity tests use (1e-4 relative).  It lives in a
file of its own, collected last, and works alone in a fresh process as well as
after the other tests.
"""
import ctypes

import numpy as np
import pytest

import gpuvoxels_gb300 as g
from gpuvoxels_gb300 import synth

pytestmark = pytest.mark.gpu

COM_RTOL = 1e-4


def _noalloc_com(L, x, y, z, m, n, out, stream=None):
    return L.vx3_center_of_mass_noalloc(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()),
                                        ctypes.c_void_p(z.data_ptr()), ctypes.c_void_p(m.data_ptr()), n,
                                        ctypes.c_void_p(out.data_ptr()), stream)


def test_noalloc_center_of_mass_matches_engine():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    L = g.library()
    c = synth.config0_creature(42)
    masses = g.inspect_vxa(c.vxa)["voxmat"][:, 10]
    with g.Context(0, 1 << 30) as ctx:
        sim = ctx.load_vxa(c.vxa, name="noalloc")
        ctx.step(sim, 300)
        expected = np.array(ctx.result(sim).current_center_of_mass)
        st = ctx.voxel_state(sim)
        vox = g.inspect_vxa(c.vxa)["voxels"]
    pos = st["pos"]
    dev = torch.device("cuda", 0)
    x = torch.tensor(np.ascontiguousarray(pos[:, 0]), dtype=torch.float64, device=dev)
    y = torch.tensor(np.ascontiguousarray(pos[:, 1]), dtype=torch.float64, device=dev)
    z = torch.tensor(np.ascontiguousarray(pos[:, 2]), dtype=torch.float64, device=dev)
    m = torch.tensor(masses[vox[:, 3]].astype(np.float32), dtype=torch.float32, device=dev)
    n = pos.shape[0]
    for call in range(2):                                   # two calls in a row share the scratch
        out = torch.full((4,), float("nan"), dtype=torch.float64, device=dev)
        rc = _noalloc_com(L, x, y, z, m, n, out)
        assert rc == 0, rc
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        np.testing.assert_allclose(got[:3], expected, rtol=COM_RTOL, atol=0)
        assert got[3] == pytest.approx(float(masses[vox[:, 3]].astype(np.float64).sum()), rel=1e-12)
    # sizes beyond the fixed scratch are refused without launching
    out = torch.zeros(4, dtype=torch.float64, device=dev)
    assert _noalloc_com(L, x, y, z, m, g.NOALLOC_MAX_POINTS + 1, out) == g.E_LIMIT
    torch.cuda.synchronize()
    assert out.cpu().numpy().tolist() == [0.0, 0.0, 0.0, 0.0]
