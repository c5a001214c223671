"""The no-allocation centre-of-mass entry point (vx3_center_of_mass_noalloc).

It serves callers that cannot allocate device memory themselves — a plugin
inside another framework whose caching allocator owns the device memory, a
real-time loop that cannot take cudaMalloc's synchronisation, a service that
accounts for every byte of its HBM budget — by keeping its scratch in a fixed
array compiled into the library.  The tests give it device buffers made by the
test (the entry point allocates nothing) and call it through the C ABI:

* twice in a row on a creature's voxels, against the engine's own centre of
  mass (vx3_get_result), within the parity tests' centre-of-mass tolerance
  (1e-4 relative);
* on synthetic points against a float64 numpy sum (1e-12 relative; the
  reduction order differs): about a million points (a fold over many blocks),
  exactly VX3_NOALLOC_MAX_POINTS (every scratch slot used), a full-size call
  followed by a small one (the small call must not read the large call's
  leftover partials), n = 0 (zeros) and a call on a non-default stream.

The file is collected last, and works alone in a fresh process as well as
after the other tests.
"""
import ctypes

import numpy as np
import pytest

import gpuvoxels_gb300 as g
from gpuvoxels_gb300 import synth

pytestmark = pytest.mark.gpu

COM_RTOL = 1e-4
SUM_RTOL = 1e-12


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _noalloc_com(L, x, y, z, m, n, out, stream=None):
    return L.vx3_center_of_mass_noalloc(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()),
                                        ctypes.c_void_p(z.data_ptr()), ctypes.c_void_p(m.data_ptr()), n,
                                        ctypes.c_void_p(out.data_ptr()), stream)


def _expected(x, y, z, m):
    w = m.astype(np.float64)
    tot = w.sum()
    if tot == 0:
        return np.zeros(4)
    return np.array([(x * w).sum() / tot, (y * w).sum() / tot, (z * w).sum() / tot, tot])


def test_noalloc_center_of_mass_matches_engine():
    torch = _torch()
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


def test_noalloc_many_blocks_limit_and_leftovers():
    torch = _torch()
    L = g.library()
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(7)
    N = g.NOALLOC_MAX_POINTS
    xs = rng.normal(0.3, 1.0, N)
    ys = rng.normal(-0.2, 2.0, N)
    zs = rng.uniform(0.0, 0.5, N)
    ms = rng.uniform(0.5, 2.0, N).astype(np.float32)
    x = torch.tensor(xs, device=dev)
    y = torch.tensor(ys, device=dev)
    z = torch.tensor(zs, device=dev)
    m = torch.tensor(ms, device=dev)
    cases = [1_000_003, N, 3_000, 0, N, 1]                  # a full-size call, then small ones after it
    for n in cases:
        out = torch.full((4,), float("nan"), dtype=torch.float64, device=dev)
        assert _noalloc_com(L, x, y, z, m, n, out) == 0, n
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        want = _expected(xs[:n], ys[:n], zs[:n], ms[:n])
        if n == 0:
            assert got.tolist() == [0.0, 0.0, 0.0, 0.0]
        else:
            np.testing.assert_allclose(got, want, rtol=SUM_RTOL, atol=1e-15, err_msg=f"n={n}")
    # the same on a stream of the caller's (the work is only enqueued there)
    s = torch.cuda.Stream(device=dev)
    out = torch.full((4,), float("nan"), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    assert _noalloc_com(L, x, y, z, m, 12_345, out, ctypes.c_void_p(s.cuda_stream)) == 0
    s.synchronize()
    np.testing.assert_allclose(out.cpu().numpy(), _expected(xs[:12_345], ys[:12_345], zs[:12_345], ms[:12_345]),
                               rtol=SUM_RTOL, atol=1e-15)
