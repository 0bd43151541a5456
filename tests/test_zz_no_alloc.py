"""uds_splat_forward_static: the EWA splatting forward that allocates nothing.

It exists for callers that cannot hand the library any scratch memory (a
plugin slot that only passes the op's inputs and outputs, a language binding
without a device allocator, a real-time loop that must not allocate after
start-up).  Its scratch is a fixed array inside libuds.so, so the test checks,
through the C ABI, that two calls in a row give the same weights as the
workspace entry point uds_splat_forward (within the 1e-6 relative L2 the EWA
tests use) and that calls above the array's 262144 (view, splat) pairs are
refused.  This file is collected last so that a failure here does not hide
the other GPU tests; it also passes on its own in a fresh process.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


@pytest.fixture(scope="module")
def L():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from unbiased_differentiable_splatting_gb300 import _lib
    return _lib.load()


def _inputs(seed, B, N, W, H, K, f):
    rng = np.random.default_rng(seed)
    z = rng.uniform(-2.4, -1.6, (B, N))
    pts = np.stack([rng.uniform(-0.5, 0.5, (B, N)) * (-z) * W / f, rng.uniform(-0.5, 0.5, (B, N)) * (-z) * H / f,
                    z], -1).astype(np.float32)
    n = rng.normal(size=(B, N, 3))
    n[..., 2] = np.abs(n[..., 2]) + 0.5
    n = (n / np.linalg.norm(n, axis=-1, keepdims=True)).astype(np.float32)
    sd = rng.uniform(0.008, 0.03, size=(1, N, 2)).astype(np.float32)
    idx = rng.integers(-1, N, size=(B, W, H, K)).astype(np.int32)
    t = lambda a: torch.as_tensor(a).to(DEV)  # noqa: E731
    return t(idx), t(pts), t(n), t(sd)


def _rel_l2(a, b):
    a = a.double()
    b = b.double()
    return float((a - b).norm() / b.norm().clamp_min(1e-30))


def test_static_matches_workspace_entry_twice(L):
    W, H, K, f = 48, 40, 8, 40.0
    stream = torch.cuda.current_stream().cuda_stream
    for seed, (B, N) in ((0, (2, 3000)), (1, (1, 5000))):
        idx, pts, nrm, sd = _inputs(seed, B, N, W, H, K, f)
        ws = torch.empty(L.uds_splat_workspace_size(B, N), dtype=torch.uint8, device=DEV)
        ref = torch.empty(idx.shape, dtype=torch.float32, device=DEV)
        st = L.uds_splat_forward(B, W, H, K, f, idx.data_ptr(), pts.data_ptr(), nrm.data_ptr(), 1, N, sd.data_ptr(),
                                 0.0, ref.data_ptr(), ws.data_ptr(), ws.numel(), stream)
        assert st == 0
        out = torch.full(idx.shape, float("nan"), dtype=torch.float32, device=DEV)
        st = L.uds_splat_forward_static(B, W, H, K, f, idx.data_ptr(), pts.data_ptr(), nrm.data_ptr(), 1, N,
                                        sd.data_ptr(), 0.0, out.data_ptr(), stream)
        assert st == 0, L.uds_last_error()
        torch.cuda.synchronize()
        assert torch.isfinite(out).all()
        assert _rel_l2(out, ref) < 1e-6
        assert torch.all(out[idx < 0] == 0)


def test_static_rejects_more_than_its_array(L):
    B, N, W, H, K, f = 2, (1 << 17) + 1, 8, 8, 2, 8.0
    dummy = torch.zeros(16, device=DEV)
    st = L.uds_splat_forward_static(B, W, H, K, f, dummy.data_ptr(), dummy.data_ptr(), dummy.data_ptr(), 1, N,
                                    dummy.data_ptr(), 0.0, dummy.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert st == 1
    assert b"262144" in L.uds_last_error()


def test_static_allocates_nothing(L):
    """After one warm call, a second call changes neither torch's allocator
    nor the device's free memory."""
    W, H, K, f, B, N = 32, 24, 4, 30.0, 2, 2000
    idx, pts, nrm, sd = _inputs(3, B, N, W, H, K, f)
    out = torch.empty(idx.shape, dtype=torch.float32, device=DEV)
    stream = torch.cuda.current_stream().cuda_stream

    def call():
        st = L.uds_splat_forward_static(B, W, H, K, f, idx.data_ptr(), pts.data_ptr(), nrm.data_ptr(), 1, N,
                                        sd.data_ptr(), 0.0, out.data_ptr(), stream)
        assert st == 0, L.uds_last_error()
        torch.cuda.synchronize()

    call()
    before = (torch.cuda.memory_allocated(), torch.cuda.mem_get_info()[0])
    call()
    after = (torch.cuda.memory_allocated(), torch.cuda.mem_get_info()[0])
    assert after == before


def test_static_per_view_std_devs_and_no_splats(L):
    """std_batch = B (per-view std-devs) against the workspace entry point,
    and N = 0: every weight is zero."""
    W, H, K, f, B, N = 40, 32, 8, 36.0, 3, 1500
    stream = torch.cuda.current_stream().cuda_stream
    idx, pts, nrm, _ = _inputs(4, B, N, W, H, K, f)
    sd = torch.as_tensor(np.random.default_rng(4).uniform(0.008, 0.03, size=(B, N, 2)).astype(np.float32)).to(DEV)
    ws = torch.empty(L.uds_splat_workspace_size(B, N), dtype=torch.uint8, device=DEV)
    ref = torch.empty(idx.shape, dtype=torch.float32, device=DEV)
    assert L.uds_splat_forward(B, W, H, K, f, idx.data_ptr(), pts.data_ptr(), nrm.data_ptr(), B, N, sd.data_ptr(),
                               0.0, ref.data_ptr(), ws.data_ptr(), ws.numel(), stream) == 0
    out = torch.full(idx.shape, float("nan"), dtype=torch.float32, device=DEV)
    assert L.uds_splat_forward_static(B, W, H, K, f, idx.data_ptr(), pts.data_ptr(), nrm.data_ptr(), B, N,
                                      sd.data_ptr(), 0.0, out.data_ptr(), stream) == 0, L.uds_last_error()
    torch.cuda.synchronize()
    assert _rel_l2(out, ref) < 1e-6
    empty = torch.full((1, W, H, K), -1, dtype=torch.int32, device=DEV)
    out0 = torch.full((1, W, H, K), float("nan"), dtype=torch.float32, device=DEV)
    assert L.uds_splat_forward_static(1, W, H, K, f, empty.data_ptr(), 0, 0, 1, 0, 0, 0.0, out0.data_ptr(),
                                      stream) == 0, L.uds_last_error()
    torch.cuda.synchronize()
    assert torch.all(out0 == 0)
