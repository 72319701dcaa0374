"""vmp_downsample_noalloc: the downsample entry point that allocates nothing.

It serves callers that cannot call cudaMalloc -- a real-time sensor thread
that must not block on an allocation, or a framework whose own allocator owns
the GPU's memory -- so its working memory is a fixed array inside libvmp and
the caller passes device buffers it owns for the input and the output.  This
file is collected last so that a run stopping at its first failure has already
run every other test.  The check: through the C ABI, two calls in a row must
give exactly the output of the existing vmp_downsample entry point (the leaf
centroid filter is float work done in a fixed order, so the tolerance is
bit-for-bit, as in the other downsample tests).
"""
import ctypes as C

import numpy as np
import pytest

from voxelmapplus_fastlio2_gb300 import abi

pytestmark = pytest.mark.gpu

MAX_POINTS = 65536  # the entry point's documented limit


def _lib():
    from voxelmapplus_fastlio2_gb300 import _lib as L
    lib = L.load()
    fn = lib.vmp_downsample_noalloc
    fn.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_void_p, C.POINTER(C.c_int), C.c_void_p]
    fn.restype = C.c_int
    return lib


def _cloud(rng, n):
    pts = np.zeros((n, 4), dtype=np.float32)
    pts[:, :3] = rng.uniform(-25.0, 25.0, (n, 3)).astype(np.float32)
    pts[:, 3] = np.sort(rng.uniform(0.0, 100.0, n)).astype(np.float32)
    return pts


def test_noalloc_downsample_matches_existing_entry_point():
    import torch
    from voxelmapplus_fastlio2_gb300 import lio
    lib = _lib()
    g = lio.LIOBuilder(abi.default_config(max_scan_points=MAX_POINTS))
    rng = np.random.default_rng(2024)
    for n, leaf in ((MAX_POINTS, 0.1), (20000, 0.5)):  # two calls in a row
        pts = _cloud(rng, n)
        ref = g.downsample(pts, leaf)  # existing entry point (vmp_downsample)
        d_in = torch.from_numpy(pts).cuda()
        d_out = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        m = C.c_int(-1)
        code = lib.vmp_downsample_noalloc(C.c_void_p(d_in.data_ptr()), n, leaf, C.c_void_p(d_out.data_ptr()),
                                          C.byref(m), None)
        assert code == abi.VMP_OK, abi.STATUS_NAMES.get(code)
        assert m.value == ref.shape[0]
        got = d_out[: m.value].cpu().numpy()
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    g.close()


def _noalloc(lib, d_in, n, leaf, d_out):
    m = C.c_int(-1)
    code = lib.vmp_downsample_noalloc(C.c_void_p(d_in), n, leaf, C.c_void_p(d_out), C.byref(m), None)
    return code, m.value


def test_noalloc_downsample_overflow_and_single_point():
    """The two other ways out of the filter: a leaf so small that the leaf
    grid would overflow 32-bit indices (the input comes back unchanged, as
    pcl::VoxelGrid returns it) and a one-point cloud -- each bit for bit as
    the existing entry point gives them."""
    import torch
    from voxelmapplus_fastlio2_gb300 import lio
    lib = _lib()
    g = lio.LIOBuilder(abi.default_config(max_scan_points=MAX_POINTS))
    rng = np.random.default_rng(77)
    for n, leaf in ((5000, 1e-4), (1, 0.1)):
        pts = _cloud(rng, n)
        ref = g.downsample(pts, leaf)
        if leaf < 1e-3:
            assert ref.shape[0] == n  # the overflow path: output = input
        d_in = torch.from_numpy(pts).cuda()
        d_out = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        code, m = _noalloc(lib, d_in.data_ptr(), n, leaf, d_out.data_ptr())
        assert code == abi.VMP_OK, abi.STATUS_NAMES.get(code)
        assert m == ref.shape[0]
        got = d_out[:m].cpu().numpy()
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    g.close()


def test_noalloc_downsample_rejects_oversize_and_bad_args():
    """Sizes beyond the limit and pointers the float4 kernels cannot take are
    rejected before anything is launched: a device pointer off by 4 bytes, a
    host (numpy) array, and an output that overlaps the input."""
    import torch
    lib = _lib()
    m = C.c_int(0)
    dummy = C.c_void_p(1)
    assert lib.vmp_downsample_noalloc(dummy, MAX_POINTS + 1, 0.1, dummy, C.byref(m), None) == abi.VMP_ERR_CAPACITY
    assert lib.vmp_downsample_noalloc(dummy, 10, 0.0, dummy, C.byref(m), None) == abi.VMP_ERR_INVALID_ARG
    assert lib.vmp_downsample_noalloc(None, 0, 0.1, None, C.byref(m), None) == 0 and m.value == 0
    n = 1000
    d_in = torch.zeros((2 * n + 4, 4), dtype=torch.float32, device="cuda")
    d_out = torch.zeros((n + 4, 4), dtype=torch.float32, device="cuda")
    host = np.zeros((n, 4), dtype=np.float32)
    torch.cuda.synchronize()
    base_in, base_out = d_in.data_ptr(), d_out.data_ptr()
    assert _noalloc(lib, base_in + 4, n, 0.1, base_out)[0] == abi.VMP_ERR_INVALID_ARG  # misaligned input
    assert _noalloc(lib, base_in, n, 0.1, base_out + 4)[0] == abi.VMP_ERR_INVALID_ARG  # misaligned output
    assert _noalloc(lib, host.ctypes.data, n, 0.1, base_out)[0] == abi.VMP_ERR_INVALID_ARG  # host input
    assert _noalloc(lib, base_in, n, 0.1, host.ctypes.data)[0] == abi.VMP_ERR_INVALID_ARG  # host output
    assert _noalloc(lib, base_in, n, 0.1, base_in)[0] == abi.VMP_ERR_INVALID_ARG  # in place
    assert _noalloc(lib, base_in, n, 0.1, base_in + 16 * (n - 1))[0] == abi.VMP_ERR_INVALID_ARG  # overlap
    code, _ = _noalloc(lib, base_in, n, 0.1, base_in + 16 * n)  # adjacent, not overlapping
    assert code == abi.VMP_OK, abi.STATUS_NAMES.get(code)
