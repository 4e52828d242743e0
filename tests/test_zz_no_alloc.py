"""The allocation-free LOD entry point against the regular one.

sl_lod_score_device_graphs_noalloc serves callers that cannot allocate device
memory where they score (a host allocator that owns the device's memory, or a
loop where an allocation's device-wide synchronisation would stall other
streams); its scratch is a fixed device array inside the library.  This test
scores two batches in a row through it, from device buffers the test itself
allocates, and checks the accumulated LOD table after each call against
sl_lod_score_graphs on the same graphs, in each LOD form, within the LOD
tolerances used by the other parity tests.  It lives in its own file, collected last.
"""
import ctypes
import sys

import numpy as np
import pytest

from conftest import load_golden
from swiftlink_gb300 import api

pytestmark = pytest.mark.gpu

FP64_LOD_TOL = 1e-10
FP32_LOD_TOL = 1e-3
LOG_ZERO = -sys.float_info.max


@pytest.fixture(scope="module", autouse=True)
def _built():
    from swiftlink_gb300 import build
    build.build()


def pack(graphs, N, F, M):
    """int32 [n][M][N][2] reference layout -> uint32 [n][M][W] device layout."""
    W = (2 * (N - F) + 31) // 32
    n = graphs.shape[0]
    bits = graphs[:, :, F:, :].reshape(n, M, 2 * (N - F)).astype(np.uint64)
    out = np.zeros((n, M, W), np.uint64)
    for b in range(2 * (N - F)):
        out[:, :, b >> 5] |= bits[:, :, b] << np.uint64(b & 31)
    return out.astype(np.uint32)


@pytest.mark.parametrize("precision,tol", [(api.SL_LOD_FP64, FP64_LOD_TOL),
                                           (api.SL_LOD_FP64_RESCALED, FP64_LOD_TOL),
                                           (api.SL_LOD_FP32_RESCALED, FP32_LOD_TOL)])
def test_noalloc_lod_matches_regular_entry_point_on_two_calls(precision, tol):
    """In each LOD form -- the plain FP64 peel, the FP64 peel with rescaling,
    and the batched FP32-rescaled peel (within the FP32 tolerance: the two
    contexts may score with different FP32 kernels) -- and on two calls in a
    row, so the second call starts from the first one's leftover scratch."""
    torch = pytest.importorskip("torch")
    g = load_golden("cfg1")
    N, F, M, n = g["N"], g["F"], g["M"], g["n_lod"]
    graphs = g["lod_graphs"]
    batches = [graphs[:2], graphs[2:]]
    fn = api.lib().sl_lod_score_device_graphs_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
    with api.Context(api.Problem.from_arrays(g), n_chains=1, lod_precision=precision) as ref_ctx, \
            api.Context(api.Problem.from_arrays(g), n_chains=1, lod_precision=precision) as ctx:
        acc = torch.full(((M - 1) * n,), LOG_ZERO, dtype=torch.float64, device="cuda")
        count = 0
        for batch in batches:
            ref_ctx.lod_score_graphs(batch)
            want_raw, want_count, tp = ref_ctx.lod_results()
            dev = torch.from_numpy(pack(batch, N, F, M).view(np.int32)).cuda()
            torch.cuda.synchronize()
            rc = fn(ctx.h, batch.shape[0], dev.data_ptr(), acc.data_ptr())
            assert rc == api.SL_OK, api.lib().sl_last_error(ctx.h)
            ctx.synchronize()
            count += batch.shape[0]
            got_raw = acc.cpu().numpy()
            assert count == want_count
            err = np.abs(api.lod_table(got_raw, count, tp) - api.lod_table(want_raw, want_count, tp)).max()
            assert err <= tol, err
            assert torch.cuda.current_device() == 0


def test_noalloc_rejects_batches_beyond_the_scratch_array():
    torch = pytest.importorskip("torch")
    g = load_golden("cfg1")
    M, n = g["M"], g["n_lod"]
    limit = (8 << 20) // 8
    too_many = limit // ((M - 1) * n) + 1
    fn = api.lib().sl_lod_score_device_graphs_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
    with api.Context(api.Problem.from_arrays(g), n_chains=1) as ctx:
        acc = torch.full(((M - 1) * n,), LOG_ZERO, dtype=torch.float64, device="cuda")
        dummy = torch.zeros(16, dtype=torch.int32, device="cuda")
        rc = fn(ctx.h, too_many, dummy.data_ptr(), acc.data_ptr())
        assert rc == api.SL_EINVAL
        assert b"scratch" in api.lib().sl_last_error(ctx.h)
