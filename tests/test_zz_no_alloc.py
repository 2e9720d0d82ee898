"""tm_observe_noalloc: observables for callers that cannot let the library
allocate device memory (a host application that owns the GPU's memory through
its own pool, or a latency-sensitive loop that must not hit cudaMalloc's
implicit synchronisation).  Its scratch is a static array in the library, so
this test checks it against the batch measurement (tm_batch_advance) on two
calls in a row -- the second call must not see the first call's leftovers.
The file sorts last so a run that stops at the first failure has already run
every other test; it also passes alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_observables_match_batch_measurement():
    torch = pytest.importorskip("torch")
    from trophic_maelstorm_gb300 import build
    build.build()
    import trophic_maelstorm_gb300 as tmg
    from trophic_maelstorm_gb300 import _lib

    ctx = tmg.Context(0)
    Ls = [1, 7, 33, 64, 200, 31]
    rng = np.random.default_rng(5)
    for precision, dtype, tdtype in ((tmg.TM_FP32, np.float32, torch.float32), (tmg.TM_FP64, np.float64, torch.float64)):
        inst = tmg.instances(Ls, range(len(Ls)), 0.72)
        fields = []
        for L in Ls:
            f = 1.0 + rng.uniform(-0.01, 0.01, (L, L))
            f[: L // 2, :] = 0.0  # absorbing half: active counts differ from L*L
            fields.append(f.astype(dtype))
        b = tmg.Batch(ctx, tmg.dp_model(), inst, precision)
        b.upload(fields)
        total, off, _ = tmg.layout(inst, 1)
        Larr = np.asarray(Ls, np.int32)
        off = np.ascontiguousarray(off, np.int64)
        dev = torch.empty(total, dtype=tdtype, device="cuda:0")
        out = torch.empty(len(Ls) * 2, dtype=torch.float64, device="cuda:0")
        for call in range(2):
            ref, _ = b.advance(0, [b.step])          # the existing measurement path
            T_ = _lib.lib()
            _lib.check(T_.tm_batch_download_device(b.handle, C.c_void_p(dev.data_ptr())), "download_device")
            out.fill_(-1.0)
            rc = T_.tm_observe_noalloc(C.c_void_p(dev.data_ptr()), precision,
                                       Larr.ctypes.data_as(C.POINTER(C.c_int32)),
                                       off.ctypes.data_as(C.POINTER(C.c_int64)), len(Ls),
                                       C.c_void_p(out.data_ptr()), C.c_void_p(ctx.stream))
            assert rc == 0, _lib.error_string(rc)
            ctx.sync()
            got = out.cpu().numpy().reshape(len(Ls), 2)
            np.testing.assert_allclose(got[:, 0], ref[0, :, 0], rtol=1e-12, atol=0)
            assert np.array_equal(got[:, 1], ref[0, :, 1]), (call, got[:, 1], ref[0, :, 1])
            b.advance(5)  # a different state for the second call
        b.close()
    # sizes beyond the built-in scratch are rejected, not truncated
    big = np.full(200000, 1024, np.int32)
    boff = np.zeros(200000, np.int64)
    rc = _lib.lib().tm_observe_noalloc(C.c_void_p(1), tmg.TM_FP32, big.ctypes.data_as(C.POINTER(C.c_int32)),
                                       boff.ctypes.data_as(C.POINTER(C.c_int64)), len(big), C.c_void_p(1), None)
    assert rc == _lib.TM_ERR_INVALID
    ctx.close()
