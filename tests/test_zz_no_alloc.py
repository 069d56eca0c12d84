"""sdpg_rgemm_device_noalloc: the GEMM for callers that cannot let the library
allocate device memory (their memory is held by their own pool allocator, or an
allocation's device synchronisation is not acceptable in their loop).

The entry point works out of one fixed device array instead of allocating; this
test calls it through the C ABI twice in a row (different precisions and shapes,
so the second call reuses the array the first call left dirty) and compares each
result with the exact product and with the allocating entry point
sdpg_rgemm_device on the same inputs, to the tolerance the GEMM tests use: 2^-(p-16) of |alpha| K max|a_i.| max|b_.j|
+ |beta c_ij| per entry (p = 32 * limbs).  It also checks that a product larger
than the fixed scratch is refused with SDPG_ERR_TOO_LARGE.  The file is named so
that pytest collects it last."""
import ctypes
import random

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bind(lib):
    c = ctypes
    f = lib.sdpg_rgemm_device_noalloc
    f.restype = c.c_int
    f.argtypes = [c.c_int, c.c_char, c.c_char, c.c_int, c.c_int, c.c_int, c.c_void_p, c.c_void_p, c.c_int,
                  c.c_void_p, c.c_int, c.c_void_p, c.c_void_p, c.c_int, c.c_void_p]
    return f


def _to_device(torch, arr):
    return torch.from_numpy(np.ascontiguousarray(arr).view(np.int32)).cuda()


def test_noalloc_gemm_matches_allocating_gemm(sdpg, exact):
    torch = pytest.importorskip("torch")
    lib = sdpg.lib()
    noalloc = _bind(lib)
    stream = torch.cuda.current_stream().cuda_stream
    cases = [(8, "N", "T", 96, 80, 120), (16, "T", "N", 40, 56, 33)]
    for call, (limbs, ta, tb, m, n, k) in enumerate(cases):
        rng = random.Random(4242 + call)
        lda = (k if ta == "T" else m) + 1
        ldb = (n if tb == "T" else k) + 2
        ldc = m + 3
        A = exact.random_ml(lda * (m if ta == "T" else k), limbs, rng, -25, 25, zero_frac=0.05)
        B = exact.random_ml(ldb * (k if tb == "T" else n), limbs, rng, -25, 25, zero_frac=0.05)
        C = exact.random_ml(ldc * n, limbs, rng, -5, 5)
        alpha = exact.random_ml(1, limbs, rng, -1, 1)
        beta = exact.random_ml(1, limbs, rng, -1, 1)
        dA, dB = _to_device(torch, A), _to_device(torch, B)
        dC_ref, dC_new = _to_device(torch, C), _to_device(torch, C)
        sdpg.check(lib.sdpg_rgemm_device(limbs, ta.encode(), tb.encode(), m, n, k, alpha.ctypes.data, dA.data_ptr(),
                                         lda, dB.data_ptr(), ldb, beta.ctypes.data, dC_ref.data_ptr(), ldc, stream))
        sdpg.check(noalloc(limbs, ta.encode(), tb.encode(), m, n, k, alpha.ctypes.data, dA.data_ptr(), lda,
                           dB.data_ptr(), ldb, beta.ctypes.data, dC_new.data_ptr(), ldc, stream))
        torch.cuda.synchronize()
        got_ref = dC_ref.cpu().numpy().view(np.uint32)
        got_new = dC_new.cpu().numpy().view(np.uint32)
        ref, scale = exact.gemm(ta, tb, m, n, k, exact.ml_decode(alpha)[0], exact.ml_decode(A), lda,
                                exact.ml_decode(B), ldb, exact.ml_decode(beta)[0], exact.ml_decode(C), ldc)
        rows = [i + j * ldc for j in range(n) for i in range(m)]
        # against the exact product, then against the allocating entry point
        err_exact = exact.max_rel_err(got_new[rows], [ref[r] for r in rows], [scale[r] for r in rows])
        assert err_exact <= 2.0 ** -(32 * limbs - 16), (call, err_exact)
        err = exact.max_rel_err(got_new[rows], exact.ml_decode(got_ref[rows]), [scale[r] for r in rows])
        assert err <= 2.0 ** -(32 * limbs - 16), (call, err)
        pad = [m + j * ldc for j in range(n)]
        assert (got_new[pad] == C[pad]).all()


def test_noalloc_gemm_rejects_products_beyond_its_scratch(sdpg):
    torch = pytest.importorskip("torch")
    lib = sdpg.lib()
    noalloc = _bind(lib)
    one = sdpg.ml_parse(["1"], 8)
    buf = torch.zeros(16, dtype=torch.int32, device="cuda")
    big = 4000  # digit planes alone would need ~1.3 GB at 256 bits
    rc = noalloc(8, b"N", b"N", big, big, big, one.ctypes.data, buf.data_ptr(), big, buf.data_ptr(), big,
                 one.ctypes.data, buf.data_ptr(), big, None)
    assert rc == -7  # SDPG_ERR_TOO_LARGE
    assert b"scratch" in lib.sdpg_last_error()
