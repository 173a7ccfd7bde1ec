"""tcgen05 tensor-core tile (3xTF32 split, FP32 accumulation in tensor memory)
against an FP64 product, through the library's self-test hook."""
import ctypes as ct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,N,K,bn", [(128, 128, 32, 128), (256, 256, 256, 256), (200, 256, 96, 256),
                                      (130, 100, 72, 128), (384, 512, 128, 256)])
def test_tc_gemm_tile(M, N, K, bn):
    torch = pytest.importorskip("torch")
    from madwave3_gb300 import load_library
    L = load_library()
    L.mw3_tc_gemm_selftest.argtypes = [ct.c_void_p] * 3 + [ct.c_int] * 4
    rng = np.random.default_rng(M * 7 + N + K)
    A = rng.standard_normal((M, K)).astype(np.float32)
    Bt = rng.standard_normal((N, K)).astype(np.float32)
    dA = torch.from_numpy(A).cuda()
    dB = torch.from_numpy(Bt).cuda()
    dC = torch.full((M, N), float("nan"), dtype=torch.float32, device="cuda")
    rc = L.mw3_tc_gemm_selftest(ct.c_void_p(dA.data_ptr()), ct.c_void_p(dB.data_ptr()), ct.c_void_p(dC.data_ptr()),
                                M, N, K, bn)
    assert rc == 0
    C = dC.cpu().numpy()
    ref = A.astype(np.float64) @ Bt.astype(np.float64).T
    err = np.abs(C - ref).max() / np.abs(ref).max()
    assert err < 5e-6, err          # FP32 accumulation over K <= 256
