"""The FMA-chain probe that gives the measured FP32 / FP64 FMA peaks."""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('prec, dt', [('FP32LOCAL', torch.float32), ('FP64', torch.float64)])
def test_fma_probe_runs_and_matches_host_recurrence(prec, dt):
    from marxs_gb300 import _abi
    lib = _abi.load()
    blocks, iters = 4, 100
    out = torch.full((blocks * 256,), float('nan'), dtype=dt, device='cuda')
    _abi.check(lib.mgpu_fma_probe(getattr(_abi, prec), blocks, iters, C.c_void_p(out.data_ptr()),
                                  None), 'mgpu_fma_probe')
    torch.cuda.synchronize()
    got = out.cpu().numpy().astype(np.float64)
    # each of the 8 chains: a <- a * b + c from a0 = (thread + k) * 1e-3
    b, c = 0.999999, 1e-7
    t = np.arange(256, dtype=np.float64)
    want = np.zeros(256)
    for k in range(8):
        a = (t + k) * 1e-3
        for _ in range(iters):
            a = a * b + c
        want += a
    rtol = 1e-5 if dt == torch.float32 else 1e-12
    np.testing.assert_allclose(got.reshape(blocks, 256), np.broadcast_to(want, (blocks, 256)),
                               rtol=rtol)


def test_fma_probe_rejects_bad_arguments():
    from marxs_gb300 import _abi
    lib = _abi.load()
    buf = torch.empty(256, dtype=torch.float32, device='cuda')
    assert lib.mgpu_fma_probe(_abi.FP32LOCAL, 0, 10, C.c_void_p(buf.data_ptr()), None) != 0
    assert lib.mgpu_fma_probe(7, 1, 10, C.c_void_p(buf.data_ptr()), None) != 0
