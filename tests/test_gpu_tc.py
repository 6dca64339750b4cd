"""tcgen05 split-precision GEMM engine vs an FP64 product (needs a GPU).

The engine stores each operand as FP16 hi + lo planes after a per-matrix
power-of-two scaling (representation error ~2^-22) and accumulates
hi*hi + hi*lo + lo*hi in FP32 tensor memory.  The FP32 accumulation bounds the
relative Frobenius error of a product with inner dimension K at about
1.2e-7 * sqrt(K) for random operands (1.9e-6 measured at K = 256); the bar
below is 2.5e-6 * sqrt(K / 256).
"""

import math

import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def tol(k):
    return 2.5e-6 * math.sqrt(k / 256.0)


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pulsesuite_gb300 import build
    build.build()


def _op(x, op):
    if op == 1:
        return x.transpose(-1, -2)
    if op == 2:
        return x.conj()
    if op == 3:
        return x.conj().transpose(-1, -2)
    return x


def _run(nk, nb, A, B, opA, opB, cplx):
    from pulsesuite_gb300 import _lib
    lib = _lib.load()
    out = torch.empty((nb, nk, nk), dtype=torch.complex128, device="cuda")
    _lib.check(lib.sbe_tc_selftest(nk, nb, _lib.ptr(A), _lib.ptr(B), opA, opB, int(cplx),
                                   _lib.ptr(out), _lib.stream_handle()), "sbe_tc_selftest")
    return out


def _rel(a, b):
    return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))


@pytest.mark.parametrize("nk", [64, 128, 256, 384])
def test_complex_products_all_ops(nk):
    g = torch.Generator(device="cpu").manual_seed(nk)
    nb = 2
    A = (torch.randn((nb, nk, nk), generator=g, dtype=torch.float64)
         + 1j * torch.randn((nb, nk, nk), generator=g, dtype=torch.float64)).cuda()
    B = (torch.randn((nb, nk, nk), generator=g, dtype=torch.float64)
         + 1j * torch.randn((nb, nk, nk), generator=g, dtype=torch.float64)).cuda()
    A[1] *= 1e-21   # second batch entry at Hamiltonian scale (J)
    B[1] *= 3e-3    # and coherence scale
    for opA in range(4):
        for opB in range(4):
            ref = _op(A, opA) @ _op(B, opB)
            out = _run(nk, nb, A, B, opA, opB, True)
            for b in range(nb):
                e = _rel(out[b], ref[b])
                assert e < tol(nk), (nk, opA, opB, b, e)


@pytest.mark.parametrize("nk", [64, 256])
def test_real_mode(nk):
    g = torch.Generator(device="cpu").manual_seed(7 + nk)
    A = torch.randn((1, nk, nk), generator=g, dtype=torch.float64).to(torch.complex128).cuda()
    B = torch.randn((1, nk, nk), generator=g, dtype=torch.float64).to(torch.complex128).cuda()
    out = _run(nk, 1, A, B, 0, 0, False)
    ref = A.real @ B.real
    assert _rel(out[0].real, ref[0]) < tol(nk)
    assert float(out.imag.abs().max()) == 0.0


def test_integer_pipe_conversions_match_hardware():
    """fp32(x) and fp64(f) of the mixed path's integer-pipe helpers vs the GPU's own
    conversions, bit for bit (FP32 subnormal results are flushed to zero by design)."""
    import numpy as np
    from pulsesuite_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(0)
    n = 1 << 16
    mant = rng.uniform(1.0, 2.0, n)
    expo = rng.integers(-140, 130, n)
    d = mant * np.exp2(expo.astype(float)) * rng.choice([-1.0, 1.0], n)
    # ties: FP32 values plus exactly half an FP32 ulp
    f = rng.uniform(1, 2, 1024).astype(np.float32).astype(np.float64)
    d[:1024] = f + np.exp2(np.floor(np.log2(f)) - 24)
    d[1024:1030] = [0.0, -0.0, np.inf, -np.inf, 3.4028234663852886e38, 1.1754943508222875e-38]
    fin = (rng.standard_normal(n) * np.exp2(rng.integers(-149, 127, n).astype(float))).astype(np.float32)
    fin[:6] = [0.0, -0.0, np.inf, 1e-45, -3e-39, 3.4e38]
    dd = torch.as_tensor(d).cuda()
    ff = torch.as_tensor(fin).cuda()
    fo = torch.empty(n, dtype=torch.float32, device="cuda")
    do = torch.empty(n, dtype=torch.float64, device="cuda")
    _lib.check(lib.sbe_convert_selftest(_lib.ptr(dd), _lib.ptr(ff), n, _lib.ptr(fo), _lib.ptr(do),
                                        _lib.stream_handle()), "sbe_convert_selftest")
    torch.cuda.synchronize()
    hw_f = dd.float()
    normal = (hw_f.abs() >= 1.1754943508222875e-38) | (hw_f == 0) | torch.isinf(hw_f)
    assert torch.equal(fo[normal].view(torch.int32), hw_f[normal].view(torch.int32))
    assert torch.all(fo[~normal] == 0)
    assert torch.equal(do.view(torch.int64), ff.double().view(torch.int64))
