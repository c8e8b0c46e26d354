"""The 5th-generation tensor-core building block (tcgen05.mma, accumulators in
tensor memory): BF16 x BF16 -> FP32 products against an exact CPU product of
the same BF16 values."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def to_bf16_bits(x):
    """round-to-nearest-even BF16 bit patterns of float32 values"""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    return r


def bf16_value(bits):
    return (bits.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


@pytest.fixture(scope="module")
def ctx():
    import ocfd
    return ocfd.Context()


@pytest.mark.parametrize("N,K", [(16, 16), (128, 16), (128, 128), (16, 128), (256, 64), (64, 256)])
def test_tc_gemm(ctx, N, K):
    import torch
    import ocfd
    from ocfd._abi import declare
    declare("ocfd_tc_gemm_bf16", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                ctypes.c_int, ctypes.c_int, ctypes.c_void_p])
    rng = np.random.default_rng(N * 1000 + K)
    A = to_bf16_bits(rng.standard_normal((128, K)))
    B = to_bf16_bits(rng.standard_normal((N, K)))
    want = bf16_value(A) @ bf16_value(B).T
    dA = torch.from_numpy(A.view(np.int16).copy()).cuda()
    dB = torch.from_numpy(B.view(np.int16).copy()).cuda()
    dC = torch.zeros((128, N), dtype=torch.float32, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    ocfd.check(ocfd.load().ocfd_tc_gemm_bf16(ctx.h, dA.data_ptr(), dB.data_ptr(), dC.data_ptr(), N, K, st),
               "ocfd_tc_gemm_bf16")
    got = dC.cpu().numpy().astype(np.float64)
    # FP32 accumulation of K exact BF16 products
    tol = 1e-6 * np.abs(bf16_value(A)) @ np.abs(bf16_value(B)).T + 1e-30
    assert (np.abs(got - want) <= 8 * tol).all(), np.abs(got - want).max()


def make_mlp(ctx, max_batch=1024, seed=11):
    import ctypes as C
    import ocfd
    from ocfd import mlp
    return mlp.Mlp(ctx, max_batch, seed)


def test_mlp_forward_vs_oracle(ctx):
    import torch
    import mlp_oracle as mo
    net = make_mlp(ctx)
    W, b = net.get_params()
    rng = np.random.default_rng(1)
    b = (0.1 * rng.standard_normal(b.shape)).astype(np.float32)
    b[mo.BOFF[4] + 10:] = 0
    net.set_params(W, b)
    X = rng.standard_normal((512, 12)).astype(np.float32)
    Y = net.forward(torch.from_numpy(X).cuda()).cpu().numpy()
    want, _ = mo.forward(W, b, X)
    err = np.abs(Y - want[:, :10]).max() / np.abs(want[:, :10]).max()
    assert err < 2e-3, err


def test_mlp_gradients_vs_oracle(ctx):
    import torch
    import mlp_oracle as mo
    net = make_mlp(ctx)
    W, b = net.get_params()
    rng = np.random.default_rng(2)
    b = (0.1 * rng.standard_normal(b.shape)).astype(np.float32)
    b[mo.BOFF[4] + 10:] = 0
    net.set_params(W, b)
    X = rng.standard_normal((512, 12)).astype(np.float32)
    T = rng.standard_normal((512, 10)).astype(np.float32)
    loss, gW, gb = net.train_step(torch.from_numpy(X).cuda(), torch.from_numpy(T).cuda(), lr=0.0, update=False,
                                  grads=True)
    wl, wW, wb = mo.train_grads(W, b, X, T)
    assert loss == pytest.approx(wl, rel=1e-4)
    for l in range(5):
        sl = slice(mo.WOFF[l], mo.WOFF[l] + mo.LN[l] * mo.LK[l])
        e = np.linalg.norm(gW[sl] - wW[sl]) / np.linalg.norm(wW[sl])
        assert e < 5e-3, (l, e)
        sb = slice(mo.BOFF[l], mo.BOFF[l] + mo.LN[l])
        e = np.linalg.norm(gb[sb] - wb[sb]) / max(np.linalg.norm(wb[sb]), 1e-30)
        assert e < 5e-3, (l, e)
    # padding rows / columns of the layout receive no gradient
    assert np.all(gW[mo.WOFF[4] + 10 * 128:mo.WOFF[4] + 16 * 128] == 0)
    assert np.all(mo.layer(gW, 0)[:, 12:] == 0)


def test_mlp_learns_smooth_map(ctx):
    """Adam on a smooth 12 -> 10 regression lowers the loss by 10x"""
    import torch
    net = make_mlp(ctx, max_batch=1024, seed=3)
    rng = np.random.default_rng(4)
    A = rng.standard_normal((12, 10)) / 4
    X = rng.standard_normal((8192, 12)).astype(np.float32)
    T = np.tanh(X @ A).astype(np.float32)
    Xd = torch.from_numpy(X).cuda()
    Td = torch.from_numpy(T).cuda()
    first = None
    for it in range(300):
        s = (it * 1024) % 8192
        loss, _, _ = net.train_step(Xd[s:s + 1024], Td[s:s + 1024], lr=2e-3)
        first = loss if first is None else first
    assert loss < first / 10, (first, loss)


def test_mlp_forward_throughput(ctx):
    """Rate of the network on the tensor cores: 2^20 rows through the five
    layers (2 (12 128 + 3 128^2 + 128 10) = 103,936 FLOP per row with the first
    layer's K padded to 16), the training forward with its stash of Z and H,
    timed with CUDA events after a warm-up, the best of three trials of five
    passes (the GPU may be shared for a moment).  The figure is printed; the
    bound only catches a broken pipeline, and no bounded wait may have run out."""
    import torch
    M = 1 << 20
    net = make_mlp(ctx, max_batch=M, seed=7)
    X = torch.randn((M, 12), dtype=torch.float32, device="cuda")
    Y = net.forward(X)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps, trials = 5, []
    for _ in range(3):
        e0.record()
        for _ in range(reps):
            Y = net.forward(X)
        e1.record()
        torch.cuda.synchronize()
        trials.append(e0.elapsed_time(e1) / reps)
    ms = min(trials)
    tflops = 103936.0 * M / (ms * 1e-3) / 1e12
    print("mlp forward: %.3f ms per 2^20 rows, %.1f TFLOP/s (trials %s ms)" %
          (ms, tflops, ", ".join("%.2f" % t for t in trials)))
    assert torch.isfinite(Y).all()
    assert ctx.check() == 0
    assert tflops > 5.0
