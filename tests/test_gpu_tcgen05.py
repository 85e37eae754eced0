"""The tcgen05 tensor-core kernels of the learned initial guess (TMEM accumulator, TMA-staged
operands in swizzled shared memory): the dense GEMM and the implicit-im2col convolution against
fp32 products of the same bf16 operands, the fused bias / ReLU / bf16 epilogue, and the whole
CNN forward on the tcgen05 path against the mma.sync path and the bf16-rounding oracle."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def N():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from astrophot_gb300 import _native

    return _native


def _status(N):
    import ctypes

    v = ctypes.c_uint32(0)
    assert N.lib().ap_tc_status(0, ctypes.byref(v)) == 0
    return v.value


# (R, S, T): one tile; ragged rows; the 64-byte and 32-byte swizzles (T = 48, 16); a ragged last
# reduction tile (288 = 4.5 x 64); narrow N tiles (S = 48 -> three 16-wide tiles); the widest
# (256) tile over a long reduction; the fc layers of the network
SHAPES = [(128, 16, 16), (136, 32, 48), (1000, 64, 288), (300, 48, 16), (256, 256, 4096), (4096, 192, 4096),
          (4096, 16, 192), (65536, 32, 16)]


@pytest.mark.parametrize("R,S,T", SHAPES)
def test_tc_gemm_matches_fp32_product(N, R, S, T):
    g = torch.Generator(device="cuda").manual_seed(R * 7 + S + T)
    A = torch.randn((R, T), device="cuda", generator=g).to(torch.bfloat16)
    W = torch.randn((S, T), device="cuda", generator=g).to(torch.bfloat16)
    want = A.float() @ W.float().T
    C = torch.full((R, S), float("nan"), device="cuda")
    rc = N.lib().ap_gemm_bf16_tc(N._ptr(A), T, N._ptr(W), T, N._ptr(C), S, R, S, T, None, None, 0, N._stream())
    assert rc == 0
    torch.cuda.synchronize()
    assert _status(N) == 0
    err = (C - want).abs().max().item()
    # the same bf16 products summed in fp32 in another order
    assert err <= 2e-5 * want.abs().max().item() * max(1.0, (T / 1024) ** 0.5), err


@pytest.mark.parametrize("R,S,T", [(136, 32, 48), (4096, 192, 4096), (1000, 64, 288)])
def test_tc_gemm_bias_relu_bf16_epilogue(N, R, S, T):
    g = torch.Generator(device="cuda").manual_seed(5 + R)
    A = torch.randn((R, T), device="cuda", generator=g).to(torch.bfloat16)
    W = torch.randn((S, T), device="cuda", generator=g).to(torch.bfloat16)
    bias = torch.randn(S, device="cuda", generator=g) * 4
    pre = A.float() @ W.float().T + bias
    act = torch.empty((R, S), dtype=torch.bfloat16, device="cuda")
    rc = N.lib().ap_gemm_bf16_tc(N._ptr(A), T, N._ptr(W), T, None, S, R, S, T, N._ptr(bias), N._ptr(act), 1,
                                 N._stream())
    assert rc == 0
    want = torch.relu(pre)
    got = act.float()
    # one bf16 rounding of an fp32 value whose sum order differs: within one bf16 step (2^-8)
    tol = 2.0 ** -8 * want.abs() + 2e-5 * pre.abs().max()
    assert bool(((got - want).abs() <= tol).all()), (got - want).abs().max().item()
    assert bool((got >= 0).all())
    # bias without ReLU into fp32
    C = torch.empty((R, S), device="cuda")
    rc = N.lib().ap_gemm_bf16_tc(N._ptr(A), T, N._ptr(W), T, N._ptr(C), S, R, S, T, N._ptr(bias), None, 0,
                                 N._stream())
    assert rc == 0
    assert (C - pre).abs().max().item() <= 2e-5 * pre.abs().max().item() * max(1.0, (T / 1024) ** 0.5)
    assert _status(N) == 0


# (batch, H, cin, S): the network's layers 2-4 (H = 32, 16, 8 -> 128-row tiles of half a stamp,
# 2 stamps, 8 stamps) with ragged batches where a tile's last stamps lie past the tensor
@pytest.mark.parametrize("B,H,cin,S", [(2, 32, 32, 64), (3, 16, 64, 128), (5, 8, 128, 256), (16, 8, 128, 256),
                                       (4, 32, 32, 64), (2, 16, 16, 32), (9, 16, 64, 128)])
def test_tc_conv_matches_conv2d(N, B, H, cin, S):
    g = torch.Generator(device="cuda").manual_seed(B * 100 + H + cin)
    x = torch.randn((B, H, H, cin), device="cuda", generator=g).to(torch.bfloat16)
    W = (torch.randn((S, 9 * cin), device="cuda", generator=g) / (3 * cin**0.5)).to(torch.bfloat16)
    bias = torch.randn(S, device="cuda", generator=g)
    # W[s][(ky * 3 + kx) * cin + c] -> conv2d weight [S][cin][3][3]
    w4 = W.float().view(S, 3, 3, cin).permute(0, 3, 1, 2)
    ref = torch.nn.functional.conv2d(x.float().permute(0, 3, 1, 2), w4, stride=2, padding=1)
    ho = H // 2
    want = ref.permute(0, 2, 3, 1).reshape(B * ho * ho, S) + bias
    C = torch.full((B * ho * ho, S), float("nan"), device="cuda")
    rc = N.lib().ap_conv3x3s2_bf16_tc(N._ptr(x), B, H, cin, N._ptr(W), S, N._ptr(C), S, N._ptr(bias), None, 0,
                                      N._stream())
    assert rc == 0
    torch.cuda.synchronize()
    assert _status(N) == 0
    err = (C - want).abs().max().item()
    assert err <= 3e-5 * want.abs().max().item(), err


def test_tc_rejects_unsupported_shapes(N):
    A = torch.zeros((128, 24), dtype=torch.bfloat16, device="cuda")
    W = torch.zeros((16, 24), dtype=torch.bfloat16, device="cuda")
    C = torch.zeros((128, 16), device="cuda")
    # T = 24 is not a multiple of 16; S = 8 below the 16-wide tile
    assert N.lib().ap_gemm_bf16_tc(N._ptr(A), 24, N._ptr(W), 24, N._ptr(C), 16, 128, 16, 24, None, None, 0,
                                   N._stream()) == 1
    assert N.lib().ap_gemm_bf16_tc(N._ptr(A), 24, N._ptr(W), 24, N._ptr(C), 16, 128, 8, 16, None, None, 0,
                                   N._stream()) == 1
    x = torch.zeros((2, 16, 16, 24), dtype=torch.bfloat16, device="cuda")
    # cin = 24 has no swizzle width
    assert N.lib().ap_conv3x3s2_bf16_tc(N._ptr(x), 2, 16, 24, N._ptr(W), 16, N._ptr(C), 16, None, None, 0,
                                        N._stream()) == 1


def test_cnn_forward_paths_agree(N):
    from astrophot_gb300 import cnn
    from oracle import cnn as C

    net = cnn.InitNet(seed=11)
    rng = np.random.default_rng(2)
    p = net.params.cpu().numpy()
    for l in range(6):
        nb = C.LAYERS[l][5]
        p[C.B_OFF[l] : C.B_OFF[l] + nb] = rng.normal(0, 0.05, nb)
    p[C.B_OFF[5] + 8 : C.B_OFF[5] + 16] = 0
    net.params = torch.tensor(p, device="cuda")
    net._sync_bf16()
    B = 48
    x = torch.tensor(rng.normal(size=(B, 64, 64)).astype(np.float32), device="cuda").reshape(-1)
    old = cnn.get_tensor_path()
    try:
        cnn.set_tensor_path("tcgen05")
        tc_infer = net.infer(x, B).cpu().numpy()
        tc_fwd = net.forward(x, B).cpu().numpy()
        cnn.set_tensor_path("mma_sync")
        ms = net.forward(x, B).cpu().numpy()
    finally:
        cnn.set_tensor_path(old)
    assert cnn.tc_status() == 0
    # the implicit-im2col convolution and the explicit one: identical MMAs on identical tiles
    assert np.array_equal(tc_infer, tc_fwd)
    # tcgen05 vs mma.sync: fp32 sums in another order, bf16 activations between layers
    assert np.linalg.norm(tc_fwd[:, :8] - ms[:, :8]) <= 6e-3 * np.linalg.norm(ms[:, :8])
    pb = C.bf16(net.params.cpu().numpy())
    emu, _ = C.forward(pb, x.cpu().numpy().reshape(B, 64, 64).astype(np.float64), round_bf16=True)
    assert np.linalg.norm(tc_infer[:, :8] - emu[:, :8]) <= 6e-3 * np.linalg.norm(emu[:, :8])
    assert np.all(tc_infer[:, 8:] == 0)
