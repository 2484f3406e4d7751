"""GPU parity tests of the tcgen05 GEMM (through the C ABI) against the FP64 CPU oracle.

bf16/f16: the oracle multiplies the same rounded inputs in FP64; the tensor
cores multiply exactly and accumulate in FP32, so |C - C64| <= 1e-5 * sum_k |a b|.
bf16x3 (fp32 inputs): the split keeps ~16 significant bits per operand, so
|C - C64| <= 1e-4 * sum_k |a b| against the FP64 product of the fp32 inputs.
Every test also checks that no bounded device wait gave up (err word stays 0).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _check(got, want, scale, tol):
    err = np.abs(got - want) / np.maximum(scale, 1e-30)
    assert err.max() <= tol, err.max()


# tile widths: 4096^3 and most small shapes take 224-column tiles (ragged last
# column), 2048 x 2048 the 256-column ones (fewer rounds of persistent tiles)
@pytest.mark.parametrize("M,N,K", [(128, 256, 64), (256, 512, 1024), (128, 256, 8), (200, 300, 72), (1, 1, 16),
                                   (384, 256, 4096), (130, 520, 136), (2048, 2048, 256)])
@pytest.mark.parametrize("dt", ["bf16", "f16"])
def test_gemm_half(umi, orc, dev, M, N, K, dt):
    import torch
    g = torch.Generator(device="cpu").manual_seed(M * 7 + N + K)
    tdt = torch.bfloat16 if dt == "bf16" else torch.float16
    A = torch.randn(M, K, generator=g).to(tdt)
    B = torch.randn(N, K, generator=g).to(tdt)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    C = umi.gemm(A.to(dev), B.to(dev), err=err).cpu().numpy()
    assert int(err.item()) == 0
    a, b = A.float().numpy(), B.float().numpy()
    want = orc.gemm_f64(a, b, b_is_nk=True)
    scale = orc.gemm_f64(np.abs(a), np.abs(b), b_is_nk=True)
    _check(C, want, scale, 1e-5)


@pytest.mark.parametrize("M,N,K", [(128, 256, 64), (256, 256, 1024), (200, 136, 48)])
def test_gemm_f32_bf16x3(umi, orc, dev, M, N, K):
    import torch
    g = np.random.default_rng(M + N + K)
    a = g.standard_normal((M, K)).astype(np.float32)
    b = g.standard_normal((N, K)).astype(np.float32)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    C = umi.gemm_f32_bf16x3(torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev), err=err).cpu().numpy()
    assert int(err.item()) == 0
    want = orc.gemm_f64(a, b, b_is_nk=True)
    scale = orc.gemm_f64(np.abs(a), np.abs(b), b_is_nk=True)
    _check(C, want, scale, 1e-4)


def test_gemm_rejects(umi, dev):
    import torch
    A = torch.zeros(128, 12, dtype=torch.bfloat16, device=dev)
    with pytest.raises(umi.UmiError):
        umi.gemm(A, A)  # K = 12 is not a multiple of 8


# ---------------------------------------------------------------- conv fprop (implicit GEMM)
def _conv_case(n, c, h, w, k, r, seed):
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    x = torch.randn(n, c, h, w, generator=g).to(torch.bfloat16)
    wt = (torch.randn(k, c, r, r, generator=g) / (r * (c ** 0.5))).to(torch.bfloat16)
    return x, wt


@pytest.mark.parametrize("n,c,h,w,k,r", [(2, 64, 16, 16, 128, 3), (1, 128, 5, 130, 64, 3), (1, 64, 7, 9, 128, 1),
                                         (1, 64, 9, 20, 200, 5), (1, 64, 1, 1, 128, 3), (3, 64, 33, 128, 128, 3),
                                         (1, 64, 6, 300, 96, 3), (2, 64, 3, 129, 16, 3)])
def test_conv2d_fprop_bf16(umi, orc, dev, n, c, h, w, k, r):
    import torch
    x, wt = _conv_case(n, c, h, w, k, r, n * 1000 + h * 10 + k)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    got = umi.conv2d_fprop_bf16(x.permute(0, 2, 3, 1).contiguous().to(dev), wt.permute(0, 2, 3, 1).contiguous().to(dev),
                                err=err).cpu().numpy()
    assert int(err.item()) == 0
    xf, wf = x.float().numpy(), wt.float().numpy()
    want = orc.conv2d_f64(xf, wf, 1, r // 2)
    scale = orc.conv2d_f64(np.abs(xf), np.abs(wf), 1, r // 2)
    _check(got, want, scale, 1e-5)


def test_conv2d_fprop_bf16_benchmark_shape_sampled(umi, dev):
    """N32 C64 128x128 K128 3x3: every output checked against an FP64 direct
    convolution computed on the GPU (torch, float64) of the same bf16 inputs."""
    import torch
    x, wt = _conv_case(32, 64, 128, 128, 128, 3, 7)
    xd, wd = x.to(dev), wt.to(dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    got = umi.conv2d_fprop_bf16(xd.permute(0, 2, 3, 1).contiguous(), wd.permute(0, 2, 3, 1).contiguous(), err=err)
    assert int(err.item()) == 0
    want = torch.nn.functional.conv2d(xd.double(), wd.double(), padding=1)
    scale = torch.nn.functional.conv2d(xd.double().abs(), wd.double().abs(), padding=1)
    rel = ((got.double() - want).abs() / scale.clamp_min(1e-30)).max().item()
    assert rel <= 1e-5, rel


# ---------------------------------------------------------------- config size: the persistent multi-tile path
def _sampled_rows_cols(orc, a, b, C, tol, nsample=64, seed=0):
    """Complete rows and columns of C (nsample of each, plus the first and last
    of each) against the FP64 product of the same inputs."""
    M, N = C.shape
    g = np.random.default_rng(seed)
    rows = np.unique(np.concatenate([[0, M - 1], g.choice(M, nsample, replace=False)]))
    cols = np.unique(np.concatenate([[0, N - 1], g.choice(N, nsample, replace=False)]))
    want_r = orc.gemm_f64(a[rows], b, b_is_nk=True)
    scale_r = orc.gemm_f64(np.abs(a[rows]), np.abs(b), b_is_nk=True)
    _check(C[rows], want_r, scale_r, tol)
    want_c = orc.gemm_f64(a, b[cols], b_is_nk=True)
    scale_c = orc.gemm_f64(np.abs(a), np.abs(b[cols]), b_is_nk=True)
    _check(C[:, cols], want_c, scale_c, tol)
    return want_r, rows


@pytest.mark.parametrize("dt", ["bf16", "f16"])
def test_gemm_half_4096_cubed(umi, orc, dev, dt):
    """M = N = K = 4096: 512 tiles of 128 x 256 over the persistent CTAs, so
    every CTA reuses both TMEM accumulators several times (the ping-pong
    between the MMA issuer and the epilogue)."""
    import torch
    M = N = K = 4096
    g = torch.Generator(device="cpu").manual_seed(4096 + (dt == "f16"))
    tdt = torch.bfloat16 if dt == "bf16" else torch.float16
    A = torch.randn(M, K, generator=g).to(tdt)
    B = torch.randn(N, K, generator=g).to(tdt)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    C = umi.gemm(A.to(dev), B.to(dev), err=err).cpu().numpy()
    assert int(err.item()) == 0
    assert np.isfinite(C).all()
    _sampled_rows_cols(orc, A.float().numpy(), B.float().numpy(), C, 1e-5)


def test_gemm_f32_bf16x3_2048(umi, orc, dev):
    import torch
    M = N = K = 2048
    g = np.random.default_rng(2048)
    a = g.standard_normal((M, K)).astype(np.float32)
    b = g.standard_normal((N, K)).astype(np.float32)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    C = umi.gemm_f32_bf16x3(torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev), err=err).cpu().numpy()
    assert int(err.item()) == 0
    _sampled_rows_cols(orc, a, b, C, 1e-4)


# ---------------------------------------------------------------- the bounded-wait timeout path
def test_gemm_epilogue_wait_times_out_and_context_stays_usable(umi, orc, dev):
    """A 1 us limit on the epilogue's wait for the first finished accumulator
    (one 128 x 256 tile with K = 4096 takes ~20 us of MMAs) makes that bounded
    wait give up: the error bit 4 comes back, umi_err_status maps it to
    UMI_ERR_TIMEOUT, the kernel returns (its copies and MMAs drained, TMEM
    freed), and the next normal call on the same stream is correct."""
    import torch
    M = N = K = 4096
    g = torch.Generator(device="cpu").manual_seed(77)
    A = torch.randn(M, K, generator=g).to(torch.bfloat16).to(dev)
    B = torch.randn(N, K, generator=g).to(torch.bfloat16).to(dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    umi.gemm_bf16_wait_limit(A, B, 1000, err=err)
    torch.cuda.synchronize()
    bits = int(err.item())
    assert bits & 4, bits
    assert bits & ~15 == 0, bits
    with pytest.raises(umi.UmiError) as ei:
        umi.check_err(err, "umi_gemm_bf16_wait_limit")
    assert "UMI_ERR_TIMEOUT" in str(ei.value)
    # the same stream, a normal call: no error bits, correct rows
    err.zero_()
    C = umi.gemm(A, B, err=err)
    umi.check_err(err, "umi_gemm_bf16")
    rows = [0, 1234, 4095]
    a, b = A[rows].float().cpu().numpy(), B.float().cpu().numpy()
    _check(C[rows].cpu().numpy(), orc.gemm_f64(a, b, b_is_nk=True), orc.gemm_f64(np.abs(a), np.abs(b), b_is_nk=True),
           1e-5)
