"""GPU parity tests of the FP32-level split-precision products (f16 hi/lo
with error correction, chunked round-to-nearest accumulation:
umi_gemm_f32_f16x3, umi_conv2d_fprop_f32_f16x3) through the C ABI against
the FP64 CPU oracle, beside the plain FP32 UMI path (the generic operator
with the reference's Gemm strategy, main/gemm.cu:8-15).

Tolerance (fp32-level): |C - C64| <= 1e-6 * sum_k |a b| for every element
(bf16x3 is held to 1e-4 of the same scale), and on the large random cases the
median of |C - C64| / |C64| <= 1e-6.  Every test also checks that no bounded
device wait gave up (err word stays 0).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-6


def _scaled_err(got, want, scale):
    return float((np.abs(got - want) / np.maximum(scale, 1e-30)).max())


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (200, 136, 48), (256, 256, 1024), (1, 1, 8), (130, 520, 136),
                                   (384, 640, 4104)])
@pytest.mark.parametrize("chunk", [0, 1, 5])
def test_gemm_f32_f16x3(umi, orc, dev, M, N, K, chunk):
    import torch
    g = np.random.default_rng(M * 3 + N + K)
    a = g.standard_normal((M, K)).astype(np.float32)
    b = g.standard_normal((N, K)).astype(np.float32)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    C = umi.gemm_f32_f16x3(torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev), chunk=chunk, err=err)
    C = C.cpu().numpy()
    assert int(err.item()) == 0
    want = orc.gemm_f64(a, b, b_is_nk=True)
    scale = orc.gemm_f64(np.abs(a), np.abs(b), b_is_nk=True)
    assert _scaled_err(C, want, scale) <= TOL


def test_gemm_f32_f16x3_4096_cubed_sampled(umi, orc, dev):
    """The configuration size: 1024 tiles of 128 x 128 over the persistent
    CTAs (every CTA reuses both chunk buffers and both correction
    accumulators many times); complete sampled rows and columns."""
    import torch
    M = N = K = 4096
    g = np.random.default_rng(4096)
    a = g.standard_normal((M, K)).astype(np.float32)
    b = g.standard_normal((N, K)).astype(np.float32)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    C = umi.gemm_f32_f16x3(torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev), err=err).cpu().numpy()
    assert int(err.item()) == 0
    rows = np.unique(np.concatenate([[0, M - 1], g.choice(M, 64, replace=False)]))
    cols = np.unique(np.concatenate([[0, N - 1], g.choice(N, 64, replace=False)]))
    want_r = orc.gemm_f64(a[rows], b, b_is_nk=True)
    assert _scaled_err(C[rows], want_r, orc.gemm_f64(np.abs(a[rows]), np.abs(b), b_is_nk=True)) <= TOL
    want_c = orc.gemm_f64(a, b[cols], b_is_nk=True)
    assert _scaled_err(C[:, cols], want_c, orc.gemm_f64(np.abs(a), np.abs(b[cols]), b_is_nk=True)) <= TOL
    med = float(np.median(np.abs(C[rows] - want_r) / np.abs(want_r)))
    assert med <= 1e-6, med


def test_gemm_f32_f16x3_more_accurate_than_tensor_core_accumulation(umi, orc, dev):
    """Chunked accumulation matters: with all-positive inputs the tensor
    core's truncating fp32 accumulation alone drifts (bf16 operands, exact
    products), while the split product stays at fp32 level."""
    import torch
    M, N, K = 128, 256, 8192
    g = np.random.default_rng(3)
    a = g.random((M, K), dtype=np.float32)
    b = g.random((N, K), dtype=np.float32)
    want = orc.gemm_f64(a, b, b_is_nk=True)
    C = umi.gemm_f32_f16x3(torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)).cpu().numpy()
    rel = np.abs(C - want) / want
    assert rel.max() <= 2e-6, rel.max()


def test_gemm_f32_f16x3_rejects(umi, dev):
    import torch
    A = torch.zeros(128, 12, device=dev)
    with pytest.raises(umi.UmiError):
        umi.gemm_f32_f16x3(A, A)  # K = 12 is not a multiple of 8
    A = torch.zeros(128, 16, device=dev)
    with pytest.raises(umi.UmiError):
        umi.gemm_f32_f16x3(A, A, chunk=65)


@pytest.mark.parametrize("n,c,h,w,k,r", [(2, 64, 16, 16, 128, 3), (1, 128, 5, 130, 64, 3), (1, 64, 7, 9, 128, 1),
                                         (1, 64, 9, 20, 200, 5), (3, 64, 33, 128, 128, 3)])
def test_conv2d_fprop_f32_f16x3(umi, orc, dev, n, c, h, w, k, r):
    import torch
    g = np.random.default_rng(n * 100 + h + k)
    x = g.standard_normal((n, c, h, w)).astype(np.float32)
    wt = (g.standard_normal((k, c, r, r)) / (r * np.sqrt(c))).astype(np.float32)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    got = umi.conv2d_fprop_f32_f16x3(torch.from_numpy(x).permute(0, 2, 3, 1).contiguous().to(dev),
                                     torch.from_numpy(wt).permute(0, 2, 3, 1).contiguous().to(dev), err=err)
    got = got.cpu().numpy()
    assert int(err.item()) == 0
    want = orc.conv2d_f64(x, wt, 1, r // 2)
    scale = orc.conv2d_f64(np.abs(x), np.abs(wt), 1, r // 2)
    assert _scaled_err(got, want, scale) <= TOL


def test_conv2d_fprop_f32_f16x3_benchmark_shape(umi, dev):
    """N32 C64 128x128 K128 3x3: every output against an FP64 convolution on
    the GPU (torch, float64) of the same fp32 inputs."""
    import torch
    gen = torch.Generator(device="cpu").manual_seed(9)
    x = torch.randn(32, 64, 128, 128, generator=gen)
    wt = torch.randn(128, 64, 3, 3, generator=gen) / 24.0
    xd, wd = x.to(dev), wt.to(dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    got = umi.conv2d_fprop_f32_f16x3(xd.permute(0, 2, 3, 1).contiguous(), wd.permute(0, 2, 3, 1).contiguous(), err=err)
    assert int(err.item()) == 0
    want = torch.nn.functional.conv2d(xd.double(), wd.double(), padding=1)
    scale = torch.nn.functional.conv2d(xd.double().abs(), wd.double().abs(), padding=1)
    rel = ((got.double() - want).abs() / scale.clamp_min(1e-30)).max().item()
    assert rel <= TOL, rel


@pytest.mark.parametrize("M,N,K", [(32, 64, 96), (17, 33, 250)])
def test_gemm_f32_generic_plain_path(umi, orc, dev, M, N, K):
    """The plain FP32 UMI path (generic operator, the reference's Gemm
    strategy on float): fp32 FMA over a blocked K loop."""
    import torch
    g = np.random.default_rng(M + N + K)
    a = g.standard_normal((M, K)).astype(np.float32)
    b = g.standard_normal((N, K)).astype(np.float32)
    C = umi.gemm_f32_generic(torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)).cpu().numpy()
    want = orc.gemm_f64(a, b, b_is_nk=True)
    assert _scaled_err(C, want, orc.gemm_f64(np.abs(a), np.abs(b), b_is_nk=True)) <= TOL
