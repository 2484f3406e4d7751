"""The allocation-free integral image, umi_iimg_u8_i32_noalloc.

It exists for callers that cannot allocate device memory (nothing to take a
workspace from, or a context where cudaMalloc is not allowed): its tile sums
go to a scratch array built into the library instead of a caller workspace.
Its results must equal those of umi_iimg_u8_i32 with a caller workspace,
bit for bit (integer arithmetic), on consecutive calls that reuse the shared
scratch.  This file sorts last so that a run stopping at the first failure
has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(umi, x, out):
    import torch
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    return umi.lib().umi_iimg_u8_i32_noalloc(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                             x.shape[0], x.shape[1], stream)


def test_noalloc_matches_workspace_entry_point_on_consecutive_calls(umi, dev):
    import torch
    # two calls in a row, different sizes, both reusing the built-in scratch
    for seed, (h, w) in enumerate([(1080, 1920), (517, 1023), (2160, 3840)]):
        x = torch.from_numpy(np.random.default_rng(100 + seed).integers(0, 256, (h, w), dtype=np.uint8)).to(dev)
        got = torch.full((h, w), -1, dtype=torch.int32, device=dev)
        assert _call(umi, x, got) == 0, umi.lib().umi_last_error_string()
        want = umi.iimg_u8_i32(x)  # the existing entry point with a caller workspace
        torch.cuda.synchronize()
        assert torch.equal(got, want), (h, w)


def test_noalloc_rejects_frames_beyond_the_scratch(umi, dev):
    import torch
    x = torch.zeros((4096, 4096), dtype=torch.uint8, device=dev)
    out = torch.empty((4096, 4096), dtype=torch.int32, device=dev)
    assert _call(umi, x, out) == 5  # UMI_ERR_NO_MEMORY
    assert b"scratch" in umi.lib().umi_last_error_string()


def test_noalloc_refuses_what_the_int32_limit_refuses(umi, dev):
    """4096x2160 tile sums fit the 1 MiB scratch, but h*w*255 >= 2^31: the
    same int32 limit as umi_iimg_u8_i32 refuses it (UMI_ERR_UNSUPPORTED);
    3840x2160 (just under the limit) is served."""
    import torch
    x = torch.zeros((2160, 4096), dtype=torch.uint8, device=dev)
    out = torch.empty((2160, 4096), dtype=torch.int32, device=dev)
    assert _call(umi, x, out) == 3  # UMI_ERR_UNSUPPORTED
    assert b"int32" in umi.lib().umi_last_error_string()
    x = torch.full((2160, 3840), 255, dtype=torch.uint8, device=dev)
    got = torch.empty((2160, 3840), dtype=torch.int32, device=dev)
    assert _call(umi, x, got) == 0
    torch.cuda.synchronize()
    assert int(got[-1, -1].item()) == 2160 * 3840 * 255
