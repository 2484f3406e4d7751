"""CPU tests of the C ABI: the library loads, exports what the header declares,
validates descriptors like the reference (with status codes instead of
abort), and rejects bad arguments before touching the GPU."""
import ctypes

import pytest

import umi_gb300 as U

PAD, WRAP = U.PAD, U.WRAP


def test_exports_every_declared_symbol(umi):
    L = umi.lib()
    names = umi.header_functions()
    assert len(names) >= 8
    for n in names:
        assert hasattr(L, n), n
    # every declared function has a ctypes signature in the bindings
    assert set(names) <= set(umi.SIGNATURES), set(names) - set(umi.SIGNATURES)


def test_status_strings(umi):
    L = umi.lib()
    assert L.umi_status_string(0) == b"UMI_OK"
    assert L.umi_status_string(1) == b"UMI_ERR_INVALID_DESC"
    assert L.umi_version() >= 100


# The descriptor of main/filter3x3.cu:37-58.
def filter3x3_desc(h=300, w=500, p2=(16, 4, 1), p3=(16, 8, 1)):
    return U.make_desc(
        p=[(1, 1, 1, 1), (1, 1, 1, 1), (h,) + p2, (w,) + p3],
        a=[(1, 1), (1, 1), (3, 3), (3, 3)],
        mems=[
            dict(p_view=[(), (), (2, 0, 1), (3, 0, 1)], a_view=[(), (), (2, -1, 1), (3, -1, 1)],
                 phys=[(1, PAD), (1, PAD), (h, PAD), (w, PAD)], stage=1),
            dict(p_view=[(), (), (2, 0, 1), (3, 0, 1)], phys=[(), (), (h, PAD), (w, PAD)], stage=2, out=True),
        ])


def test_plan_filter3x3(umi):
    p = umi.plan_build(filter3x3_desc())
    assert p.n_threads == 256
    assert list(p.grid) == [1, 1, 19, 32]
    assert p.n_cta == 19 * 32
    assert p.n_ablock == 1 and p.ablock_size == 9
    m = p.mem[0]
    assert list(m.base) == [0, 0, -1, -1]
    assert m.pcoef[2][2] == 1 and m.pcoef[3][3] == 1
    assert m.acoef[2][2] == 1 and m.acoef[3][3] == 1
    assert m.pad_mask == 0xf
    assert list(m.rowstride) == [300 * 500, 300 * 500, 500, 1]
    o = p.mem[1]
    # leading sizes left at 0 ({} in the reference's initialiser): rowstride = product of later sizes
    assert o.is_output == 1 and list(o.rowstride) == [0, 300 * 500, 500, 1]
    assert all(o.acoef[k][d] == 0 for k in range(4) for d in range(4))  # Post output: no a-index term


def test_plan_expand(umi):
    # main/gemm.cu:37: Expand 0x1124 -> E0=1, E1=1, E2=2, E3=4 points per thread
    d = filter3x3_desc(h=100, w=200)
    d.expand = 0x1124
    p = umi.plan_build(d)
    assert list(p.expand) == [1, 1, 2, 4]
    assert p.grid[2] == -(-100 // 32) and p.grid[3] == -(-200 // 64)


def test_iimg_pass2_warp_shuf_zero_accepted(umi):
    # main/iimg.cu:61 leaves warp_shuf = 0: the reference divides by zero
    # (SIGFPE at src/UMI.cpp:59); here 0 reads as 1.
    d = U.make_desc(
        p=[(1, 1, 1), (1, 1, 1), (1, 1, 1), (500, 128, 32)], a=[(1, 1), (1, 1), (1, 1), (300, 32)],
        mems=[dict(p_view=[(), (), (), (2, 0, 1)], a_view=[(), (), (), (3, 0, 1)],
                   phys=[(1, PAD), (1, PAD), (500, PAD), (300, PAD)], stage=1),
              dict(p_view=[(), (), (), (3, 0, 1)], a_view=[(), (), (), (2, 0, 1)],
                   phys=[(1, PAD), (1, PAD), (300, PAD), (500, PAD)], stage=1, out=True)])
    p = umi.plan_build(d)
    assert p.n_threads == 128
    assert p.mem[1].acoef[2][3] == 1  # Loop output: a-index term kept


@pytest.mark.parametrize("case", ["shuf_not_pow2", "warp_product", "block_not_divisible", "too_many_threads",
                                  "zero_block", "a_block_zero", "expand_zero", "bad_phys_dim", "bad_mode",
                                  "too_many_ptrs"])
def test_plan_rejects(umi, case):
    d = filter3x3_desc()
    if case == "shuf_not_pow2":
        d.p[3].warp_shuf = 3
    elif case == "warp_product":
        d.p[3].warp_size = 4
    elif case == "block_not_divisible":
        d.p[2].block_size = 6
    elif case == "too_many_threads":
        d.p[2].block_size = 64; d.p[3].block_size = 32
    elif case == "zero_block":
        d.p[1].block_size = 0
    elif case == "a_block_zero":
        d.a[2].block_size = 0
    elif case == "expand_zero":
        d.expand = 0x1110
    elif case == "bad_phys_dim":
        d.mem[0].p_view[2].physical_dim_id = 4
    elif case == "bad_mode":
        d.mem[0].phys[2].mode = 7
    elif case == "too_many_ptrs":
        d.mem[0].n_ptr = 5
    with pytest.raises(U.UmiError) as e:
        umi.plan_build(d)
    assert e.value.status == 1  # UMI_ERR_INVALID_DESC
    assert umi.lib().umi_last_error_string()


def test_plan_empty_parallel_space(umi):
    d = filter3x3_desc(h=0)
    p = umi.plan_build(d)
    assert p.n_cta == 0


def test_null_arguments_rejected_without_gpu(umi):
    L = umi.lib()
    assert L.umi_plan_build(None, None) == 2
    assert L.umi_full_me_u8(None, None, 64, 64, 16, 32, None, None, None) == 2
    assert L.umi_iimg_u8_i32(None, None, 10, 10, None, 0, None) == 2
    w9 = (ctypes.c_float * 9)()
    assert L.umi_filter3x3_f32(None, None, 4, 4, w9, 0.0, None) == 2


def test_unsupported_rejected_without_gpu(umi):
    L = umi.lib()
    buf = ctypes.create_string_buffer(64)
    assert L.umi_full_me_u8(buf, buf, 64, 64, 12, 32, None, buf, None) == 3
    assert L.umi_full_me_u8(buf, buf, 64, 64, 16, 65, None, buf, None) == 3
    assert b"search range" in L.umi_last_error_string()


def test_iimg_workspace_contract(umi):
    L = umi.lib()
    n = L.umi_iimg_u8_i32_workspace_bytes(1080, 1920)
    assert 0 < n < 1080 * 1920  # small next to the frame
    assert L.umi_iimg_u8_i32_workspace_bytes(0, 5) == 0
    buf = ctypes.create_string_buffer(64)
    # too small a workspace is reported before any launch
    ws = (ctypes.c_char * 32).from_buffer(buf)
    p = ctypes.addressof(ws)
    p16 = (p + 15) & ~15
    assert L.umi_iimg_u8_i32(ctypes.c_void_p(p16), ctypes.c_void_p(p16), 1080, 1920, ctypes.c_void_p(p16), 16,
                             None) == 5
