"""Row-band split of one frame across ranks (one GPU per rank).

The rows of a frame (block rows for motion estimation) are divided into
contiguous bands, one per rank, as evenly as possible.  Each rank runs the
unchanged single-GPU operator on its band plus a halo of the rows that the
band's outputs read, so that every output equals the whole-frame result bit
for bit:

* full search (``me_band``): the halo is the search range rounded up to whole
  block rows, so the slice starts on a block row and its blocks are the
  frame's blocks shifted by whole rows; only the band's blocks are searched
  (``umi_full_me_u8_list``).  Reference rows are clamped only at the frame's
  own top and bottom: an interior slice holds every row its candidates read.
* 3x3 filter (``filter3x3_band``): a halo of one row; the slice's first and
  last rows are padded by the kernel, but they are not outputs.
* integral image (``iimg_band``): no halo and one exchange.  A band's integral
  image equals the integral image of its own rows plus, in every row, the sum
  of the last rows of the bands above it (an exclusive scan over ranks of one
  row each, made by ``all_gather``).  Frames are limited as for the
  whole-frame operator (sums within int32).

``gather_rows`` assembles the bands on every rank.  Nothing waits on another
rank inside a kernel: the only collectives are ``torch.distributed``
all_gather calls between launches.  Without an initialised process group
(or with ``group`` / ``world`` of one) every function works on the local
process alone, so several bands can be run one after another on one GPU.
"""
from __future__ import annotations

from dataclasses import dataclass

import umi_gb300 as U


def split(n: int, world: int, rank: int) -> tuple[int, int]:
    """Rows [lo, hi) of rank `rank` when n rows are split into `world` bands."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of {world}")
    return n * rank // world, n * (rank + 1) // world


@dataclass(frozen=True)
class MeBand:
    by0: int    # first block row of the band
    by1: int    # one past its last block row
    s0: int     # first pixel row of the slice (a multiple of the block size)
    s1: int     # one past its last pixel row
    first: int  # slice block index of the band's first block
    count: int  # blocks in the band


def me_band_plan(h: int, w: int, block: int, search: int, world: int, rank: int) -> MeBand:
    """The slice of rank `rank` for the full search of an h x w frame."""
    nby, nbx = h // block, w // block
    by0, by1 = split(nby, world, rank)
    halo = -(-search // block) * block
    s0 = max(0, by0 * block - halo)
    s1 = by1 * block + halo
    if s1 >= h or by1 == nby:  # the bottom band keeps the frame's last rows (partial block rows included)
        s1 = h
    return MeBand(by0, by1, s0, s1, (by0 - s0 // block) * nbx, (by1 - by0) * nbx)


def me_band(cur, ref, world: int, rank: int, block: int = 16, search: int = 32, stream=None):
    """Motion vectors (count, 3) int32 [dy, dx, sad] of the band's blocks, in
    raster order: rows by0 .. by1 - 1 of the whole frame's result."""
    import torch
    h, w = cur.shape
    pl = me_band_plan(h, w, block, search, world, rank)
    out_rows = ((pl.s1 - pl.s0) // block) * (w // block)
    if pl.count == 0:
        return torch.empty((0, 3), dtype=torch.int32, device=cur.device)
    blocks = torch.arange(pl.first, pl.first + pl.count, dtype=torch.int32, device=cur.device)
    n = torch.tensor([pl.count], dtype=torch.int32, device=cur.device)
    out = torch.empty((out_rows, 3), dtype=torch.int32, device=cur.device)
    U.full_me_u8_list(cur[pl.s0:pl.s1], ref[pl.s0:pl.s1], blocks, n, out, block=block, search=search, stream=stream)
    return out[pl.first:pl.first + pl.count]


def filter3x3_band(img, w9, world: int, rank: int, pad: float = 0.0, stream=None):
    """Rows [y0, y1) of the whole frame's 3x3 filter output (float32)."""
    h = img.shape[0]
    y0, y1 = split(h, world, rank)
    if y1 == y0:
        return img[0:0].clone()
    s0, s1 = max(0, y0 - 1), min(h, y1 + 1)
    out = U.filter3x3_f32(img[s0:s1], w9, pad, stream=stream)
    return out[y0 - s0:y1 - s0]


def iimg_band_local(img, world: int, rank: int, stream=None):
    """Integral image of the rank's own rows (no carry from the bands above).
    Frames the whole-frame operator refuses (sums that could exceed int32:
    more than 2^31 / 255 pixels) are refused here too."""
    import torch
    h, w = img.shape
    if h * w > (1 << 31) // 255:
        raise U.UmiError(U.UMI_ERR_UNSUPPORTED, "iimg_band", f"{h}x{w} frame: sums could exceed int32")
    y0, y1 = split(h, world, rank)
    if y1 == y0:
        return torch.empty((0, w), dtype=torch.int32, device=img.device)
    return U.iimg_u8_i32(img[y0:y1], stream=stream)


def band_totals(local):
    """The band's last integral-image row (its column totals), zeros for an empty band."""
    import torch
    if local.shape[0] == 0:
        return torch.zeros((local.shape[1],), dtype=torch.int32, device=local.device)
    return local[-1].clone()


def exchange_totals(totals, group=None) -> list:
    """Every rank's band totals, in rank order (all_gather; the local row
    alone without a process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size(group) == 1:
        return [totals]
    got = [torch.empty_like(totals) for _ in range(dist.get_world_size(group))]
    dist.all_gather(got, totals.contiguous(), group=group)
    return got


def add_carry(local, all_totals, rank: int):
    """local + (sum of the totals of ranks < rank) in every row, in place
    (int32; sums past int32 wrap, two's complement)."""
    import torch
    if rank > 0 and local.shape[0] > 0:
        carry = torch.stack(list(all_totals[:rank])).sum(0, dtype=torch.int64)
        carry = ((carry + 2 ** 31) % 2 ** 32 - 2 ** 31).to(torch.int32)  # two's-complement wrap
        local += carry
    return local


def iimg_band(img, world: int, rank: int, group=None, stream=None):
    """Rows [y0, y1) of the whole frame's integral image: the band's own
    integral image plus the exchanged totals of the bands above."""
    local = iimg_band_local(img, world, rank, stream=stream)
    return add_carry(local, exchange_totals(band_totals(local), group), rank)


def gather_rows(part, group=None):
    """The bands of all ranks stacked in rank order (all_gather of parts
    padded to the longest band), or `part` itself without a process group."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size(group) == 1:
        return part
    world = dist.get_world_size(group)
    n = torch.tensor([part.shape[0]], dtype=torch.int64, device=part.device)
    sizes = [torch.empty_like(n) for _ in range(world)]
    dist.all_gather(sizes, n, group=group)
    sizes = [int(s.item()) for s in sizes]
    mx = max(sizes)
    buf = torch.zeros((mx,) + tuple(part.shape[1:]), dtype=part.dtype, device=part.device)
    buf[:part.shape[0]] = part
    got = [torch.empty_like(buf) for _ in range(world)]
    dist.all_gather(got, buf, group=group)
    return torch.cat([g[:s] for g, s in zip(got, sizes)])
