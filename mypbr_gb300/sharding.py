"""Splitting one frame over ranks (one process per GPU).

Pixels and samples of camera::render (camera.h:95-139 of the reference) are
independent, so a frame shards two ways with no exchange while rendering:

* row bands: rank r renders rows [first, first + count) of the image
  (mypbr_render_opts.first_row / row_count); the bands are gathered once at the
  end. Random numbers are keyed by (pixel, pass), so a band renders exactly
  the pixels a full render would.
* sample shards: every rank renders the whole image with its own seed; the
  frames merge as an average weighted by their sample counts.
"""
import numpy as np


def row_band(rank, world, height):
    """(first_row, row_count) of rank's band: contiguous, sizes differing by at most one."""
    if not (0 <= rank < world) or height < 1:
        raise ValueError("bad rank / world / height")
    base, extra = divmod(height, world)
    first = rank * base + min(rank, extra)
    return first, base + (1 if rank < extra else 0)


def sample_seed(base_seed, rank):
    """An independent seed per rank for sample sharding."""
    return (int(base_seed) + 0x9E3779B97F4A7C15 * (rank + 1)) % (1 << 64)


def merge_sample_shards(means, spps):
    """Merges per-rank mean images rendered with independent seeds: the
    sample-weighted average, the mean a single render of sum(spps) samples
    estimates."""
    spps = np.asarray(spps, dtype=np.float64)
    acc = sum(m * s for m, s in zip(means, spps))
    return acc / spps.sum()


def assemble_row_bands(bands, world, height):
    """Stacks the bands of ranks 0..world-1 (each (count, W, ...)) into the image."""
    out = []
    for r in range(world):
        first, count = row_band(r, world, height)
        if bands[r].shape[0] != count:
            raise ValueError(f"band of rank {r} has {bands[r].shape[0]} rows, expected {count}")
        out.append(bands[r])
    return np.concatenate(out, axis=0)


def gather_row_bands(band, rank, world, height, group=None):
    """torch.distributed all_gather of row bands (padded to equal size) into the
    full image on every rank. band: numpy (count, W, C)."""
    import torch
    import torch.distributed as dist
    first, count = row_band(rank, world, height)
    rows = -(-height // world)
    w = band.shape[1:]
    buf = torch.zeros((rows,) + tuple(w), dtype=torch.float64)
    buf[:count] = torch.from_numpy(np.ascontiguousarray(band))
    parts = [torch.zeros_like(buf) for _ in range(world)]
    dist.all_gather(parts, buf, group=group)
    bands = [parts[r][:row_band(r, world, height)[1]].numpy() for r in range(world)]
    return assemble_row_bands(bands, world, height)
