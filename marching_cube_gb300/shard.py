"""Host-side split of one extraction over several devices or processes.

A volume's cubes are cut into z-slabs at multiples of the brick depth (8);
each rank runs the slab extraction (extract_slab / mcg_mc_extract_slab) on
its slab, and the ranks exchange one number each -- their vertex totals --
to place their soups in the whole volume's soup: rank r's soup starts at the
sum of the totals of ranks 0..r-1.  Concatenated in rank order the slabs'
soups are the whole volume's soup.
"""
import torch

BRICK_DEPTH = 8


def slab_bounds(nz, parts):
    """[(z0, z1)] for `parts` slabs covering the cube layers 0 <= z < nz - 1,
    every z0 a multiple of BRICK_DEPTH; slabs differ by at most one brick
    layer (trailing slabs may be empty, (z, z))."""
    layers = max(nz - 1, 0)
    bricks = (layers + BRICK_DEPTH - 1) // BRICK_DEPTH
    out = []
    b0 = 0
    for r in range(parts):
        nb = bricks // parts + (1 if r < bricks % parts else 0)
        z0 = min(b0 * BRICK_DEPTH, layers)
        z1 = min((b0 + nb) * BRICK_DEPTH, layers)
        out.append((z0, z1))
        b0 += nb
    return out


def exchange_offsets(local_vertices, group=None):
    """One all-gather of the per-rank vertex totals: returns (offset, total)
    of this rank's soup in the whole soup."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    mine = torch.tensor([int(local_vertices)], dtype=torch.int64)
    if dist.get_backend(group) == "nccl":
        mine = mine.cuda()
    every = [torch.zeros_like(mine) for _ in range(world)]
    dist.all_gather(every, mine, group=group)
    counts = [int(t.item()) for t in every]
    return sum(counts[:rank]), sum(counts)
