"""Launch-configuration autotuner for the Swift step.

The knobs that change the frame time without changing what the step computes (every candidate
is a valid coloring of the same constraints; results are then those of that coloring):
  * tile size of the tile-local Gauss-Seidel schedule (xrt_set_tile_vertices): small tiles keep
    more SMs busy when one garment is latency-bound, large tiles cut halo traffic and barriers
    per constraint when a batch of garments is throughput-bound;
  * programmatic dependent launch (xrt_set_dependent_launch);
  * threads per block of the per-vertex kernels (xrt_set_vertex_block), tuned at the chosen tile
    size and launch mode; results are identical for every value.
The block size of the tile kernels (256 / 512 threads) and their one- or two-lane bend
projection follow from the tile schedule inside the library.  The LBVH keeps one triangle per
leaf, as the reference builds it (BVH.cu:689-694): the candidate lists must equal the
reference's leaf-by-leaf traversal, so the leaf size is not a free knob here.

Each candidate is built by the caller's `make(tile_vertices)` (a started ClothSolver), stepped
`warmup` frames, then `frames` frames timed with CUDA events on the library's stream; the
fastest mean frame time wins.  For a batch, `make` can build a representative subset of its
instances (see `subset`), which is what the batched benchmark does.
"""
import numpy as np

DEFAULT_TILES = (256, 512, 768, 1024, 2048)
DEFAULT_VERTEX_BLOCKS = (64, 128, 256)


def time_frames(solver, frames, targets=None, first=0):
    """Mean device time of `frames` frames (ms); `targets(k)` -> device pointer or None."""
    import torch
    _, _, sp = solver.device_state()
    dev = torch.device("cuda", solver.device)
    stream = torch.cuda.ExternalStream(sp, device=dev)
    lib = solver._lib
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(frames)]
    torch.cuda.synchronize(dev)
    with torch.cuda.stream(stream):
        for k, (a, b) in enumerate(ev):
            if targets is not None:
                ptr = targets(first + k)
                if ptr is not None:
                    lib.xrt_set_obstacle_targets_device(solver._h, ptr)
            a.record(stream)
            solver.step()
            b.record(stream)
    torch.cuda.synchronize(dev)
    solver.synchronize()
    return sum(a.elapsed_time(b) for a, b in ev) / frames


def tune(make, tiles=DEFAULT_TILES, pdl=(True, False), frames=3, warmup=1, targets=None,
         vertex_blocks=DEFAULT_VERTEX_BLOCKS):
    """Returns ({"tile_vertices": t, "dependent_launch": d, "vertex_block": b},
    [(tile, pdl, vertex block, ms_per_frame), ...]).  Tile size and launch mode are tuned at the
    default vertex block (128), then the vertex block at the chosen pair."""
    trials = []
    for t in tiles:
        s = make(t)
        for d in pdl:
            s.set_dependent_launch(d)
            time_frames(s, warmup, targets, first=0)
            ms = time_frames(s, frames, targets, first=warmup)
            trials.append((t, d, 128, ms))
        s.close()
    t, d, _, _ = min(trials, key=lambda r: r[3])
    s = make(t)
    s.set_dependent_launch(d)
    for b in vertex_blocks:
        if b == 128:
            continue
        s.set_vertex_block(b)
        time_frames(s, warmup, targets, first=0)
        trials.append((t, d, b, time_frames(s, frames, targets, first=warmup)))
    s.close()
    best = min((r for r in trials if r[0] == t and r[1] == d), key=lambda r: r[3])
    return {"tile_vertices": t, "dependent_launch": d, "vertex_block": best[2]}, trials


def subset(n_items, count):
    """`count` evenly spaced indices of `n_items` (all when count >= n_items)."""
    if count >= n_items:
        return list(range(n_items))
    return sorted(set(np.linspace(0, n_items - 1, count).round().astype(int).tolist()))
