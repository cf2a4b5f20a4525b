"""Launch-configuration autotuner for the Swift step.

The two knobs that change the frame time without changing what the step computes (every
candidate is a valid coloring of the same constraints; results are then those of that coloring):
  * tile size of the tile-local Gauss-Seidel schedule (xrt_set_tile_vertices): small tiles keep
    more SMs busy when one garment is latency-bound, large tiles cut halo traffic and barriers
    per constraint when a batch of garments is throughput-bound;
  * programmatic dependent launch (xrt_set_dependent_launch).
The block size of the tile kernels (256 / 512 threads) and their one- or two-lane bend
projection follow from the tile schedule inside the library.

Each candidate is built by the caller's `make(tile_vertices)` (a started ClothSolver), stepped
`warmup` frames, then `frames` frames timed with CUDA events on the library's stream; the
fastest mean frame time wins.  For a batch, `make` can build a representative subset of its
instances (see `subset`), which is what the batched benchmark does.
"""
import numpy as np

DEFAULT_TILES = (256, 512, 1024, 2048)


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


def tune(make, tiles=DEFAULT_TILES, pdl=(True, False), frames=3, warmup=1, targets=None):
    """Returns ({"tile_vertices": t, "dependent_launch": d}, [(tile, pdl, ms_per_frame), ...])."""
    trials = []
    for t in tiles:
        s = make(t)
        for d in pdl:
            s.set_dependent_launch(d)
            time_frames(s, warmup, targets, first=0)
            ms = time_frames(s, frames, targets, first=warmup)
            trials.append((t, d, ms))
        s.close()
    t, d, _ = min(trials, key=lambda r: r[2])
    return {"tile_vertices": t, "dependent_launch": d}, trials


def subset(n_items, count):
    """`count` evenly spaced indices of `n_items` (all when count >= n_items)."""
    if count >= n_items:
        return list(range(n_items))
    return sorted(set(np.linspace(0, n_items - 1, count).round().astype(int).tolist()))
