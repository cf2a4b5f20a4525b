"""Generates the golden fixtures of the CPU oracle (tests/golden/*.npz).

    python -m tests.golden.make_golden

Each case is a small seeded input; the fixture records the oracle's output so that any change to
the oracle's arithmetic or ordering shows up as a test failure (test_oracle_cpu.py).  Keys starting
with "approx_" hold results that go through the host's acosf (bend rest angles and frames with
bending) and are compared with an absolute tolerance of 1e-5; everything else bit for bit.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle import oracle as orc  # noqa: E402
from xrtailor_gb300 import scenes  # noqa: E402


def _soup(n, seed, size=0.05, flat=None):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-1, 1, size=(n, 1, 3))
    p = c + rng.normal(0, size, size=(n, 3, 3))
    if flat is not None:
        p[:, :, flat] = 0.0
    return p.astype(np.float32).reshape(n, 9)


def lbvh_soup():
    b = orc.OracleLbvh()
    p = _soup(700, 21)
    b.build(p, scr=0.001)
    t = b.export()
    rng = np.random.default_rng(22)
    q = rng.uniform(-1, 1, size=(64, 3)).astype(np.float32)
    cnt, cand = b.query(0, q)
    segs = np.concatenate([q, q + 0.2], 1).astype(np.float32)
    scnt, scand = b.query(1, segs)
    pred = (p + rng.normal(0, 0.02, p.shape)).astype(np.float32)
    b.refit(pred)
    r = b.export()
    return dict(morton=t["morton"], objects=t["objects"], nodes=t["nodes"], aabbs=t["aabbs"],
                iesc=t["iesc"], eesc=t["eesc"], pcount=cnt, pcand=cand[:, :8], scount=scnt,
                scand=scand[:, :8], refit_aabbs=r["aabbs"])


def lbvh_duplicates():
    b = orc.OracleLbvh()
    base = _soup(120, 23)
    b.build(np.concatenate([base, base]), scr=0.0)
    t = b.export()
    return dict(morton=t["morton"], objects=t["objects"], nodes=t["nodes"], iesc=t["iesc"],
                eesc=t["eesc"], unique=np.array([t["unique"]], np.int32))


def _frame_case(bending):
    cloth = scenes.grid_cloth(12, 1.0, origin=(0.0, 0.35, 0.0), jitter=1e-3, seed=5)
    cloth.fixed_indices = scenes.two_corner_pins(12)
    cloth.attached_indices = scenes.two_corner_pins(12)
    sphere = scenes.icosphere(2, 0.3, center=(0.5, 0.0, 0.5))
    p = scenes._params(num_substeps=3, num_iterations=4, stretch_compliance=1e-8,
                       bend_compliance=1e-6, num_collision_passes=3, solve_bending=int(bending),
                       long_range_stretchiness=1.05)
    o = orc.OracleSolver(p)
    o.add_cloth(cloth, particle_diameter=0.03)
    o.add_obstacle(sphere)
    o.start()
    for _ in range(6):
        o.step()
    c = o.export_contacts()
    pre = "approx_" if bending else ""
    out = {pre + "positions": o.host_positions(), pre + "velocities": o.host_velocities(),
           "edges": o.edges()[0], "rtri": o.obstacle_rtri(), "colors0": o.coloring(0)}
    if not bending:
        out.update(vf_index=c["vf_index"], rt_index=c["rt_index"], ee=c["ee"],
                   neighbors=o.export_neighbors()[:4096])
    else:
        b, th = o.bends()
        out.update(bends=b, approx_theta=th, colors1=o.coloring(1))
    return out


def frame_no_bending():
    return _frame_case(False)


def frame_bending():
    return _frame_case(True)


CASES = {"lbvh_soup": lbvh_soup, "lbvh_duplicates": lbvh_duplicates,
         "frame_no_bending": frame_no_bending, "frame_bending": frame_bending}


def main():
    for name, fn in CASES.items():
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **fn())
        print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
