"""Frame cache (include/xrt_cache.h): every recorded frame equals the state read right after
that frame, bit for bit, while the copies overlap the following frames; the OBJ export writes
the reference's format (ObjSequenceExporter.cpp:21-46)."""
import numpy as np
import pytest

from tests.helpers import bits
from xrtailor_gb300 import ClothSolver, XrtError, scenes

pytestmark = pytest.mark.gpu


def _solver():
    sc = scenes.plain_small(24)
    s = ClothSolver(scenes.scene_params(sc, bend_compliance=100.0, num_substeps=4,
                                        num_iterations=4, num_collision_passes=4))
    s.add_cloth(sc.cloth, particle_diameter=sc.particle_diameter)
    s.add_obstacle(sc.obstacle)
    s.start()
    return s, sc


def test_cached_frames_equal_the_frames(xrt):
    s, sc = _solver()
    t, _ = _solver()
    s.cache_begin(5, cloth=True, obstacle=True, normals=True)
    want = []
    for f in range(7):                      # two past the capacity: not recorded
        s.step()
        t.step()
        want.append((t.host_positions(), t.host_normals(), t.obstacle_positions(),
                     t.obstacle_normals()))
    assert s.cache_count() == 5
    for f in range(5):
        got = s.cache_read(f)
        for k, w in zip(("cloth_positions", "cloth_normals", "obstacle_positions",
                         "obstacle_normals"), want[f]):
            np.testing.assert_array_equal(bits(got[k]), bits(w), err_msg=(f, k))
    # recording does not change the frames
    np.testing.assert_array_equal(bits(s.host_positions()), bits(t.host_positions()))
    s.cache_end()


def test_obj_export_format(xrt, tmp_path):
    s, sc = _solver()
    s.cache_begin(3, cloth=True, normals=True)
    s.step(3)
    s.cache_export_obj(str(tmp_path))
    tri = sc.cloth.triangles
    for f in range(3):
        fr = s.cache_read(f)
        lines = (tmp_path / f"{f:06d}.obj").read_text().splitlines()
        V = len(fr["cloth_positions"])
        assert lines[0] == "# Generated by XRTailor" and lines[1] == "o mesh"
        v = [ln for ln in lines if ln.startswith("v ")]
        vn = [ln for ln in lines if ln.startswith("vn ")]
        fc = [ln for ln in lines if ln.startswith("f ")]
        assert len(v) == V and len(vn) == V and len(fc) == len(tri) and "s 1" in lines
        assert v[7] == "v %.6f %.6f %.6f" % tuple(float(x) for x in fr["cloth_positions"][7])
        assert vn[3] == "vn %.6f %.6f %.6f" % tuple(float(x) for x in fr["cloth_normals"][3])
        assert fc[5] == "f %d %d %d" % tuple(int(i) + 1 for i in tri[5])
    with pytest.raises(XrtError):
        s.cache_export_obj(str(tmp_path), obstacle=True)   # the obstacle was not cached
    with pytest.raises(XrtError):
        s.cache_read(3)
