"""C-ABI checks that need no GPU: the library loads, exports every declared entry point, the
ctypes structs match the C layout, and product entry points fail loudly without a device."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "xrt.h")


def declared_symbols():
    import glob
    syms = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        syms |= set(re.findall(r"^(?:xrt_status|const char\*)\s+(xrt_[a-z0-9_]+)\s*\(", text,
                               flags=re.M))
    return sorted(syms)


def test_every_declared_symbol_is_exported(xrt):
    syms = declared_symbols()
    assert len(syms) >= 40
    missing = [s for s in syms if not hasattr(xrt, s)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", os.path.join(ROOT, "xrtailor_gb300", "libxrt.so")],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (xrt_[a-z0-9_]+)", out))
    assert set(syms) <= exported


def test_ctypes_bindings_cover_header(xrt):
    from xrtailor_gb300 import _lib
    assert sorted(_lib.SIGNATURES) == declared_symbols()


def test_struct_layouts_match_c(xrt):
    from xrtailor_gb300 import _lib
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "xrt.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu\n", sizeof(xrt_swift_params), sizeof(xrt_cloth_desc),
         sizeof(xrt_obstacle_desc), sizeof(xrt_sizes), offsetof(xrt_swift_params, frame_time),
         offsetof(xrt_cloth_desc, particle_diameter));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        vals = [int(v) for v in subprocess.run([exe], capture_output=True, text=True,
                                               check=True).stdout.split()]
    assert vals == [C.sizeof(_lib.SwiftParams), C.sizeof(_lib.ClothDesc), C.sizeof(_lib.ObstacleDesc),
                    C.sizeof(_lib.Sizes), _lib.SwiftParams.frame_time.offset,
                    _lib.ClothDesc.particle_diameter.offset]


def test_default_params_are_the_reference_effective_defaults(xrt):
    from xrtailor_gb300 import _lib
    p = _lib.SwiftParams()
    assert xrt.xrt_default_params(C.byref(p)) == 0
    assert (p.num_substeps, p.num_iterations, p.max_neighbor_size, p.inter_leaved_hash) == (1, 200, 64, 3)
    assert p.relaxation_factor == pytest.approx(0.25)      # SimParams default, config key ignored
    assert p.geodesic_lra == 1                              # SimParams default, config key ignored
    assert p.bvh_tolerance == pytest.approx(0.003)          # SwiftModeCollisionSettings default
    assert p.bend_compliance == pytest.approx(100.0)
    assert p.long_range_stretchiness == pytest.approx(1.1)
    assert p.frame_time == pytest.approx(1.0 / 60.0)
    v = C.c_int32()
    assert xrt.xrt_get_version(C.byref(v)) == 0 and v.value == 1


def test_oracle_defaults_equal_the_library_defaults(xrt, oracle_lib):
    """The oracle restates the defaults itself (CPU runs load nothing from libxrt.so); both
    restatements must agree field for field, bit for bit."""
    from oracle.oracle import default_fem_material, default_params
    from xrtailor_gb300 import _lib
    a, b = _lib.SwiftParams(), default_params()
    assert xrt.xrt_default_params(C.byref(a)) == 0
    assert bytes(a) == bytes(b)
    m = _lib.FemMaterial()
    assert xrt.xrt_default_fem_material(C.byref(m)) == 0
    assert bytes(m) == bytes(default_fem_material())


def _gpu_present():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_gpu_present(), reason="checks the no-device path")
def test_create_fails_loudly_without_device(xrt):
    from xrtailor_gb300 import _lib
    h = C.c_void_p()
    assert xrt.xrt_create(C.byref(h), 0) == _lib.XRT_ERR_NO_DEVICE
    assert not h.value
    b = C.c_void_p()
    assert xrt.xrt_lbvh_create(C.byref(b), 0) == _lib.XRT_ERR_NO_DEVICE
    from xrtailor_gb300 import ClothSolver, XrtError
    with pytest.raises(XrtError):
        ClothSolver()


def test_null_arguments_are_rejected(xrt):
    from xrtailor_gb300 import _lib
    assert xrt.xrt_default_params(None) == _lib.XRT_ERR_INVALID_ARGUMENT
    assert xrt.xrt_create(None, 0) == _lib.XRT_ERR_INVALID_ARGUMENT
    assert xrt.xrt_step_frame(None) == _lib.XRT_ERR_INVALID_ARGUMENT
    assert xrt.xrt_set_params(None, None) == _lib.XRT_ERR_INVALID_ARGUMENT
    assert xrt.xrt_destroy(None) == 0
