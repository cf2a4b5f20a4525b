"""xrt_lbvh_build_noalloc: the LBVH build for callers that may not allocate GPU memory, such as
engines or plugin hosts that own the memory budget and forbid allocation after start-up.  Its
output must equal the allocating entry point's (xrt_lbvh_build + xrt_lbvh_export) bit for bit,
call after call, although every call reuses the same fixed device array.

This file is collected last on purpose: if it fails, a run that stops at the first failure has
already run every other test."""
import numpy as np
import pytest

from tests.helpers import bits, prim_soup

pytestmark = pytest.mark.gpu

MAX_PRIMS = 65536


def _allocating(prims, pred, scr):
    from xrtailor_gb300 import Lbvh
    b = Lbvh()
    b.build(prims, pred, scr)
    out = b.export()
    b.close()
    return out


def _noalloc(xrt, prims, pred, scr):
    import torch
    n = prims.shape[0]
    nn = 2 * n - 1
    dev = torch.device("cuda:0")
    d_prims = torch.from_numpy(np.ascontiguousarray(prims)).to(dev)
    d_pred = None if pred is None else torch.from_numpy(np.ascontiguousarray(pred)).to(dev)
    out = dict(morton=torch.empty(n, dtype=torch.int32, device=dev),
               objects=torch.empty(n, dtype=torch.int32, device=dev),
               nodes=torch.empty((nn, 4), dtype=torch.int32, device=dev),
               aabbs=torch.empty((nn, 6), dtype=torch.float32, device=dev),
               iesc=torch.empty(max(n - 1, 1), dtype=torch.int32, device=dev),
               eesc=torch.empty(n, dtype=torch.int32, device=dev))
    stream = torch.cuda.current_stream(dev)
    # one primitive has no internal node: the internal escape table may then be NULL
    iesc = None if n == 1 else out["iesc"].data_ptr()
    rc = xrt.xrt_lbvh_build_noalloc(
        d_prims.data_ptr(), None if d_pred is None else d_pred.data_ptr(), n, float(scr),
        out["morton"].data_ptr(), out["objects"].data_ptr(), out["nodes"].data_ptr(),
        out["aabbs"].data_ptr(), iesc, out["eesc"].data_ptr(), stream.cuda_stream)
    assert rc == 0, rc
    torch.cuda.synchronize(dev)
    h = {k: v.cpu().numpy() for k, v in out.items()}
    h["morton"] = h["morton"].view(np.uint32)
    h["objects"] = h["objects"].view(np.uint32)
    h["nodes"] = h["nodes"].view(np.uint32)
    h["iesc"] = h["iesc"][: max(n - 1, 0)]
    return h


def _same(a, b):
    for k in ("morton", "objects", "nodes", "iesc", "eesc"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    np.testing.assert_array_equal(bits(a["aabbs"]), bits(b["aabbs"]))


def test_noalloc_build_matches_allocating_build_on_consecutive_calls(xrt):
    rng = np.random.default_rng(41)
    big = prim_soup(6000, seed=41)
    big_pred = (big + rng.normal(0, 0.02, big.shape)).astype(np.float32)
    small = prim_soup(1500, seed=42)
    dup = np.concatenate([small[:400], small[:400]])  # equal Morton codes (64-bit keys)
    cases = [(big, big_pred, 0.001), (small, None, 0.0), (dup, None, 0.0), (big, big_pred, 0.001)]
    first = None
    for prims, pred, scr in cases:  # consecutive calls share the fixed array
        got = _noalloc(xrt, prims, pred, scr)
        _same(got, _allocating(prims, pred, scr))
        if first is None:
            first = got
    _same(got, first)  # the last call repeats the first input


def test_noalloc_build_at_the_limit_and_at_one_primitive(xrt):
    # the largest accepted input fills the fixed layout (32 radix tiles of the histogram); one
    # primitive has a single leaf and no internal node; the two calls in a row share the array
    rng = np.random.default_rng(43)
    full = prim_soup(MAX_PRIMS, seed=43)
    full_pred = (full + rng.normal(0, 0.01, full.shape)).astype(np.float32)
    one = prim_soup(1, seed=44)
    for prims, pred, scr in ((full, full_pred, 0.002), (one, None, 0.0), (full, full_pred, 0.002)):
        _same(_noalloc(xrt, prims, pred, scr), _allocating(prims, pred, scr))


def test_noalloc_build_rejects_more_than_the_limit(xrt):
    from xrtailor_gb300 import _lib
    import torch
    dev = torch.device("cuda:0")
    buf = torch.zeros(16, dtype=torch.float32, device=dev)
    p = buf.data_ptr()
    rc = xrt.xrt_lbvh_build_noalloc(p, None, MAX_PRIMS + 1, 0.0, p, p, p, p, p, p, None)
    assert rc == _lib.XRT_ERR_FACE_CAPACITY
    rc = xrt.xrt_lbvh_build_noalloc(None, None, 10, 0.0, p, p, p, p, p, p, None)
    assert rc == _lib.XRT_ERR_INVALID_ARGUMENT
