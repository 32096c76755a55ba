"""prtcl_gpu_field_upload_noalloc against prtcl_gpu_field_upload.

Both entry points must leave the same device contents (compared bit for bit
after a download), on two calls in a row, with the second call smaller than
the first (vectors and matrices alike) so that bytes the first call left in
the fixed staging array would show up if they were read.  Counts above the
staging limit are refused and leave the field unchanged; so is a call on a
stream that is being captured into a CUDA graph.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STAGE_BYTES = 8 << 20


def _upload_noalloc(model, group, field, a):
    from prtcl_gb300._lib import check, load
    n = model.get_group(group).item_count
    check(load().prtcl_gpu_field_upload_noalloc(model._h, group.encode(), field.encode(), a.ctypes.data, n, None))


def _model():
    from prtcl_gb300.core import Model
    m = Model()
    g = m.add_group("f", "fluid")
    for suffix in ("a", "b"):
        g.varying.add_field("x_" + suffix, "f32", (3,))
        g.varying.add_field("m_" + suffix, "f32", (3, 3))
        g.varying.add_field("s_" + suffix, "f32", ())
        g.varying.add_field("i_" + suffix, "i32", ())
    return m, g


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.mark.parametrize("first,second", [(600_000, 350_000)])
def test_noalloc_upload_matches_upload(gpu_lib, first, second):
    m, g = _model()
    rng = np.random.default_rng(7)
    for call, n in enumerate((first, second)):
        g.resize(n)
        # a matrix field of n items needs 36 n staging bytes: keep it inside,
        # and make the second matrix call smaller than the first as well
        nm = min(n, STAGE_BYTES // 36) // (1 + call)
        x = rng.standard_normal((n, 3)).astype(np.float32)
        mat = rng.standard_normal((n, 9)).astype(np.float32)
        s = rng.standard_normal(n).astype(np.float32)
        ints = rng.integers(-2**31, 2**31 - 1, n, dtype=np.int64).astype(np.int32)
        f = g.varying
        f.get_field("x_a").upload(x)
        _upload_noalloc(m, "f", "x_b", x)
        f.get_field("s_a").upload(s)
        _upload_noalloc(m, "f", "s_b", s)
        f.get_field("i_a").upload(ints)
        _upload_noalloc(m, "f", "i_b", ints)
        for name in ("x", "s", "i"):
            a = f.get_field(name + "_a").download()
            bb = f.get_field(name + "_b").download()
            assert np.array_equal(_bits(a), _bits(bb)), (call, name)
        np.testing.assert_array_equal(_bits(f.get_field("x_b").download()), _bits(x))
        # matrices, on a group small enough for the staging array
        g.resize(nm)
        f.get_field("m_a").upload(mat[:nm])
        _upload_noalloc(m, "f", "m_b", mat[:nm])
        a = f.get_field("m_a").download()
        bb = f.get_field("m_b").download()
        assert np.array_equal(_bits(a), _bits(bb)), (call, "m")
        np.testing.assert_array_equal(_bits(bb), _bits(mat[:nm]))


def test_noalloc_upload_limit(gpu_lib):
    from prtcl_gb300 import PrtclGpuError
    m, g = _model()
    n = STAGE_BYTES // 12 + 1   # one vector item more than the array holds
    g.resize(n)
    x = np.ones((n, 3), np.float32)
    g.varying.get_field("x_a").upload(np.zeros((n, 3), np.float32))
    with pytest.raises(PrtclGpuError, match="no-alloc upload"):
        _upload_noalloc(m, "f", "x_a", x)
    assert not g.varying.get_field("x_a").download().any()
    # scalar fields are copied without staging: no limit applies
    s = np.arange(n, dtype=np.float32)
    _upload_noalloc(m, "f", "s_a", s)
    np.testing.assert_array_equal(g.varying.get_field("s_a").download(), s)
    # a count that does not match the group is an error, as for the ordinary upload
    from prtcl_gb300._lib import load
    rc = load().prtcl_gpu_field_upload_noalloc(m._h, b"f", b"s_a", s.ctypes.data, n - 1, None)
    assert rc != 0


def test_noalloc_upload_refused_under_capture(gpu_lib):
    """The call synchronises its stream, which a capture forbids: it returns
    an error before touching the stream, and the field keeps its values."""
    import torch
    from prtcl_gb300._lib import load
    m, g = _model()
    g.resize(1000)
    x = np.ones((1000, 3), np.float32)
    g.varying.get_field("x_a").upload(np.zeros((1000, 3), np.float32))
    s = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=s, capture_error_mode="relaxed"):
        rc = load().prtcl_gpu_field_upload_noalloc(m._h, b"f", b"x_a", x.ctypes.data, 1000,
                                                   C.c_void_p(s.cuda_stream))
    assert rc != 0
    assert "captured" in load().prtcl_gpu_last_error().decode()
    assert not g.varying.get_field("x_a").download().any()
