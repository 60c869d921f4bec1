"""The batch case table on the host (no GPU): nr_batch_prepare issues no GPU
work, so its argument checks and step count run here, and the launching
calls refuse a table that nr_batch_prepare did not write before they touch
CUDA.  The workspaces are host buffers: prepare only carves pointers."""
import ctypes

import numpy as np
import pytest

from conftest import golden
from test_oracle_golden import geom_of


@pytest.fixture(scope="module")
def native(native_lib_path):
    from newrecon_gb300 import native

    native.load(native_lib_path)
    return native


def _aligned(nbytes, align=256):
    raw = np.zeros(nbytes + align, np.uint8)
    off = (-raw.ctypes.data) % align
    return raw, raw.ctypes.data + off


def make_cases(native, spec):
    """spec: (subset_num, n_iters, potential) per case, on the tiny geometry."""
    from newrecon_gb300.geometry import POTENTIALS, NrBatchCase, NrOstrParams

    g = geom_of(golden("tiny"))
    keep = []
    arr = (NrBatchCase * len(spec))()
    for k, (m, iters, pot) in enumerate(spec):
        p = NrOstrParams(m, POTENTIALS[pot], 0, 0, 1.0, 0.002)
        gc = g.to_c()
        size = ctypes.c_size_t(0)
        native.call("nr_ostr_workspace_size", ctypes.byref(gc), ctypes.byref(p), ctypes.byref(size))
        ws, ws_ptr = _aligned(int(size.value))
        x, x_ptr = _aligned(4 * g.n_voxels)
        keep += [ws, x]
        arr[k] = NrBatchCase(gc, p, iters, ctypes.c_void_p(x_ptr), ctypes.c_void_p(ws_ptr),
                             int(size.value))
    return arr, keep


def table_for(native, n):
    size = ctypes.c_size_t(0)
    native.call("nr_batch_table_size", n, ctypes.byref(size))
    return _aligned(int(size.value), 8), int(size.value)


def test_prepare_returns_the_longest_case(native):
    spec = [(3, 2, "lange"), (6, 3, "huber"), (2, 1, "hyperbola"), (6, 1, "q2"), (1, 4, "huber")]
    arr, keep = make_cases(native, spec)
    (buf, ptr), size = table_for(native, len(spec))
    steps = ctypes.c_int32(0)
    native.call("nr_batch_prepare", arr, len(spec), ctypes.c_void_p(ptr), size,
                ctypes.byref(steps), None)
    assert steps.value == max(m * it for m, it, _ in spec)


def test_prepare_rejects_bad_cases(native):
    from newrecon_gb300.native import NrError

    arr, keep = make_cases(native, [(3, 2, "lange"), (6, 1, "huber")])
    (buf, ptr), size = table_for(native, 2)
    steps = ctypes.c_int32(0)
    for n in (0, 65):
        with pytest.raises(NrError) as e:
            native.call("nr_batch_prepare", arr, n, ctypes.c_void_p(ptr), size,
                        ctypes.byref(steps), None)
        assert e.value.code == 2
    with pytest.raises(NrError) as e:  # table too small
        native.call("nr_batch_prepare", arr, 2, ctypes.c_void_p(ptr), size - 8,
                    ctypes.byref(steps), None)
    assert e.value.code == 6
    with pytest.raises(NrError) as e:  # table misaligned
        native.call("nr_batch_prepare", arr, 2, ctypes.c_void_p(ptr + 4), size,
                    ctypes.byref(steps), None)
    assert e.value.code == 6
    arr[1].p.potential = 7  # unknown potential
    with pytest.raises(NrError) as e:
        native.call("nr_batch_prepare", arr, 2, ctypes.c_void_p(ptr), size, ctypes.byref(steps),
                    None)
    assert e.value.code == 2
    arr[1].p.potential = 3
    arr[1].n_iters = -1
    with pytest.raises(NrError) as e:
        native.call("nr_batch_prepare", arr, 2, ctypes.c_void_p(ptr), size, ctypes.byref(steps),
                    None)
    assert e.value.code == 2
    arr[1].n_iters = 1
    arr[1].p.upd_planes = 12  # not a slab depth the update is built for
    with pytest.raises(NrError) as e:
        native.call("nr_batch_prepare", arr, 2, ctypes.c_void_p(ptr), size, ctypes.byref(steps),
                    None)
    assert e.value.code == 2
    arr[1].p.upd_planes = 32
    arr[1].p.upd_tile = 3  # not an update tile
    with pytest.raises(NrError) as e:
        native.call("nr_batch_prepare", arr, 2, ctypes.c_void_p(ptr), size, ctypes.byref(steps),
                    None)
    assert e.value.code == 2
    arr[1].p.upd_tile = 1
    native.call("nr_batch_prepare", arr, 2, ctypes.c_void_p(ptr), size, ctypes.byref(steps), None)
    arr[1].ws_bytes -= 256  # workspace too small for its geometry
    with pytest.raises(NrError) as e:
        native.call("nr_batch_prepare", arr, 2, ctypes.c_void_p(ptr), size, ctypes.byref(steps),
                    None)
    assert e.value.code == 6


def test_launching_calls_refuse_foreign_tables(native):
    """A zeroed or misaligned table is refused before any CUDA call (so this
    runs without a GPU)."""
    from newrecon_gb300.native import NrError

    (buf, ptr), size = table_for(native, 4)
    graph = ctypes.c_void_p(0)
    calls = [
        ("nr_batch_step", (ctypes.c_void_p(ptr), 0, None)),
        ("nr_batch_finish", (ctypes.c_void_p(ptr), None)),
        ("nr_batch_graph_create", (ctypes.c_void_p(ptr), 1, ctypes.c_void_p(1),
                                   ctypes.byref(graph))),
    ]
    for name, args in calls:
        with pytest.raises(NrError) as e:
            native.call(name, *args)
        assert e.value.code == 2, name
    with pytest.raises(NrError):
        native.call("nr_batch_step", ctypes.c_void_p(ptr + 4), 0, None)
    # a real table with its case permutation broken is refused too
    arr, keep = make_cases(native, [(3, 2, "lange"), (6, 1, "huber")])
    steps = ctypes.c_int32(0)
    native.call("nr_batch_prepare", arr, 2, ctypes.c_void_p(ptr), size, ctypes.byref(steps), None)
    before = buf.copy()
    words = np.frombuffer(buf, np.int32, count=size // 4, offset=ptr - buf.ctypes.data)
    n_idx = 0
    assert words[n_idx] == 2
    words[n_idx] = 70  # more cases than the table can hold
    with pytest.raises(NrError) as e:
        native.call("nr_batch_step", ctypes.c_void_p(ptr), 0, None)
    assert e.value.code == 2
    buf[:] = before


def test_batch_mode_choice():
    """"auto" runs cases that each fill the GPU (2^26 voxels or more) one after
    another and smaller ones by shared launches; explicit modes are kept."""
    from newrecon_gb300.ostr import Batch

    big, small = Batch.SEQUENTIAL_VOXELS, Batch.SEQUENTIAL_VOXELS - 1
    assert Batch.choose_mode([2048 * 1024 * 70] * 4) == "sequential"
    assert Batch.choose_mode([big, big]) == "sequential"
    assert Batch.choose_mode([big, small]) == "shared"
    assert Batch.choose_mode([1024 * 512 * 60]) == "shared"
    assert Batch.choose_mode([big], "shared") == "shared"
    assert Batch.choose_mode([small], "sequential") == "sequential"
    with pytest.raises(ValueError):
        Batch.choose_mode([big], "persistent")
