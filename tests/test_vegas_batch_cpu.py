"""Host-side checks of the batched VEGAS C ABI (tq_vegas_batch_table_size):
the item validation runs on the host before anything touches a device, so
these run without a GPU.  The pointers are placeholders that are never
dereferenced (nothing here launches or copies)."""
import ctypes

import pytest

from torchquad_gb300 import _lib as L

FAKE = 0x1000  # a non-null placeholder address


def _item(dim=3, dtype=L.TQ_F64, n_bins=50, n_strat=4, family=L.TQ_FN_GAUSSIAN, ws_bytes=1 << 30,
          warm=100, expected=1000):
    it = L.VegasItem()
    st = it.st
    st.dim, st.dtype, st.n_bins, st.n_strat = dim, dtype, n_bins, n_strat
    st.n_cubes = n_strat**dim
    for name in ("x_edges", "dx_edges", "weights", "counts", "dh", "jf", "jf2", "neval", "cube_start",
                 "rng_offset", "stats", "flags", "scalars", "domain", "control"):
        setattr(st, name, FAKE)
    st.n_stat_slots = 30
    it.params, it.workspace, it.workspace_bytes = FAKE, FAKE, ws_bytes
    it.warm_samples, it.expected_points = warm, expected
    it.family, it.use_grid_improve, it.use_warmup = family, 1, 1
    return it


def _size(*items):
    arr = (L.VegasItem * len(items))(*items)
    return L.lib().tq_vegas_batch_table_size(arr, len(items))


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import torchquad_gb300.build as B

    B.build()
    L.load(B.lib_path())


def test_valid_batch_has_a_table():
    a = _size(_item(), _item(dim=5, n_bins=1024, family=L.TQ_FN_OSCILLATORY))
    b = _size(_item())
    assert a > b > 0


@pytest.mark.parametrize("bad", [
    dict(n_bins=1025),                      # maps of at most 1024 intervals
    dict(family=7),                         # unknown integrand family
    dict(dim=0),                            # dimension out of range
    dict(dim=L.TQ_MAX_DIM + 1),
    dict(ws_bytes=16),                      # workspace smaller than tq_vegas_workspace_size
    dict(warm=-1),
])
def test_invalid_items_are_rejected(bad):
    assert _size(_item(), _item(**bad)) == 0


def test_mixed_dtypes_are_rejected():
    assert _size(_item(dtype=L.TQ_F64), _item(dtype=L.TQ_F32)) == 0


def test_inconsistent_cube_count_is_rejected():
    it = _item()
    it.st.n_cubes += 1
    assert _size(it) == 0


def test_empty_batch_is_rejected():
    assert L.lib().tq_vegas_batch_table_size(ctypes.cast(None, ctypes.POINTER(L.VegasItem)), 0) == 0
