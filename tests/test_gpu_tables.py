"""GPU FP64 table fill against the oracle's FP64 fill and the reference's
stored float32 tables (tests/golden/tables.npz)."""
import numpy as np
import pytest

import mcd_oracle as O
from mcd import _lib, tables

from _gpu_util import GOLDEN_TABLES

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", list(GOLDEN_TABLES))
@pytest.mark.parametrize("kind", ["Moller", "Gryz"])
def test_table_fill(golden, name, kind):
    T = golden["tables"]
    key = name + "/" + kind
    sp = str(T[key + "/species"])
    m = _lib.material(sp)
    dt = tables.DeviceTable(kind, m, T[key + "/Ws"], T[key + "/Es"], "cuda", keep_fp64=True)
    cdf32 = dt.cdf.cpu().numpy()
    cdf64 = dt.cdf64.cpu().numpy()
    nvalid = dt.nvalid.cpu().numpy()
    # unmasked counts: exact, against the reference
    assert np.array_equal(nvalid, T[key + "/nvalid"])
    assert np.array_equal((cdf32 != 0).sum(axis=1), nvalid)
    # FP64 values against the oracle's FP64 fill (sequential cumsum)
    ocdf, valid = O.table_cdf(kind, O.Material(sp), T[key + "/Ws"], T[key + "/Es"])
    v = valid
    assert np.max(np.abs(cdf64[v] - ocdf[v])) < 1e-13
    assert np.all(cdf32[~v] == 0) and np.all(cdf64[~v] == 0)
    # float32 table: the oracle's rounding almost everywhere, the reference's within one step
    o32 = O.table_store32(ocdf, valid)
    assert np.mean(cdf32 != o32) < 1e-4
    rows = T[key + "/rows"]
    d = np.abs(cdf32[rows].astype(np.float64) - T[key + "/cdf_rows"].astype(np.float64))
    assert d.max() <= 2.0 ** -24 + 1e-12
    assert np.max(np.abs(cdf32.astype(np.float64).sum(axis=1) - T[key + "/rowsum"])) < 1e-5
    # every valid row ends at exactly 1
    last = cdf32[np.arange(cdf32.shape[0]), np.maximum(nvalid - 1, 0)]
    assert np.all(last[nvalid > 0] == 1.0)
