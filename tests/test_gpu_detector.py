"""Detector projection (mcd_project_detector, projOnDetector of
MC/tools/rotation.py:78-102) against the reference's own outputs and the
oracle: FP64 to 1e-9 um, FP32 to 2e-3 um (the outputs are ~5600 um, whose
float32 spacing is 4.9e-4 um); ragged and unaligned sizes take the scalar
path; empty input launches nothing."""
import numpy as np
import pytest
import torch

import mcd_oracle as O
from mcd import _lib, detector, engine
from _gpu_util import input_par

pytestmark = pytest.mark.gpu


def planes(d, dtype):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(d, dtype=np.float64).T)).to("cuda", dtype)


def test_reference_vectors_fp64(golden):
    P = golden["physics"]
    d = P["det/dirs"]
    for a in P["det/alphas"]:
        ref = P["det/xy/%g" % a]
        got = detector.project(planes(d, torch.float64), a, P["det/xy_PC"], float(P["det/L"])).cpu().numpy().T
        assert np.max(np.abs(got - ref)) <= 1e-9, a


def test_reference_signature(golden):
    P = golden["physics"]
    d = P["det/dirs"]
    a = float(P["det/alphas"][0])
    res = detector.projOnDetector(list(d), a, P["det/xy_PC"], float(P["det/L"]))
    assert isinstance(res, list) and len(res) == len(d) and res[0].shape == (2,)
    assert np.max(np.abs(np.array(res) - P["det/xy/%g" % a])) <= 1e-9
    # the module's default geometry is the reference's (parameters.py:22-33)
    assert a == detector.ALPHA
    assert np.allclose(P["det/xy_PC"], detector.XY_PC, rtol=0, atol=0)
    assert float(P["det/L"]) == detector.L


@pytest.mark.parametrize("n", [1, 3, 5, 64, 1000, (1 << 20) + 3])
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_sizes_and_precisions(n, dtype):
    rng = np.random.default_rng(n)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    ref = O.proj_on_detector(d, 20.0, detector.XY_PC, detector.L)
    got = detector.project(planes(d, dtype)).cpu().numpy().astype(np.float64).T
    tol = 1e-9 if dtype == torch.float64 else 2e-3
    assert np.max(np.abs(got - ref)) <= tol


def test_unaligned_planes_and_empty_input():
    rng = np.random.default_rng(3)
    d = rng.normal(size=(4099, 3))
    buf = torch.zeros(3 * 4099 + 1, dtype=torch.float32, device="cuda")
    view = buf[1:].view(3, 4099)                    # base 4 bytes past a 16-byte boundary
    view.copy_(planes(d, torch.float32))
    out = torch.zeros(2 * 4099 + 1, dtype=torch.float32, device="cuda")[1:].view(2, 4099)
    detector.project(view, out=out)
    ref = O.proj_on_detector(d.astype(np.float32).astype(np.float64), 20.0, detector.XY_PC, detector.L)
    assert np.max(np.abs(out.cpu().numpy().astype(np.float64).T - ref)) <= 2e-3
    empty = torch.zeros((3, 0), dtype=torch.float32, device="cuda")
    assert detector.project(empty).shape == (2, 0)
    L = _lib.lib()
    assert L.mcd_project_detector(None, -1, _lib.FP32, 20.0, 0.0, 0.0, 0.0, None, None) == _lib.EINVAL
    assert L.mcd_project_detector(None, 4, 7, 20.0, 0.0, 0.0, 0.0, None, None) == _lib.EINVAL


def test_projects_transport_output():
    """Exit directions of backscattered electrons straight from the transport
    buffers, projected without leaving the GPU."""
    p = input_par("Si", 20000.0, 1000.0, 70.0)
    n = 20000
    sim = engine.make_sim(p, n, seed=4)
    mat = _lib.material("Si")
    from mcd.tables import ds_tables
    tabs = ds_tables(mat, p["E0"], p["Emin"], p["Wc"], p["tol_E"], p["tol_W"])
    bufs = engine.RunBuffers(n, _lib.FP32, True, 0)
    bufs.zero()
    engine.launch(sim, mat, tabs, bufs)
    dirs = bufs.el["dir"].view(3, n)
    xy = detector.project(dirs).cpu().numpy().T
    d = dirs.cpu().numpy().T.astype(np.float64)
    ref = O.proj_on_detector(d, detector.ALPHA, detector.XY_PC, detector.L)
    assert np.max(np.abs(xy - ref)) <= 2e-3
    bks = bufs.el["outcome"].cpu().numpy() == _lib.OUT_BKS
    assert bks.sum() > 0.2 * n
